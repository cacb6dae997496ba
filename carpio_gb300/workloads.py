"""Seeded synthetic inputs with the shapes and value distributions of the
benchmarked workloads (no external data sets are involved)."""
import numpy as np

from .batch import DIRICHLET, NEUMANN, Problem


def gaussian_source(nx, ny, rng, n=8, box=((0.0, 0.0), (1.0, 1.0)),
                    widths=(0.02, 0.2)):
    """Sum of `n` Gaussians at the cell centres of a uniform nx x ny grid:
    centres uniform in the box, widths uniform in `widths`, amplitudes
    N(0, 1); the mean is removed so the all-Neumann problem is solvable."""
    (x0, y0), (x1, y1) = box
    xc = x0 + (np.arange(nx) + 0.5) * (x1 - x0) / nx
    yc = y0 + (np.arange(ny) + 0.5) * (y1 - y0) / ny
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    f = np.zeros((nx, ny))
    for _ in range(n):
        cx = rng.uniform(x0, x1)
        cy = rng.uniform(y0, y1)
        w = rng.uniform(*widths)
        a = rng.normal()
        f += a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * w * w))
    return f - f.mean()


def uneven_batch(count=512, sizes=tuple(range(32, 513, 16)), seed=0,
                 p_neumann=0.5):
    """The batched-Poisson workload: `count` square problems on [0,1]^2 with
    side N drawn uniformly from `sizes`, boundary all Dirichlet-0 or all
    Neumann-0 (mean removal) with probability p_neumann, source a zero-mean
    sum of 8 Gaussians. Returns (problems, sources)."""
    rng = np.random.default_rng(seed)
    problems, sources = [], []
    for _ in range(count):
        n = int(rng.choice(sizes))
        neumann = rng.random() < p_neumann
        bc = [(NEUMANN, 0.0)] * 4 if neumann else [(DIRICHLET, 0.0)] * 4
        problems.append(Problem(n, n, bc=bc))
        sources.append(gaussian_source(n, n, rng))
    return problems, sources
