"""Small fixed workloads of single kernels, for profilers and timing.

    python profile_cases.py unet N
        two forwards of the trained U-Net on one N x N field (the tcgen05
        3x3 convolutions and the network's elementwise kernels)
    python profile_cases.py batch COUNT N [cluster]
        one batched persistent solve of COUNT all-Neumann N x N problems with
        Gaussian sources to 1e-8 (the default kernel, one CTA per problem
        with the multigrid preconditioner; `cluster`: thread-block clusters
        of 16 CTAs)

    python profile_cases.py advect N STEPS
        STEPS steps of the stand-alone Advection_ on N x N (rotating cone,
        van Leer): the tile wavefront k_advect_tiles
    python profile_cases.py ic N KIND
        one structure-level IC_CGS / IC_CG solve of an N x N Dirichlet-0
        Poisson problem with a unit source to 1e-8 (the factor's triangular
        solves as the five-point wavefront)

Each prints one line with its timing and exits 0 on success.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def unet(n):
    import torch
    from carpio_gb300.unet import load_trained
    net = load_trained()
    x = torch.randn(1, n, n, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
    z = torch.empty_like(x)
    for _ in range(2):
        net.forward(x, out=z)
    torch.cuda.synchronize()
    print(f"unet {n}x{n}: mean |z| {float(z.abs().mean()):.4e}")


def batch(count, n, cluster=False):
    from carpio_gb300 import workloads
    from carpio_gb300.batch import BatchedPoisson, Problem, NEUMANN
    rng = np.random.default_rng(1)
    probs = [Problem(n, n, bc=[(NEUMANN, 0.0)] * 4) for _ in range(count)]
    srcs = [workloads.gaussian_source(n, n, rng) for _ in probs]
    bp = BatchedPoisson(probs, tol=1e-8,
                        tiles=dict(threads=512, cluster=16) if cluster else None)
    bp.upload(0, srcs)
    bp.zero(1)
    bp.run()
    st = bp.stats[0]
    print(f"batch {count} x {n}^2: {bp.ms:.2f} ms, {st['iters']} iterations, "
          f"{1000 * st['ms'] / max(st['iters'], 1):.2f} us/iteration")


def advect(n, steps):
    import time
    import bench
    g, eq = bench.advection_case(n)
    t0 = time.perf_counter()
    eq.run(steps)
    ms = 1e3 * (time.perf_counter() - t0) / steps
    print(f"advect {n}x{n}: {ms:.2f} ms per step")


def ic(n, kind):
    import bench
    g, p = bench.ic_case(n, kind)
    rc = p.run()
    print(f"{kind} {n}x{n}: code {rc}, {p.stats.iters} iterations, {p.stats.ms:.2f} ms")


def main(argv=None):
    a = list(sys.argv[1:] if argv is None else argv)
    if a[:1] == ["unet"] and len(a) == 2:
        unet(int(a[1]))
    elif a[:1] == ["batch"] and len(a) in (3, 4):
        batch(int(a[1]), int(a[2]), len(a) > 3 and a[3] == "cluster")
    elif a[:1] == ["advect"] and len(a) == 3:
        advect(int(a[1]), int(a[2]))
    elif a[:1] == ["ic"] and len(a) == 3:
        ic(int(a[1]), a[2])
    else:
        sys.exit(__doc__)


if __name__ == "__main__":
    main()
