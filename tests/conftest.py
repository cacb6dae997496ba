"""Shared test helpers. Tests marked `gpu` need a CUDA device (GB300) and the
built library; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Parity bar of the plain FP64 path against the FP64 reference: relative L2.
PLAIN_RTOL = 1e-10


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (sm_103a) and libcarpio_gpu.so")


def golden(name):
    path = os.path.join(GOLDEN, name + ".npz")
    with np.load(path) as d:
        return {k: d[k] for k in d.files}


def golden_names(prefix):
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.startswith(prefix) and f.endswith(".npz"))


def fixture_sizes(d, nx, ny, gl):
    """the normal cells' sizes of a fixture's stretched grid, or None"""
    if "stretch" in d and float(d["stretch"]):
        return d["grid_sx"][gl:gl + nx], d["grid_sy"][gl:gl + ny]
    return None


def gpu_grid(d, nx, ny, gl):
    """the library grid of a fixture: uniform on [0,1]^2 or from sizes"""
    from carpio_gb300 import structure as S
    sz = fixture_sizes(d, nx, ny, gl)
    if sz is None:
        return S.Grid((0.0, 0.0), (1.0, 1.0), (nx, ny), gl)
    return S.Grid.from_sizes((0.0, 0.0), gl, sz[0], sz[1])


def oracle_grid(d, nx, ny, gl):
    """the oracle grid of a fixture"""
    from oracle import restate as R
    sz = fixture_sizes(d, nx, ny, gl)
    if sz is None:
        return R.Grid(nx, ny, gl)
    return R.Grid(nx, ny, gl, csx=sz[0], csy=sz[1])


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library on a CUDA device; fails (does not skip) without one."""
    from carpio_gb300 import _lib
    L = _lib.load()
    n = L.carpio_gpu_device_count()
    if n < 1:
        pytest.fail("no CUDA device visible: gpu tests need a GB300")
    return L


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """(Re)build libcarpio_gpu.so if its sources changed (no-op when fresh),
    so the ABI tests always load the library the sources describe."""
    from carpio_gb300 import compile as c
    c.build()


def advect_case(d):
    """the stand-alone Advection_ set-ups of the advect_* fixtures, as the
    harness writes them: initial functions of u, v, phi and the boundary
    conditions of phi (a BoundaryIndex of the library's Python mirror)"""
    from carpio_gb300 import structure as S
    case = str(d["case"])
    bi = S.BoundaryIndex()
    if case == "band":
        fu = lambda t, x, y, z: 1.0
        fv = lambda t, x, y, z: 1.0
        fphi = lambda t, x, y, z: 0.0
        b0 = S.BoundaryCondition()
        b0.set_default_1_bc(0)
        b1 = S.BoundaryCondition()
        b1.set_default_1_bc(lambda t, x, y, z: 1.0 if (y >= 0.0 and y <= 0.3) else 0.0)
        bi.insert(0, 0, "phi", b1)
        for k in (1, 2, 3):
            bi.insert(0, k, "phi", b0)
    elif case == "rotate":
        fu = lambda t, x, y, z: -(y - 0.5)
        fv = lambda t, x, y, z: x - 0.5

        def fphi(t, x, y, z):
            dx, dy = x - 0.5, y - 0.75
            r2 = dx * dx + dy * dy
            return 1.0 - r2 / 0.04 if r2 < 0.04 else 0.0
    else:
        raise ValueError(case)
    return dict(u=fu, v=fv, phi=fphi, bi=bi)
