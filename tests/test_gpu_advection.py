"""Stand-alone Advection_ (s_advection.hpp:22-216) on the GPU through the
library's Python mirror and C ABI, against the reference's own runs
(advect_* fixtures): the in-place sweep reproduces the reference's cell
order, so phi, the face velocities and the ghost-filled cell velocities are
bit-identical."""
import ctypes

import numpy as np
import pytest

from conftest import advect_case, bits_equal, golden, golden_names, gpu_grid

pytestmark = pytest.mark.gpu


def make(d):
    from carpio_gb300 import structure as S
    n = int(d["n"])
    g = gpu_grid(d, n, n, 2)
    c = advect_case(d)
    eq = S.Advection(g)
    eq.set_time(int(d["steps"]) - 1, float(d["dt"]))
    for k in ("u", "v", "phi"):
        eq.initial_CS(k, c[k])
    for (seg, name), bc in c["bi"]._m.items():
        eq.add_bc(0, seg, name, bc)
    eq.set_advection_scheme(str(d["scheme"]))
    return g, eq


@pytest.mark.parametrize("name", golden_names("advect_"))
def test_advection_matches_reference(name):
    d = golden(name)
    g, eq = make(d)
    eq.run()
    assert bits_equal(eq.get_CS("phi"), d["phi"])
    for k in ("u", "v", "uf", "vf"):
        assert bits_equal(eq.get_CS(k), d[k]), k


def test_advection_split_runs_match_one_run():
    """run(k) calls continue from where the last one stopped"""
    d = golden("advect_40_quick_rotate")
    g, eq = make(d)
    steps = int(d["steps"])
    eq.run(steps // 3)
    eq.run(steps - steps // 3)
    assert bits_equal(eq.get_CS("phi"), d["phi"])


def test_advection_arguments():
    from carpio_gb300 import _lib
    from carpio_gb300 import structure as S
    L = _lib.load()
    g1 = S.Grid((0.0, 0.0), (1.0, 1.0), (8, 8), 1)
    h = ctypes.c_void_p()
    assert L.carpio_gpu_advection_create(g1.handle, ctypes.byref(h)) == 0
    try:
        # minmod is not one of Advection_'s schemes; radius-2 schemes need gl 2
        assert L.carpio_gpu_advection_set_scheme(h, 9) == _lib.EINVAL
        assert L.carpio_gpu_advection_set_scheme(h, 4) == _lib.EINVAL
        assert L.carpio_gpu_advection_set_scheme(h, 1) == 0
        # stepping before initial()
        assert L.carpio_gpu_advection_step(h, 0.1, 1) == _lib.EINVAL
        bc = _lib.BC()
        for k in range(4):
            bc.type[k], bc.value[k] = 3, 0.0
        assert L.carpio_gpu_advection_set_bc(h, 2, ctypes.byref(bc), None) == _lib.EINVAL
        assert L.carpio_gpu_advection_initial(h, None, None, None) == 0
        assert L.carpio_gpu_advection_step(h, 0.1, 3) == 0
        out = g1.zeros()
        assert L.carpio_gpu_advection_get(h, None, None, None, None, _lib.ptr(out)) == 0
        assert not out.any()   # zero velocity, zero phi, Neumann 0
    finally:
        L.carpio_gpu_advection_destroy(h)


def oracle_bc(c):
    from oracle import restate as R
    o = R.BC()
    for k in range(4):
        o.type[k], o.value[k] = c.type[k], c.value[k]
    return o


@pytest.mark.parametrize("nx,ny,scheme,ly,dt", [(7, 19, "VanLeer", 0.7, 0.01),
                                                (1, 9, "QUICK", 0.7, 0.01),
                                                (13, 2, "upwind1", 0.7, 0.01),
                                                (16, 16, "center4", 0.7, 0.01),
                                                (161, 130, "VanLeer", 0.7, 1e-3),
                                                (190, 100, "superbee", 0.7, 1e-3),
                                                (256, 128, "VanLeer", 0.5, 1e-3),
                                                (96, 300, "WAHYD", 0.7, 1e-3)])
def test_advection_ragged_grids_match_oracle(nx, ny, scheme, ly, dt):
    """ragged and one-cell-wide grids, random velocity and phi fields, a
    Dirichlet function BC and Neumann values: the GPU sweep against the
    oracle's sequential loop, bit for bit. The larger grids run the row-
    pipelined sweep: a last band of one row (161) and of 30 rows (190),
    power-of-two spacings (256 x 128 on 1 x 0.5), three full bands (96)."""
    from carpio_gb300 import structure as S
    from oracle import restate as R
    rng = np.random.default_rng(nx * 100 + ny)
    g = S.Grid((0.0, 0.0), (1.0, ly), (nx, ny), 2)
    og = R.Grid(nx, ny, 2, 0.0, 1.0, 0.0, ly)
    assert bits_equal(og.cx, g.cx) and bits_equal(og.sy, g.sy)
    eq = S.Advection(g)
    eq.set_time(11, dt)
    u0, v0, p0 = (rng.uniform(-1, 1, g.N()) for _ in range(3))
    eq.initial_CS("u", 0.0)
    bi = S.BoundaryIndex()
    b_fun = S.BoundaryCondition()
    b_fun.set_default_1_bc(lambda t, x, y, z: 0.5 + y)
    b_n = S.BoundaryCondition()
    b_n.set_default_2_bc(0.25)
    for seg, b in ((0, b_fun), (1, b_n), (2, b_n), (3, b_fun)):
        eq.add_bc(0, seg, "phi", b)
        bi.insert(0, seg, "phi", b)
    eq.set_advection_scheme(scheme)
    # the library's initial() with explicit fields in place of functions
    eq.initial_fields(u0, v0, p0)
    eq.run()
    # the oracle: default (Neumann 0) velocity BCs, C2F, 12 in-place steps
    nb = oracle_bc(S.BoundaryIndex().to_c("u"))
    u = R.apply_bc(og, nb, u0)
    v = R.apply_bc(og, nb, v0)
    uf, vf = R.c2f(og, u, v)
    gv = bi.ghost_values(g, "phi", 0.0)
    phi = R.advect_run(og, scheme.lower(), oracle_bc(bi.to_c("phi", functions=True)),
                       uf, vf, dt, 12, p0, gv)
    assert bits_equal(eq.get_CS("uf"), uf) and bits_equal(eq.get_CS("vf"), vf)
    assert bits_equal(eq.get_CS("phi"), phi)


@pytest.mark.parametrize("n,scheme", [(520, "VanLeer"), (560, "CUI")])
def test_advection_grid_wide_sweep_matches_oracle(n, scheme):
    """grids whose diagonals are long run the sweep over all SMs (grid
    barriers between diagonals): still the oracle's sequential values, bit
    for bit"""
    from carpio_gb300 import structure as S
    from oracle import restate as R
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 2)
    og = R.Grid(n, n, 2)
    eq = S.Advection(g)
    eq.set_time(1, 0.25 / n)
    eq.set_advection_scheme(scheme)
    X, Y = np.meshgrid(g.cx, g.cy, indexing="ij")
    u0, v0 = -(Y - 0.5), X - 0.5
    r2 = (X - 0.5) ** 2 + (Y - 0.75) ** 2
    p0 = np.where(r2 < 0.04, 1.0 - r2 / 0.04, 0.0)
    eq.initial_fields(u0, v0, p0)
    eq.run()
    nb = oracle_bc(S.BoundaryIndex().to_c("u"))
    uf, vf = R.c2f(og, R.apply_bc(og, nb, u0), R.apply_bc(og, nb, v0))
    phi = R.advect_run(og, scheme.lower(), nb, uf, vf, 0.25 / n, 2, p0)
    assert bits_equal(eq.get_CS("phi"), phi)
