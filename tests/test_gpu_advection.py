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
