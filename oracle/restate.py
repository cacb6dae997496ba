"""ctypes wrapper of the C restatement (oracle/restate.c). TEST INFRASTRUCTURE.

Arrays follow the reference's layouts: cell and face fields are full
(nx+2gl) x (ny+2gl) float64 arrays with y contiguous (SpaceT,
lib/algebra/space.hpp:184-209); solver vectors number cells x fastest.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "librestate.so")
_lib = None

CG, JACOBI, DIA_BICGSTAB, BICGSTAB, IC_CGS, IC_CG = 0, 1, 2, 3, 4, 5
KINDS = {"cg": CG, "jacobi": JACOBI, "dia_bicgstab": DIA_BICGSTAB,
         "bicgstab": BICGSTAB, "ic_cgs": IC_CGS, "ic_cg": IC_CG}
SCHEMES = {"upwind1": 0, "center": 1, "center4": 2, "upwind2": 3,
           "vanleer": 4, "superbee": 5, "wahyd": 6, "quick": 7, "cui": 8,
           "minmod": 9}
EZERODIAG = -4

_d = ctypes.POINTER(ctypes.c_double)
_u = ctypes.POINTER(ctypes.c_uint32)
_i = ctypes.POINTER(ctypes.c_int)


class BC(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int * 4), ("value", ctypes.c_double * 4)]


class NSCfg(ctypes.Structure):
    _fields_ = [("rho", ctypes.c_double), ("mu", ctypes.c_double),
                ("cfl", ctypes.c_double), ("diff_number", ctypes.c_double),
                ("diff_coef", ctypes.c_double), ("scheme", ctypes.c_int),
                ("cg_max_iter", ctypes.c_int), ("cg_tol", ctypes.c_double),
                ("threads", ctypes.c_int), ("proj_kind", ctypes.c_int),
                ("proj_nomean", ctypes.c_int), ("mu_field", ctypes.c_void_p)]


def build():
    """Compile librestate.so in place (make -C oracle restate)."""
    subprocess.run(["make", "-s", "-C", _HERE, "restate"], check=True)


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "restate.c")
        if (not os.path.exists(_SO)
                or os.path.getmtime(_SO) < os.path.getmtime(src)):
            build()
        L = ctypes.CDLL(_SO)
        L.rs_krylov_csr.argtypes = [ctypes.c_int, ctypes.c_int, _u, _u, _d, _d,
                                    _d, _i, _d, _d, ctypes.c_int, _i,
                                    ctypes.c_int]
        L.rs_krylov_csr.restype = ctypes.c_int
        L.rs_dot.argtypes = [ctypes.c_int, _d, _d]
        L.rs_dot.restype = ctypes.c_double
        L.rs_nrm2.argtypes = [ctypes.c_int, _d]
        L.rs_nrm2.restype = ctypes.c_double
        L.rs_residual.argtypes = [ctypes.c_int, _u, _u, _d, _d, _d, ctypes.c_int]
        L.rs_residual.restype = ctypes.c_double
        L.rs_grid_uniform.argtypes = [ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, _d, _d]
        L.rs_grid_sizes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    _d, _d, _d]
        L.rs_assemble_poisson.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _d, _d, _d,
            ctypes.POINTER(BC), ctypes.c_double, _d, ctypes.c_double, _u, _u,
            _d, _d, _d]
        L.rs_assemble_poisson.restype = ctypes.c_int
        L.rs_apply_bc.argtypes = [ctypes.c_int] * 3 + [_d] * 4 + [
            ctypes.POINTER(BC), _d]
        L.rs_apply_bc_gv.argtypes = [ctypes.c_int] * 3 + [_d] * 4 + [
            ctypes.POINTER(BC), _d, _d]
        L.rs_advect_run.argtypes = [ctypes.c_int] * 4 + [_d] * 4 + [
            ctypes.POINTER(BC), _d, _d, _d, ctypes.c_double, ctypes.c_int, _d]
        L.rs_kim_run.argtypes = (
            [ctypes.c_int] * 3 + [_d] * 4
            + [ctypes.POINTER(BC), ctypes.POINTER(BC), ctypes.POINTER(NSCfg),
               ctypes.c_int, ctypes.c_int, ctypes.c_double] + [_d] * 10 + [_i, _d])
        L.rs_kim_run.restype = ctypes.c_int
        L.rs_grad.argtypes = [ctypes.c_int] * 3 + [_d] * 5
        L.rs_div.argtypes = [ctypes.c_int] * 3 + [_d] * 5
        L.rs_f2c.argtypes = [ctypes.c_int] * 3 + [_d] * 4
        L.rs_c2f.argtypes = [ctypes.c_int] * 3 + [_d] * 6
        L.rs_diffusion.argtypes = [ctypes.c_int] * 3 + [_d] * 4 + [
            ctypes.c_double, _d, _d]
        L.rs_diffusion_var.argtypes = [ctypes.c_int] * 3 + [_d] * 7
        L.rs_advection.argtypes = [ctypes.c_int] * 4 + [_d] * 8
        L.rs_max_magnitude.argtypes = [ctypes.c_int] * 3 + [_d] * 2
        L.rs_max_magnitude.restype = ctypes.c_double
        L.rs_ns_run.argtypes = (
            [ctypes.c_int] * 3 + [_d] * 4
            + [ctypes.POINTER(BC), ctypes.POINTER(BC), ctypes.POINTER(NSCfg),
               ctypes.c_int, _d] + [_d] * 6 + [_d, _i, _d])
        L.rs_ns_run.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t=_d):
    return a.ctypes.data_as(t)


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


def make_bc(types, values):
    bc = BC()
    for s in range(4):
        bc.type[s] = int(types[s])
        bc.value[s] = float(values[s])
    return bc


class Grid:
    """Grid arrays with ghosts as Grid_ builds them: uniform
    (_set_uniform_grid, lib/structure/s_grid.hpp:372-395) or, given the
    normal cells' sizes csx, csy, non-uniform (_set_non_uniform_grid,
    s_grid.hpp:397-434; nx, ny are then their lengths)."""

    def __init__(self, nx, ny, gl, x0=0.0, x1=1.0, y0=0.0, y1=1.0, csx=None, csy=None):
        if csx is not None:
            csx = np.ascontiguousarray(csx, dtype=np.float64)
            csy = np.ascontiguousarray(csy, dtype=np.float64)
            nx, ny = csx.size, csy.size
        self.nx, self.ny, self.gl = nx, ny, gl
        L = lib()
        self.cx = np.zeros(nx + 2 * gl)
        self.sx = np.zeros(nx + 2 * gl)
        self.cy = np.zeros(ny + 2 * gl)
        self.sy = np.zeros(ny + 2 * gl)
        if csx is not None:
            L.rs_grid_sizes(nx, gl, x0, _p(csx), _p(self.cx), _p(self.sx))
            L.rs_grid_sizes(ny, gl, y0, _p(csy), _p(self.cy), _p(self.sy))
        else:
            L.rs_grid_uniform(nx, gl, x0, x1, _p(self.cx), _p(self.sx))
            L.rs_grid_uniform(ny, gl, y0, y1, _p(self.cy), _p(self.sy))

    @property
    def shape(self):
        return (self.nx + 2 * self.gl, self.ny + 2 * self.gl)

    def zeros(self):
        return np.zeros(self.shape)

    def args(self):
        return (self.nx, self.ny, self.gl)

    def geo(self):
        return (_p(self.cx), _p(self.sx), _p(self.cy), _p(self.sy))

    def interior(self, f):
        g = self.gl
        return f[g:g + self.nx, g:g + self.ny]


def residual(rowptr, colind, val, x, b, full=False):
    """carpio::Residual restated: nrm2(b - A x) / nrm2(b)"""
    rp = np.ascontiguousarray(rowptr, dtype=np.uint32)
    ci = np.ascontiguousarray(colind, dtype=np.uint32)
    return lib().rs_residual(len(rp) - 1, _p(rp, _u), _p(ci, _u), _p(_f64(val)),
                             _p(_f64(x)), _p(_f64(b)), 1 if full else 0)


def krylov_csr(kind, rowptr, colind, val, b, x0, max_iter, tol,
               hist_cap=None, threads=1):
    """carpio::CG/Jacobi/Dia_BiCGSTAB/BiCGSTAB restated. Returns
    (code, x, iters, tol_out, hist)."""
    L = lib()
    rowptr = np.ascontiguousarray(rowptr, dtype=np.uint32)
    colind = np.ascontiguousarray(colind, dtype=np.uint32)
    val = _f64(val)
    b = _f64(b)
    x = _f64(x0).copy()
    n = b.size
    mi = ctypes.c_int(int(max_iter))
    t = ctypes.c_double(float(tol))
    cap = int(max_iter) + 1 if hist_cap is None else int(hist_cap)
    hist = np.zeros(max(cap, 1))
    hl = ctypes.c_int(0)
    code = L.rs_krylov_csr(KINDS.get(kind, kind), n, _p(rowptr, _u),
                           _p(colind, _u), _p(val), _p(b), _p(x),
                           ctypes.byref(mi), ctypes.byref(t), _p(hist), cap,
                           ctypes.byref(hl), int(threads))
    return code, x, mi.value, t.value, hist[:min(hl.value, cap)]


def assemble_poisson(grid, bc, beta=1.0, src=None, src_value=0.0, bfield=None):
    """StencilPoisson_ + GhostRegular_ assembled as Solver_::_build_matrix;
    bfield: a beta field (full field with ghosts) instead of the uniform beta"""
    L = lib()
    n = grid.nx * grid.ny
    rp = np.zeros(n + 1, dtype=np.uint32)
    ci = np.zeros(5 * n, dtype=np.uint32)
    va = np.zeros(5 * n)
    b = np.zeros(n)
    s = None if src is None else _f64(src)
    nz = L.rs_assemble_poisson(*grid.args(), *grid.geo(), ctypes.byref(bc),
                               float(beta),
                               _p(s) if s is not None else None,
                               float(src_value), _p(rp, _u), _p(ci, _u),
                               _p(va), _p(b),
                               _p(_f64(bfield)) if bfield is not None else None)
    return rp, ci[:nz].copy(), va[:nz].copy(), b


def field_to_vec(grid, f):
    """interior of a field -> solver vector (x fastest)"""
    return np.ascontiguousarray(grid.interior(f).T).reshape(-1)


def vec_to_field(grid, vec, f=None):
    f = grid.zeros() if f is None else f
    g = grid.gl
    f[g:g + grid.nx, g:g + grid.ny] = vec.reshape(grid.ny, grid.nx).T
    return f


def apply_bc(grid, bc, f, gv=None):
    f = _f64(f).copy()
    if gv is None:
        lib().rs_apply_bc(*grid.args(), *grid.geo(), ctypes.byref(bc), _p(f))
    else:
        lib().rs_apply_bc_gv(*grid.args(), *grid.geo(), ctypes.byref(bc),
                             _p(_f64(gv)), _p(f))
    return f


def advect_run(grid, scheme, bc, uf, vf, dt, steps, phi, gv=None):
    """Advection_::run_one_step (s_advection.hpp:185-212) `steps` times on
    a copy of phi; gv: optional per-ghost boundary values (a cell field)"""
    phi = _f64(phi).copy()
    lib().rs_advect_run(SCHEMES.get(scheme, scheme), *grid.args(), *grid.geo(),
                        ctypes.byref(bc), None if gv is None else _p(_f64(gv)),
                        _p(_f64(uf)), _p(_f64(vf)), float(dt), int(steps), _p(phi))
    return phi


def grad(grid, phi):
    gx, gy = grid.zeros(), grid.zeros()
    lib().rs_grad(*grid.args(), _p(grid.cx), _p(grid.cy), _p(_f64(phi)),
                  _p(gx), _p(gy))
    return gx, gy


def div(grid, fx, fy):
    out = grid.zeros()
    lib().rs_div(*grid.args(), _p(grid.sx), _p(grid.sy), _p(_f64(fx)),
                 _p(_f64(fy)), _p(out))
    return out


def f2c(grid, fx, fy):
    a, b = grid.zeros(), grid.zeros()
    lib().rs_f2c(*grid.args(), _p(_f64(fx)), _p(_f64(fy)), _p(a), _p(b))
    return a, b


def c2f(grid, u, v, fx=None, fy=None):
    fx = grid.zeros() if fx is None else _f64(fx).copy()
    fy = grid.zeros() if fy is None else _f64(fy).copy()
    lib().rs_c2f(*grid.args(), _p(grid.sx), _p(grid.sy), _p(_f64(u)),
                 _p(_f64(v)), _p(fx), _p(fy))
    return fx, fy


def diffusion(grid, mu, f):
    out = grid.zeros()
    lib().rs_diffusion(*grid.args(), *grid.geo(), float(mu), _p(_f64(f)),
                       _p(out))
    return out


def diffusion_var(grid, mu, f):
    """NablaMuNabla with a mu field (s_operation.hpp:630-662)"""
    out = grid.zeros()
    lib().rs_diffusion_var(*grid.args(), *grid.geo(), _p(_f64(mu)), _p(_f64(f)),
                           _p(out))
    return out


def advection(grid, scheme, uf, vf, f):
    out = grid.zeros()
    lib().rs_advection(SCHEMES.get(scheme, scheme), *grid.args(), *grid.geo(),
                       _p(_f64(uf)), _p(_f64(vf)), _p(_f64(f)), _p(out))
    return out


def max_magnitude(grid, u, v):
    return lib().rs_max_magnitude(*grid.args(), _p(_f64(u)), _p(_f64(v)))


def cavity_bcs():
    """lid-driven cavity: u = 1 on segment 3 (y+), no-slip elsewhere"""
    return make_bc([1, 1, 1, 1], [0, 0, 0, 1]), make_bc([1] * 4, [0] * 4)


def ns_run(grid, state, steps, *, Re=1000.0, mu=1.0, cfl=0.5,
           diff_number=0.25, diff_coef=None, scheme="vanleer",
           cg_max_iter=100000, cg_tol=1e-10, threads=1, bc_u=None, bc_v=None,
           proj="cg", proj_mean=True, mu_field=None):
    """Runs `steps` explicit projection steps in place on
    state = dict(dt=float, u, v, uf, vf, phi, p). Returns (code, step_dt,
    step_iters, step_resid)."""
    if bc_u is None or bc_v is None:
        bc_u, bc_v = cavity_bcs()
    cfg = NSCfg(rho=Re, mu=mu, cfl=cfl, diff_number=diff_number,
                diff_coef=(1.0 / Re) if diff_coef is None else diff_coef,
                scheme=SCHEMES.get(scheme, scheme), cg_max_iter=cg_max_iter,
                cg_tol=cg_tol, threads=threads, proj_kind=KINDS[proj],
                proj_nomean=0 if proj_mean else 1)
    if mu_field is not None:
        mu_field = _f64(mu_field)
        cfg.mu_field = mu_field.ctypes.data
    for k in ("u", "v", "uf", "vf", "phi", "p"):
        state[k] = _f64(state[k])
    dt = ctypes.c_double(state["dt"])
    sdt = np.zeros(max(steps, 1))
    sit = np.zeros(max(steps, 1), dtype=np.int32)
    sres = np.zeros(max(steps, 1))
    code = lib().rs_ns_run(*grid.args(), *grid.geo(), ctypes.byref(bc_u),
                           ctypes.byref(bc_v), ctypes.byref(cfg), int(steps),
                           ctypes.byref(dt), *(_p(state[k]) for k in (
                               "u", "v", "uf", "vf", "phi", "p")),
                           _p(sdt), _p(sit, _i), _p(sres))
    state["dt"] = dt.value
    return code, sdt[:steps], sit[:steps], sres[:steps]


def new_state(grid, dt0):
    return dict(dt=float(dt0), u=grid.zeros(), v=grid.zeros(),
                uf=grid.zeros(), vf=grid.zeros(), phi=grid.zeros(),
                p=grid.zeros())


def kim_run(grid, state, steps, dt, *, Re=1000.0, mu=1.0, scheme="vanleer",
            cg_max_iter=100000, cg_tol=1e-10, threads=1, bc_u=None, bc_v=None,
            proj="cg", proj_mean=True):
    """NS_kim_ steps (s_ns_kim.hpp:130-280) in place on state = dict(step=int,
    u, v, uf, vf, phi, p, us, vs, usf, vsf); dt fixed (the stepper has no
    restrict_time). Returns (code, step_iters, step_resid)."""
    if bc_u is None or bc_v is None:
        bc_u, bc_v = cavity_bcs()
    cfg = NSCfg(rho=Re, mu=mu, scheme=SCHEMES.get(scheme, scheme),
                cg_max_iter=cg_max_iter, cg_tol=cg_tol, threads=threads,
                proj_kind=KINDS[proj], proj_nomean=0 if proj_mean else 1)
    keys = ("u", "v", "uf", "vf", "phi", "p", "us", "vs", "usf", "vsf")
    for k in keys:
        state[k] = _f64(state[k])
    sit = np.zeros(max(steps, 1), dtype=np.int32)
    sres = np.zeros(max(steps, 1))
    code = lib().rs_kim_run(*grid.args(), *grid.geo(), ctypes.byref(bc_u),
                            ctypes.byref(bc_v), ctypes.byref(cfg), int(steps),
                            1 if state["step"] == 0 else 0, float(dt),
                            *(_p(state[k]) for k in keys), _p(sit, _i), _p(sres))
    state["step"] += steps
    return code, sit[:steps], sres[:steps]
