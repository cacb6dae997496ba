"""Structure-level mirror of lib/structure over the C ABI: Grid_, BoundaryCondition,
Poisson_ (s_poisson.hpp) and NS_explicit_ (s_ns_explicit.hpp), on the GPU.

Fields are numpy arrays (or CUDA tensors) of the reference's SpaceT shape
(nx+2gl, ny+2gl), y contiguous, ghosts included.
"""
import ctypes
import os
import sys

import numpy as np

from . import _lib


class Grid:
    """Grid_<2>(pmin, pmax, n, gl) with uniform cells (s_grid.hpp:25-34), or
    Grid.from_sizes(pmin, gl, csx, csy) from the normal cells' sizes
    (Grid_<2>(min, gl, csx, csy), s_grid.hpp:35-48, 397-434)."""

    def __init__(self, pmin, pmax, n, gl, _sizes=None):
        L = _lib.load()
        self.nx, self.ny = int(n[0]), int(n[1])
        self.gl = int(gl)
        h = ctypes.c_void_p()
        if _sizes is None:
            rc = L.carpio_gpu_grid_create_uniform(
                self.nx, self.ny, self.gl, float(pmin[0]), float(pmax[0]),
                float(pmin[1]), float(pmax[1]), ctypes.byref(h))
        else:
            csx, csy = _sizes
            rc = L.carpio_gpu_grid_create(self.nx, self.ny, self.gl, float(pmin[0]),
                                          float(pmin[1]), _lib.ptr(csx), _lib.ptr(csy),
                                          ctypes.byref(h))
        if rc:
            raise _lib.CarpioGpuError(rc, "grid_create")
        self.handle = h
        self.cx = np.zeros(self.nx + 2 * self.gl)
        self.sx = np.zeros(self.nx + 2 * self.gl)
        self.cy = np.zeros(self.ny + 2 * self.gl)
        self.sy = np.zeros(self.ny + 2 * self.gl)
        L.carpio_gpu_grid_coords(h, _lib.ptr(self.cx), _lib.ptr(self.sx),
                                 _lib.ptr(self.cy), _lib.ptr(self.sy))

    @classmethod
    def from_sizes(cls, pmin, gl, csx, csy):
        csx = np.ascontiguousarray(csx, dtype=np.float64)
        csy = np.ascontiguousarray(csy, dtype=np.float64)
        return cls(pmin, None, (csx.size, csy.size), gl, _sizes=(csx, csy))

    def N(self):
        return (self.nx + 2 * self.gl, self.ny + 2 * self.gl)

    def zeros(self):
        return np.zeros(self.N())

    def interior(self, f):
        g = self.gl
        return f[g:g + self.nx, g:g + self.ny]

    def __del__(self):
        # no CUDA calls while the interpreter shuts down: the runtime may be
        # gone already; the process exit releases the device memory
        h = getattr(self, "handle", None)
        if h is not None and _lib._lib is not None and not sys.is_finalizing():
            _lib._lib.carpio_gpu_grid_destroy(h)
            self.handle = None


def Output_Scalar(filename, grid, field):
    """structure::Output_Scalar (s_io_file.hpp:43-71): writes the field (the
    grid's layout with ghosts, host or device) in the reference's text
    format"""
    f = np.ascontiguousarray(field, dtype=np.float64)
    if f.shape != grid.N():
        raise ValueError(f"field shape {f.shape} != grid {grid.N()}")
    rc = _lib.load().carpio_gpu_output_scalar(grid.handle, os.fsencode(filename), _lib.ptr(f))
    if rc:
        raise _lib.CarpioGpuError(rc, "output_scalar")


class BoundaryCondition:
    """BoundaryCondition (s_boundary.hpp:10-130); default Neumann 0. The
    value is a number or a function f(t, x, y, z) (set_default_1_bc(Fun),
    s_boundary.hpp:109-114); functions are taken by Advection only."""
    BC1, BC2 = 1, 2

    def __init__(self):
        self.type, self.value = 2, 0.0

    @staticmethod
    def _val(val):
        return val if callable(val) else float(val)

    def set_default_1_bc(self, val):
        self.type, self.value = 1, self._val(val)

    def set_default_2_bc(self, val):
        self.type, self.value = 2, self._val(val)

    def get_val(self, t, x, y, z):
        return float(self.value(t, x, y, z)) if callable(self.value) else self.value


class BoundaryIndex:
    """BoundaryIndex (s_boundary.hpp:132-234) for one shape (0): per
    variable name and segment, default Neumann 0."""

    def __init__(self):
        self._m = {}

    def insert(self, shape, seg, name, bc):
        if shape != 0 or seg not in (0, 1, 2, 3):
            raise ValueError("regular grids have shape 0, segments 0..3")
        self._m[(seg, name)] = bc

    def find(self, seg, name):
        return self._m.get((seg, name), BoundaryCondition())

    def has_function(self, name):
        return any(callable(self.find(s, name).value) for s in range(4))

    def to_c(self, name, functions=False):
        c = _lib.BC()
        for s in range(4):
            bc = self.find(s, name)
            if callable(bc.value) and not functions:
                raise ValueError(f"{name}: function boundary values are taken "
                                 "by Advection only")
            c.type[s] = bc.type
            c.value[s] = 0.0 if callable(bc.value) else bc.value
        return c

    def ghost_values(self, grid, name, t):
        """the value Equation_::apply_bc (s_equation.hpp:340-378) takes for
        every ghost cell: BC::get_val at time t at the face of the ghost's
        source cell on the ghost's side, on both axes (Grid_::f_,
        s_grid.hpp:200-211; z = -0.5 / +0.5 in 2-D). A field of the grid's
        layout, zero in the normal cells."""
        nx, ny, gl = grid.nx, grid.ny, grid.gl
        gv = grid.zeros()
        NI, NJ = gv.shape
        # the ghost frame only: full rows I < gl, I >= NI - gl, and the
        # columns J < gl, J >= NJ - gl of the other rows
        frame = [(I, J) for I in list(range(gl)) + list(range(NI - gl, NI)) for J in range(NJ)]
        frame += [(I, J) for I in range(gl, NI - gl)
                  for J in list(range(gl)) + list(range(NJ - gl, NJ))]
        for I, J in frame:
            i, j = I - gl, J - gl
            if i < 0 or i >= nx:
                seg, hi = (0, False) if i < 0 else (1, True)
                oi, oj = (0 if i < 0 else nx - 1), j
            else:
                seg, hi = (2, False) if j < 0 else (3, True)
                oi, oj = i, (0 if j < 0 else ny - 1)
            cx, hx = grid.cx[oi + gl], grid.sx[oi + gl] * 0.5
            cy, hy = grid.cy[oj + gl], grid.sy[oj + gl] * 0.5
            x = cx + hx if hi else cx - hx
            y = cy + hy if hi else cy - hy
            z = 0.5 if hi else 0.0 - 0.5
            gv[I, J] = self.find(seg, name).get_val(t, x, y, z)
        return gv


def solver_cfg(name="CG", max_iter=1000, tol=1e-3, mean_removal=False,
               precision="fp64", inner_tol=0.0, inner_max_iter=0, flags=0,
               poly_degree=0, poly_ratio=0.0, precond="default"):
    c = _lib.SolverCfg()
    c.poly_degree = int(poly_degree)
    c.poly_ratio = float(poly_ratio)
    c.precond = _lib.PRECOND[precond]
    c.kind = _lib.KINDS[name]
    c.precision = _lib.MIXED if precision == "mixed" else _lib.FP64
    c.max_iter = int(max_iter)
    c.tol = float(tol)
    c.mean_removal = 1 if mean_removal else 0
    c.inner_tol = float(inner_tol)
    c.inner_max_iter = int(inner_max_iter)
    c.flags = int(flags)
    return c


def learned_cfg(use_net=True, smooth=4, omega=0.8, memory=2, stall=20, fallback=True):
    c = _lib.LearnedCfg()
    c.use_net, c.smooth, c.omega = int(bool(use_net)), int(smooth), float(omega)
    c.memory, c.stall, c.fallback = int(memory), int(stall), int(bool(fallback))
    return c


class Poisson:
    """Poisson_<2> (s_poisson.hpp:265-594) with the GPU solver behind
    Solver_<2>::solve. set_solver accepts "CG", "Jacobi", "Dia_BiCGSTAB",
    "BiCGSTAB" and "IC_CGS", "IC_CG" (the carpio:: solvers; the IC ones in
    FP64, through the CSR layer)."""

    def __init__(self, grid):
        self.grid = grid
        self._bi = BoundaryIndex()
        self.beta = 1.0
        self.cfg = solver_cfg()
        self.source = None
        self.phi = None
        self.stats = _lib.SolverStats()
        self.lresid = []

    def add_bc(self, shape, seg, name, bc):
        self._bi.insert(shape, seg, name, bc)

    def set_uniform_beta(self, beta=1.0):
        self.beta = float(beta)

    def set_source(self, source):
        """a full field, or f(x, y) evaluated at the cell centres"""
        if callable(source):
            g = self.grid
            X, Y = np.meshgrid(g.cx, g.cy, indexing="ij")
            source = np.asarray(source(X, Y), dtype=np.float64)
        self.source = source

    def set_depend(self, phi, beta, source):
        self.phi = phi
        if beta is not None:
            raise NotImplementedError("variable beta is not on the GPU path")
        self.source = source

    def set_solver(self, name, any_=None, max_iter=1000, tol=1e-3, **kw):
        self.cfg = solver_cfg(name, max_iter, tol, **kw)

    def set_beta(self, field):
        """a beta field (full field with ghosts), as set_depend(phi, spbeta,
        source) gives the reference's Poisson_; None: back to the uniform
        beta"""
        self.beta_field = field

    def set_uniform_alpha(self, a=1.0):
        """Poisson_::set_uniform_alpha (s_poisson.hpp:461-471): the
        StencilHelmholtz_ rows with a uniform alpha"""
        self.alpha = float(a)

    def unset_uniform_alpha(self):
        self.alpha = None

    def set_learned(self, net, use_net=True, smooth=4, omega=0.8, memory=2,
                    stall=20, fallback=True):
        """solve with flexible CG preconditioned by the U-Net `net`
        (carpio_gb300.unet.UNet; None: back to the plain solver)"""
        self.learned = None if net is None and use_net else (
            net, learned_cfg(use_net, smooth, omega, memory, stall, fallback))

    def run(self):
        L = _lib.load()
        if self.phi is None:
            self.phi = self.grid.zeros()
        if self.source is None:
            self.source = self.grid.zeros()
        bc = self._bi.to_c("phi")
        if getattr(self, "learned", None) is not None:
            net, lc = self.learned
            cap = self.cfg.max_iter + 2
            hist = np.zeros(max(cap, 1))
            rc = L.carpio_gpu_poisson_solve_learned(
                self.grid.handle, ctypes.byref(bc), self.beta, _lib.ptr(self.source),
                _lib.ptr(self.phi), ctypes.byref(self.cfg),
                net.handle if net is not None else None, ctypes.byref(lc),
                _lib.ptr(hist), cap, ctypes.byref(self.stats))
            if rc < 0:
                raise _lib.CarpioGpuError(rc, "poisson_solve_learned")
            self.lresid = hist[:min(self.stats.outer_iters + 1, cap)].tolist()
            return rc
        cap = self.cfg.max_iter + 2
        hist = np.zeros(max(cap, 1))
        if getattr(self, "beta_field", None) is not None:
            bf = np.ascontiguousarray(self.beta_field, dtype=np.float64)
            rc = L.carpio_gpu_poisson_solve_beta(
                self.grid.handle, ctypes.byref(bc), _lib.ptr(bf),
                _lib.ptr(self.source), _lib.ptr(self.phi), ctypes.byref(self.cfg),
                _lib.ptr(hist), cap, ctypes.byref(self.stats))
        elif getattr(self, "alpha", None) is not None:
            rc = L.carpio_gpu_helmholtz_solve(
                self.grid.handle, ctypes.byref(bc), self.alpha, self.beta,
                _lib.ptr(self.source), _lib.ptr(self.phi), ctypes.byref(self.cfg),
                _lib.ptr(hist), cap, ctypes.byref(self.stats))
        else:
            rc = L.carpio_gpu_poisson_solve(
                self.grid.handle, ctypes.byref(bc), self.beta,
                _lib.ptr(self.source), _lib.ptr(self.phi), ctypes.byref(self.cfg),
                _lib.ptr(hist), cap, ctypes.byref(self.stats))
        if rc < 0:
            raise _lib.CarpioGpuError(rc, "poisson_solve")
        self.lresid = hist[:min(self.stats.hist_len, cap)].tolist()
        return rc

    def get_CS(self, name):
        if name == "phi":
            return self.phi
        if name == "source":
            return self.source
        raise KeyError(name)


class NS_explicit:
    """NS_explicit_<2> (s_ns_explicit.hpp) stepping on the GPU. Configure as
    the reference's examples do, then run(steps)."""

    def __init__(self, grid):
        self.grid = grid
        self._bi = BoundaryIndex()
        self.rho, self.mu = 1.0, 1.0
        self.cfl = 0.5
        self.diff_number, self.diff_coef = 1e10, 1.0
        self.scheme = "upwind1"
        self.proj = solver_cfg("CG", 1000, 1e-3, mean_removal=True)
        self.dt0 = None
        self.max_step = 0
        self.handle = None
        self.step_dt, self.step_iters, self.step_resid = [], [], []

    def add_bc(self, shape, seg, name, bc):
        self._bi.insert(shape, seg, name, bc)

    def set_time(self, max_step, dt):
        self.max_step, self.dt0 = int(max_step), float(dt)

    def set_uniform_rho(self, rho=1.0):
        self.rho = float(rho)

    def set_uniform_mu(self, mu=1.0):
        self.mu = float(mu)
        self._mu_fun = None

    def unset_uniform_mu(self):
        """with initial_CS("mu", f): a mu field (s_ns.hpp:111-118, 277-280)"""
        self._mu_fun = getattr(self, "_mu_fun", None) or (lambda t, x, y, z: 1.0)

    def initial_CS(self, name, fun):
        if name != "mu":
            raise ValueError("NS_explicit.initial_CS takes the mu field only")
        self._mu_fun = fun if callable(fun) else (lambda t, x, y, z, v=float(fun): v)

    def _mu_field(self):
        """set_CS("mu", f): f at every cell centre, ghosts included, t = 0"""
        g, f = self.grid, self._mu_fun
        out = g.zeros()
        for I in range(out.shape[0]):
            for J in range(out.shape[1]):
                out[I, J] = f(0.0, g.cx[I], g.cy[J], 0.0)
        return out

    def set_CFL_number(self, v=0.5):
        self.cfl = float(v)

    def set_diffusion_number(self, v=1e10, coe=1.0):
        self.diff_number, self.diff_coef = float(v), float(coe)

    def set_advection_scheme(self, name):
        if name not in _lib.SCHEMES:
            raise ValueError(f"unknown scheme {name}")
        self.scheme = name

    def set_learned(self, net, use_net=True, smooth=4, omega=0.8, memory=2,
                    stall=20, fallback=True):
        """project with flexible CG preconditioned by the U-Net `net`
        (None: back to the configured projection solver)"""
        if self.handle is None:
            self.initial()
        self._learned = (net, learned_cfg(use_net, smooth, omega, memory, stall, fallback))
        rc = _lib.load().carpio_gpu_ns_set_learned(
            self.handle, net.handle if net is not None else None,
            ctypes.byref(self._learned[1]))
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_set_learned")

    def set_projection_solver(self, name="CG", max_iter=1000, tol=1e-3,
                              precision="fp64", mean_removal=None, **kw):
        """NS_::set_projection_solver (s_ns.hpp:120-130). "CG" is the
        drop-in (with mean removal by default); "IC_CGS" / "IC_CG" are the
        reference's shipped solvers (Solver_IC_CGS_, s_solver.hpp:329-352,
        removes no mean), FP64 only; "Dia_BiCGSTAB" / "BiCGSTAB" as the
        drop-in's other kinds (mean removal by default)."""
        if mean_removal is None:
            mean_removal = name in ("CG", "Dia_BiCGSTAB", "BiCGSTAB")
        self.proj = solver_cfg(name, max_iter, tol, mean_removal=mean_removal,
                               precision=precision, **kw)

    def initial(self):
        L = _lib.load()
        c = _lib.NSCfg()
        c.rho, c.mu, c.cfl = self.rho, self.mu, self.cfl
        c.diff_number, c.diff_coef = self.diff_number, self.diff_coef
        c.scheme = _lib.SCHEMES[self.scheme]
        c.bc_u = self._bi.to_c("u")
        c.bc_v = self._bi.to_c("v")
        c.projection = self.proj
        h = ctypes.c_void_p()
        rc = L.carpio_gpu_ns_create(self.grid.handle, ctypes.byref(c),
                                    self.dt0, ctypes.byref(h))
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_create")
        self.handle = h
        if getattr(self, "_mu_fun", None) is not None:
            rc = L.carpio_gpu_ns_set_mu_field(h, _lib.ptr(self._mu_field()))
            if rc:
                raise _lib.CarpioGpuError(rc, "ns_set_mu_field")

    def run(self, steps=None):
        """Equation_::run: max_step + 1 steps (s_time.hpp:335-341) unless
        `steps` is given."""
        if self.handle is None:
            self.initial()
        n = self.max_step + 1 if steps is None else int(steps)
        dts = np.zeros(max(n, 1))
        its = np.zeros(max(n, 1), dtype=np.int32)
        res = np.zeros(max(n, 1))
        rc = _lib.load().carpio_gpu_ns_run(self.handle, n, _lib.ptr(dts),
                                           _lib.ptr(its), _lib.ptr(res))
        if rc < 0:
            raise _lib.CarpioGpuError(rc, "ns_run")
        self.step_dt += dts[:n].tolist()
        self.step_iters += its[:n].tolist()
        self.step_resid += res[:n].tolist()
        return rc

    def profile(self):
        """per-step device times of the last run (carpio_gpu_ns_profile)"""
        n = ctypes.c_int(0)
        _lib.load().carpio_gpu_ns_profile(self.handle, 0, ctypes.byref(n),
                                          None, None, None, None)
        m = n.value
        solve, step = np.zeros(max(m, 1)), np.zeros(max(m, 1))
        inner = np.zeros(max(m, 1), dtype=np.int32)
        outer = np.zeros(max(m, 1), dtype=np.int32)
        rc = _lib.load().carpio_gpu_ns_profile(
            self.handle, m, ctypes.byref(n), _lib.ptr(solve), _lib.ptr(step),
            _lib.ptr(inner), _lib.ptr(outer))
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_profile")
        return dict(solve_ms=solve[:m], step_ms=step[:m], inner=inner[:m],
                    outer=outer[:m])

    def set_state(self, dt, **fields):
        args = [fields.get(k) for k in ("u", "v", "uf", "vf", "phi", "p")]
        rc = _lib.load().carpio_gpu_ns_set_state(
            self.handle, float(dt), *[_lib.ptr(a) if a is not None else None
                                      for a in args])
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_set_state")

    def state(self, out=None):
        """the fields (and dt) as host arrays; `out`: a dict of arrays to
        fill instead (e.g. pinned torch tensors; the returned dict holds
        them plus dt, `out` itself is not changed)"""
        g = self.grid
        if out is None:
            out = {k: g.zeros() for k in ("u", "v", "uf", "vf", "phi", "p")}
        dt = ctypes.c_double()
        rc = _lib.load().carpio_gpu_ns_get_state(
            self.handle, ctypes.byref(dt),
            *[_lib.ptr(out[k]) for k in ("u", "v", "uf", "vf", "phi", "p")])
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_get_state")
        res = dict(out)
        res["dt"] = dt.value
        return res

    def get_CS(self, name):
        return self.state()[name]

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and _lib._lib is not None and not sys.is_finalizing():
            _lib._lib.carpio_gpu_ns_destroy(h)
            self.handle = None


class Advection:
    """Stand-alone Advection_<2> (s_advection.hpp:22-216) on the GPU:
    initial_CS for u, v and phi (numbers or functions f(t, x, y, z)),
    add_bc, set_advection_scheme, set_time, then run(); get_CS reads the
    fields. The velocity field stays fixed; phi is updated in place in the
    reference's cell order, so results are bit-identical to it."""
    SCHEMES = ("upwind1", "center", "center4", "upwind2", "VanLeer",
               "superbee", "WAHYD", "QUICK", "CUI")

    def __init__(self, grid):
        L = _lib.load()
        self.grid = grid
        self._bi = BoundaryIndex()
        self._fun = {"u": 0.0, "v": 0.0, "phi": 0.0}
        self.scheme = "upwind1"
        self.max_step, self.dt = 0, None
        self.t, self.step = 0.0, 0
        h = ctypes.c_void_p()
        rc = L.carpio_gpu_advection_create(grid.handle, ctypes.byref(h))
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_create")
        self.handle = h
        self._ready = False

    def set_time(self, max_step, dt):
        self.max_step, self.dt = int(max_step), float(dt)

    def initial_CS(self, name, val):
        if name not in self._fun:
            raise ValueError(f"unknown field {name}")
        self._fun[name] = val

    def add_bc(self, shape, seg, name, bc):
        self._bi.insert(shape, seg, name, bc)

    def set_advection_scheme(self, name):
        if name not in self.SCHEMES:
            raise ValueError(f"unknown scheme {name}")
        rc = _lib.load().carpio_gpu_advection_set_scheme(
            self.handle, _lib.SCHEMES[name])
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_set_scheme")
        self.scheme = name

    def _field(self, name):
        """set_CS (s_equation.hpp:266-287): the function at every cell
        centre, ghosts included, at the current time"""
        g, f = self.grid, self._fun[name]
        if not callable(f):
            return np.full(g.N(), float(f))
        out = g.zeros()
        for I in range(out.shape[0]):
            for J in range(out.shape[1]):
                out[I, J] = f(self.t, g.cx[I], g.cy[J], 0.0)
        return out

    def _set_bc(self, name, t):
        k = ("u", "v", "phi").index(name)
        gv = self._bi.ghost_values(self.grid, name, t) \
            if self._bi.has_function(name) else None
        c = self._bi.to_c(name, functions=True)
        rc = _lib.load().carpio_gpu_advection_set_bc(
            self.handle, k, ctypes.byref(c), _lib.ptr(gv) if gv is not None else None)
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_set_bc")

    def initial(self):
        for nm in ("u", "v", "phi"):
            self._set_bc(nm, self.t)
        fs = [self._field(nm) for nm in ("u", "v", "phi")]
        rc = _lib.load().carpio_gpu_advection_initial(
            self.handle, *[_lib.ptr(f) for f in fs])
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_initial")
        self._ready = True

    def initial_fields(self, u, v, phi):
        """initial() from arrays (the grid's layout, ghosts included, host
        or device) in place of the initial_CS functions"""
        for nm in ("u", "v", "phi"):
            self._set_bc(nm, self.t)
        rc = _lib.load().carpio_gpu_advection_initial(
            self.handle, _lib.ptr(u), _lib.ptr(v), _lib.ptr(phi))
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_initial")
        self._ready = True

    def run(self, steps=None):
        """Equation_::run (s_equation.hpp:132-178): initial() on the first
        call, then max_step + 1 steps (Time_::is_end is current > max,
        s_time.hpp:74-80) unless `steps` is given. Function BCs of phi are
        evaluated at each step's time, as apply_bc does."""
        if self.dt is None:
            raise ValueError("set_time first")
        if not self._ready:
            self.initial()
        n = self.max_step + 1 if steps is None else int(steps)
        L = _lib.load()
        if self._bi.has_function("phi"):
            for _ in range(n):
                self._set_bc("phi", self.t)
                rc = L.carpio_gpu_advection_step(self.handle, self.dt, 1)
                if rc:
                    raise _lib.CarpioGpuError(rc, "advection_step")
                self.t += self.dt
                self.step += 1
        else:
            rc = L.carpio_gpu_advection_step(self.handle, self.dt, n)
            if rc:
                raise _lib.CarpioGpuError(rc, "advection_step")
            for _ in range(n):
                self.t += self.dt
            self.step += n
        return 0

    def get_CS(self, name):
        names = ("u", "v", "uf", "vf", "phi")
        if name not in names:
            raise ValueError(f"unknown field {name}")
        out = self.grid.zeros()
        args = [_lib.ptr(out) if nm == name else None for nm in names]
        rc = _lib.load().carpio_gpu_advection_get(self.handle, *args)
        if rc:
            raise _lib.CarpioGpuError(rc, "advection_get")
        return out

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and _lib._lib is not None and not sys.is_finalizing():
            _lib._lib.carpio_gpu_advection_destroy(h)
            self.handle = None


class NS_kim(NS_explicit):
    """NS_kim_<2> (s_ns_kim.hpp, Kim and Moin 1985) stepping on the GPU:
    configured like NS_explicit; the time-step restriction settings are
    ignored, as the reference's stepper does not call restrict_time."""

    def initial(self):
        super().initial()
        rc = _lib.load().carpio_gpu_ns_set_stepper(self.handle, 1)
        if rc:
            raise _lib.CarpioGpuError(rc, "ns_set_stepper")


def operator(grid, which, a=None, b=None, c=None, scheme=0, coef=0.0,
             bc=None, out1=None, out2=None, rho=None):
    """carpio_gpu_operator on host fields; returns (out1, out2, scalar).
    `rho`: the density of operator 9 (default 1)."""
    L = _lib.load()
    o1 = grid.zeros() if out1 is None else np.array(out1, dtype=np.float64)
    o2 = grid.zeros() if out2 is None else np.array(out2, dtype=np.float64)
    s = ctypes.c_double(0.0 if rho is None else float(rho))
    sch = _lib.SCHEMES[scheme] if isinstance(scheme, str) else int(scheme)
    keep = [None if x is None else np.ascontiguousarray(x, dtype=np.float64)
            for x in (a, b, c)]
    rc = L.carpio_gpu_operator(
        grid.handle, int(which), sch, float(coef),
        ctypes.byref(bc) if bc is not None else None,
        *[_lib.ptr(x) if x is not None else None for x in keep],
        _lib.ptr(o1), _lib.ptr(o2), ctypes.byref(s))
    if rc:
        raise _lib.CarpioGpuError(rc, f"operator {which}")
    return o1, o2, s.value
