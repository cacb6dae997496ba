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
    """BoundaryCondition (s_boundary.hpp:10-130); default Neumann 0."""
    BC1, BC2 = 1, 2

    def __init__(self):
        self.type, self.value = 2, 0.0

    def set_default_1_bc(self, val):
        self.type, self.value = 1, float(val)

    def set_default_2_bc(self, val):
        self.type, self.value = 2, float(val)


class BoundaryIndex:
    """BoundaryIndex (s_boundary.hpp:132-234) for one shape (0): per
    variable name and segment, default Neumann 0."""

    def __init__(self):
        self._m = {}

    def insert(self, shape, seg, name, bc):
        if shape != 0 or seg not in (0, 1, 2, 3):
            raise ValueError("regular grids have shape 0, segments 0..3")
        self._m[(seg, name)] = bc

    def to_c(self, name):
        c = _lib.BC()
        for s in range(4):
            bc = self._m.get((s, name), BoundaryCondition())
            c.type[s] = bc.type
            c.value[s] = bc.value
        return c


def solver_cfg(name="CG", max_iter=1000, tol=1e-3, mean_removal=False,
               precision="fp64", inner_tol=0.0, inner_max_iter=0, flags=0,
               poly_degree=0, poly_ratio=0.0):
    c = _lib.SolverCfg()
    c.poly_degree = int(poly_degree)
    c.poly_ratio = float(poly_ratio)
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
    "BiCGSTAB" (the carpio:: solvers)."""

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
                              precision="fp64", **kw):
        self.proj = solver_cfg(name, max_iter, tol, mean_removal=True,
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
             bc=None, out1=None, out2=None):
    """carpio_gpu_operator on host fields; returns (out1, out2, scalar)."""
    L = _lib.load()
    o1 = grid.zeros() if out1 is None else np.array(out1, dtype=np.float64)
    o2 = grid.zeros() if out2 is None else np.array(out2, dtype=np.float64)
    s = ctypes.c_double(0.0)
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
