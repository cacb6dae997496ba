"""Batched Poisson solves (carpio_gpu_batch_*, include/carpio_gpu.h).

Many independent Poisson_::run() problems on uniform grids of uneven sizes in
one persistent launch of thread-block clusters, replayed from a CUDA graph.
Each problem is solved as carpio_gpu_poisson_solve solves one grid with the
MIXED CG (FP32 inner iterations inside FP64 residuals and mean removal), to the
reference's relative-residual test. The reference has no batched solver; a
loop of Poisson_::run() calls is what this replaces.

Fields are given per problem as interior arrays of shape (nx, ny) (y
contiguous), on the host (numpy) or on the device (torch CUDA tensors).
"""
import ctypes
import sys

import numpy as np

from . import _lib

DIRICHLET, NEUMANN = 1, 2


class Problem:
    """One Poisson_ problem of a batch: an nx x ny uniform grid on `box`,
    boundary conditions per segment (x-, x+, y-, y+) as (type, value) with
    type 1 Dirichlet / 2 Neumann, uniform beta. `mean_removal` defaults to
    True exactly for all-Neumann boundaries (the null space)."""

    def __init__(self, nx, ny, box=((0.0, 0.0), (1.0, 1.0)), bc=None,
                 beta=1.0, mean_removal=None):
        self.nx, self.ny = int(nx), int(ny)
        self.box = ((float(box[0][0]), float(box[0][1])),
                    (float(box[1][0]), float(box[1][1])))
        self.bc = list(bc) if bc is not None else [(DIRICHLET, 0.0)] * 4
        if len(self.bc) != 4:
            raise ValueError("bc needs one (type, value) per segment")
        self.beta = float(beta)
        neumann = all(t == NEUMANN for t, _ in self.bc)
        self.mean_removal = neumann if mean_removal is None else bool(mean_removal)

    def to_c(self):
        p = _lib.BatchProblem()
        p.nx, p.ny = self.nx, self.ny
        (p.xmin, p.ymin), (p.xmax, p.ymax) = self.box
        for k, (t, v) in enumerate(self.bc):
            p.bc.type[k] = int(t)
            p.bc.value[k] = float(v)
        p.mean_removal = 1 if self.mean_removal else 0
        p.beta = self.beta
        return p


def _problems_c(problems):
    arr = (_lib.BatchProblem * len(problems))()
    for i, pr in enumerate(problems):
        arr[i] = pr.to_c()
    return arr


def _tiles_c(tiles):
    t = _lib.BatchTiles()
    if tiles:
        t.threads = int(tiles.get("threads", 0))
        t.cluster = int(tiles.get("cluster", 0))
        t.cells_per_cta = int(tiles.get("cells_per_cta", 0))
        t.use_graph = int(tiles.get("use_graph", 0))
    return t


def _check(rc, what):
    if rc < 0:
        raise _lib.CarpioGpuError(rc, what)
    return rc


def plan(problems, tiles, clusters):
    """Host-only planning: team size and cluster slot of every problem and the
    estimated makespan (ms) for `clusters` clusters of the given tiles."""
    L = _lib.load()
    n = len(problems)
    team = np.zeros(n, np.int32)
    slot = np.zeros(n, np.int32)
    est = ctypes.c_double()
    t = _tiles_c(tiles)
    _check(L.carpio_gpu_batch_plan(n, _problems_c(problems), ctypes.byref(t),
                                   int(clusters),
                                   team.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   slot.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   ctypes.byref(est)), "carpio_gpu_batch_plan")
    return team, slot, est.value


def shard(problems, world):
    """Host-only: the rank (0..world-1) of every problem, balancing estimated
    work across processes (largest first onto the least-loaded rank)."""
    L = _lib.load()
    n = len(problems)
    out = np.zeros(n, np.int32)
    _check(L.carpio_gpu_batch_shard(n, _problems_c(problems) if n else None,
                                    int(world),
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))),
           "carpio_gpu_batch_shard")
    return out


class BatchedPoisson:
    """A planned batch with its device fields. solve() = upload sources (and
    initial guesses), run, download solutions."""

    def __init__(self, problems, tol=1e-8, max_iter=100000, inner_tol=3e-2,
                 flags=0, tiles=None):
        self._L = _lib.load()
        self.problems = list(problems)
        self.n = len(self.problems)
        cfg = _lib.SolverCfg()
        cfg.kind = _lib.CG
        cfg.precision = _lib.MIXED
        cfg.max_iter = int(max_iter)
        cfg.tol = float(tol)
        cfg.mean_removal = 0
        cfg.inner_tol = float(inner_tol)
        cfg.inner_max_iter = 0
        cfg.flags = int(flags)
        self._h = ctypes.c_void_p()
        t = _tiles_c(tiles)
        _check(self._L.carpio_gpu_batch_create(
            self.n, _problems_c(self.problems), ctypes.byref(cfg),
            ctypes.byref(t) if tiles else None, ctypes.byref(self._h)),
            "carpio_gpu_batch_create")
        self.stats = None
        self.ms = None

    def _ptrs(self, fields):
        if len(fields) != self.n:
            raise ValueError("one field per problem")
        keep, ptrs = [], (ctypes.c_void_p * self.n)()
        for i, (f, pr) in enumerate(zip(fields, self.problems)):
            if hasattr(f, "data_ptr"):
                if tuple(f.shape) != (pr.nx, pr.ny) or not f.is_contiguous():
                    raise ValueError(f"field {i}: want contiguous ({pr.nx}, {pr.ny})")
                ptrs[i] = f.data_ptr()
            else:
                a = np.ascontiguousarray(f, dtype=np.float64)
                if a.shape != (pr.nx, pr.ny):
                    raise ValueError(f"field {i}: want shape ({pr.nx}, {pr.ny})")
                keep.append(a)
                ptrs[i] = a.ctypes.data
        return ptrs, keep

    def upload(self, which, fields):
        ptrs, keep = self._ptrs(fields)
        _check(self._L.carpio_gpu_batch_upload(self._h, int(which), ptrs),
               "carpio_gpu_batch_upload")
        del keep

    def download(self, which=1):
        out = [np.empty((p.nx, p.ny)) for p in self.problems]
        ptrs = (ctypes.c_void_p * self.n)(*[a.ctypes.data for a in out])
        _check(self._L.carpio_gpu_batch_download(self._h, int(which), ptrs),
               "carpio_gpu_batch_download")
        return out

    def field_address(self, which, i):
        """device address of problem i's field (one ghost layer, zero ring)"""
        p = ctypes.c_void_p()
        _check(self._L.carpio_gpu_batch_field(self._h, int(which), int(i),
                                              ctypes.byref(p)),
               "carpio_gpu_batch_field")
        return p.value

    def zero(self, which):
        _check(self._L.carpio_gpu_batch_zero(self._h, int(which)),
               "carpio_gpu_batch_zero")

    def run(self):
        """Solves every problem on the device fields; returns the batch code
        (0 all converged, 1 some reached max_iter). Per-problem stats in
        self.stats, device ms of the launch in self.ms."""
        st = (_lib.SolverStats * self.n)()
        ms = ctypes.c_double()
        rc = self._L.carpio_gpu_batch_run(self._h, st, ctypes.byref(ms))
        _check(rc, "carpio_gpu_batch_run")
        self.stats = [dict(code=s.code, iters=s.iters, resid=s.tol_out,
                           updates=s.outer_iters, ms=s.ms) for s in st]
        self.ms = ms.value
        return rc

    def solve(self, sources, phi0=None):
        self.upload(0, sources)
        if phi0 is None:
            self.zero(1)
        else:
            self.upload(1, phi0)
        self.run()
        return self.download(1)

    def autotune(self, max_candidates=18):
        _check(self._L.carpio_gpu_batch_autotune(self._h, int(max_candidates)),
               "carpio_gpu_batch_autotune")
        return self.info()

    def info(self):
        inf = _lib.BatchInfo()
        _check(self._L.carpio_gpu_batch_get_info(self._h, ctypes.byref(inf)),
               "carpio_gpu_batch_get_info")
        t = inf.tiles
        return dict(threads=t.threads, cluster=t.cluster,
                    cells_per_cta=t.cells_per_cta, use_graph=t.use_graph >= 0,
                    clusters=inf.clusters, ctas=inf.ctas,
                    smem_bytes=inf.smem_bytes, teams=list(inf.teams),
                    est_ms=inf.est_ms, candidates=inf.candidates,
                    tuned_ms=inf.tuned_ms)

    def close(self):
        if self._h:
            self._L.carpio_gpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        if not sys.is_finalizing():
            try:
                self.close()
            except Exception:
                pass
