"""Benchmark of the projection hot path: lid-driven cavity steps/s at 1024^2.

Workload (the 1024^2 cavity configuration): uniform 1024x1024 cells on
[0,1]^2, gl = 2, Re = 1000 (rho = 1000, mu = 1), lid u = 1 on the top wall,
no-slip elsewhere, van Leer TVD advection, explicit diffusion, CFL 0.5 and
diffusion number 0.25, dt0 = 0.5 h; all-Neumann pressure Poisson solved to
1e-8 relative residual with mean removal, FP32 inner CG inside FP64
iterative refinement. Synthetic state: the cavity started from rest; W
warm-up steps, then K timed steps. One "step" = NS_explicit_::run_one_step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's CPU implementation of the same step
(its restatement in oracle/: CSR assembly + carpio::CG to 1e-8 with mean
removal, FP64, on all host threads) on rank 0: W untimed steps from rest,
then K timed full steps. The reference has no GPU path.

The line also carries: `roofline` of the projection solve on the Krylov bytes
of the measurement contract (40 B/cell per FP32 CG iteration, 40 B/cell per
FP64 refinement step), `accuracy` (the mixed against the FP64 projection
after the same steps, and both against the CPU oracle on the first step),
`cpu_baseline` (the oracle timed on steps 2..4 from rest), and the legs of
the other configurations (FP64 projection, Poisson to 1e-8, learned,
batched, next rows).

Timing: CUDA events on the library's launching stream around each step
(carpio_gpu_ns_profile), max over ranks. The per-step working set (10
fields + the Krylov vectors, ~200 MB) is larger than the 129 MB L2, so no
flush is inserted between steps. e2e: the same steps through the public API
with pinned host buffers, the step's inputs (u, v, uf, vf, phi, dt) copied
host->device before and the full state device->host after every step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 1024
TOL = 1e-8
RE = 1000.0
METRIC = "cavity_steps_per_s_1024"
# kernels the library launches per projection step (restrict_time, 3 ghost
# fills, predictor, C2F, the persistent projection solve, correction)
LAUNCHES_PER_STEP = 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="FP64 residual replacement after this FP32 reduction (0: library default)")
    ap.add_argument("--poly-degree", type=int, default=0,
                    help="band-local Chebyshev degree of the FP32 CG (0 default, -1 none)")
    ap.add_argument("--poly-ratio", type=float, default=0.0)
    ap.add_argument("--precond", default="default",
                    choices=["default", "spectral", "chebyshev", "multigrid"],
                    help="the mixed solve's FP32 stage (default: spectral where it "
                         "applies, else multigrid)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64 comparison, Poisson, learned, batched, next-row and CPU legs")
    ap.add_argument("--oracle-steps", type=int, default=3,
                    help="accuracy run: steps also run by the CPU oracle")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of the bench line: run the mixed and the FP64 "
                         "projections side by side for this many steps and print "
                         "their per-step relative L2 differences and solve times")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def config(n):
    """the workload, identical in both arms (what is solved, not how)"""
    return {"workload": f"lid-driven cavity {n}x{n}, Re 1000, van Leer, "
                        f"all-Neumann pressure Poisson to {TOL:g} relative "
                        f"residual with mean removal",
            "n": n, "Re": RE, "scheme": "VanLeer", "tol": TOL,
            "cfl": 0.5, "diffusion_number": 0.25, "dt0": 0.5 / n,
            "start": "from rest; W untimed steps, then K timed steps",
            "l2": "per-step working set ~200 MB > 129 MB L2; no flush",
            "parallelism": "replicas"}


def spectral_applies(n):
    """the cavity's pressure operator (uniform grid and coefficient, all
    Neumann) takes the spectral preconditioner when its side is a power of
    two"""
    return PRECOND[0] in ("default", "spectral") and n >= 2 and (n & (n - 1)) == 0


def solver_desc(precision, inner_tol, n=1024):
    """how our arm solves the projection"""
    if precision != "mixed":
        pre = None
    elif spectral_applies(n):
        pre = ("spectral: M = A^-1 through the DCT-II of both axes (FP32 FFTs "
               "in shared memory, two grid barriers per application), iterative "
               "refinement with double-float residuals")
    elif PRECOND[0] in ("multigrid", "default", "spectral"):
        pre = ("geometric multigrid V(1,1)-cycle (damped Jacobi, bilinear "
               "prolongation, restriction its transpose)")
    elif POLY[0] < 0:
        pre = "none"
    else:
        pre = (f"band-local Chebyshev degree {POLY[0] or 5}, "
               f"interval [2/{POLY[1] or 30:g}, 2] of D^-1 A")
    return {"precision": precision, "inner_tol": inner_tol, "fp32_preconditioner": pre}


# preconditioner of the on-chip FP32 CG: band-local Chebyshev (degree, ratio;
# 0 = defaults) and the choice between it and the multigrid V-cycle
POLY = [0, 0.0]
PRECOND = ["default"]


def make_cavity(n, precision, inner_tol):
    from carpio_gb300 import structure as S
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 2)
    ns = S.NS_explicit(g)
    ns.set_advection_scheme("VanLeer")
    ns.set_time(0, 0.5 / n)
    bc0, bc1 = S.BoundaryCondition(), S.BoundaryCondition()
    bc0.set_default_1_bc(0.0)
    bc1.set_default_1_bc(1.0)
    for s in range(3):
        ns.add_bc(0, s, "u", bc0)
    ns.add_bc(0, 3, "u", bc1)
    for s in range(4):
        ns.add_bc(0, s, "v", bc0)
    ns.set_uniform_rho(RE)
    ns.set_diffusion_number(0.25, 1.0 / RE)
    ns.set_projection_solver("CG", 200000, TOL, precision=precision,
                             inner_tol=inner_tol, poly_degree=POLY[0], poly_ratio=POLY[1],
                             precond=PRECOND[0])
    ns.initial()
    return g, ns


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def poly_degree(n=1024):
    """degree of the FP32 CG's band-local Chebyshev preconditioner in use
    (-1: the multigrid V-cycle, -2: the spectral preconditioner)"""
    if spectral_applies(n):
        return -2
    if PRECOND[0] in ("multigrid", "default", "spectral"):
        return -1
    return 0 if POLY[0] < 0 else (POLY[0] or 5)


def solve_bytes(precision, inner, outer, deg=0):
    """Algorithmic bytes per cell of one projection-solve launch, split into
    the Krylov part (the per-kernel figures of the measurement contract) and
    the band-local preconditioner's passes, which that table does not list.

    Krylov: FP32 inner CG iteration 40 B (K1: p = z + beta p, q = A p, p.q;
    K2: x += alpha p, r -= alpha q, r.r; 4 B vectors, neighbours counted
    once); FP64 refinement step 40 B (r = b - A x, update x, mean removal),
    one more for the first residual; FP64 CG iteration 80 B.
    Preconditioner, per FP32 iteration: first Chebyshev step 20 B (read r,
    D; write d, z, r_k), each further step 28 B (read d, r_k, z, D; write d,
    r_k, z), the (r, z) dot 8 B; the multigrid V-cycle (deg = -1) 32 B per
    fine cell (write r and the pre-smoothed z; read z and D, write the
    residual; read it for the restriction; read z and D for the post-
    smoothing) and a quarter of that again per coarser level (x 4/3); the
    spectral preconditioner (deg = -2) 32 B per cell and application (rows:
    read r, write the workspace; columns: read and write it twice; rows back:
    read it, write z), applied once per FP32 iteration and once per
    refinement that does not converge (the first residual's included)."""
    if precision == "mixed":
        krylov = 40 * inner + 40 * (outer + 1)
        if deg > 0:
            pre = (20 + 28 * (deg - 1) + 8) * inner
        elif deg == -2:
            pre = 32 * (inner + outer)
        elif deg < 0:
            pre = 32 * 4 / 3 * inner
        else:
            pre = 0
        return krylov, pre
    return 80 * inner, 0


def traffic_per_launch(n, precision):
    """DRAM bytes of one projection-solve launch from the committed ncu
    capture of this kernel at this size, or None"""
    if precision != "mixed":
        return None
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        rec = t["launches"][str(n)]
        return float(rec["dram_bytes"])
    except (OSError, KeyError, ValueError):
        return None


def oracle_cavity(n, threads):
    """the reference's CPU step (oracle restatement of NS_explicit_ with CSR
    assembly + carpio::CG to 1e-8 and mean removal, FP64) on a cavity of n^2
    from rest; returns (grid, state, step function) where step() runs one
    full step and returns (seconds, CG iterations, code)"""
    from oracle import restate as R
    R.lib()
    g = R.Grid(n, n, 2)
    st = R.new_state(g, 0.5 / n)

    def step():
        t0 = time.perf_counter()
        code, _, its, _ = R.ns_run(g, st, 1, scheme="vanleer", cg_tol=TOL,
                                   cg_max_iter=200000, threads=threads)
        return time.perf_counter() - t0, int(its[0]), int(code)
    return g, st, step


def run_reference(a):
    """the reference arm: the reference algorithm on the host cores, W
    untimed steps from rest, then K timed full steps"""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = a.n
    _, _, step = oracle_cavity(n, threads)
    for _ in range(a.warmup):
        step()
    t, its = [], []
    for _ in range(a.steps):
        dt, it, code = step()
        assert code == 0, f"reference step failed: code {code}"
        t.append(dt)
        its.append(it)
    el = float(np.sum(t))
    v = a.steps / el
    sample = (f"steps {a.warmup + 1}..{a.warmup + a.steps} of the {n}^2 cavity from "
              f"rest, each a full step (FP64 CG to {TOL:g}, mean removal; "
              f"{int(np.mean(its))} CG iterations a step on average), oracle "
              f"restatement of the reference on {threads} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s",
        "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * el / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (cavity from rest)",
        "config": config(n),
        "solver": {"precision": "fp64", "kind": "carpio::CG with mean removal"},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "cg_iters_per_step": float(np.mean(its)),
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def rel_l2(x, y):
    ref = np.linalg.norm(y)
    return float(np.linalg.norm(x - y) / ref) if ref > 0 else float(np.linalg.norm(x))


def cpu_baseline_leg(n, threads, gpu_step1):
    """The reference's CPU step on the host cores, on a bounded sample: the
    oracle runs steps 1..4 of the cavity from rest, full steps; steps 2..4
    are timed. Step 1 also checks the GPU's first step (FP64 and mixed
    projections) against the oracle: relative L2 of u, v, p."""
    g, st, step = oracle_cavity(n, threads)
    step()
    check = {}
    for label, fields in gpu_step1.items():
        check[label] = {k: rel_l2(fields[k], g.interior(st[k])) for k in ("u", "v", "p")}
    t, its = [], []
    for _ in range(3):
        dt, it, _ = step()
        t.append(dt)
        its.append(it)
    return {"value": len(t) / float(np.sum(t)), "unit": "steps/s", "cores": threads,
            "kind": "port",
            "sample": f"steps 2..4 of the {n}^2 cavity from rest, full steps "
                      f"(FP64 CG to {TOL:g} with mean removal, {int(np.mean(its))} "
                      f"CG iterations a step), oracle restatement on {threads} threads"}, check


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
        return
    POLY[0], POLY[1] = a.poly_degree, a.poly_ratio
    PRECOND[0] = a.precond
    if a.accuracy_steps > 0:
        accuracy_run(a)
        return
    ws, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from carpio_gb300 import _lib
    _lib.load()
    n = a.n
    g, ns = make_cavity(n, a.precision, a.inner_tol)
    # warm-up (also builds the coefficient cache)
    if a.warmup > 0:
        rc = ns.run(a.warmup)
        assert rc == 0, f"warm-up failed: {_lib.strerror(rc)}"
    clocks = Clocks(local)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # the state before the timed steps, in pinned host memory: the e2e leg
    # replays the same steps from it through the public API
    st = ns.state()
    host = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory()
            for k in ("u", "v", "uf", "vf", "phi", "p")}
    dt0 = st["dt"]
    snap = {k: v.clone() for k, v in host.items()}
    barrier()
    clocks.start()
    t0 = time.perf_counter()
    rc = ns.run(a.steps)
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    assert rc == 0, f"timed steps failed: {_lib.strerror(rc)}"
    prof = ns.profile()
    dev_s = float(np.sum(prof["step_ms"])) / 1e3
    elapsed = dev_s
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = ws * a.steps / elapsed
    inner = float(np.mean(prof["inner"]))
    outer = float(np.mean(prof["outer"]))
    solve_ms = float(np.mean(prof["solve_ms"]))
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * elapsed / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if a.precision == "mixed" else "f64",
        "data": "synthetic (cavity from rest)",
        "config": config(n),
        "solver": solver_desc(a.precision, a.inner_tol, n),
        "gpu_launches": LAUNCHES_PER_STEP * a.steps,
        "clocks": clk,
        "wall_ms_per_step": 1e3 * wall / a.steps,
        "projection": {"solve_ms": solve_ms, "inner_iters": inner,
                       "outer_iters": outer,
                       "us_per_inner_iter": 1e3 * solve_ms / max(inner, 1.0),
                       "share_of_step": solve_ms / (1e3 * dev_s / a.steps)},
    }
    # roofline of the dominant kernel (the persistent projection solve) on
    # the Krylov bytes of the measurement contract; the preconditioner's
    # passes are reported beside it
    peak, how = peaks()
    kry, pre = solve_bytes(a.precision, inner, outer,
                           poly_degree(n) if a.precision == "mixed" else 0)
    achieved = kry * n * n / (solve_ms / 1e3) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak,
                       "unit": "GB/s", "frac": achieved / peak,
                       "peak_source": how,
                       "traffic": traffic_per_launch(n, a.precision),
                       "algorithmic_bytes_per_launch": kry * n * n,
                       "bytes_model": ("40 B/cell per FP32 CG iteration + 40 B/cell per "
                                       "FP64 refinement step" if a.precision == "mixed"
                                       else "80 B/cell per FP64 CG iteration"),
                       "preconditioner_bytes_per_launch": pre * n * n,
                       "kernel": ("k_poisson_mixed_tile" if a.precision == "mixed"
                                  else "k_poisson") + " (persistent projection solve)"}
    if a.precision == "mixed":
        out["roofline"]["note"] = (
            "the solve's vectors stay in shared memory, registers and L2: DRAM "
            "traffic is `traffic`, far below the algorithmic bytes; the kernel "
            "is bound by grid synchronisation latency and its spectral "
            "applications (with the spectral preconditioner: iterative "
            "refinement, per refinement one application with two grid "
            "barriers, a grid barrier and one residual all-reduce; the "
            "residuals in double-float on the FP32 pipe)")
    # e2e through the public API with host buffers: the timed steps again,
    # from the same starting state, each step copying its inputs in from
    # pinned host memory (u, v, uf, vf, phi and dt; p is only an output:
    # the step overwrites every element of it) and the whole state back out
    for k, v in snap.items():
        host[k].copy_(v)
    dt = dt0
    ins = ("u", "v", "uf", "vf", "phi")
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        ns.set_state(dt, **{k: host[k] for k in ins})
        rc = ns.run(1)
        if rc != 0:
            break
        dt = ns.state(out=host)["dt"]
    barrier()
    e_el = time.perf_counter() - t0
    assert rc == 0, f"e2e steps failed: {_lib.strerror(rc)}"
    nbytes = sum(v.numel() * v.element_size() for v in host.values())
    nin = sum(host[k].numel() * host[k].element_size() for k in ins)
    out["e2e"] = {"value": ws * a.steps / e_el, "unit": "steps/s",
                  "h2d_bytes_per_step": nin + 8,
                  "d2h_bytes_per_step": nbytes + 8,
                  "steps": a.steps}
    if not a.no_extras and rank == 0:
        # the other projection on the same workload, same GPU, same steps
        other = "fp64" if a.precision == "mixed" else "mixed"
        g2, ns2 = make_cavity(n, other, a.inner_tol)
        ns2.run(a.warmup)
        torch.cuda.synchronize()
        ns2.run(a.steps)
        p2 = ns2.profile()
        leg = {"steps_per_s": a.steps / (float(np.sum(p2["step_ms"])) / 1e3),
               "solve_ms": float(np.mean(p2["solve_ms"])),
               "iters": float(np.mean(p2["inner"]))}
        if other == "fp64":
            # k_poisson's own roofline: 80 B/cell per FP64 CG iteration
            gbs = 80.0 * leg["iters"] * n * n / (leg["solve_ms"] / 1e3) / 1e9
            leg["roofline"] = {"achieved": gbs, "peak": peak, "frac": gbs / peak,
                               "unit": "GB/s", "peak_source": how,
                               "us_per_iter": 1e3 * leg["solve_ms"] / max(leg["iters"], 1.0)}
        out[f"{other}_projection"] = leg
        # accuracy: the two projections after the same W + K steps
        s1, s2 = ns.state(), ns2.state()
        out["accuracy"] = {
            f"{a.precision}_vs_{other}_after_{a.warmup + a.steps}_steps":
                {k: rel_l2(g.interior(s1[k]), g2.interior(s2[k])) for k in ("u", "v", "p")}}
        del ns2
        # Poisson ms to 1e-8 on the same divergence field: FP64 CG vs mixed
        # vs the learned preconditioner, and on a held-out 512^2 field
        out["poisson_ms_to_1e-8"] = poisson_leg(n, a.inner_tol)
        out["poisson_512_heldout"] = heldout_leg(512)
        out["learned_cavity"] = learned_cavity_leg(n, a.inner_tol)
        out["unet_forward"] = unet_leg(n)
        out["batched_512"] = batched_leg()
        out["next_rows"] = next_rows_leg()
        if ws == 1:
            # the first step of both projections from rest, for the check
            # against the CPU oracle inside the CPU-baseline leg
            first = {}
            for prec in ("fp64", "mixed"):
                gq, nq = make_cavity(n, prec, a.inner_tol)
                assert nq.run(1) == 0
                sq = nq.state()
                first[prec] = {k: gq.interior(sq[k]) for k in ("u", "v", "p")}
                del nq
            threads = os.cpu_count() or 1
            cb, check = cpu_baseline_leg(n, threads, first)
            cb["next_rows"] = cpu_next_rows(threads)
            out["cpu_baseline"] = cb
            for prec, errs in check.items():
                out["accuracy"][f"{prec}_vs_cpu_oracle_step1"] = errs
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cone_fields(g):
    """solid rotation of a cone on a grid's cells (ghosts included):
    u = -(y - 1/2), v = x - 1/2, phi = 1 - r^2 / 0.04 within r < 0.2 of
    (0.5, 0.75)"""
    X, Y = np.meshgrid(g.cx, g.cy, indexing="ij")
    dx, dy = X - 0.5, Y - 0.75
    r2 = dx * dx + dy * dy
    return -(Y - 0.5), X - 0.5, np.where(r2 < 0.04, 1.0 - r2 / 0.04, 0.0)


def advection_case(n):
    """stand-alone Advection_ on n^2: the rotating cone, van Leer, the
    default (Neumann 0) boundaries, dt = 0.25 / n"""
    from carpio_gb300 import structure as S
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 2)
    eq = S.Advection(g)
    eq.set_time(0, 0.25 / n)
    eq.set_advection_scheme("VanLeer")
    eq.initial_fields(*cone_fields(g))
    return g, eq


def ic_case(n, kind):
    """the shipped IC solvers at the structure level: n^2 Dirichlet-0
    Poisson with a unit source, to 1e-8 (FP64)"""
    from carpio_gb300 import structure as S
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 1)
    p = S.Poisson(g)
    bc = S.BoundaryCondition()
    bc.set_default_1_bc(0.0)
    for seg in range(4):
        p.add_bc(0, seg, "phi", bc)
    p.set_source(np.ones(g.N()))
    p.set_solver(kind, max_iter=10000, tol=TOL)
    return g, p


def next_rows_leg(steps=5):
    """The rows beyond the projection path, on the GPU: stand-alone
    Advection_ (1024^2 rotating cone), the NS_kim_ stepper (256^2 cavity),
    the structure-level IC_CGS / IC_CG (128^2 Poisson); wall time of the
    synchronous calls, after one warm-up"""
    import torch
    out = {}
    n = 1024
    g, eq = advection_case(n)
    eq.run(1)
    t0 = time.perf_counter()
    eq.run(steps)
    ms = 1e3 * (time.perf_counter() - t0) / steps
    out["advection_1024"] = {"ms_per_step": ms, "mcell_steps_per_s": n * n / ms / 1e3,
                             "steps": steps, "scheme": "VanLeer",
                             "kernel": "k_advect_rows (one lane per grid row, four warps "
                                       "per band computing one TVD face each)"}
    del eq
    from carpio_gb300 import structure as S
    m = 256
    gk = S.Grid((0.0, 0.0), (1.0, 1.0), (m, m), 2)
    ns = S.NS_kim(gk)
    ns.set_advection_scheme("VanLeer")
    ns.set_time(0, 0.5 / m)
    bc0, bc1 = S.BoundaryCondition(), S.BoundaryCondition()
    bc0.set_default_1_bc(0.0)
    bc1.set_default_1_bc(1.0)
    for sg in range(3):
        ns.add_bc(0, sg, "u", bc0)
    ns.add_bc(0, 3, "u", bc1)
    for sg in range(4):
        ns.add_bc(0, sg, "v", bc0)
    ns.set_uniform_rho(RE)
    ns.set_projection_solver("CG", 200000, TOL)
    ns.initial()
    ns.run(1)
    torch.cuda.synchronize()
    ns.run(steps)
    pk = ns.profile()
    out["ns_kim_256"] = {"steps_per_s": steps / (float(np.sum(pk["step_ms"])) / 1e3),
                         "projection_iters": float(np.mean(pk["inner"])), "steps": steps}
    del ns
    for kind in ("IC_CGS", "IC_CG"):
        gi, p = ic_case(128, kind)
        p.run()
        gi, p = ic_case(128, kind)   # a fresh solve from phi = 0
        t0 = time.perf_counter()
        p.run()
        out[f"{kind.lower()}_128"] = {"ms": 1e3 * (time.perf_counter() - t0),
                                      "iters": int(p.stats.iters),
                                      "resid": float(p.stats.tol_out),
                                      "code": int(p.stats.code)}
    return out


def cpu_next_rows(threads):
    """The same rows on the host, by the oracle restatement: Advection_ one
    step at 1024^2 and IC_CGS / IC_CG on the assembled 128^2 system on one
    thread (the reference's loops are sequential), an NS_kim_ step at 256^2
    with the projection CG on all threads."""
    from oracle import restate as R
    out = {}
    n = 1024
    og = R.Grid(n, n, 2)
    u, v, phi = cone_fields(og)
    nb = R.BC()
    for k in range(4):
        nb.type[k], nb.value[k] = 2, 0.0
    u = R.apply_bc(og, nb, u)
    v = R.apply_bc(og, nb, v)
    uf, vf = R.c2f(og, u, v)
    t0 = time.perf_counter()
    R.advect_run(og, "vanleer", nb, uf, vf, 0.25 / n, 1, phi)
    ms = 1e3 * (time.perf_counter() - t0)
    out["advection_1024"] = {"ms_per_step": ms, "cores": 1, "sample": "one step"}
    # NS_kim_: one step of the 256^2 cavity (dt 0.5 / 256) after one from rest
    k = 256
    gk = R.Grid(k, k, 2)
    stk = {nm: gk.zeros() for nm in ("u", "v", "uf", "vf", "phi", "p", "us", "vs",
                                     "usf", "vsf")}
    stk["step"] = 0
    R.kim_run(gk, stk, 1, 0.5 / k, Re=RE, scheme="vanleer", cg_tol=TOL,
              cg_max_iter=200000, threads=threads)
    t0 = time.perf_counter()
    R.kim_run(gk, stk, 1, 0.5 / k, Re=RE, scheme="vanleer", cg_tol=TOL,
              cg_max_iter=200000, threads=threads)
    out["ns_kim_256"] = {"steps_per_s": 1.0 / (time.perf_counter() - t0),
                         "cores": threads, "sample": "the second step from rest"}
    m = 128
    gi = R.Grid(m, m, 1)
    db = R.BC()
    for k in range(4):
        db.type[k], db.value[k] = 1, 0.0
    rp, ci, va, b = R.assemble_poisson(gi, db, 1.0, None, 1.0)
    for kind in ("ic_cgs", "ic_cg"):
        t0 = time.perf_counter()
        code, x, its, tol_out, _ = R.krylov_csr(kind, rp, ci, va, b, np.zeros(b.size),
                                                10000, TOL)
        out[f"{kind}_128"] = {"ms": 1e3 * (time.perf_counter() - t0), "iters": int(its),
                              "cores": 1, "sample": "one solve, assembled system"}
    return out


def poisson_leg(n, inner_tol):
    """Poisson time to 1e-8 relative residual on a synthetic smooth field
    (sum of 8 seeded Gaussians, zero mean, all-Neumann): FP64 CG vs FP32
    inner / FP64 refinement, device time of the solve."""
    from carpio_gb300 import structure as S
    rng = np.random.default_rng(1234)
    g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 2)
    X, Y = np.meshgrid(g.cx, g.cy, indexing="ij")
    src = np.zeros(g.N())
    for _ in range(8):
        cx, cy = rng.uniform(0, 1, 2)
        w = rng.uniform(0.02, 0.2)
        src += rng.normal() * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    res = {}
    for prec in ("fp64", "mixed"):
        P = S.Poisson(g)
        P.set_depend(g.zeros(), None, src)
        P.set_solver("CG", None, 200000, TOL, mean_removal=True, precision=prec,
                     inner_tol=inner_tol, poly_degree=POLY[0], poly_ratio=POLY[1],
                     precond=PRECOND[0])
        P.run()   # warm-up
        P.set_depend(g.zeros(), None, src)
        rc = P.run()
        res[prec] = {"ms": P.stats.ms, "iters": P.stats.iters,
                     "outer": P.stats.outer_iters, "resid": P.stats.tol_out,
                     "code": rc}
    if learned_ok(n):
        from carpio_gb300.unet import load_trained
        net = load_trained()
        for label, use in (("learned", True), ("fcg_without_net", False)):
            P = S.Poisson(g)
            P.set_depend(g.zeros(), None, src)
            P.set_solver("CG", None, 200000, TOL, mean_removal=True, precision="mixed",
                         inner_tol=inner_tol)
            P.set_learned(net if use else None, use_net=use, fallback=True)
            P.run()   # warm-up
            P.set_depend(g.zeros(), None, src)
            rc = P.run()
            res[label] = {"ms": P.stats.ms, "iters": P.stats.iters,
                          "fcg_iters": P.stats.outer_iters,
                          "fallback_iters": P.stats.iters - P.stats.outer_iters,
                          "resid": P.stats.tol_out, "code": rc}
    res["speedup_mixed_over_fp64"] = res["fp64"]["ms"] / res["mixed"]["ms"]
    if "learned" in res:
        res["speedup_learned_over_fp64"] = res["fp64"]["ms"] / res["learned"]["ms"]
    return res


def learned_ok(n):
    h3 = n // 8
    return n % 8 == 0 and n >= 16 and min(h3, 128) * min(h3, 128 // min(h3, 128)) == 128


def heldout_leg(n):
    """a held-out 512^2 random potential field (the training generator with
    an unseen seed): iterations and device ms to 1e-8 of FP64 CG, the mixed
    CG, flexible CG with the trained network and without it"""
    from carpio_gb300 import structure as S, train as T
    from carpio_gb300.unet import load_trained
    net = load_trained()
    phi = T.random_potentials(1, n, seed=20251203)[0]
    b = T.neumann_laplacian(phi).cpu().numpy()
    res = {}
    for label in ("fp64", "mixed", "learned", "fcg_without_net"):
        g = S.Grid((0.0, 0.0), (1.0, 1.0), (n, n), 1)
        P = S.Poisson(g)
        for seg in range(4):
            bc = S.BoundaryCondition()
            bc.set_default_2_bc(0.0)
            P.add_bc(0, seg, "phi", bc)
        src = g.zeros()
        src[1:-1, 1:-1] = -b * n * n
        P.set_solver("CG", None, 200000, TOL, mean_removal=True,
                     precision="fp64" if label == "fp64" else "mixed")
        if label in ("learned", "fcg_without_net"):
            P.set_learned(net if label == "learned" else None,
                          use_net=label == "learned", fallback=True)
        for _ in range(2):   # warm-up, then the measured solve
            P.set_depend(g.zeros(), None, src)
            rc = P.run()
        x = g.interior(P.phi)
        err = float(np.linalg.norm(x - phi.cpu().numpy()) / np.linalg.norm(phi.cpu().numpy()))
        res[label] = {"ms": P.stats.ms, "iters": P.stats.iters,
                      "fcg_iters": P.stats.outer_iters if "learned" in label or "fcg" in label else None,
                      "resid": P.stats.tol_out, "code": rc, "rel_l2_vs_exact": err}
    res["iters_ratio_fp64_over_learned"] = res["fp64"]["iters"] / max(1, res["learned"]["iters"])
    return res


def learned_cavity_leg(n, inner_tol, steps=2, warmup=1):
    """cavity steps/s with the learned projection (flexible CG + network,
    fallback to the plain CG), same workload"""
    if not learned_ok(n):
        return None
    from carpio_gb300.unet import load_trained
    import torch
    net = load_trained()
    g, ns = make_cavity(n, "mixed", inner_tol)
    ns.set_learned(net, fallback=True)
    ns.run(warmup)
    torch.cuda.synchronize()
    ns.run(steps)
    pr = ns.profile()
    return {"steps_per_s": steps / (float(np.sum(pr["step_ms"])) / 1e3),
            "solve_ms": float(np.mean(pr["solve_ms"])),
            "iters": float(np.mean(pr["inner"])),
            "fcg_iters": float(np.mean(pr["outer"])), "steps": steps}


def unet_leg(n):
    """device time of one U-Net application at n^2 and its tensor-core rate"""
    import torch
    from carpio_gb300.unet import load_trained
    if not learned_ok(n):
        return None
    net = load_trained()
    x = torch.randn(1, n, n, device="cuda")
    z = torch.empty_like(x)
    for _ in range(3):
        net.forward(x, out=z)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        net.forward(x, out=z)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # multiply-adds of the 13 tensor-core layers per pixel of their level
    macs = 0
    for (ci0, ci1, co), lvl in zip(
            [(32, 0, 32), (32, 0, 64), (64, 0, 64), (64, 0, 128), (128, 0, 128),
             (128, 0, 256), (256, 0, 256), (256, 128, 128), (128, 0, 128),
             (128, 64, 64), (64, 0, 64), (64, 32, 32), (32, 0, 32)],
            [0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0]):
        macs += 9 * (ci0 + ci1) * co * (n >> lvl) ** 2
    peak, how = bf16_peak()
    tflops = 2.0 * macs / (ms / 1e3) / 1e12
    return {"ms": ms, "tensor_gflop": 2.0 * macs / 1e9, "tflops": tflops,
            "peak_tflops": peak, "frac": tflops / peak, "peak_source": how,
            "note": "host-launched layers (stream-ordered), wall of 10 forwards / 10"}


def bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def batched_leg(count=512, reps=2):
    """512 uneven Poisson problems (side N uniform in {32, 48, ..., 512}, 8
    Gaussians, Dirichlet-0 or all-Neumann, FP32 inner / FP64 refinement to
    1e-8): one persistent cluster launch replayed from a CUDA graph vs a loop
    of single solves on the same device-resident inputs"""
    import torch
    from carpio_gb300 import batch, structure as S, workloads
    probs, srcs = workloads.uneven_batch(count, seed=0)
    bp = batch.BatchedPoisson(probs, tol=TOL)
    bp.upload(0, srcs)
    ms = []
    for _ in range(reps + 1):
        bp.zero(1)
        rc = bp.run()
        ms.append(bp.ms)
    info = bp.info()
    iters = sum(s["iters"] for s in bp.stats)
    cells = sum(p.nx * p.ny for p in probs)
    cell_iters = sum(s["iters"] * p.nx * p.ny for s, p in zip(bp.stats, probs))
    t_batch = min(ms[1:])
    # the same problems one at a time through carpio_gpu_poisson_solve
    t0 = time.perf_counter()
    dev_ms = 0.0
    for i, p in enumerate(probs):
        g = S.Grid(p.box[0], p.box[1], (p.nx, p.ny), 1)
        P = S.Poisson(g)
        for seg, (tt, v) in enumerate(p.bc):
            bc = S.BoundaryCondition()
            (bc.set_default_1_bc if tt == 1 else bc.set_default_2_bc)(v)
            P.add_bc(0, seg, "phi", bc)
        src = torch.zeros(p.nx + 2, p.ny + 2, dtype=torch.float64, device="cuda")
        src[1:-1, 1:-1] = torch.from_numpy(srcs[i])
        P.set_depend(torch.zeros_like(src), None, src)
        P.set_solver("CG", None, 200000, TOL, mean_removal=p.mean_removal,
                     precision="mixed")
        P.run()
        dev_ms += P.stats.ms
    loop_wall = 1e3 * (time.perf_counter() - t0)
    return {"problems": count, "cells": cells, "code": rc,
            "persistent_graph_ms": t_batch, "loop_single_solves_ms": loop_wall,
            "loop_device_ms": dev_ms, "speedup": loop_wall / t_batch,
            "inner_iters": iters, "cell_iters_per_s": cell_iters / (t_batch / 1e3),
            "max_resid": max(s["resid"] for s in bp.stats),
            "tiles": {k: info[k] for k in ("threads", "cluster", "cells_per_cta",
                                           "clusters", "ctas", "smem_bytes", "teams")}}


def accuracy_run(a):
    """the mixed projection against the FP64 projection on the same cavity,
    step by step: relative L2 of u, v, p and the solve times"""
    import torch
    n, steps = a.n, a.accuracy_steps
    gm, nm = make_cavity(n, "mixed", a.inner_tol)
    gf, nf = make_cavity(n, "fp64", a.inner_tol)
    # the CPU oracle (reference algorithm: CSR assembly + CG with mean
    # removal, FP64) on the first steps
    ko = min(a.oracle_steps, steps)
    if ko > 0:
        from oracle import restate as R
        go = R.Grid(n, n, 2)
        so = R.new_state(go, 0.5 / n)
    rows = []

    def rel(x, y):
        ref = np.linalg.norm(y)
        return float(np.linalg.norm(x - y) / ref) if ref > 0 else 0.0
    for st in range(steps):
        nm.run(1)
        nf.run(1)
        pm, pf = nm.profile(), nf.profile()
        sm, sf = nm.state(), nf.state()
        row = {"step": st + 1,
               "solve_ms_mixed": float(pm["solve_ms"][0]),
               "solve_ms_fp64": float(pf["solve_ms"][0]),
               "iters_mixed": int(pm["inner"][0]), "iters_fp64": int(pf["inner"][0])}
        for k in ("u", "v", "p"):
            row[f"rel_l2_{k}"] = rel(gm.interior(sm[k]), gf.interior(sf[k]))
        if st < ko:
            R.ns_run(go, so, 1, scheme="vanleer", cg_tol=TOL, threads=os.cpu_count() or 1)
            for k in ("u", "v", "p"):
                ref = go.interior(so[k])
                row[f"oracle_rel_l2_{k}_mixed"] = rel(gm.interior(sm[k]), ref)
                row[f"oracle_rel_l2_{k}_fp64"] = rel(gf.interior(sf[k]), ref)
        rows.append(row)
    summ = {f"max_rel_l2_{k}": max(r[f"rel_l2_{k}"] for r in rows) for k in ("u", "v", "p")}
    summ["solve_ms_mixed_mean"] = float(np.mean([r["solve_ms_mixed"] for r in rows]))
    summ["solve_ms_fp64_mean"] = float(np.mean([r["solve_ms_fp64"] for r in rows]))
    print(json.dumps({"accuracy": f"mixed vs fp64 projection, {n}^2 cavity "
                      f"(CPU oracle on the first {ko} steps)",
                      "steps": steps, "summary": summ, "rows": rows}), flush=True)


if __name__ == "__main__":
    main()
