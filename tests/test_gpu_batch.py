"""GPU checks of the batched Poisson solver (carpio_gpu_batch_*): every
problem of an uneven batch against the oracle (the reference's assembly and
FP64 CG, with mean removal for all-Neumann problems), with the default
kernel (one CTA per problem, multigrid-preconditioned) and with the cluster
kernel (teams of up to 16 CTAs that share reductions and halo rows through
distributed shared memory); repeatability, graph vs plain launch, limits."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rel_l2
from oracle import restate as R

pytestmark = pytest.mark.gpu

TOL = 1e-8
# two solutions that each meet a 1e-8 relative residual differ by at most
# cond(A) * 1e-8; on these grids (N <= 130) well below this
SOL_RTOL = 1e-5


def problem_set(seed, sizes, mixed_bc=True):
    from carpio_gb300.batch import DIRICHLET, NEUMANN, Problem
    from carpio_gb300.workloads import gaussian_source
    rng = np.random.default_rng(seed)
    probs, srcs = [], []
    for k, n in enumerate(sizes):
        kind = k % 4
        if kind == 0:
            p = Problem(n, n, bc=[(DIRICHLET, 0.0)] * 4)
        elif kind == 1:
            p = Problem(n, n, bc=[(NEUMANN, 0.0)] * 4)
        elif kind == 2 and mixed_bc:
            # non-square cells count, non-unit box, non-zero boundary values
            p = Problem(n, max(3, n // 2 + 1), box=((-1.0, 0.5), (1.0, 2.0)),
                        bc=[(DIRICHLET, 1.0), (DIRICHLET, -0.5), (NEUMANN, 0.75),
                            (NEUMANN, -1.25)])
        else:
            p = Problem(n + 3, n, bc=[(DIRICHLET, 0.0)] * 4, beta=2.0)
        probs.append(p)
        srcs.append(gaussian_source(p.nx, p.ny, rng, box=p.box))
    return probs, srcs


def oracle(p, src, tol=1e-12, threads=4):
    """(A as scipy CSR, b, x) in the reference's vector order (x fastest)."""
    og = R.Grid(p.nx, p.ny, 1, p.box[0][0], p.box[1][0], p.box[0][1], p.box[1][1])
    f = og.zeros()
    og.interior(f)[:] = src
    types = [t for t, _ in p.bc]
    vals = [v for _, v in p.bc]
    rp, ci, va, b = R.assemble_poisson(og, R.make_bc(types, vals), p.beta, src=f)
    if p.mean_removal:
        b = b - b.mean()
    code, x, it, t, _ = R.krylov_csr("cg", rp, ci, va, b, np.zeros(b.size),
                                     200000, tol, threads=threads)
    assert code == 0
    if p.mean_removal:
        x = x - x.mean()
    A = sp.csr_matrix((va, ci.astype(np.int64), rp.astype(np.int64)),
                      shape=(b.size, b.size))
    return A, b, x


def vec(sol):
    return np.ascontiguousarray(np.asarray(sol).T).reshape(-1)


def nrm2(v):
    # BLAS_Level1.hpp:569: the last element is left out
    return np.sqrt(np.sum(v[:-1] ** 2)) if v.size > 1 else abs(v[0])


def check(probs, srcs, sols, stats, tol=TOL):
    for i, (p, src, sol, st) in enumerate(zip(probs, srcs, sols, stats)):
        A, b, x = oracle(p, src)
        xv = vec(sol)
        r = b - A @ xv
        nb = nrm2(b) or 1.0
        true_res = nrm2(r) / nb
        assert st["code"] == 0, (i, st)
        assert true_res <= tol * 1.02, (i, true_res, st)
        assert abs(true_res - st["resid"]) <= 1e-3 * max(true_res, 1e-300) + 1e-15, (i, true_res, st)
        assert rel_l2(xv, x) <= SOL_RTOL, (i, rel_l2(xv, x))
        if p.mean_removal:
            assert abs(xv.mean()) <= 1e-12 * max(1.0, np.abs(xv).max())


def test_uneven_batch_matches_oracle(gpu_lib):
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(0, [8, 17, 32, 40, 64, 96, 130, 24, 48, 77, 5, 2])
    bp = BatchedPoisson(probs, tol=TOL)
    sols = bp.solve(srcs)
    check(probs, srcs, sols, bp.stats)
    assert all(s["iters"] > 0 and s["updates"] >= 1 for s in bp.stats)
    info = bp.info()
    assert info["ctas"] == info["clusters"] * info["cluster"]
    assert sum(info["teams"]) == len(probs)


@pytest.mark.parametrize("tiles", [
    dict(threads=512, cluster=16, cells_per_cta=256),    # teams of 2..16 CTAs
    dict(threads=256, cluster=8, cells_per_cta=512),
    dict(threads=512, cluster=4, cells_per_cta=1024),
    dict(threads=256, cluster=2, cells_per_cta=16384),
    dict(threads=512, cluster=16, cells_per_cta=16384, use_graph=-1),
])
def test_teams_of_many_ctas_match_oracle(gpu_lib, tiles):
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(1, [16, 33, 64, 100, 128, 40, 72, 90])
    bp = BatchedPoisson(probs, tol=TOL, tiles=tiles)
    info = bp.info()
    assert info["threads"] == tiles["threads"] and info["cluster"] == tiles["cluster"]
    if tiles["cells_per_cta"] <= 1024:
        assert sum(info["teams"][1:]) > 0, info     # some teams span CTAs
    sols = bp.solve(srcs)
    check(probs, srcs, sols, bp.stats)


def test_repeatable_and_graph_equals_plain_launch(gpu_lib):
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(2, [64, 48, 96, 33, 128, 20])
    tiles = dict(threads=512, cluster=8, cells_per_cta=1024)
    a = BatchedPoisson(probs, tol=TOL, tiles=tiles)
    s1 = a.solve(srcs)
    s2 = a.solve(srcs)
    b = BatchedPoisson(probs, tol=TOL, tiles=dict(tiles, use_graph=-1))
    s3 = b.solve(srcs)
    for x, y, z in zip(s1, s2, s3):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
        assert np.array_equal(x.view(np.uint64), z.view(np.uint64))


def test_team_of_sixteen_on_the_largest_grids(gpu_lib):
    from carpio_gb300.batch import BatchedPoisson, DIRICHLET, NEUMANN, Problem
    from carpio_gb300.workloads import gaussian_source
    rng = np.random.default_rng(7)
    probs = [Problem(512, 512, bc=[(NEUMANN, 0.0)] * 4),
             Problem(448, 448, bc=[(DIRICHLET, 0.0)] * 4)]
    srcs = [gaussian_source(p.nx, p.ny, rng) for p in probs]
    bp = BatchedPoisson(probs, tol=TOL, tiles=dict(threads=512, cluster=16,
                                                   cells_per_cta=16384))
    assert bp.info()["teams"][4] == 2
    sols = bp.solve(srcs)
    for p, src, sol, st in zip(probs, srcs, sols, bp.stats):
        A, b, x = oracle(p, src, tol=1e-11, threads=16)
        xv = vec(sol)
        assert st["code"] == 0
        assert nrm2(b - A @ xv) / nrm2(b) <= TOL * 1.02
        assert rel_l2(xv, x) <= 1e-4


def test_matches_single_grid_solver(gpu_lib):
    """each problem of the batch and carpio_gpu_poisson_solve (MIXED) on the
    same grid agree to what the 1e-8 tolerance allows"""
    from carpio_gb300 import structure as S
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(3, [40, 64, 96, 50])
    bp = BatchedPoisson(probs, tol=TOL)
    sols = bp.solve(srcs)
    for p, src, sol in zip(probs, srcs, sols):
        g = S.Grid(p.box[0], p.box[1], (p.nx, p.ny), 1)
        P = S.Poisson(g)
        for seg, (t, v) in enumerate(p.bc):
            bc = S.BoundaryCondition()
            (bc.set_default_1_bc if t == 1 else bc.set_default_2_bc)(v)
            P.add_bc(0, seg, "phi", bc)
        f = g.zeros()
        f[1:-1, 1:-1] = src
        P.set_uniform_beta(p.beta)
        P.set_depend(g.zeros(), None, f)
        P.set_solver("CG", None, 100000, TOL, mean_removal=p.mean_removal,
                     precision="mixed")
        assert P.run() == 0
        assert rel_l2(sol, g.interior(P.phi)) <= SOL_RTOL


def test_zero_source_and_warm_start(gpu_lib):
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(4, [32, 48, 64, 24], mixed_bc=False)
    bp = BatchedPoisson(probs, tol=TOL)
    zeros = [np.zeros((p.nx, p.ny)) for p in probs]
    sols = bp.solve(zeros)
    assert all(s["iters"] == 0 and s["code"] == 0 for s in bp.stats)
    assert all(np.all(s == 0) for s in sols)
    # warm start from the converged solutions: at most a few iterations
    sols = bp.solve(srcs)
    bp.solve(srcs, phi0=sols)
    assert all(s["code"] == 0 and s["iters"] <= 5 for s in bp.stats), bp.stats


def test_rejects_what_does_not_fit(gpu_lib):
    """the cluster kernel keeps a problem on chip: 1024^2 fits no team of 16
    CTAs; the block size must be one it is built for"""
    from carpio_gb300 import _lib
    from carpio_gb300.batch import BatchedPoisson, Problem
    with pytest.raises(_lib.CarpioGpuError):
        BatchedPoisson([Problem(1024, 1024)], tol=TOL,
                       tiles=dict(threads=512, cluster=16, cells_per_cta=16384))
    with pytest.raises(_lib.CarpioGpuError):
        BatchedPoisson([Problem(64, 64)], tol=TOL, tiles=dict(threads=384))
    with pytest.raises(_lib.CarpioGpuError):
        BatchedPoisson([Problem(64, 64)], tol=TOL,
                       tiles=dict(threads=384, cluster=8, cells_per_cta=4096))


def test_autotune_keeps_a_valid_configuration(gpu_lib):
    from carpio_gb300.batch import BatchedPoisson
    probs, srcs = problem_set(5, [32, 64, 100, 128, 48, 80, 16, 130])
    bp = BatchedPoisson(probs, tol=TOL)
    bp.upload(0, srcs)
    bp.zero(1)
    info = bp.autotune(max_candidates=4)
    assert 1 <= info["candidates"] <= 4 and info["tuned_ms"] > 0
    # the tuned configuration solves from the restored initial guess
    bp.run()
    check(probs, srcs, bp.download(1), bp.stats)
    # a new batch with the same shapes starts from the tuned configuration
    bp2 = BatchedPoisson(probs, tol=TOL)
    i2 = bp2.info()
    assert (i2["threads"], i2["cluster"], i2["cells_per_cta"]) == \
        (info["threads"], info["cluster"], info["cells_per_cta"])


def test_watchdog_expiry_is_reported(gpu_lib):
    """a solve deadline of 1 ms expires (checked every 256 iterations by
    every CTA); the launch returns ETIMEOUT and the context stays usable"""
    from carpio_gb300 import _lib
    from carpio_gb300.batch import BatchedPoisson, NEUMANN, Problem
    from carpio_gb300.workloads import gaussian_source
    rng = np.random.default_rng(9)
    probs = [Problem(384, 384, bc=[(NEUMANN, 0.0)] * 4), Problem(96, 96)]
    srcs = [gaussian_source(p.nx, p.ny, rng) for p in probs]
    bp = BatchedPoisson(probs, tol=TOL, tiles=dict(threads=512, cluster=16,
                                                   cells_per_cta=4096))
    bp.upload(0, srcs)
    bp.zero(1)
    try:
        assert gpu_lib.carpio_gpu_set_watchdog(2000, 1) == 0
        with pytest.raises(_lib.CarpioGpuError) as e:
            bp.run()
        assert e.value.code == _lib.ETIMEOUT
    finally:
        gpu_lib.carpio_gpu_set_watchdog(2000, 600000)
    bp.zero(1)
    assert bp.run() == 0


def test_multigrid_kernel_graph_repeatable_and_large(gpu_lib):
    """the default kernel (one CTA per problem, V-cycle preconditioner):
    bitwise repeatable, the captured graph equals a plain launch, a few
    V-cycles per problem, and problems too large for a cluster team (512^2,
    1024 x 256) solved like carpio_gpu_poisson_solve solves them"""
    from carpio_gb300 import structure as S
    from carpio_gb300.batch import BatchedPoisson, NEUMANN, Problem
    from carpio_gb300.workloads import gaussian_source
    probs, srcs = problem_set(11, [64, 96, 130, 48, 33, 16])
    a = BatchedPoisson(probs, tol=TOL)
    s1 = a.solve(srcs)
    s2 = a.solve(srcs)
    b = BatchedPoisson(probs, tol=TOL, tiles=dict(use_graph=-1))
    s3 = b.solve(srcs)
    for x, y, z in zip(s1, s2, s3):
        assert np.array_equal(x, y) and np.array_equal(x, z)
    assert a.info()["cluster"] == 1 and a.info()["teams"][0] == len(probs)
    check(probs, srcs, s1, a.stats)
    for p, st in zip(probs, a.stats):
        if p.nx % 8 == 0 and p.ny % 8 == 0:
            assert st["iters"] <= 60, (p.nx, p.ny, st)
    rng = np.random.default_rng(12)
    big = [Problem(512, 512, bc=[(NEUMANN, 0.0)] * 4), Problem(1024, 256)]
    bsrc = [gaussian_source(p.nx, p.ny, rng) for p in big]
    bp = BatchedPoisson(big, tol=TOL)
    sols = bp.solve(bsrc)
    for p, src, sol, st in zip(big, bsrc, sols, bp.stats):
        assert st["code"] == 0 and st["resid"] <= TOL
        g = S.Grid(p.box[0], p.box[1], (p.nx, p.ny), 1)
        P = S.Poisson(g)
        for seg, (t, v) in enumerate(p.bc):
            bc = S.BoundaryCondition()
            (bc.set_default_1_bc if t == 1 else bc.set_default_2_bc)(v)
            P.add_bc(0, seg, "phi", bc)
        f = g.zeros()
        f[1:-1, 1:-1] = src
        P.set_depend(g.zeros(), None, f)
        P.set_solver("CG", None, 100000, 1e-10, mean_removal=p.mean_removal,
                     precision="mixed")
        assert P.run() == 0
        assert rel_l2(sol, g.interior(P.phi)) <= 1e-4
