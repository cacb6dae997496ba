"""CPU checks of the batched solver's host side: the planner that places
problems on cluster team slots, the work-balanced split across processes
(also run as two gloo ranks), and argument validation. No device needed."""
import os
import socket

import numpy as np
import pytest

from carpio_gb300 import _lib
from carpio_gb300.batch import DIRICHLET, NEUMANN, Problem, plan, shard

SLOTS = 16   # slot index = cluster * 16 + slot within the cluster


def square_batch(count, seed, sizes=tuple(range(32, 513, 16))):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(sizes))
        t = NEUMANN if rng.random() < 0.5 else DIRICHLET
        out.append(Problem(n, n, bc=[(t, 0.0)] * 4))
    return out


def rows_max(nx, t):
    return -(-nx // t)


@pytest.mark.parametrize("tiles,clusters,nmax", [
    (dict(threads=512, cluster=16, cells_per_cta=16384), 7, 512),
    (dict(threads=512, cluster=16, cells_per_cta=4096), 7, 512),
    (dict(threads=256, cluster=16, cells_per_cta=8192), 9, 352),
    (dict(threads=512, cluster=8, cells_per_cta=16384), 15, 352),
    (dict(threads=512, cluster=16, cells_per_cta=16384), 40, 512),
])
def test_plan_places_every_problem_on_a_valid_team(tiles, clusters, nmax):
    probs = square_batch(200, seed=1, sizes=tuple(range(32, nmax + 1, 16)))
    team, slot, est = plan(probs, tiles, clusters)
    T, S = tiles["threads"], tiles["cluster"]
    hard = min(16384, 32 * T)
    assert est > 0
    cl_team = {}
    for p, t, s in zip(probs, team, slot):
        assert t in (1, 2, 4, 8, 16) and t <= S and t <= p.nx
        cells = rows_max(p.nx, t) * p.ny
        assert cells <= hard
        # the smallest team that meets the target (or the largest allowed)
        if t > 1:
            assert rows_max(p.nx, t // 2) * p.ny > tiles["cells_per_cta"] or \
                rows_max(p.nx, t // 2) * p.ny > hard
        c, k = divmod(int(s), SLOTS)
        assert 0 <= c < clusters
        assert cl_team.setdefault(c, t) == t, "one team size per cluster"
        assert k < S // t
    # deterministic
    team2, slot2, est2 = plan(probs, tiles, clusters)
    assert np.array_equal(team, team2) and np.array_equal(slot, slot2) and est == est2


def test_plan_makespan_shrinks_with_clusters():
    probs = square_batch(300, seed=2)
    tiles = dict(threads=512, cluster=16, cells_per_cta=16384)
    ests = [plan(probs, tiles, c)[2] for c in (5, 7, 14, 28)]
    assert all(a >= b for a, b in zip(ests, ests[1:])), ests
    assert ests[-1] < ests[0]


def test_plan_merges_team_sizes_when_clusters_are_few():
    probs = square_batch(64, seed=3)
    tiles = dict(threads=512, cluster=16, cells_per_cta=16384)
    team, slot, _ = plan(probs, tiles, 2)
    assert len({int(s) // SLOTS for s in slot}) <= 2
    assert len(set(team.tolist())) <= 2


def test_plan_rejects_what_fits_no_team():
    tiles = dict(threads=512, cluster=16, cells_per_cta=16384)
    with pytest.raises(_lib.CarpioGpuError):
        plan([Problem(1024, 1024)], tiles, 7)        # needs 64 CTAs
    with pytest.raises(_lib.CarpioGpuError):          # 512^2 needs 32 CTAs of 256 threads
        plan([Problem(512, 512)], dict(tiles, threads=256), 7)
    with pytest.raises(_lib.CarpioGpuError):
        plan([Problem(64, 64)], dict(tiles, threads=384), 7)
    with pytest.raises(_lib.CarpioGpuError):
        plan([Problem(0, 64)], tiles, 7)
    with pytest.raises(_lib.CarpioGpuError):
        plan([Problem(8, 8, bc=[(3, 0.0)] * 4)], tiles, 7)
    with pytest.raises(_lib.CarpioGpuError):
        plan([Problem(8, 8, beta=0.0)], tiles, 7)


def work(p):
    n = max(p.nx, p.ny)
    neumann = all(t == NEUMANN for t, _ in p.bc)
    return p.nx * p.ny * (int((4.9 if neumann else 2.9) * n) + 10)


def test_shard_balances_work():
    probs = square_batch(512, seed=4)
    for world in (1, 2, 3, 8):
        r = shard(probs, world)
        assert r.min() >= 0 and r.max() < world
        loads = np.zeros(world)
        for p, k in zip(probs, r):
            loads[k] += work(p)
        # LPT: no rank exceeds another by more than the largest item
        assert loads.max() - loads.min() <= max(work(p) for p in probs)
    assert len(shard([], 4)) == 0


def test_create_validates_before_device_work():
    import ctypes
    L = _lib.load()
    h = ctypes.c_void_p()
    cfg = _lib.SolverCfg()
    cfg.kind, cfg.precision, cfg.max_iter, cfg.tol = _lib.CG, _lib.FP64, 10, 1e-8
    probs = (_lib.BatchProblem * 1)(Problem(8, 8).to_c())
    # FP64 precision is not what the batch solves
    assert L.carpio_gpu_batch_create(1, probs, ctypes.byref(cfg), None,
                                     ctypes.byref(h)) == _lib.EINVAL
    cfg.precision, cfg.kind = _lib.MIXED, _lib.JACOBI
    assert L.carpio_gpu_batch_create(1, probs, ctypes.byref(cfg), None,
                                     ctypes.byref(h)) == _lib.EINVAL
    assert L.carpio_gpu_batch_create(0, probs, ctypes.byref(cfg), None,
                                     ctypes.byref(h)) == _lib.EINVAL
    for fn in ("carpio_gpu_batch_destroy",):
        assert getattr(L, fn)(None) == _lib.EINVAL
    assert L.carpio_gpu_batch_run(None, None, None) == _lib.EINVAL
    assert L.carpio_gpu_batch_zero(None, 1) == _lib.EINVAL
    assert L.carpio_gpu_batch_autotune(None, 4) == _lib.EINVAL


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                            rank=rank, world_size=world)
    probs = square_batch(128, seed=5)
    r = shard(probs, world)
    mine = [i for i in range(len(probs)) if r[i] == rank]
    gathered = [None] * world
    dist.all_gather_object(gathered, (mine, r.tolist()))
    np.save(os.path.join(out_dir, f"rank{rank}.npy"),
            np.array([len(g[0]) for g in gathered] + [int(g[1] == gathered[0][1]) for g in gathered]))
    if rank == 0:
        allidx = sorted(i for g in gathered for i in g[0])
        assert allidx == list(range(len(probs)))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_across_two_gloo_ranks(tmp_path):
    """Each rank derives its own share with no data-path collective; the
    shares are disjoint, cover the batch, and every rank computes the same
    assignment."""
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
             join=True)
    for rank in range(world):
        v = np.load(tmp_path / f"rank{rank}.npy")
        counts, agree = v[:world], v[world:]
        assert counts.sum() == 128 and all(agree)
