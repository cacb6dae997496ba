"""carpio_gpu_krylov_csr_noalloc: the CSR Krylov solve for callers that cannot
allocate device memory mid-solve (a framework owning all device memory
through its own pool; a time-stepping service that forbids cudaMalloc after
start-up). It is checked against the allocating entry point,
carpio_gpu_krylov_csr, on two calls in a row through the C ABI. Collected
last on purpose: a failure here comes after every other test has run."""
import ctypes

import numpy as np
import pytest

from conftest import PLAIN_RTOL, golden, rel_l2

pytestmark = pytest.mark.gpu


def noalloc_solve(L, kind, d, tol, max_iter, stream=None):
    """one call of the no-alloc entry point on device copies of a fixture's
    system, on `stream` (a torch.cuda.Stream) or the default stream"""
    torch = pytest.importorskip("torch")
    dev = "cuda"
    rp = torch.from_numpy(d["rowptr"].astype(np.int32)).to(dev)
    ci = torch.from_numpy(d["colind"].astype(np.int32)).to(dev)
    va = torch.from_numpy(d["val"]).to(dev)
    b = torch.from_numpy(d["b"]).to(dev)
    x = torch.zeros_like(b)
    hist = torch.zeros(max_iter + 2, dtype=torch.float64, device=dev)
    mi, t, hl = ctypes.c_int(max_iter), ctypes.c_double(tol), ctypes.c_int(0)
    torch.cuda.synchronize()
    code = L.carpio_gpu_krylov_csr_noalloc(
        kind, b.numel(), va.numel(), ctypes.c_void_p(rp.data_ptr()),
        ctypes.c_void_p(ci.data_ptr()), ctypes.c_void_p(va.data_ptr()),
        ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
        ctypes.byref(mi), ctypes.byref(t), ctypes.c_void_p(hist.data_ptr()),
        hist.numel(), ctypes.byref(hl), 0,
        None if stream is None else ctypes.c_void_p(stream.cuda_stream))
    return code, x.cpu().numpy(), mi.value, t.value, hist[:hl.value].cpu().numpy()


def alloc_solve(kind, d, tol, max_iter):
    from carpio_gb300 import algebra
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    x = np.zeros(A.iLen())
    lr = []
    code, it, t = algebra.krylov(kind, A, x, d["b"].copy(), max_iter, tol, lr)
    return code, x, it, t, np.asarray(lr)


def check_same(name, kind, tol, r1, r2):
    c1, x1, it1, t1, h1 = r1
    c2, x2, it2, t2, h2 = r2
    assert c1 == c2 == 0, (name, kind, c1, c2)
    bar = 1e-9 if "bus685" in name else PLAIN_RTOL   # as in test_gpu_csr
    if kind == 1:
        bar = 1e-8   # Jacobi stops at tol; its iterates differ by rounding only
    assert rel_l2(x1, x2) <= bar, (name, kind, rel_l2(x1, x2))
    assert abs(len(h1) - len(h2)) <= max(3, len(h2) // 20)
    assert t1 < tol or (kind in (0, 1) and t1 <= tol)


# (fixture, kind, tol, max_iter): CG 0, JACOBI 1, DIA_BICGSTAB 2, BICGSTAB 3
CASES = [("csr_pde225_dia_bicgstab", 2, 1e-13, 2000),
         ("csr_bus685_cg", 0, 1e-13, 20000),
         ("csr_pde225_jacobi", 1, 1e-10, 20000),
         ("csr_pde225_bicgstab", 3, 1e-13, 2000)]


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib):
    """every kind, each called twice in a row (the second call reuses the
    array the first one left behind), against carpio_gpu_krylov_csr"""
    L = gpu_lib
    for name, kind, tol, max_iter in CASES:
        d = golden(name)
        ref = alloc_solve(kind, d, tol, max_iter)
        for _ in range(2):
            check_same(name, kind, tol, noalloc_solve(L, kind, d, tol, max_iter), ref)


def test_noalloc_on_a_stream_after_a_failed_call(gpu_lib):
    """on a caller's stream: a call that stops at max_iter (code 1) leaves
    the shared array dirty; the next call starts clean and matches the
    allocating entry point"""
    torch = pytest.importorskip("torch")
    L = gpu_lib
    s = torch.cuda.Stream()
    for name, kind, tol, max_iter in CASES[1:3]:
        d = golden(name)
        code, _, it, _, _ = noalloc_solve(L, kind, d, tol, 1, stream=s)
        assert code == 1 and it == 1
        check_same(name, kind, tol, noalloc_solve(L, kind, d, tol, max_iter, stream=s),
                   alloc_solve(kind, d, tol, max_iter))


def test_noalloc_rejects_oversize_and_host_arrays(gpu_lib):
    torch = pytest.importorskip("torch")
    from carpio_gb300 import _lib
    L = gpu_lib
    n = 32769
    rp = torch.arange(n + 1, dtype=torch.int32, device="cuda")
    ci = torch.arange(n, dtype=torch.int32, device="cuda")
    va = torch.ones(n, dtype=torch.float64, device="cuda")
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    mi, t = ctypes.c_int(10), ctypes.c_double(1e-8)
    args = [ctypes.c_void_p(a.data_ptr()) for a in (rp, ci, va, b, x)]
    assert L.carpio_gpu_krylov_csr_noalloc(0, n, n, *args, ctypes.byref(mi),
                                           ctypes.byref(t), None, 0, None, 0,
                                           None) == _lib.EINVAL
    hb = np.ones(4)
    assert L.carpio_gpu_krylov_csr_noalloc(
        0, 4, 4, args[0], args[1], args[2], ctypes.c_void_p(hb.ctypes.data),
        args[4], ctypes.byref(mi), ctypes.byref(t), None, 0, None, 0,
        None) == _lib.EINVAL
    # pinned host memory is addressable by the GPU but is not device memory
    hp = torch.ones(4, dtype=torch.float64).pin_memory()
    assert L.carpio_gpu_krylov_csr_noalloc(
        0, 4, 4, args[0], args[1], args[2], ctypes.c_void_p(hp.data_ptr()),
        args[4], ctypes.byref(mi), ctypes.byref(t), None, 0, None, 0,
        None) == _lib.EINVAL
