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


def noalloc_solve(L, kind, d, tol, max_iter):
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
        hist.numel(), ctypes.byref(hl), 0, None)
    return code, x.cpu().numpy(), mi.value, t.value, hist[:hl.value].cpu().numpy()


def alloc_solve(kind, d, tol, max_iter):
    from carpio_gb300 import algebra
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    x = np.zeros(A.iLen())
    lr = []
    code, it, t = algebra.krylov(kind, A, x, d["b"].copy(), max_iter, tol, lr)
    return code, x, it, t, np.asarray(lr)


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib):
    L = gpu_lib
    cases = [("csr_pde225_dia_bicgstab", 2, 1e-13, 2000),
             ("csr_bus685_cg", 0, 1e-13, 20000)]
    for name, kind, tol, max_iter in cases:   # two calls in a row
        d = golden(name)
        c1, x1, it1, t1, h1 = noalloc_solve(L, kind, d, tol, max_iter)
        c2, x2, it2, t2, h2 = alloc_solve(kind, d, tol, max_iter)
        assert c1 == c2 == 0
        bar = 1e-9 if "bus685" in name else PLAIN_RTOL   # as in test_gpu_csr
        assert rel_l2(x1, x2) <= bar, (name, rel_l2(x1, x2))
        assert abs(len(h1) - len(h2)) <= max(3, len(h2) // 20)
        assert t1 < tol or (kind == 0 and t1 <= tol)


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
