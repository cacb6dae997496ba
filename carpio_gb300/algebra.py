"""Algebra-level mirror of lib/algebra (solver_matrix.hpp, matrix_SparCompRow.hpp)
over the C ABI: the carpio:: free-function Krylov solvers on a CSR matrix,
with the reference's in/out semantics and return codes.

    code, max_iter, tol = CG(A, x, b, max_iter, tol, lresid)

x is updated in place (numpy array or CUDA tensor); lresid, when given, is a
list that receives the residual history like std::list<Float>& lresid.
"""
import ctypes

import numpy as np

from . import _lib


class MatrixSCR:
    """MatrixSCR_ (lib/algebra/matrix_SparCompRow.hpp:27-36): val_, rowptr_,
    colind_ with 32-bit unsigned indices (St)."""

    def __init__(self, rowptr, colind, val):
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.uint32)
        self.colind = np.ascontiguousarray(colind, dtype=np.uint32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        if self.rowptr.size < 1 or self.colind.size != self.val.size:
            raise ValueError("inconsistent CSR arrays")

    def iLen(self):
        return self.rowptr.size - 1

    def NumNonzeros(self):
        return self.val.size

    def __matmul__(self, x):
        """MatrixSCR_::operator* on the host (for checks only)"""
        x = np.asarray(x, dtype=np.float64)
        y = np.zeros(self.iLen())
        for i in range(self.iLen()):
            s, e = self.rowptr[i], self.rowptr[i + 1]
            y[i] = np.dot(self.val[s:e], x[self.colind[s:e]])
        return y


def _as_f64(a, name):
    if hasattr(a, "data_ptr"):
        import torch
        if a.dtype != torch.float64 or not a.is_contiguous():
            raise TypeError(f"{name} must be a contiguous float64 tensor")
        return a
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 \
            or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a contiguous float64 numpy array")
    return a


def krylov(kind, A, x, b, max_iter, tol, lresid=None, flags=0):
    """Runs carpio_gpu_krylov_csr. Returns (code, max_iter_out, tol_out);
    raises CarpioGpuError for negative (library) codes."""
    L = _lib.load()
    x = _as_f64(x, "x")
    b = _as_f64(b, "b")
    n = A.iLen()
    mi = ctypes.c_int(int(max_iter))
    t = ctypes.c_double(float(tol))
    cap = int(max_iter) + 2 if lresid is not None else 0
    hist = np.zeros(max(cap, 1))
    hl = ctypes.c_int(0)
    code = L.carpio_gpu_krylov_csr(
        _lib.KINDS[kind] if isinstance(kind, str) else int(kind), n,
        A.NumNonzeros(), _lib.ptr(A.rowptr), _lib.ptr(A.colind),
        _lib.ptr(A.val), _lib.ptr(b), _lib.ptr(x), ctypes.byref(mi),
        ctypes.byref(t), _lib.ptr(hist) if cap else None, cap,
        ctypes.byref(hl), int(flags))
    if code < 0:
        raise _lib.CarpioGpuError(code, f"carpio_gpu_krylov_csr({kind})")
    if lresid is not None:
        lresid.extend(hist[:min(hl.value, cap)].tolist())
    return code, mi.value, t.value


def CG(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::CG (solver_matrix.hpp:264-316)"""
    return krylov(_lib.CG, A, x, b, max_iter, tol, lresid, flags)


def Jacobi(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::Jacobi (solver_matrix.hpp:192-260)"""
    return krylov(_lib.JACOBI, A, x, b, max_iter, tol, lresid, flags)


def Dia_BiCGSTAB(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::Dia_BiCGSTAB (solver_matrix.hpp:599-672)"""
    return krylov(_lib.DIA_BICGSTAB, A, x, b, max_iter, tol, lresid, flags)


def BiCGSTAB(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::BiCGSTAB (solver_matrix.hpp:674-745)"""
    return krylov(_lib.BICGSTAB, A, x, b, max_iter, tol, lresid, flags)


def Residual(A, x, b, flags=0):
    """carpio::Residual (solver_matrix.hpp:583-597): nrm2(b - A x) / nrm2(b)
    with nrm2's drop-last quirk, on the GPU (carpio_gpu_residual)"""
    L = _lib.load()
    x = _as_f64(x, "x")
    b = _as_f64(b, "b")
    r = ctypes.c_double(0.0)
    code = L.carpio_gpu_residual(A.iLen(), A.NumNonzeros(), _lib.ptr(A.rowptr),
                                 _lib.ptr(A.colind), _lib.ptr(A.val), _lib.ptr(x),
                                 _lib.ptr(b), int(flags), ctypes.byref(r))
    if code < 0:
        raise _lib.CarpioGpuError(code, "carpio_gpu_residual")
    return r.value


class Solver_Jacobi_:
    """carpio::Solver_Jacobi_ (solver_matrix.hpp:820-910): class form with
    num_iter() / residual() / get_residual_array()."""

    def __init__(self, max_iter=100, tol=1e-3):
        self._max_iter, self._tol = int(max_iter), float(tol)
        self._num_iter, self._resid, self._lresid = 0, 1e10, []

    def solve(self, A, x, b):
        self._lresid = []
        code, it, t = Jacobi(A, x, b, self._max_iter, self._tol, self._lresid)
        # the class form reports max_iter on exhaustion (solver_matrix.hpp:905)
        self._num_iter = it
        self._resid = t
        return code

    def num_iter(self):
        return self._num_iter

    def residual(self):
        return self._resid

    def get_residual_array(self):
        return np.asarray(self._lresid)


def IC_CGS(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::IC_CGS (solver_matrix.hpp:376-438) with ICPre
    (preconditioner.hpp:97-177)"""
    return krylov(_lib.IC_CGS, A, x, b, max_iter, tol, lresid, flags)


def IC_CG(A, x, b, max_iter, tol, lresid=None, flags=0):
    """carpio::IC_CG (solver_matrix.hpp:318-374) with ICPre"""
    return krylov(_lib.IC_CG, A, x, b, max_iter, tol, lresid, flags)
