"""GPU parity of the algebra-level drop-in (carpio_gpu_krylov_csr) against the
reference's own runs (golden fixtures) and the oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import golden, golden_names, rel_l2
from oracle import restate as R

pytestmark = pytest.mark.gpu


def true_resid(A, x, b):
    r = b - A @ x
    nb = np.linalg.norm(b[:-1])
    return np.linalg.norm(r[:-1]) / (nb if nb else 1.0)


@pytest.mark.parametrize("name", golden_names("csr_"))
def test_csr_matches_reference(gpu_lib, name):
    from carpio_gb300 import algebra, _lib
    d = golden(name)
    kind = str(d["case_args"][4])
    max_iter, tol = int(d["case_args"][5]), float(d["case_args"][6])
    if "aborted" in d:
        # DiaPre exits the reference process on a zero diagonal; the library
        # returns CARPIO_GPU_EZERODIAG instead (test_csr_zero_diagonal_is_an_error)
        assert "Diagonal preconditioner failure" in str(d["message"])
        return
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    b = d["b"].copy()
    x = d["x0"].copy()
    lr = []
    k = "jacobi" if kind == "jacobi_class" else kind
    code, it, t = algebra.krylov(k, A, x, b, max_iter, tol, lr)
    assert code == int(d["ret"])
    # iteration counts: the parallel sums round differently; allow a few
    # iterations either way on long runs, exact on short ones
    ref_it = int(d["max_iter_out"])
    assert abs(it - ref_it) <= max(2, ref_it // 1000), (it, ref_it)
    assert len(lr) == pytest.approx(int(d["lresid_len"]), abs=max(2, ref_it // 1000))
    if code == 0:
        stop = "<=" if k in ("cg", "jacobi") else "<"
        assert (t <= tol) if stop == "<=" else (t < tol)
    # solutions: both satisfy the same stopping test; the difference is
    # bounded by the solver tolerance, not by rounding
    assert rel_l2(x, d["x"]) <= max(1e-10, 50 * tol), rel_l2(x, d["x"])


def test_csr_zero_diagonal_is_an_error(gpu_lib):
    from carpio_gb300 import algebra, _lib
    # 3x3 with a missing diagonal in row 1
    A = algebra.MatrixSCR([0, 2, 3, 5], [0, 1, 0, 1, 2], [2.0, 1.0, 1.0, 1.0, 3.0])
    for solver in (algebra.Dia_BiCGSTAB, algebra.BiCGSTAB, algebra.Jacobi):
        x = np.zeros(3)
        with pytest.raises(_lib.CarpioGpuError) as e:
            solver(A, x, np.ones(3), 100, 1e-10)
        assert e.value.code == _lib.EZERODIAG
        assert np.all(x == 0)


def test_csr_rejects_bad_inputs(gpu_lib):
    from carpio_gb300 import algebra, _lib
    A = algebra.MatrixSCR([0, 1, 2], [0, 1], [1.0, 2.0])
    b = np.array([1.0, np.nan])
    with pytest.raises(_lib.CarpioGpuError) as e:
        algebra.CG(A, np.zeros(2), b, 10, 1e-10)
    assert e.value.code == _lib.ENONFINITE
    with pytest.raises(_lib.CarpioGpuError) as e:
        algebra.krylov(7, A, np.zeros(2), np.ones(2), 10, 1e-10)
    assert e.value.code == _lib.EINVAL


def test_csr_single_row_uses_abs(gpu_lib):
    # nrm2 of a length-1 vector is |x0| (BLAS_Level1.hpp:567)
    from carpio_gb300 import algebra
    A = algebra.MatrixSCR([0, 1], [0], [4.0])
    x = np.zeros(1)
    code, it, t = algebra.CG(A, x, np.array([2.0]), 10, 1e-12)
    c2, x2, it2, t2, _ = R.krylov_csr("cg", A.rowptr, A.colind, A.val,
                                      np.array([2.0]), np.zeros(1), 10, 1e-12)
    assert (code, it) == (c2, it2)
    assert x[0] == pytest.approx(0.5, rel=1e-15)


def test_csr_initial_guess_already_converged(gpu_lib):
    from carpio_gb300 import algebra
    d = golden("csr_bus685_cg")
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    x = d["x"].copy()
    lr = []
    code, it, t = algebra.CG(A, x, d["b"].copy(), 100, 1e-6, lr)
    assert code == 0 and it == 0 and lr == []
    # Dia_BiCGSTAB appends the initial residual in that case (:612-617)
    lr = []
    x = d["x"].copy()
    code, it, t = algebra.Dia_BiCGSTAB(A, x, d["b"].copy(), 100, 1e-6, lr)
    assert code == 0 and it == 0 and len(lr) == 1


def test_csr_max_iter_exhausted(gpu_lib):
    from carpio_gb300 import algebra
    d = golden("csr_bus685_cg")
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    x = np.zeros_like(d["b"])
    lr = []
    code, it, t = algebra.CG(A, x, d["b"].copy(), 5, 1e-14, lr)
    c2, x2, it2, t2, h2 = R.krylov_csr("cg", A.rowptr, A.colind, A.val, d["b"],
                                       np.zeros_like(d["b"]), 5, 1e-14)
    assert code == c2 == 1 and it == it2 == 5 and len(lr) == 5
    assert rel_l2(x, x2) < 1e-9
    assert np.allclose(lr, h2, rtol=1e-9)


def test_csr_device_pointers_and_repeatability(gpu_lib):
    torch = pytest.importorskip("torch")
    from carpio_gb300 import algebra
    d = golden("csr_pde225_dia_bicgstab")
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    xs = []
    for _ in range(3):
        x = torch.zeros(d["b"].size, dtype=torch.float64, device="cuda")
        b = torch.from_numpy(d["b"].copy()).cuda()
        algebra.Dia_BiCGSTAB(A, x, b, 1000, 1e-10)
        xs.append(x.cpu().numpy())
    # the reductions are fixed trees: runs are bitwise repeatable
    assert np.array_equal(xs[0].view(np.uint64), xs[1].view(np.uint64))
    assert np.array_equal(xs[0].view(np.uint64), xs[2].view(np.uint64))
    assert rel_l2(xs[0], d["x"]) < 1e-8


def test_csr_class_jacobi_matches_reference_test(gpu_lib):
    """test/algebra/_test_solver.hpp:129-163: Solver_Jacobi_ on 685_bus,
    b = 1, x0 = 1, tol 1e-6."""
    from carpio_gb300 import algebra
    d = golden("csr_bus685_jacobi_class")
    A = algebra.MatrixSCR(d["rowptr"], d["colind"], d["val"])
    s = algebra.Solver_Jacobi_(100000, 1e-6)
    x = np.ones(A.iLen())
    code = s.solve(A, x, np.ones(A.iLen()))
    assert code == 0
    assert abs(s.num_iter() - int(d["max_iter_out"])) <= 60
    assert s.residual() <= 1e-6
    assert rel_l2(x, d["x"]) < 1e-6
