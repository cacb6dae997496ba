// carpio_gpu.hpp -- C++ host adapters over the C ABI (carpio_gpu.h) with the
// signatures of the reference's solver entry points, so a C++ caller of
// hyperpower/carpios switches by changing the namespace:
//
//   carpio::CG(A, x, b, max_iter, tol, lresid)          lib/algebra/solver_matrix.hpp:264
//   carpio_gpu::CG(A, x, b, max_iter, tol, lresid)      this header
//
// MAT is any CSR type with the MatrixSCR_ accessors iLen(), NumNonzeros(),
// row_ptr(i), col_ind(k), val(k) (lib/algebra/matrix_SparCompRow.hpp);
// ARR any vector with size() and operator[] (ArrayListV,
// lib/algebra/array_list.hpp). Header-only; link with -lcarpio_gpu.
#ifndef CARPIO_GPU_HPP
#define CARPIO_GPU_HPP

#include <cstdint>
#include <list>
#include <stdexcept>
#include <string>
#include <vector>

#include "carpio_gpu.h"

namespace carpio_gpu {

// Raised for the negative (library) codes; the reference's own codes 0..3
// are returned as the reference returns them.
struct Error : std::runtime_error {
	int code;
	explicit Error(int c)
		: std::runtime_error(std::string("carpio_gpu: ") + carpio_gpu_strerror(c)),
		  code(c) {}
};

template<class MAT, class ARR>
int krylov(int kind, const MAT& A, ARR& x, const ARR& b, int& max_iter,
		double& tol, std::list<double>& lresid, uint32_t flags = 0) {
	const int n = (int)A.iLen();
	const int nnz = (int)A.NumNonzeros();
	std::vector<uint32_t> rp(n + 1), ci(nnz);
	std::vector<double> va(nnz), xv(n), bv(n), hist(max_iter > 0 ? max_iter + 2 : 1);
	for (int i = 0; i <= n; ++i) rp[i] = (uint32_t)A.row_ptr(i);
	for (int k = 0; k < nnz; ++k) {
		ci[k] = (uint32_t)A.col_ind(k);
		va[k] = (double)A.val(k);
	}
	for (int i = 0; i < n; ++i) {
		xv[i] = (double)x[i];
		bv[i] = (double)b[i];
	}
	int hl = 0;
	int code = carpio_gpu_krylov_csr(kind, n, nnz, rp.data(), ci.data(),
			va.data(), bv.data(), xv.data(), &max_iter, &tol, hist.data(),
			(int)hist.size(), &hl, flags);
	if (code < 0) throw Error(code);
	for (int i = 0; i < n; ++i) x[i] = xv[i];
	for (int k = 0; k < hl && k < (int)hist.size(); ++k) lresid.push_back(hist[k]);
	return code;
}

template<class MAT, class ARR>
int CG(const MAT& A, ARR& x, const ARR& b, int& max_iter, double& tol,
		std::list<double>& lresid) {
	return krylov(CARPIO_GPU_CG, A, x, b, max_iter, tol, lresid);
}
template<class MAT, class ARR>
int Jacobi(const MAT& A, ARR& x, const ARR& b, int& max_iter, double& tol,
		std::list<double>& lresid) {
	return krylov(CARPIO_GPU_JACOBI, A, x, b, max_iter, tol, lresid);
}
template<class MAT, class ARR>
int Dia_BiCGSTAB(const MAT& A, ARR& x, const ARR& b, int& max_iter,
		double& tol, std::list<double>& lresid) {
	return krylov(CARPIO_GPU_DIA_BICGSTAB, A, x, b, max_iter, tol, lresid);
}
template<class MAT, class ARR>
int BiCGSTAB(const MAT& A, ARR& x, const ARR& b, int& max_iter, double& tol,
		std::list<double>& lresid) {
	return krylov(CARPIO_GPU_BICGSTAB, A, x, b, max_iter, tol, lresid);
}
// IC(0)-preconditioned solvers (solver_matrix.hpp:318-438): the factor is
// computed on the host in ICPre's order, the triangular solves run on the GPU
template<class MAT, class ARR>
int IC_CGS(const MAT& A, ARR& x, const ARR& b, int& max_iter, double& tol,
		std::list<double>& lresid) {
	return krylov(CARPIO_GPU_IC_CGS, A, x, b, max_iter, tol, lresid);
}
template<class MAT, class ARR>
int IC_CG(const MAT& A, ARR& x, const ARR& b, int& max_iter, double& tol,
		std::list<double>& lresid) {
	return krylov(CARPIO_GPU_IC_CG, A, x, b, max_iter, tol, lresid);
}

// RAII handles for the structure level.
class Grid {
public:
	Grid(int nx, int ny, int gl, double x0, double x1, double y0, double y1) {
		int c = carpio_gpu_grid_create_uniform(nx, ny, gl, x0, x1, y0, y1, &g_);
		if (c) throw Error(c);
	}
	~Grid() { if (g_) carpio_gpu_grid_destroy(g_); }
	Grid(const Grid&) = delete;
	Grid& operator=(const Grid&) = delete;
	carpio_gpu_grid* get() const { return g_; }
private:
	carpio_gpu_grid* g_ = nullptr;
};

// Poisson_::run() for a set_depend'ed field: source and phi are full
// SpaceT fields (nx+2gl) x (ny+2gl), y contiguous; phi's normal cells are
// the initial guess and receive the solution.
inline int poisson_solve(Grid& g, const carpio_gpu_bc& bc, double beta,
		const double* source, double* phi, const carpio_gpu_solver_cfg& cfg,
		carpio_gpu_solver_stats* stats = nullptr) {
	int c = carpio_gpu_poisson_solve(g.get(), &bc, beta, source, phi, &cfg,
			nullptr, 0, stats);
	if (c < 0) throw Error(c);
	return c;
}

}  // namespace carpio_gpu

#endif
