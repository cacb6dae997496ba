// Algebra-level drop-in: carpio::CG / Jacobi / Dia_BiCGSTAB / BiCGSTAB
// (lib/algebra/solver_matrix.hpp) on a MatrixSCR_ CSR matrix, one persistent
// cooperative launch per solve.
#include "internal.hpp"

#include <cmath>
#include <mutex>

namespace {

using namespace cg_dev;

__global__ void __launch_bounds__(kThreads) k_csr_solve(CsrOp op, FlatSpace sp,
		Vecs<double> v, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	krylov_run<double>(sp, op, v, sc, gc, bank);
}

struct CsrWs {
	std::mutex mu;
	cudaStream_t s = nullptr;
	cg_host::LaunchWs lw;
	cg_host::DevBuf rp, ci, va, vec, hist;
};

// Never destroyed: freeing device memory from a static destructor can run
// after the CUDA runtime has shut down at process exit.
CsrWs& ws() {
	static CsrWs* w = new CsrWs();
	return *w;
}

bool finite_all(const double* p, int n) {
	for (int i = 0; i < n; ++i)
		if (!std::isfinite(p[i])) return false;
	return true;
}

}  // namespace

extern "C" int carpio_gpu_krylov_csr(int kind, int n, int nnz,
		const uint32_t* rowptr, const uint32_t* col, const double* val,
		const double* b, double* x, int* max_iter, double* tol,
		double* resid_hist, int hist_cap, int* hist_len, uint32_t flags) {
	using namespace cg_host;
	if (n <= 0 || nnz < 0 || !rowptr || (!col && nnz) || (!val && nnz) || !b
			|| !x || !max_iter || !tol || kind < 0 || kind > 3)
		return CARPIO_GPU_EINVAL;
	if (hist_cap < 0 || (hist_cap > 0 && !resid_hist)) return CARPIO_GPU_EINVAL;
	CsrWs& w = ws();
	std::lock_guard<std::mutex> lock(w.mu);
	if (!w.s) CG_CK(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking));
	cudaStream_t s = w.s;
	// host inputs are checked for NaN/Inf before any work (the reference
	// would propagate them silently)
	if (!is_device_ptr(b) && !finite_all(b, n)) return CARPIO_GPU_ENONFINITE;
	if (!is_device_ptr(x) && !finite_all(x, n)) return CARPIO_GPU_ENONFINITE;
	if (val && !is_device_ptr(val) && !finite_all(val, nnz)) return CARPIO_GPU_ENONFINITE;
	int rc;
	if ((rc = to_device(w.rp, rowptr, sizeof(uint32_t) * (n + 1), s))) return rc;
	if ((rc = to_device(w.ci, col, sizeof(uint32_t) * (size_t)nnz, s))) return rc;
	if ((rc = to_device(w.va, val, sizeof(double) * (size_t)nnz, s))) return rc;
	const int nvec = 13;
	if ((rc = w.vec.ensure(sizeof(double) * (size_t)n * nvec))) return rc;
	double* base = w.vec.as<double>();
	Vecs<double> v;
	double** slots[nvec] = { &v.x, &v.b, &v.r, &v.p, &v.q, &v.z, &v.rt, &v.ph,
		&v.s, &v.sh, &v.t, &v.v, &v.d };
	for (int i = 0; i < nvec; ++i) *slots[i] = base + (size_t)i * n;
	CG_CK(cudaMemcpyAsync(v.x, x, sizeof(double) * n, cudaMemcpyDefault, s));
	CG_CK(cudaMemcpyAsync(v.b, b, sizeof(double) * n, cudaMemcpyDefault, s));
	int blocks = coop_blocks((const void*)k_csr_solve, n, 2);
	if ((rc = w.lw.ensure(blocks))) return rc;
	if ((rc = w.hist.ensure(sizeof(double) * (size_t)(hist_cap > 0 ? hist_cap : 1)))) return rc;
	CG_CK(cudaMemsetAsync(w.lw.ctl.p, 0, sizeof(Ctl), s));
	CsrOp op{ w.rp.as<uint32_t>(), w.ci.as<uint32_t>(), w.va.as<double>() };
	FlatSpace sp{ n };
	SolveCtl sc;
	sc.kind = kind;
	sc.max_iter = *max_iter;
	sc.tol = *tol;
	sc.flags = flags;
	sc.hist = hist_cap > 0 ? w.hist.as<double>() : nullptr;
	sc.hist_cap = hist_cap;
	sc.out = &w.lw.ctl.as<Ctl>()->out;
	GridCtl gc = make_gridctl(w.lw);
	void* args[] = { &op, &sp, &v, &sc, &gc };
	CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve, blocks,
			kThreads, args, 0, s));
	CG_CK(cudaMemcpyAsync(w.lw.host_ctl, w.lw.ctl.p, sizeof(Ctl),
			cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	const Ctl& c = *w.lw.host_ctl;
	if (c.err) return c.err;
	int code = c.out.code;
	if (code < 0) return code;
	CG_CK(cudaMemcpyAsync(x, v.x, sizeof(double) * n, cudaMemcpyDefault, s));
	int keep = c.out.hist_len < hist_cap ? c.out.hist_len : hist_cap;
	if (keep > 0)
		CG_CK(cudaMemcpyAsync(resid_hist, sc.hist, sizeof(double) * keep,
				cudaMemcpyDefault, s));
	CG_CK(cudaStreamSynchronize(s));
	*max_iter = c.out.iters;
	*tol = c.out.tol;
	if (hist_len) *hist_len = c.out.hist_len;
	return code;
}
