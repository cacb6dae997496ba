// Algebra-level drop-in: carpio::CG / Jacobi / Dia_BiCGSTAB / BiCGSTAB and
// IC_CGS / IC_CG (lib/algebra/solver_matrix.hpp) on a MatrixSCR_ CSR
// matrix, one persistent cooperative launch per solve.
#include "internal.hpp"
#include "ic.cuh"
#include "mixed.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

namespace {

using namespace cg_dev;

__global__ void __launch_bounds__(kThreads) k_csr_solve(CsrOp op, FlatSpace sp,
		Vecs<double> v, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	krylov_run<double>(sp, op, v, sc, gc, bank);
}

// CARPIO_GPU_FLAG_MIXED: the kind's FP32 iterations inside FP64 refinement
__global__ void __launch_bounds__(kThreads) k_csr_solve_mixed(CsrOp op, FlatSpace sp,
		Vecs<double> v, MixedT<CsrOp32> mx, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	mixed_run(sp, op, v, mx, sc, false, gc, bank);
}

__global__ void k_to_float(const double* a, float* b, int n) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		b[i] = (float)a[i];
}

__global__ void __launch_bounds__(1024) k_csr_solve_ic(CsrOp op, IcOp ic,
		Vecs<double> v, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	if (sc.kind == CARPIO_GPU_IC_CGS) ic_cgs_run<false>(ic.n, op, ic, v, sc, gc, bank);
	else ic_cg_run<false>(ic.n, op, ic, v, sc, gc, bank);
}

// the five-point wavefront (ic.grid): block 0 holds one lane per grid row
__global__ void __launch_bounds__(kIcGridThreads, 1) k_csr_solve_ic_grid(CsrOp op, IcOp ic,
		Vecs<double> v, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	if (sc.kind == CARPIO_GPU_IC_CGS) ic_cgs_run<true>(ic.n, op, ic, v, sc, gc, bank);
	else ic_cg_run<true>(ic.n, op, ic, v, sc, gc, bank);
}

// carpio::Residual (solver_matrix.hpp:583-597), first part: r = b - A x per
// row in MatrixSCR_::operator*'s order (matrix_SparCompRow.hpp:236-249: from
// 0, s += x[col] * val, two roundings per term, so r is bit-exact), and per
// block the sums of squares nrm2 takes of b and of r (BLAS_Level1.hpp:556-577:
// the last element left out unless `full`; one element: |x[0]|).
__global__ void __launch_bounds__(kThreads) k_residual_part(CsrOp op, int n,
		const double* x, const double* b, int full, double* part) {
	double s[2] = { 0.0, 0.0 };
	const int counted = (full || n == 1) ? n : n - 1;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		double ax = 0.0;
		for (uint32_t e = op.rp[i]; e < op.rp[i + 1]; ++e)
			ax = __dadd_rn(ax, __dmul_rn(x[op.ci[e]], op.va[e]));
		const double r = __dsub_rn(b[i], ax);
		if (i < counted) {
			s[0] = fma(b[i], b[i], s[0]);
			s[1] = fma(r, r, s[1]);
		}
	}
	block_sum<double, 2>(s);
	if (threadIdx.x == 0) {
		part[2 * blockIdx.x] = s[0];
		part[2 * blockIdx.x + 1] = s[1];
	}
}

// second part, one warp: the partials in a fixed order, then
// nrm2(r) / nrm2(b) with normb = 1 when it is 0
__global__ void k_residual_final(int nb, const double* part, double* out) {
	double sb = 0.0, sr = 0.0;
	for (int k = threadIdx.x; k < nb; k += 32) {
		sb += part[2 * k];
		sr += part[2 * k + 1];
	}
	for (int o = 16; o > 0; o >>= 1) {
		sb += __shfl_down_sync(0xffffffffu, sb, o);
		sr += __shfl_down_sync(0xffffffffu, sr, o);
	}
	if (threadIdx.x == 0) {
		double normb = sqrt(sb);
		if (normb == 0.0) normb = 1;
		out[0] = sqrt(sr) / normb;
	}
}

struct CsrWs {
	std::mutex mu;
	cudaStream_t s = nullptr;
	cg_host::LaunchWs lw;
	cg_host::DevBuf rp, ci, va, vec, hist;
	cg_host::DevBuf icd, icu[3], icl[3], icf[2], icb[2];   // IC factor, levels
	cg_host::DevBuf ick[2], icn[2], icc[2], icv[2];         // packed level rows
	cg_host::DevBuf icg[3];                                 // five-point factor
	cg_host::DevBuf rx, rb, rpart;   // Residual: staged x, b; partials + result
	cg_host::DevBuf va32, vec32;     // MIXED: FP32 values and vectors
};

// ICPre (preconditioner.hpp:97-136): the upper triangle with its diagonal,
// columns ascending per row, factored by ICFactor (:20-48) in its order.
// Returns false when a row has no diagonal (the reference exits).
struct IcHost {
	std::vector<uint32_t> pntr, indx;
	std::vector<double> val;
};

bool ic_factor(int n, const uint32_t* rp, const uint32_t* ci, const double* va, IcHost& f) {
	f.pntr.assign(n + 1, 0);
	f.indx.clear();
	f.val.clear();
	for (int k = 0; k < n; ++k) {
		std::vector<std::pair<uint32_t, double> > row;
		for (uint32_t j = rp[k]; j < rp[k + 1]; ++j)
			if (ci[j] >= (uint32_t)k) row.push_back({ ci[j], va[j] });
		std::sort(row.begin(), row.end(),
				[](const std::pair<uint32_t, double>& a, const std::pair<uint32_t, double>& b) {
					return a.first < b.first;
				});
		for (auto& e : row) { f.indx.push_back(e.first); f.val.push_back(e.second); }
		f.pntr[k + 1] = (uint32_t)f.indx.size();
		if (row.empty() || row[0].first != (uint32_t)k) return false;
	}
	std::vector<uint32_t>& pntr = f.pntr;
	std::vector<uint32_t>& indx = f.indx;
	std::vector<double>& val = f.val;
	// the factorisation, step for step as ICFactor; indx is read one entry
	// past a row's end there, so keep a sentinel past the last entry
	indx.push_back(0);
	for (int k = 0; k < n - 1; ++k) {
		const uint32_t d = pntr[k];
		double z = val[d] = std::sqrt(val[d]);
		for (uint32_t i = d + 1; i < pntr[k + 1]; ++i) val[i] /= z;
		for (uint32_t i = d + 1; i < pntr[k + 1]; ++i) {
			z = val[i];
			const uint32_t h = indx[i];
			uint32_t g = i;
			for (uint32_t j = pntr[h]; j < pntr[h + 1]; ++j)
				for (; g < pntr[k + 1] && indx[g + 1] <= indx[j]; ++g)
					if (indx[g] == indx[j]) val[j] -= z * val[g];
		}
	}
	val[pntr[n - 1]] = std::sqrt(val[pntr[n - 1]]);
	indx.pop_back();
	return true;
}

// rows grouped by level: level[i] ascending, rows ascending within a level
void by_level(const std::vector<int>& level, std::vector<uint32_t>& ptr,
		std::vector<uint32_t>& rows) {
	const int nl = level.empty() ? 0 : *std::max_element(level.begin(), level.end()) + 1;
	ptr.assign(nl + 1, 0);
	for (int l : level) ++ptr[l + 1];
	for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
	rows.assign(level.size(), 0);
	std::vector<uint32_t> pos(ptr.begin(), ptr.end() - 1);
	for (size_t i = 0; i < level.size(); ++i) rows[pos[level[i]]++] = (uint32_t)i;
}

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
			|| !x || !max_iter || !tol || kind < 0 || kind > CARPIO_GPU_IC_CG)
		return CARPIO_GPU_EINVAL;
	if (hist_cap < 0 || (hist_cap > 0 && !resid_hist)) return CARPIO_GPU_EINVAL;
	const bool mixed = (flags & CARPIO_GPU_FLAG_MIXED) != 0;
	if (mixed && kind != CARPIO_GPU_CG && kind != CARPIO_GPU_DIA_BICGSTAB
			&& kind != CARPIO_GPU_BICGSTAB)
		return CARPIO_GPU_EINVAL;
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
	const bool ic = kind == CARPIO_GPU_IC_CGS || kind == CARPIO_GPU_IC_CG;
	const void* kern = ic ? (const void*)k_csr_solve_ic
	                      : mixed ? (const void*)k_csr_solve_mixed : (const void*)k_csr_solve;
	int blocks = coop_blocks(kern, n, 2);
	if ((rc = w.lw.ensure(blocks))) return rc;
	if ((rc = w.hist.ensure(sizeof(double) * (size_t)(hist_cap > 0 ? hist_cap : 1)))) return rc;
	CG_CK(cudaMemsetAsync(w.lw.ctl.p, 0, sizeof(Ctl), s));
	CsrOp op{ w.rp.as<uint32_t>(), w.ci.as<uint32_t>(), w.va.as<double>() };
	FlatSpace sp{ n };
	IcOp icop{};
	if (ic) {
		// the factor on the host (from host copies of the matrix)
		std::vector<uint32_t> hrp(n + 1), hci(nnz);
		std::vector<double> hva(nnz);
		CG_CK(cudaMemcpy(hrp.data(), rowptr, sizeof(uint32_t) * (n + 1), cudaMemcpyDefault));
		if (nnz) {
			CG_CK(cudaMemcpy(hci.data(), col, sizeof(uint32_t) * nnz, cudaMemcpyDefault));
			CG_CK(cudaMemcpy(hva.data(), val, sizeof(double) * nnz, cudaMemcpyDefault));
		}
		IcHost f;
		if (!ic_factor(n, hrp.data(), hci.data(), hva.data(), f)) return CARPIO_GPU_EZERODIAG;
		std::vector<double> dg(n);
		std::vector<uint32_t> up(n + 1, 0), ui, lcount(n + 1, 0);
		std::vector<double> uv;
		for (int i = 0; i < n; ++i) {
			dg[i] = f.val[f.pntr[i]];
			for (uint32_t e = f.pntr[i] + 1; e < f.pntr[i + 1]; ++e) {
				ui.push_back(f.indx[e]);
				uv.push_back(f.val[e]);
				++lcount[f.indx[e] + 1];
			}
			up[i + 1] = (uint32_t)ui.size();
		}
		// forward: the rows updating row k, ascending (transpose of the factor)
		std::vector<uint32_t> lp(n + 1, 0);
		for (int k = 0; k < n; ++k) lp[k + 1] = lp[k] + lcount[k + 1];
		std::vector<uint32_t> li(lp[n]), fill(lp.begin(), lp.end() - 1);
		std::vector<double> lv(lp[n]);
		for (int i = 0; i < n; ++i)
			for (uint32_t e = up[i]; e < up[i + 1]; ++e) {
				const uint32_t k = ui[e];
				li[fill[k]] = (uint32_t)i;
				lv[fill[k]++] = uv[e];
			}
		std::vector<int> lf(n, 0), lb(n, 0);
		for (int k = 0; k < n; ++k)
			for (uint32_t e = lp[k]; e < lp[k + 1]; ++e) lf[k] = std::max(lf[k], lf[li[e]] + 1);
		for (int i = n - 1; i >= 0; --i)
			for (uint32_t e = up[i]; e < up[i + 1]; ++e) lb[i] = std::max(lb[i], lb[ui[e]] + 1);
		std::vector<uint32_t> fptr, frows, bptr, brows;
		by_level(lf, fptr, frows);
		by_level(lb, bptr, brows);
		auto put = [&](DevBuf& d, const void* p, size_t bytes) {
			return to_device(d, p, bytes ? bytes : 8, s);
		};
		if ((rc = put(w.icd, dg.data(), sizeof(double) * n))) return rc;
		if ((rc = put(w.icu[0], up.data(), sizeof(uint32_t) * up.size()))) return rc;
		if ((rc = put(w.icu[1], ui.data(), sizeof(uint32_t) * ui.size()))) return rc;
		if ((rc = put(w.icu[2], uv.data(), sizeof(double) * uv.size()))) return rc;
		if ((rc = put(w.icl[0], lp.data(), sizeof(uint32_t) * lp.size()))) return rc;
		if ((rc = put(w.icl[1], li.data(), sizeof(uint32_t) * li.size()))) return rc;
		if ((rc = put(w.icl[2], lv.data(), sizeof(double) * lv.size()))) return rc;
		if ((rc = put(w.icf[0], fptr.data(), sizeof(uint32_t) * fptr.size()))) return rc;
		if ((rc = put(w.icf[1], frows.data(), sizeof(uint32_t) * frows.size()))) return rc;
		if ((rc = put(w.icb[0], bptr.data(), sizeof(uint32_t) * bptr.size()))) return rc;
		if ((rc = put(w.icb[1], brows.data(), sizeof(uint32_t) * brows.size()))) return rc;
		CG_CK(cudaStreamSynchronize(s));   // host vectors go out of scope
		icop.n = n;
		icop.d = w.icd.as<double>();
		icop.up = w.icu[0].as<uint32_t>();
		icop.ui = w.icu[1].as<uint32_t>();
		icop.uv = w.icu[2].as<double>();
		icop.lp = w.icl[0].as<uint32_t>();
		icop.li = w.icl[1].as<uint32_t>();
		icop.lv = w.icl[2].as<double>();
		icop.fptr = w.icf[0].as<uint32_t>();
		icop.frows = w.icf[1].as<uint32_t>();
		icop.nfl = (int)fptr.size() - 1;
		icop.bptr = w.icb[0].as<uint32_t>();
		icop.brows = w.icb[1].as<uint32_t>();
		icop.nbl = (int)bptr.size() - 1;
		// a five-point factor in natural order (every upper entry of row i at
		// i + 1 within a grid row, or at i + m, one m for all rows): the
		// wavefront sweeps of ic_sweep_grid, one lane per grid row
		int gm = 0;
		bool grid = !(flags & CARPIO_GPU_FLAG_NO_TILE);
		for (int i = 0; i < n && grid; ++i)
			for (uint32_t e = up[i]; e < up[i + 1]; ++e) {
				const long d = (long)ui[e] - i;
				if (d == 1) continue;
				if (!gm) gm = (int)d;
				else if (d != gm) { grid = false; break; }
			}
		grid = grid && gm >= 2 && n % gm == 0 && n / gm <= kIcGridThreads;
		for (int i = 0; i < n && grid; ++i) {
			int near = 0, far = 0;
			for (uint32_t e = up[i]; e < up[i + 1]; ++e) {
				if (ui[e] == (uint32_t)i + 1) ++near;
				else ++far;
			}
			if (near > 1 || far > 1 || (near && (i + 1) % gm == 0)) grid = false;
		}
		if (grid) {
			std::vector<double> gf(2 * (size_t)n, 0.0), gb(2 * (size_t)n, 0.0), rd(n);
			for (int i = 0; i < n; ++i) {
				rd[i] = 1.0 / dg[i];
				for (uint32_t e = up[i]; e < up[i + 1]; ++e) {
					const uint32_t c = ui[e];
					if (c == (uint32_t)i + 1) {
						gf[2 * (size_t)c + 1] = uv[e] / dg[c];
						gb[2 * (size_t)i] = uv[e] / dg[i];
					} else {
						gf[2 * (size_t)c] = uv[e] / dg[c];
						gb[2 * (size_t)i + 1] = uv[e] / dg[i];
					}
				}
			}
			if ((rc = put(w.icg[0], gf.data(), sizeof(double) * gf.size()))) return rc;
			if ((rc = put(w.icg[1], gb.data(), sizeof(double) * gb.size()))) return rc;
			if ((rc = put(w.icg[2], rd.data(), sizeof(double) * rd.size()))) return rc;
			CG_CK(cudaStreamSynchronize(s));
			icop.grid = 1;
			icop.gm = gm;
			icop.gR = n / gm;
			icop.gf = w.icg[0].as<double2>();
			icop.gb = w.icg[1].as<double2>();
			icop.grd = w.icg[2].as<double>();
		}
		// every level ends in a barrier: one block (block barriers, ~0.15 us)
		// when that beats the grid (grid barriers, ~1.5 us, but all SMs on
		// the ~10 vector passes of an iteration); a rough cost model, it
		// only picks between two correct launch shapes
		const double nlev = (double)icop.nfl + icop.nbl;
		const double t1 = nlev * 0.15 + 10.0 * n / kThreads * 0.05;
		const double tb = nlev * 1.5 + 10.0 * ((double)n / ((double)blocks * kThreads) * 0.05 + 1.5);
		if (t1 < tb && !grid) blocks = 1;
		// one block whose vector fits in shared memory: the level sweeps
		// run there on rows packed in level order (ic.cuh ic_apply_smem)
		if (blocks == 1 && sizeof(double) * (size_t)n <= 200 * 1024) {
			for (int pass = 0; pass < 2; ++pass) {
				const std::vector<uint32_t>& rows = pass == 0 ? frows : brows;
				const std::vector<uint32_t>& ep = pass == 0 ? lp : up;
				const std::vector<uint32_t>& ec = pass == 0 ? li : ui;
				const std::vector<double>& ev = pass == 0 ? lv : uv;
				const size_t np = rows.size();
				std::vector<uint32_t> pk(np), pc(np * kIcInline, 0);
				std::vector<int> pn(np);
				std::vector<double> pv(np * kIcInline, 0.0);
				for (size_t t = 0; t < np; ++t) {
					const uint32_t k = rows[t];
					pk[t] = k;
					pn[t] = (int)(ep[k + 1] - ep[k]);
					for (uint32_t e = ep[k], m = 0; e < ep[k + 1] && m < (uint32_t)kIcInline; ++e, ++m) {
						pc[t * kIcInline + m] = ec[e];
						pv[t * kIcInline + m] = ev[e];
					}
				}
				if ((rc = put(w.ick[pass], pk.data(), sizeof(uint32_t) * np))) return rc;
				if ((rc = put(w.icn[pass], pn.data(), sizeof(int) * np))) return rc;
				if ((rc = put(w.icc[pass], pc.data(), sizeof(uint32_t) * pc.size()))) return rc;
				if ((rc = put(w.icv[pass], pv.data(), sizeof(double) * pv.size()))) return rc;
				CG_CK(cudaStreamSynchronize(s));
			}
			icop.smem = 1;
			icop.fk = w.ick[0].as<uint32_t>();
			icop.bk = w.ick[1].as<uint32_t>();
			icop.fn = w.icn[0].as<int>();
			icop.bn = w.icn[1].as<int>();
			icop.fc = w.icc[0].as<uint32_t>();
			icop.bc = w.icc[1].as<uint32_t>();
			icop.fv = w.icv[0].as<double>();
			icop.bv = w.icv[1].as<double>();
		}
	}
	SolveCtl sc;
	sc.kind = kind;
	sc.max_iter = *max_iter;
	sc.tol = *tol;
	sc.flags = flags;
	sc.hist = hist_cap > 0 ? w.hist.as<double>() : nullptr;
	sc.hist_cap = hist_cap;
	sc.out = &w.lw.ctl.as<Ctl>()->out;
	GridCtl gc = make_gridctl(w.lw);
	if (ic) {
		void* args[] = { &op, &icop, &v, &sc, &gc };
		if (icop.grid) {
			// block 0 runs the sweeps with one lane per grid row; the vector
			// passes spread over blocks of the same size
			const void* gk = (const void*)k_csr_solve_ic_grid;
			int per_sm = 0;
			CG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gk, kIcGridThreads, 0));
			const int gb = (int)std::max(1L, std::min((long)std::max(per_sm, 1) * sm_count(),
					((long)n + kIcGridThreads - 1) / kIcGridThreads));
			if ((rc = w.lw.ensure(gb))) return rc;
			gc = make_gridctl(w.lw);
			CG_CK(cudaLaunchCooperativeKernel(gk, gb, kIcGridThreads, args, 0, s));
		} else if (icop.smem) {
			// one block of 1024 threads with the vector in shared memory
			const int sm = (int)(sizeof(double) * (size_t)n);
			CG_CK(cudaFuncSetAttribute((const void*)k_csr_solve_ic,
					cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
			CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve_ic, 1, 1024, args, sm, s));
		} else {
			CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve_ic, blocks,
					kThreads, args, 0, s));
		}
	} else if (mixed) {
		// FP32 copies of the values; 13 FP32 vectors (CG uses four)
		if ((rc = w.va32.ensure(sizeof(float) * (size_t)(nnz ? nnz : 1)))) return rc;
		if ((rc = w.vec32.ensure(sizeof(float) * (size_t)n * 13))) return rc;
		if (nnz) {
			const int nb = std::max(1, std::min((nnz + kThreads - 1) / kThreads, 4 * sm_count()));
			k_to_float<<<nb, kThreads, 0, s>>>(w.va.as<double>(), w.va32.as<float>(), nnz);
			CG_CK(cudaGetLastError());
		}
		MixedT<CsrOp32> mx;
		std::memset(&mx, 0, sizeof mx);
		mx.op32 = CsrOp32{ w.rp.as<uint32_t>(), w.ci.as<uint32_t>(), w.va32.as<float>() };
		float* fb = w.vec32.as<float>();
		float** fs[13] = { &mx.f.x, &mx.f.r, &mx.f.p, &mx.f.q, &mx.f.b, &mx.f.z,
			&mx.f.rt, &mx.f.ph, &mx.f.s, &mx.f.sh, &mx.f.t, &mx.f.v, &mx.f.d };
		for (int i = 0; i < 13; ++i) *fs[i] = fb + (size_t)i * n;
		mx.inner_tol = 1e-4;
		mx.inner_max = 1 << 30;
		void* args[] = { &op, &sp, &v, &mx, &sc, &gc };
		CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve_mixed, blocks,
				kThreads, args, 0, s));
	} else {
		void* args[] = { &op, &sp, &v, &sc, &gc };
		CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve, blocks,
				kThreads, args, 0, s));
	}
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

extern "C" int carpio_gpu_residual(int n, int nnz, const uint32_t* rowptr,
		const uint32_t* col, const double* val, const double* x, const double* b,
		uint32_t flags, double* resid) {
	using namespace cg_host;
	if (n <= 0 || nnz < 0 || !rowptr || (!col && nnz) || (!val && nnz) || !x || !b
			|| !resid)
		return CARPIO_GPU_EINVAL;
	CsrWs& w = ws();
	std::lock_guard<std::mutex> lock(w.mu);
	if (!w.s) CG_CK(cudaStreamCreateWithFlags(&w.s, cudaStreamNonBlocking));
	cudaStream_t s = w.s;
	int rc;
	if ((rc = to_device(w.rp, rowptr, sizeof(uint32_t) * (n + 1), s))) return rc;
	if ((rc = to_device(w.ci, col, sizeof(uint32_t) * (size_t)nnz, s))) return rc;
	if ((rc = to_device(w.va, val, sizeof(double) * (size_t)nnz, s))) return rc;
	if ((rc = to_device(w.rx, x, sizeof(double) * n, s))) return rc;
	if ((rc = to_device(w.rb, b, sizeof(double) * n, s))) return rc;
	const int nb = std::max(1, std::min((n + kThreads - 1) / kThreads, 4 * sm_count()));
	if ((rc = w.rpart.ensure(sizeof(double) * (2 * (size_t)nb + 1)))) return rc;
	double* part = w.rpart.as<double>();
	CsrOp op{ w.rp.as<uint32_t>(), w.ci.as<uint32_t>(), w.va.as<double>() };
	k_residual_part<<<nb, kThreads, 0, s>>>(op, n, w.rx.as<double>(), w.rb.as<double>(),
			(flags & CARPIO_GPU_FLAG_FULL_NRM2) ? 1 : 0, part);
	CG_CK(cudaGetLastError());
	k_residual_final<<<1, 32, 0, s>>>(nb, part, part + 2 * nb);
	CG_CK(cudaGetLastError());
	double r = 0.0;
	CG_CK(cudaMemcpyAsync(&r, part + 2 * nb, sizeof r, cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	*resid = r;
	return 0;
}
