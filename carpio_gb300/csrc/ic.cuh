// IC(0)-preconditioned Krylov solvers of the reference: carpio::IC_CG and
// carpio::IC_CGS (lib/algebra/solver_matrix.hpp:318-438) with ICPre
// (lib/algebra/preconditioner.hpp:20-177). The incomplete Cholesky factor is
// computed on the host in the reference's order (csr.cu); here it is applied
// by level-scheduled triangular solves inside the persistent solver launch:
// the rows of one level depend only on rows of earlier levels, so a level is
// one parallel pass and levels are separated by grid barriers.
#pragma once

#include "krylov.cuh"

namespace cg_dev {

// ICPre's factor, rearranged for level scheduling. Forward solve (the
// reference's column sweep, y[indx] -= z val) gathered per row k: the rows
// i < k that update k (lp/li/lv, i ascending, i.e. the reference's order of
// updates); backward solve per row i: its off-diagonal entries (up/ui/uv,
// columns ascending).
constexpr int kIcInline = 4;   // entries of a row packed inline (one block)

struct IcOp {
	int n;
	const double* d;                                  // val_[pntr_[i]]
	const uint32_t *lp, *li; const double* lv;
	const uint32_t *up, *ui; const double* uv;
	const uint32_t *fptr, *frows; int nfl;            // forward levels
	const uint32_t *bptr, *brows; int nbl;            // backward levels
	// one-block launches: the solve vector in shared memory, and every
	// level position's row packed (row, diagonal, entry count, up to
	// kIcInline (column, value) pairs; longer rows read the lists above)
	// so that the next level's data loads while the current level runs
	int smem;                                         // 1: use the path below
	const uint32_t *fk, *bk;                          // row of each position
	const int *fn, *bn;                               // its entry count
	const uint32_t *fc, *bc;                          // [position][kIcInline]
	const double *fv, *bv;
	// five-point factors in natural order (row k = j m + i coupled to k - 1
	// and k + 1 within a grid row of length m, to k - m and k + m across
	// rows, nothing wrapping around a row end): the two triangular solves run
	// as a skewed wavefront in block 0 (ic_sweep_grid)
	int grid;                                         // 1: use that path
	int gm, gR;                                       // row length m, rows R
	const double2* gf;      // forward {U(k-m, k), U(k-1, k)} / d_k, 0 where absent
	const double2* gb;      // backward {U(k, k+1), U(k, k+m)} / d_k, 0 where absent
	const double* grd;      // 1 / d_k
};

// One level position's packed row, loaded ahead of its level.
struct IcRow {
	uint32_t k;
	int cnt;
	double d;
	uint32_t c[kIcInline];
	double v[kIcInline];
};

__device__ __forceinline__ void ic_load_row(const IcOp& ic, bool fwd, uint32_t pos, IcRow& r) {
	const uint32_t* K = fwd ? ic.fk : ic.bk;
	const int* N = fwd ? ic.fn : ic.bn;
	const uint32_t* Cc = fwd ? ic.fc : ic.bc;
	const double* V = fwd ? ic.fv : ic.bv;
	r.k = __ldg(K + pos);
	r.cnt = __ldg(N + pos);
	r.d = __ldg(ic.d + r.k);
#pragma unroll
	for (int m = 0; m < kIcInline; ++m) {
		r.c[m] = __ldg(Cc + (size_t)pos * kIcInline + m);
		r.v[m] = __ldg(V + (size_t)pos * kIcInline + m);
	}
}

// ic_apply on one block with the vector in shared memory (sm: n doubles).
// The operations and their order are those of the global-memory path.
__device__ void ic_apply_smem(const IcOp& ic, const double* in, double* out, double* sm) {
	const int T = blockDim.x, tid = threadIdx.x;
	for (int t = tid; t < ic.n; t += T) sm[t] = ldcg(in + t);
	__syncthreads();
	for (int pass = 0; pass < 2; ++pass) {
		const bool fwd = pass == 0;
		const uint32_t* ptr = fwd ? ic.fptr : ic.bptr;
		const int nl = fwd ? ic.nfl : ic.nbl;
		IcRow cur, nxt;
		uint32_t lo = ptr[0], hi = ptr[nl > 0 ? 1 : 0];
		if (nl > 0 && lo + tid < hi) ic_load_row(ic, fwd, lo + tid, cur);
		for (int l = 0; l < nl; ++l) {
			// the next level's first row for this thread (every thread that
			// has one there, whether or not it has a row at this level), in
			// flight while this level computes
			const uint32_t lo2 = hi, hi2 = l + 1 < nl ? ptr[l + 2] : hi;
			if (lo2 + tid < hi2) ic_load_row(ic, fwd, lo2 + tid, nxt);
			// rows wider than the block run in several rounds
			for (uint32_t pos = lo + tid; pos < hi; pos += T) {
				IcRow r;
				if (pos == lo + tid) r = cur;
				else ic_load_row(ic, fwd, pos, r);
				if (fwd) {
					double y = sm[r.k];
					if (r.cnt <= kIcInline) {
#pragma unroll
						for (int m = 0; m < kIcInline; ++m)
							if (m < r.cnt) y = __dsub_rn(y, __dmul_rn(sm[r.c[m]], r.v[m]));
					} else {
						for (uint32_t e = ic.lp[r.k]; e < ic.lp[r.k + 1]; ++e)
							y = __dsub_rn(y, __dmul_rn(sm[ic.li[e]], ic.lv[e]));
					}
					sm[r.k] = __ddiv_rn(y, r.d);
				} else {
					double z = 0.0;
					if (r.cnt <= kIcInline) {
#pragma unroll
						for (int m = 0; m < kIcInline; ++m)
							if (m < r.cnt) z = __dadd_rn(z, __dmul_rn(sm[r.c[m]], r.v[m]));
					} else {
						for (uint32_t e = ic.up[r.k]; e < ic.up[r.k + 1]; ++e)
							z = __dadd_rn(z, __dmul_rn(sm[ic.ui[e]], ic.uv[e]));
					}
					sm[r.k] = __ddiv_rn(__dsub_rn(sm[r.k], z), r.d);
				}
			}
			__syncthreads();
			cur = nxt;
			lo = lo2;
			hi = hi2;
		}
	}
	for (int t = tid; t < ic.n; t += T) out[t] = sm[t];
	__syncthreads();
}

// ------------------------------------------------- five-point wavefront --
// The triangular solves of a factor with the five-point pattern, in one
// block: lane l of warp w owns grid row j = 32 w + l and walks its m cells in
// order, skewed one step behind lane l - 1 (forward; ahead of it backward),
// so that the row neighbour's value is in the lane's own register and the
// value across rows arrives by one warp shuffle from the previous step. The
// warps run in lockstep over global steps, warp w kIcLag steps behind warp
// w - 1, with a barrier of the sweeping warps every kIcSync steps: lane 31's
// value of column t (forward) goes into a shared-memory ring at one step and
// the next warp's lane 0 reads it kIcSync steps later, after that barrier.
// No flags, no per-step fences. Inputs, coefficients and reciprocals of the
// next kIcAhead cells wait in registers.
// The arithmetic is the reference's update (ICPre::solve,
// preconditioner.hpp:143-161), y_k = (x_k - sum_i U(i, k) y_i) / d_k, with
// the division distributed: the host scales each coefficient by 1 / d_k and
// the lane forms x_k / d_k while it waits, so that a step's dependent chain
// is two fused multiply-adds (the row neighbour's, then the shuffled one);
// the result is within a few roundings of the reference's.
constexpr int kIcRing = 64;          // ring columns per warp boundary
constexpr int kIcAhead = 8;          // cells loaded ahead of their step
constexpr int kIcSync = 8;           // steps between barriers (divides kIcAhead)
constexpr int kIcLag = 31 + kIcSync; // steps between neighbouring warps
constexpr int kIcGridThreads = 512;  // block size of the wavefront launch: rows <= 512
static_assert(kIcAhead % kIcSync == 0 && 2 * kIcSync <= kIcRing, "ring");

__device__ __forceinline__ void ic_bar(int threads) {
	asm volatile("bar.sync 1, %0;" :: "r"(threads) : "memory");
}

// out = M^-1 in for a five-point factor (ic.grid), run by one block of at
// least 32 * ceil(R / 32) threads; `in` and `out` in global memory
// (distinct arrays). Ends with a block barrier.
__device__ void ic_sweep_grid(const IcOp& ic, const double* in, double* out) {
	__shared__ double ring[kIcGridThreads / 32][kIcRing];   // [boundary][column mod ring]
	const int m = ic.gm, R = ic.gR, W = (R + 31) >> 5;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if (warp < W) {
		const int j = warp * 32 + lane;
		const bool act = j < R;
		const int nsteps = (W - 1) * kIcLag + m + 31;
		for (int pass = 0; pass < 2; ++pass) {
			const bool fwd = pass == 0;
			// forward: lane 0 takes row j - 1 from warp - 1's lane 31 through
			// ring `warp`, lane 31 feeds ring warp + 1; backward: lane 31 takes
			// row j + 1 from warp + 1's lane 0 through ring warp + 1, lane 0
			// feeds ring `warp`
			const int skew = fwd ? lane : 31 - lane;
			const int off = (fwd ? warp : W - 1 - warp) * kIcLag + skew;
			const bool edge_lane = fwd ? lane == 0 : lane == 31;
			const bool cons_lane = fwd ? (lane == 0 && warp > 0) : (lane == 31 && warp + 1 < W);
			const bool prod_lane = fwd ? (lane == 31 && warp + 1 < W) : (lane == 0 && warp > 0);
			const int cb = fwd ? warp : warp + 1;     // ring read
			const int pb = fwd ? warp + 1 : warp;     // ring written
			const double* src = fwd ? in : out;
			const double2* cf = fwd ? ic.gf : ic.gb;
			const size_t row = (size_t)j * m;
			auto cell = [&](int t) { return row + (size_t)(fwd ? t : m - 1 - t); };
			double pin[kIcAhead], pc0[kIcAhead], pc1[kIcAhead], prd[kIcAhead];
#pragma unroll
			for (int u = 0; u < kIcAhead; ++u) {
				const int t = u - off;
				pin[u] = pc0[u] = pc1[u] = prd[u] = 0.0;
				if (act && t >= 0 && t < m) {
					const size_t k = cell(t);
					const double2 c = __ldg(cf + k);
					pin[u] = ldcg(src + k);
					pc0[u] = c.x;
					pc1[u] = c.y;
					prd[u] = __ldg(ic.grd + k);
				}
			}
			double res = 0.0;                          // the previous step's value
			for (int S0 = 0; S0 < nsteps; S0 += kIcAhead) {
#pragma unroll
				for (int u = 0; u < kIcAhead; ++u) {
					const int t = S0 + u - off;        // this lane's cell
					double nb = fwd ? __shfl_up_sync(0xffffffffu, res, 1)
					                : __shfl_down_sync(0xffffffffu, res, 1);
					if (edge_lane) nb = 0.0;           // no row beyond the edge
					const bool on = act && t >= 0 && t < m;
					if (on) {
						if (cons_lane) nb = ring[cb][t & (kIcRing - 1)];
						const double own = t > 0 ? res : 0.0;   // the row neighbour
						double y = pin[u] * prd[u];
						if (fwd) {
							y = fma(-pc1[u], own, y);     // U(k-1, k) / d_k z_{k-1}
							y = fma(-pc0[u], nb, y);      // U(k-m, k) / d_k z_{k-m}
						} else {
							y = fma(-pc0[u], own, y);     // U(k, k+1) / d_k z_{k+1}
							y = fma(-pc1[u], nb, y);      // U(k, k+m) / d_k z_{k+m}
						}
						out[cell(t)] = y;
						res = y;
						if (prod_lane) ring[pb][t & (kIcRing - 1)] = y;
					}
					// the slot's next cell: kIcAhead steps on
					const int tn = t + kIcAhead;
					if (act && tn >= 0 && tn < m) {
						const size_t k = cell(tn);
						const double2 c = __ldg(cf + k);
						pin[u] = ldcg(src + k);
						pc0[u] = c.x;
						pc1[u] = c.y;
						prd[u] = __ldg(ic.grd + k);
					}
					if ((u % kIcSync) == kIcSync - 1) ic_bar(W * 32);
				}
			}
			ic_bar(W * 32);   // the forward's writes before the backward's reads
		}
	}
	__syncthreads();
}

#define GLOOP(cnt)                                                             \
	for (int t = blockIdx.x * blockDim.x + threadIdx.x, _c = (cnt); t < _c;  \
			t += gridDim.x * blockDim.x)

// out = M^-1 in (ICPre::solve); exact IEEE operations in the reference's
// order, so the result does not depend on the level split
// GRID: the launch uses the five-point wavefront (ic.grid set)
template<bool GRID>
__device__ bool ic_apply(const IcOp& ic, const double* in, double* out,
		const GridCtl& gc) {
	if constexpr (GRID) {
		// block 0 sweeps; the callers' grid barrier before ordered `in`
		if (blockIdx.x == 0) ic_sweep_grid(ic, in, out);
		return grid_sync<true>(gc);
	}
	if (ic.smem && gridDim.x == 1) {
		extern __shared__ double ic_sm[];
		// the block barrier before (the callers' grid_sync<true>) ordered
		// `in`; the one at the end orders `out` for the next pass
		ic_apply_smem(ic, in, out, ic_sm);
		return true;
	}
	GLOOP(ic.n) out[t] = in[t];
	if (!grid_sync<true>(gc)) return false;
	for (int l = 0; l < ic.nfl; ++l) {
		const uint32_t b0 = ic.fptr[l];
		GLOOP((int)(ic.fptr[l + 1] - b0)) {
			const uint32_t k = ic.frows[b0 + t];
			double y = ldcg(out + k);
			for (uint32_t e = ic.lp[k]; e < ic.lp[k + 1]; ++e)
				y = __dsub_rn(y, __dmul_rn(ldcg(out + ic.li[e]), ic.lv[e]));
			out[k] = __ddiv_rn(y, ic.d[k]);
		}
		if (!grid_sync<true>(gc)) return false;
	}
	for (int l = 0; l < ic.nbl; ++l) {
		const uint32_t b0 = ic.bptr[l];
		GLOOP((int)(ic.bptr[l + 1] - b0)) {
			const uint32_t i = ic.brows[b0 + t];
			double z = 0.0;
			for (uint32_t e = ic.up[i]; e < ic.up[i + 1]; ++e)
				z = __dadd_rn(z, __dmul_rn(ldcg(out + ic.ui[e]), ic.uv[e]));
			out[i] = __ddiv_rn(__dsub_rn(ldcg(out + i), z), ic.d[i]);
		}
		if (!grid_sync<true>(gc)) return false;
	}
	return true;
}

// grid sums of NV products (full dot products, dot() of BLAS_Level1)
template<int NV>
__device__ __forceinline__ bool dots(const double* const (&a)[NV], const double* const (&b)[NV],
		int n, const GridCtl& gc, int& bank, double (&res)[NV]) {
	double acc[NV];
#pragma unroll
	for (int m = 0; m < NV; ++m) acc[m] = 0.0;
	GLOOP(n) {
#pragma unroll
		for (int m = 0; m < NV; ++m) acc[m] = fma(ldcg(a[m] + t), ldcg(b[m] + t), acc[m]);
	}
	if (!grid_allreduce<double, NV, true>(acc, gc, bank)) return false;
#pragma unroll
	for (int m = 0; m < NV; ++m) res[m] = acc[m];
	return true;
}

// nrm2 with the reference's quirk (the last element left out unless FULL_NRM2
// or n == 1), as a relative residual
__device__ __forceinline__ bool nrm2_rel(const double* r, int n, bool full, double normb,
		const GridCtl& gc, int& bank, double& resid) {
	double acc[1] = { 0.0 };
	GLOOP(n) {
		if (t != n - 1 || full) { const double x = ldcg(r + t); acc[0] = fma(x, x, acc[0]); }
	}
	if (!grid_allreduce<double, 1, true>(acc, gc, bank)) return false;
	resid = sqrt(acc[0]) / normb;
	return true;
}

// r = b - A x; normb = nrm2(b) (1 when zero); resid = nrm2(r) / normb
template<class Op>
__device__ bool ic_start(const Op& op, const Vecs<double>& v, int n, bool full,
		const GridCtl& gc, int& bank, double& normb, double& resid) {
	double acc[2] = { 0.0, 0.0 };
	GLOOP(n) {
		const double bb = v.b[t];
		const double rr = bb - op.apply(v.x, t, t);
		v.r[t] = rr;
		if (t != n - 1 || full) { acc[0] = fma(bb, bb, acc[0]); acc[1] = fma(rr, rr, acc[1]); }
	}
	if (!grid_allreduce<double, 2, true>(acc, gc, bank)) return false;
	normb = sqrt(acc[0]);
	if (normb == 0.0) normb = 1;
	resid = sqrt(acc[1]) / normb;
	return true;
}

// carpio::IC_CG (solver_matrix.hpp:318-374)
template<bool GRID, class Op>
__device__ void ic_cg_run(int n, const Op& op, const IcOp& ic, const Vecs<double>& v,
		const SolveCtl& sc, const GridCtl& gc, int& bank) {
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || n == 1;
	int hl = 0;
	double normb, resid;
	if (!ic_start(op, v, n, full, gc, bank, normb, resid)) return;
	if (resid <= sc.tol) { finish(sc, 0, 0, resid, hl); return; }
	double rho_1 = 0.0;
	for (int it = 1; it <= sc.max_iter; ++it) {
		if (!grid_sync<true>(gc)) return;
		if (!ic_apply<GRID>(ic, v.r, v.z, gc)) return;           // z = M^-1 r
		double rz[1];
		{
			const double* a[1] = { v.r };
			const double* b[1] = { v.z };
			if (!dots<1>(a, b, n, gc, bank, rz)) return;
		}
		const double rho = rz[0];
		const double beta = it == 1 ? 0.0 : rho / rho_1;
		GLOOP(n) v.p[t] = it == 1 ? v.z[t] : fma(beta, v.p[t], v.z[t]);
		if (!grid_sync<true>(gc)) return;
		GLOOP(n) v.q[t] = op.apply(v.p, t, t);
		if (!grid_sync<true>(gc)) return;
		double pq[1];
		{
			const double* a[1] = { v.p };
			const double* b[1] = { v.q };
			if (!dots<1>(a, b, n, gc, bank, pq)) return;
		}
		const double alpha = rho / pq[0];
		GLOOP(n) {
			v.x[t] = fma(alpha, v.p[t], v.x[t]);
			v.r[t] = fma(-alpha, v.q[t], v.r[t]);
		}
		if (!grid_sync<true>(gc)) return;
		if (!nrm2_rel(v.r, n, full, normb, gc, bank, resid)) return;
		hist_push(sc, hl, resid);
		if (resid <= sc.tol) { finish(sc, 0, it, resid, hl); return; }
		rho_1 = rho;
	}
	finish(sc, 1, sc.max_iter, resid, hl);
}

// carpio::IC_CGS (solver_matrix.hpp:376-438); rtilde = rt, u = s, phat = ph,
// vhat = v, uhat = sh, qhat = t, u + q = d
template<bool GRID, class Op>
__device__ void ic_cgs_run(int n, const Op& op, const IcOp& ic, const Vecs<double>& v,
		const SolveCtl& sc, const GridCtl& gc, int& bank) {
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || n == 1;
	int hl = 0;
	double normb, resid;
	if (!ic_start(op, v, n, full, gc, bank, normb, resid)) return;
	GLOOP(n) v.rt[t] = v.r[t];
	if (resid <= sc.tol) { finish(sc, 0, 0, resid, hl); return; }
	double rho_2 = 0.0;
	for (int it = 1; it <= sc.max_iter; ++it) {
		if (!grid_sync<true>(gc)) return;
		double r1[1];
		{
			const double* a[1] = { v.rt };
			const double* b[1] = { v.r };
			if (!dots<1>(a, b, n, gc, bank, r1)) return;
		}
		const double rho_1 = r1[0];
		if (rho_1 == 0.0) {
			// the reference returns with max_iter unchanged
			if (!nrm2_rel(v.r, n, full, normb, gc, bank, resid)) return;
			finish(sc, 2, sc.max_iter, resid, hl);
			return;
		}
		if (it == 1) {
			GLOOP(n) { const double r = v.r[t]; v.s[t] = r; v.p[t] = r; }
		} else {
			const double beta = rho_1 / rho_2;
			GLOOP(n) {
				const double u = fma(beta, v.q[t], v.r[t]);
				v.s[t] = u;
				v.p[t] = fma(beta, fma(beta, v.p[t], v.q[t]), u);
			}
		}
		if (!grid_sync<true>(gc)) return;
		if (!ic_apply<GRID>(ic, v.p, v.ph, gc)) return;          // phat = M^-1 p
		GLOOP(n) v.v[t] = op.apply(v.ph, t, t);            // vhat = A phat
		if (!grid_sync<true>(gc)) return;
		double rv[1];
		{
			const double* a[1] = { v.rt };
			const double* b[1] = { v.v };
			if (!dots<1>(a, b, n, gc, bank, rv)) return;
		}
		const double alpha = rho_1 / rv[0];
		GLOOP(n) {
			const double q = fma(-alpha, v.v[t], v.s[t]);
			v.q[t] = q;
			v.d[t] = v.s[t] + q;                           // u + q
		}
		if (!grid_sync<true>(gc)) return;
		if (!ic_apply<GRID>(ic, v.d, v.sh, gc)) return;          // uhat = M^-1 (u + q)
		GLOOP(n) {
			v.x[t] = fma(alpha, v.sh[t], v.x[t]);
			v.t[t] = op.apply(v.sh, t, t);                 // qhat = A uhat
		}
		if (!grid_sync<true>(gc)) return;
		GLOOP(n) v.r[t] = fma(-alpha, v.t[t], v.r[t]);
		if (!grid_sync<true>(gc)) return;
		rho_2 = rho_1;
		if (!nrm2_rel(v.r, n, full, normb, gc, bank, resid)) return;
		hist_push(sc, hl, resid);
		if (resid < sc.tol) { finish(sc, 0, it, resid, hl); return; }
	}
	finish(sc, 1, sc.max_iter, resid, hl);
}

#undef GLOOP

}  // namespace cg_dev
