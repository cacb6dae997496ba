// Persistent Krylov engine: one cooperative launch runs a whole solve.
//
// The algorithms restate lib/algebra/solver_matrix.hpp step by step
// (CG :264-316, Jacobi :192-260, Dia_BiCGSTAB :599-672, BiCGSTAB :674-745):
// same recurrences, same stopping tests (<= for CG/Jacobi, < for BiCGSTAB),
// the same nrm2 that leaves out the last element (BLAS_Level1.hpp:569), the
// same early exits and the same values left in max_iter/tol. They differ
// from the CPU only in the order of the additions inside each dot product
// (parallel trees) and in using fused multiply-adds.
//
// Each block owns a fixed strided set of cells for the whole solve, so every
// element-wise phase reads only values its own thread wrote; a grid barrier
// separates the phases that read neighbours (the operator) from the ones that
// write them. Every block evaluates the scalar recurrences from the same
// all-reduced bits, so all blocks take the same branches.
#pragma once

#include "common.cuh"

namespace cg_dev {

// ------------------------------------------------------------ index spaces --
// Flat vectors of length n (the CSR layer): element k at k.
struct FlatSpace {
	int n;
	__device__ __forceinline__ int count() const { return n; }
	__device__ __forceinline__ int addr(int k) const { return k; }
	__device__ __forceinline__ int last_addr() const { return n - 1; }
};

// Normal cells of a field with gl ghost layers and row pitch P (doubles or
// floats): cell (i, j) at (i + gl) * P + (j + gl). Cells are visited y
// fastest (k = i * ny + j) so consecutive threads touch consecutive
// addresses. The reference's last solver element (x-fastest numbering) is
// cell (nx-1, ny-1), also the last k here.
struct GridSpace {
	int nx, ny, gl, P;
	__device__ __forceinline__ int count() const { return nx * ny; }
	__device__ __forceinline__ int addr(int k) const {
		int i = k / ny;
		return (i + gl) * P + (k - i * ny) + gl;
	}
	__device__ __forceinline__ void ij(int k, int& i, int& j) const {
		i = k / ny;
		j = k - i * ny;
	}
	__device__ __forceinline__ int last_addr() const {
		return (nx - 1 + gl) * P + (ny - 1 + gl);
	}
};

// ---------------------------------------------------------------- operators --
// Matrix-free StencilPoisson_ operator: (A p)(i,j) = D p + ax[i] pW
// + ax[i+1] pE + ay[j] pS + ay[j+1] pN. ax/ay are the reference's off-diagonal
// coefficients (-beta*a/d) per face, 0 on boundary faces (their ghost entries
// are folded into D by the ghost substitution). Vectors keep a zero ghost ring.
template<class R, bool NU = false>
struct StencilOp {
	GridSpace sp;
	const R* D;
	const R* ax;  // [nx+1]: x-face coefficients of row 0
	const R* ay;  // [ny+1]: y-face coefficients of column 0
	// general rows (NU: non-uniform grids, variable beta): each cell's own
	// four off-diagonal coefficients, arrays in the field layout (x-, x+,
	// y-, y+ one field apart); unused (null) when ax / ay describe the rows
	const R* cf = nullptr;
	size_t cfs = 0;                // distance between the four arrays
	__device__ __forceinline__ void coeffs(int i, int j, int a, R& xm, R& xp, R& ym, R& yp) const {
		if constexpr (NU) {
			xm = cf[a];
			xp = cf[cfs + a];
			ym = cf[2 * cfs + a];
			yp = cf[3 * cfs + a];
		} else {
			xm = ax[i];
			xp = ax[i + 1];
			ym = ay[j];
			yp = ay[j + 1];
		}
	}
	__device__ __forceinline__ R apply(const R* p, int k, int a) const {
		int i, j;
		sp.ij(k, i, j);
		R xm, xp, ym, yp;
		coeffs(i, j, a, xm, xp, ym, yp);
		R c = D[a] * ldcg(p + a);
		c = fma(xm, ldcg(p + a - sp.P), c);
		c = fma(xp, ldcg(p + a + sp.P), c);
		c = fma(ym, ldcg(p + a - 1), c);
		c = fma(yp, ldcg(p + a + 1), c);
		return c;
	}
	// sum of T x over the off-diagonal entries with T = -a / D (Jacobi)
	__device__ __forceinline__ R jacobi_tx(const R* x, int k, int a) const {
		int i, j;
		sp.ij(k, i, j);
		R xm, xp, ym, yp;
		coeffs(i, j, a, xm, xp, ym, yp);
		R d = D[a], s = 0;
		s = fma(-xm / d, ldcg(x + a - sp.P), s);
		s = fma(-ym / d, ldcg(x + a - 1), s);
		s = fma(-yp / d, ldcg(x + a + 1), s);
		s = fma(-xp / d, ldcg(x + a + sp.P), s);
		return s;
	}
	__device__ __forceinline__ R diag(int k, int a) const { return D[a]; }
};

// CSR (MatrixSCR_) operator, one row per thread visit.
struct CsrOp {
	const uint32_t* rp;
	const uint32_t* ci;
	const double* va;
	__device__ __forceinline__ double apply(const double* p, int k, int) const {
		double s = 0.0;
		for (uint32_t e = rp[k]; e < rp[k + 1]; ++e) s = fma(va[e], ldcg(p + ci[e]), s);
		return s;
	}
	__device__ __forceinline__ double diag(int k, int) const {
		for (uint32_t e = rp[k]; e < rp[k + 1]; ++e)
			if ((int)ci[e] == k) return va[e];
		return 0.0;
	}
	__device__ __forceinline__ double jacobi_tx(const double* x, int k, int) const {
		double d = diag(k, k), s = 0.0;
		for (uint32_t e = rp[k]; e < rp[k + 1]; ++e)
			if ((int)ci[e] != k) s = fma(-va[e] / d, ldcg(x + ci[e]), s);
		return s;
	}
};

// ------------------------------------------------------------------ vectors --
template<class R>
struct Vecs {
	R *x, *b, *r, *p, *q, *z;          // z: Jacobi's new iterate
	R *rt, *ph, *s, *sh, *t, *v, *d;   // BiCGSTAB; d: DiaPre diagonal
};

struct SolveOut {
	int code;
	int iters;
	double tol;
	int hist_len;
	int outer;
	int inner;
};

struct SolveCtl {
	int kind;
	int max_iter;
	double tol;
	uint32_t flags;
	double* hist;
	int hist_cap;
	SolveOut* out;
};

__device__ __forceinline__ void hist_push(const SolveCtl& sc, int& len, double v) {
	if (blockIdx.x == 0 && threadIdx.x == 0 && sc.hist && len < sc.hist_cap)
		sc.hist[len] = v;
	++len;
}

__device__ __forceinline__ void finish(const SolveCtl& sc, int code, int iters,
		double tol, int hist_len) {
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		sc.out->code = code;
		sc.out->iters = iters;
		sc.out->tol = tol;
		sc.out->hist_len = hist_len;
	}
}

#define KLOOP(sp)                                                              \
	for (int k = blockIdx.x * blockDim.x + threadIdx.x, _n = (sp).count();     \
			k < _n; k += gridDim.x * blockDim.x)

// Sum of squares over the vector with the reference's nrm2 (last element
// left out unless FULL_NRM2 or n == 1) -> [0]; the full sum -> [1].
template<class R, class Sp>
__device__ __forceinline__ bool norms2(const Sp& sp, const R* y, bool full,
		const GridCtl& gc, int& bank, double& excl, double& all) {
	const int la = sp.last_addr();
	R acc[1] = { 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		if (a != la || full) { R v = y[a]; acc[0] = fma(v, v, acc[0]); }
	}
	if (!grid_allreduce<R, 1>(acc, gc, bank)) return false;
	R yl = ldcg(y + la);
	excl = (double)acc[0];
	all = full ? excl : (double)(acc[0] + yl * yl);
	return true;
}

// ------------------------------------------------------------------------ CG --
// The scalar recurrences (divisions, sqrt, the stopping test) run in thread 0
// of each block and reach the other threads through shared memory: every
// block still derives them from the same all-reduced bits.
template<class R, class Sp, class Op>
__device__ void cg_run(const Sp& sp, const Op& op, const Vecs<R>& v,
		const SolveCtl& sc, const GridCtl& gc, int& bank) {
	__shared__ R s_sc[4];
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
	const int la = sp.last_addr();
	int hl = 0;
	// r = b - A x ; nrm2(b), nrm2(r)
	R acc[2] = { 0, 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		R bb = v.b[a];
		R rr = bb - op.apply(v.x, k, a);
		v.r[a] = rr;
		if (a != la || full) { acc[0] = fma(bb, bb, acc[0]); acc[1] = fma(rr, rr, acc[1]); }
	}
	if (!grid_allreduce<R, 2>(acc, gc, bank)) return;
	double normb = 1, resid = 0;
	if (threadIdx.x == 0) {
		R rl = ldcg(v.r + la);
		normb = sqrt((double)acc[0]);
		if (normb == 0.0) normb = 1;
		resid = sqrt((double)acc[1]) / normb;
		s_sc[0] = resid <= sc.tol ? R(1) : R(0);
		s_sc[1] = full ? acc[1] : acc[1] + rl * rl;   // rho = (r, r)
	}
	__syncthreads();
	if (s_sc[0] != R(0)) { finish(sc, 0, 0, resid, hl); return; }
	R rho = s_sc[1], beta = 0, alpha;
	for (int it = 1; it <= sc.max_iter; ++it) {
		if (it == 1) {
			KLOOP(sp) { int a = sp.addr(k); v.p[a] = v.r[a]; }
		} else {
			KLOOP(sp) { int a = sp.addr(k); v.p[a] = fma(beta, v.p[a], v.r[a]); }
		}
		if (!grid_sync(gc)) return;
		R pq[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			R qq = op.apply(v.p, k, a);
			v.q[a] = qq;
			pq[0] = fma(v.p[a], qq, pq[0]);
		}
		if (!grid_allreduce<R, 1>(pq, gc, bank)) return;
		if (threadIdx.x == 0) s_sc[2] = rho / pq[0];
		__syncthreads();
		alpha = s_sc[2];
		R rr[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			v.x[a] = fma(alpha, v.p[a], v.x[a]);
			R r2 = fma(-alpha, v.q[a], v.r[a]);
			v.r[a] = r2;
			if (a != la || full) rr[0] = fma(r2, r2, rr[0]);
		}
		if (!grid_allreduce<R, 1>(rr, gc, bank)) return;
		if (threadIdx.x == 0) {
			R rl = ldcg(v.r + la);
			resid = sqrt((double)rr[0]) / normb;
			hist_push(sc, hl, resid);
			R rho_new = full ? rr[0] : rr[0] + rl * rl;
			s_sc[0] = resid <= sc.tol ? R(1) : R(0);
			s_sc[1] = rho_new;
			s_sc[3] = rho_new / rho;   // beta of the next iteration
		}
		__syncthreads();
		if (s_sc[0] != R(0)) { finish(sc, 0, it, resid, hl); return; }
		rho = s_sc[1];
		beta = s_sc[3];
	}
	finish(sc, 1, sc.max_iter, resid, hl);
}

// -------------------------------------------------------------------- Jacobi --
// newx = T x + C with T = -(A - D)/D, C = b/D; r = b - A newx. On convergence
// the returned x is the previous iterate, as in the reference (x = newx
// happens only after the convergence test).
template<class R, class Sp, class Op>
__device__ void jacobi_run(const Sp& sp, const Op& op, const Vecs<R>& v,
		const SolveCtl& sc, const GridCtl& gc, int& bank) {
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
	const int la = sp.last_addr();
	int hl = 0;
	R acc[3] = { 0, 0, 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		R bb = v.b[a];
		R rr = bb - op.apply(v.x, k, a);
		if (a != la || full) { acc[0] = fma(bb, bb, acc[0]); acc[1] = fma(rr, rr, acc[1]); }
		if (op.diag(k, a) == R(0)) acc[2] = 1;
	}
	if (!grid_allreduce<R, 3>(acc, gc, bank)) return;
	double normb = sqrt((double)acc[0]);
	if (normb == 0.0) normb = 1;
	double resid = sqrt((double)acc[1]) / normb;
	if (resid <= sc.tol) { finish(sc, 0, 0, resid, hl); return; }
	if (acc[2] != R(0)) { finish(sc, CARPIO_GPU_EZERODIAG, sc.max_iter, resid, hl); return; }
	R* cur = v.x;
	R* nxt = v.z;
	int code = 1, iters = sc.max_iter;
	for (int it = 1; it <= sc.max_iter; ++it) {
		KLOOP(sp) {
			int a = sp.addr(k);
			R d = op.diag(k, a);
			nxt[a] = op.jacobi_tx(cur, k, a) + v.b[a] / d;
		}
		if (!grid_sync(gc)) return;
		R rr[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			R r2 = v.b[a] - op.apply(nxt, k, a);
			if (a != la || full) rr[0] = fma(r2, r2, rr[0]);
		}
		if (!grid_allreduce<R, 1>(rr, gc, bank)) return;
		resid = sqrt((double)rr[0]) / normb;
		hist_push(sc, hl, resid);
		if (resid <= sc.tol) { code = 0; iters = it; break; }
		R* t = cur; cur = nxt; nxt = t;
	}
	if (cur != v.x) { KLOOP(sp) { int a = sp.addr(k); v.x[a] = cur[a]; } }
	finish(sc, code, iters, resid, hl);
}

// ------------------------------------------------------------------ BiCGSTAB --
// inv = 1: Dia_BiCGSTAB (M^-1 = 1/diag); inv = 2: BiCGSTAB ("M^-1" = diag).
template<class R, class Sp, class Op>
__device__ void bicgstab_run(int inv, const Sp& sp, const Op& op,
		const Vecs<R>& v, const SolveCtl& sc, const GridCtl& gc, int& bank) {
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
	const int la = sp.last_addr();
	int hl = 0;
	R acc[3] = { 0, 0, 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		R bb = v.b[a];
		R rr = bb - op.apply(v.x, k, a);
		v.r[a] = rr;
		v.rt[a] = rr;
		R d = op.diag(k, a);
		if (d == R(0)) acc[2] = 1;
		v.d[a] = inv == 1 ? R(1) / d : d;
		if (a != la || full) { acc[0] = fma(bb, bb, acc[0]); acc[1] = fma(rr, rr, acc[1]); }
	}
	if (!grid_allreduce<R, 3>(acc, gc, bank)) return;
	R rl = ldcg(v.r + la);
	if (acc[2] != R(0)) { finish(sc, CARPIO_GPU_EZERODIAG, sc.max_iter, sc.tol, hl); return; }
	double normb = sqrt((double)acc[0]);
	if (normb == 0.0) normb = 1;
	double resid = sqrt((double)acc[1]) / normb;
	if (resid <= sc.tol) {
		if (inv == 1) hist_push(sc, hl, resid);
		finish(sc, 0, 0, resid, hl);
		return;
	}
	R rho_1 = full ? acc[1] : acc[1] + rl * rl;   // dot(rtilde, r) with rtilde = r
	R rho_2 = 0, alpha = 0, omega = 0;
	for (int it = 1; it <= sc.max_iter; ++it) {
		if (rho_1 == R(0)) {
			double nr = 0, dummy;
			if (!norms2(sp, v.r, full, gc, bank, nr, dummy)) return;
			finish(sc, 2, sc.max_iter, sqrt(nr) / normb, hl);
			return;
		}
		if (it == 1) {
			KLOOP(sp) { int a = sp.addr(k); v.p[a] = v.r[a]; v.ph[a] = v.r[a] * v.d[a]; }
		} else {
			R beta = (rho_1 / rho_2) * (alpha / omega);
			KLOOP(sp) {
				int a = sp.addr(k);
				R pp = fma(beta, fma(-omega, v.v[a], v.p[a]), v.r[a]);
				v.p[a] = pp;
				v.ph[a] = pp * v.d[a];
			}
		}
		if (!grid_sync(gc)) return;
		R rv[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			R vv = op.apply(v.ph, k, a);
			v.v[a] = vv;
			rv[0] = fma(v.rt[a], vv, rv[0]);
		}
		if (!grid_allreduce<R, 1>(rv, gc, bank)) return;
		alpha = rho_1 / rv[0];
		R ss[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			R s = fma(-alpha, v.v[a], v.r[a]);
			v.s[a] = s;
			v.sh[a] = s * v.d[a];
			if (a != la || full) ss[0] = fma(s, s, ss[0]);
		}
		if (!grid_allreduce<R, 1>(ss, gc, bank)) return;
		resid = sqrt((double)ss[0]) / normb;
		if (resid < sc.tol) {
			KLOOP(sp) { int a = sp.addr(k); v.x[a] = fma(alpha, v.ph[a], v.x[a]); }
			if (inv == 1) hist_push(sc, hl, resid);
			finish(sc, 0, sc.max_iter, resid, hl);   // max_iter left unchanged
			return;
		}
		R ts[2] = { 0, 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			R tt = op.apply(v.sh, k, a);
			v.t[a] = tt;
			ts[0] = fma(tt, v.s[a], ts[0]);
			ts[1] = fma(tt, tt, ts[1]);
		}
		if (!grid_allreduce<R, 2>(ts, gc, bank)) return;
		omega = ts[0] / ts[1];
		R rr[2] = { 0, 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			v.x[a] = v.x[a] + fma(alpha, v.ph[a], omega * v.sh[a]);
			R r2 = fma(-omega, v.t[a], v.s[a]);
			v.r[a] = r2;
			if (a != la || full) rr[0] = fma(r2, r2, rr[0]);
			rr[1] = fma(v.rt[a], r2, rr[1]);
		}
		if (!grid_allreduce<R, 2>(rr, gc, bank)) return;
		rho_2 = rho_1;
		rho_1 = rr[1];
		resid = sqrt((double)rr[0]) / normb;
		hist_push(sc, hl, resid);
		if (resid < sc.tol) { finish(sc, 0, it, resid, hl); return; }
		if (omega == R(0)) {
			double nr = 0, dummy;
			if (!norms2(sp, v.r, full, gc, bank, nr, dummy)) return;
			finish(sc, 3, sc.max_iter, sqrt(nr) / normb, hl);
			return;
		}
	}
	finish(sc, 1, sc.max_iter, resid, hl);
}

template<class R, class Sp, class Op>
__device__ __forceinline__ void krylov_run(const Sp& sp, const Op& op,
		const Vecs<R>& v, const SolveCtl& sc, const GridCtl& gc, int& bank) {
	switch (sc.kind) {
	case CARPIO_GPU_CG: cg_run<R>(sp, op, v, sc, gc, bank); break;
	case CARPIO_GPU_JACOBI: jacobi_run<R>(sp, op, v, sc, gc, bank); break;
	case CARPIO_GPU_DIA_BICGSTAB: bicgstab_run<R>(1, sp, op, v, sc, gc, bank); break;
	case CARPIO_GPU_BICGSTAB: bicgstab_run<R>(2, sp, op, v, sc, gc, bank); break;
	default: finish(sc, CARPIO_GPU_EINVAL, 0, 0.0, 0);
	}
}

}  // namespace cg_dev
