// FP32 inner iterations inside FP64 iterative refinement, for any index
// space (GridSpace, FlatSpace) and operator pair (the FP64 operator for the
// residual b - A x, its FP32 copy for the inner solve): the mixed-precision
// solver of the structured Poisson path and of the CSR layer.
//
// The FP64 side restates the reference's stopping test (nrm2 of b - A x over
// nrm2 of b, the last element left out, solver_matrix.hpp:264-316); the
// inner solves are the kind's own recurrences (CG :264-316, Dia_BiCGSTAB
// :599-672, BiCGSTAB :674-745) in FP32 with FP32 accumulation, on the
// residual scaled to unit norm, until it has dropped by inner_tol.
#pragma once

#include "krylov.cuh"

namespace cg_dev {

template<class Op32>
struct MixedT {
	Op32 op32;
	Vecs<float> f;         // e (x), r, p, q; BiCGSTAB: rt, ph, s, sh, t, v, d
	double inner_tol;
	int inner_max;
	int pdeg;              // on-chip path: degree of the band-local Chebyshev
	                       // preconditioner (0 = none)
	float pratio;          // its eigenvalue interval [2 / pratio, 2] of D^-1 A
};

// FP32 copy of a MatrixSCR_ operator: the same rows, float values.
struct CsrOp32 {
	const uint32_t* rp;
	const uint32_t* ci;
	const float* va;
	__device__ __forceinline__ float apply(const float* p, int k, int) const {
		float s = 0.f;
		for (uint32_t e = rp[k]; e < rp[k + 1]; ++e) s = fmaf(va[e], ldcg(p + ci[e]), s);
		return s;
	}
	__device__ __forceinline__ float diag(int k, int) const {
		for (uint32_t e = rp[k]; e < rp[k + 1]; ++e)
			if ((int)ci[e] == k) return va[e];
		return 0.f;
	}
};

// FP32 CG on A32 e = r32 from e = 0 (one inner solve of the refinement).
// Returns the number of iterations, or -1 on a barrier error.
template<class Sp, class Op32>
__device__ int inner_cg(const Sp& sp, const MixedT<Op32>& m, int cap,
		const GridCtl& gc, int& bank) {
	const Vecs<float>& f = m.f;
	const Op32& op = m.op32;
	float rr0[1] = { 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		float r = f.r[a];
		f.x[a] = 0.f;
		f.p[a] = r;
		rr0[0] = fmaf(r, r, rr0[0]);
	}
	if (!grid_allreduce<float, 1>(rr0, gc, bank)) return -1;
	float rho = rr0[0];
	const float stop = (float)(m.inner_tol * m.inner_tol) * rho;
	int it = 0;
	while (it < cap && rho > stop && rho > 0.f) {
		float pq[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			float q = op.apply(f.p, k, a);
			f.q[a] = q;
			pq[0] = fmaf(f.p[a], q, pq[0]);
		}
		if (!grid_allreduce<float, 1>(pq, gc, bank)) return -1;
		float alpha = rho / pq[0];
		float rr[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			f.x[a] = fmaf(alpha, f.p[a], f.x[a]);
			float r = fmaf(-alpha, f.q[a], f.r[a]);
			f.r[a] = r;
			rr[0] = fmaf(r, r, rr[0]);
		}
		if (!grid_allreduce<float, 1>(rr, gc, bank)) return -1;
		float beta = rr[0] / rho;
		rho = rr[0];
		++it;
		if (it < cap && rho > stop) {
			KLOOP(sp) { int a = sp.addr(k); f.p[a] = fmaf(beta, f.p[a], f.r[a]); }
			if (!grid_sync(gc)) return -1;
		}
	}
	return it;
}

// FP32 BiCGSTAB on A32 e = r32 from e = 0 (one inner solve of the
// refinement), the recurrences of bicgstab_run (Dia_BiCGSTAB,
// solver_matrix.hpp:599-672, inv = 1: M^-1 = 1/diag; BiCGSTAB, :674-745,
// inv = 2: "M^-1" = diag) with FP32 vectors, FP32 accumulation and the full
// 2-norm; it stops once the FP32 residual has dropped by inner_tol (the
// early exit on |s| included) or on a breakdown. Returns the number of
// iterations (e holds the correction), or -1 on a barrier error; *brk gets
// 2 (rho = 0) or 3 (omega = 0) when a breakdown ended it.
template<class Sp, class Op32>
__device__ int inner_bicgstab(const Sp& sp, const MixedT<Op32>& m, int inv,
		int cap, const GridCtl& gc, int& bank, int* brk) {
	const Vecs<float>& f = m.f;
	const Op32& op = m.op32;
	*brk = 0;
	float acc[1] = { 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		float r = f.r[a];
		f.x[a] = 0.f;
		f.rt[a] = r;
		float d = op.diag(k, a);
		f.d[a] = inv == 1 ? 1.f / d : d;
		acc[0] = fmaf(r, r, acc[0]);
	}
	if (!grid_allreduce<float, 1>(acc, gc, bank)) return -1;
	float rho_1 = acc[0];
	const float stop = (float)(m.inner_tol * m.inner_tol) * acc[0];
	float rho_2 = 0.f, alpha = 0.f, omega = 0.f;
	int it = 0;
	while (it < cap) {
		if (rho_1 == 0.f) { *brk = 2; break; }
		if (it == 0) {
			KLOOP(sp) { int a = sp.addr(k); f.p[a] = f.r[a]; f.ph[a] = f.r[a] * f.d[a]; }
		} else {
			const float beta = (rho_1 / rho_2) * (alpha / omega);
			KLOOP(sp) {
				int a = sp.addr(k);
				float pp = fmaf(beta, fmaf(-omega, f.v[a], f.p[a]), f.r[a]);
				f.p[a] = pp;
				f.ph[a] = pp * f.d[a];
			}
		}
		if (!grid_sync(gc)) return -1;
		float rv[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			float vv = op.apply(f.ph, k, a);
			f.v[a] = vv;
			rv[0] = fmaf(f.rt[a], vv, rv[0]);
		}
		if (!grid_allreduce<float, 1>(rv, gc, bank)) return -1;
		alpha = rho_1 / rv[0];
		// (rt, v) = 0 in FP32: a breakdown the FP64 recurrences would not
		// meet at these sizes; stop with the iterate so far (the next
		// refinement restarts from the true residual)
		if (!isfinite(alpha)) { *brk = 2; break; }
		float ss[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			float sv = fmaf(-alpha, f.v[a], f.r[a]);
			f.s[a] = sv;
			f.sh[a] = sv * f.d[a];
			ss[0] = fmaf(sv, sv, ss[0]);
		}
		if (!grid_allreduce<float, 1>(ss, gc, bank)) return -1;
		++it;
		if (ss[0] <= stop) {
			KLOOP(sp) { int a = sp.addr(k); f.x[a] = fmaf(alpha, f.ph[a], f.x[a]); }
			break;
		}
		float ts[2] = { 0, 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			float tt = op.apply(f.sh, k, a);
			f.t[a] = tt;
			ts[0] = fmaf(tt, f.s[a], ts[0]);
			ts[1] = fmaf(tt, tt, ts[1]);
		}
		if (!grid_allreduce<float, 2>(ts, gc, bank)) return -1;
		omega = ts[0] / ts[1];
		if (!isfinite(omega)) {
			// t = 0: keep the half step x + alpha ph and stop
			KLOOP(sp) { int a = sp.addr(k); f.x[a] = fmaf(alpha, f.ph[a], f.x[a]); }
			*brk = 3;
			break;
		}
		float rr[2] = { 0, 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			f.x[a] = f.x[a] + fmaf(alpha, f.ph[a], omega * f.sh[a]);
			float r2 = fmaf(-omega, f.t[a], f.s[a]);
			f.r[a] = r2;
			rr[0] = fmaf(r2, r2, rr[0]);
			rr[1] = fmaf(f.rt[a], r2, rr[1]);
		}
		if (!grid_allreduce<float, 2>(rr, gc, bank)) return -1;
		rho_2 = rho_1;
		rho_1 = rr[1];
		if (rr[0] <= stop) break;
		if (omega == 0.f) { *brk = 3; break; }
	}
	return it;
}

// FP32 inner CG inside FP64 iterative refinement: r = b - A x, the stopping
// test and the update of x in FP64; the correction solve in FP32 with FP32
// accumulation, on the residual scaled to unit norm.
template<class Sp, class Op64, class Op32>
__device__ void mixed_run(const Sp& sp, const Op64& op,
		const Vecs<double>& v, const MixedT<Op32>& m, const SolveCtl& sc,
		bool mean, const GridCtl& gc, int& bank) {
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
	const int la = sp.last_addr();
	const double n = (double)sp.count();
	int hl = 0, total = 0, outer = 0, code = 1;
	double acc[1] = { 0 };
	KLOOP(sp) {
		int a = sp.addr(k);
		double bb = v.b[a];
		if (a != la || full) acc[0] = fma(bb, bb, acc[0]);
	}
	if (!grid_allreduce<double, 1>(acc, gc, bank)) return;
	double normb = sqrt(acc[0]);
	if (normb == 0.0) normb = 1;
	double resid = 0;
	// The FP32 BiCGSTAB recursion can drift from the true residual and, near a
	// breakdown, return a correction that makes x worse. Its inner solves are
	// kept short, x is saved before each one (in v.p, unused here), and a
	// correction after which the FP64 residual did not drop is undone and
	// retried with half the cap.
	const bool bicg = sc.kind != CARPIO_GPU_CG;
	int bcap = m.inner_max < 100 ? m.inner_max : 100;
	int rejects = 0;
	bool restored = false;
	double best = 0.0;
	for (;;) {
		double rs[3] = { 0, 0, 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			double r = v.b[a] - op.apply(v.x, k, a);
			v.r[a] = r;
			if (a != la || full) rs[0] = fma(r, r, rs[0]);
			rs[1] += r;
			rs[2] = fma(r, r, rs[2]);
		}
		if (!grid_allreduce<double, 3>(rs, gc, bank)) return;
		resid = sqrt(rs[0]) / normb;
		hist_push(sc, hl, resid);
		if (bicg && outer > 0 && !restored && !(resid < best)) {
			if (++rejects > 8 || total >= sc.max_iter) { resid = best; break; }
			KLOOP(sp) { int a = sp.addr(k); v.x[a] = v.p[a]; }
			if (!grid_sync(gc)) return;
			bcap = bcap > 8 ? bcap / 2 : 4;
			restored = true;
			continue;
		}
		restored = false;
		if (!(resid == resid)) break;   // NaN: code 1 with the NaN residual
		if (resid <= sc.tol) {
			if (blockIdx.x == 0 && threadIdx.x == 0) { sc.out->outer = outer; sc.out->inner = total; }
			finish(sc, 0, total, resid, hl);
			return;
		}
		best = resid;
		if (total >= sc.max_iter) break;
		double mr = mean ? rs[1] / n : 0.0;
		double rn = sqrt(mean ? fmax(rs[2] - rs[1] * mr, 0.0) : rs[2]);
		if (!(rn > 0.0)) break;
		double sc_in = 1.0 / rn;
		KLOOP(sp) {
			int a = sp.addr(k);
			m.f.r[a] = (float)((v.r[a] - mr) * sc_in);
			if (bicg) v.p[a] = v.x[a];
		}
		if (!grid_sync(gc)) return;
		const int cap = min(bicg ? bcap : m.inner_max, sc.max_iter - total);
		int brk = 0;
		int it = sc.kind == CARPIO_GPU_CG
				? inner_cg(sp, m, cap, gc, bank)
				: inner_bicgstab(sp, m, sc.kind == CARPIO_GPU_DIA_BICGSTAB ? 1 : 2, cap,
						gc, bank, &brk);
		if (it < 0) return;
		total += it;
		++outer;
		KLOOP(sp) { int a = sp.addr(k); v.x[a] = fma(rn, (double)m.f.x[a], v.x[a]); }
		if (!grid_sync(gc)) return;
		// a breakdown before any progress ends the solve with the
		// reference's code for it; after progress the next refinement
		// restarts the inner solve from the new residual
		if (brk && it <= 1) { code = brk; break; }
		if (it == 0) break;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) { sc.out->outer = outer; sc.out->inner = total; }
	finish(sc, code, total, resid, hl);
}

}  // namespace cg_dev
