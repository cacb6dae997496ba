// Structure-level Poisson solve on the GPU: the matrix-free form of
// StencilPoisson_ + GhostRegular_ (lib/structure/s_poisson.hpp:60-114,
// s_ghost.hpp:140-179, 334-357) behind structure::Solver_<2>::solve
// (s_solver.hpp:77-171), in one persistent cooperative launch.
//
// Coefficients are computed on the host with the reference's formulas in the
// reference's order, so D, the face coefficients and the right-hand side
// carry the same bits as the CSR the reference assembles; only the Krylov
// sums are ordered differently.
#include "internal.hpp"
#include "poisson_rhs.cuh"
#include "mixed.cuh"
#include "mg.cuh"
#include "dct.cuh"
#include "dfloat.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

namespace {

using namespace cg_dev;

// ------------------------------------------------------------ device side --
template<bool NU>
using MixedArgsT = MixedT<StencilOp<float, NU>>;
using MixedArgs = MixedArgsT<false>;
// the uniform and non-uniform specialisations differ in code only, so one
// host-side argument block serves the kernels of either
static_assert(sizeof(MixedArgsT<true>) == sizeof(MixedArgs), "layout");
static_assert(sizeof(StencilOp<double, true>) == sizeof(StencilOp<double>), "layout");

template<int SRC, int KIND, bool NU>
__global__ void __launch_bounds__(kThreads) k_poisson(StencilOp<double, NU> op,
		Vecs<double> v, RhsArgs ra, MixedArgsT<NU> mx, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	const GridSpace& sp = op.sp;
	// prologue: b (bit-exact row constants), x0 from phi
	double s[1] = { 0 };
	KLOOP(sp) {
		int i, j;
		sp.ij(k, i, j);
		int a = sp.addr(k);
		double bb = rhs_at<SRC>(sp, ra, i, j, a);
		v.b[a] = bb;
		v.x[a] = ra.phi[a];
		s[0] += bb;
	}
	if (ra.mean) {
		// null-space removal of b: b - mean(b)
		if (!grid_allreduce<double, 1>(s, gc, bank)) return;
		double m = s[0] / (double)sp.count();
		KLOOP(sp) { int a = sp.addr(k); v.b[a] = v.b[a] - m; }
	}
	if (!grid_sync(gc)) return;
	if (KIND == 4) mixed_run(sp, op, v, mx, sc, ra.mean != 0, gc, bank);
	else krylov_run<double>(sp, op, v, sc, gc, bank);
	if (read_err(gc)) {
		if (blockIdx.x == 0 && threadIdx.x == 0) sc.out->code = read_err(gc);
		return;
	}
	// epilogue: mean removal of x, x back into phi
	double mx0 = 0.0;
	if (ra.mean) {
		double t[1] = { 0 };
		KLOOP(sp) { int a = sp.addr(k); t[0] += v.x[a]; }
		if (!grid_allreduce<double, 1>(t, gc, bank)) {
			if (blockIdx.x == 0 && threadIdx.x == 0) sc.out->code = read_err(gc);
			return;
		}
		mx0 = t[0] / (double)sp.count();
	}
	KLOOP(sp) { int a = sp.addr(k); ra.phi[a] = ra.mean ? v.x[a] - mx0 : v.x[a]; }
}

// ------------------------------------------------ tile-resident FP32 CG --
// The mixed solve with its Krylov state on chip: FP32 CG with reliable
// updates. Whenever the FP32 residual has dropped by inner_tol since the last
// update (or looks converged), the FP32 iterate is added into the FP64
// solution, the true residual b - A x is recomputed in FP64 and replaces r,
// and CG continues with its search direction (no restart). The stopping test
// is always made on the FP64 residual. (Variants with one reduction per
// iteration -- Chronopoulos-Gear, or |r - alpha q|^2 by recurrence -- lose
// too much in FP32 at the condition numbers of these grids.)
//
// One CTA per SM owns a band of x-rows [r0, r1). Thread t owns the columns
// t, t + T, ... (< ny) of every row of the band, so a cell's row and column
// are loop indices and its x and q sit in registers; r and p live in shared
// memory, p with one halo row above and below. p's halo rows are advanced
// locally with the same FMA the neighbour band applies to the same inputs
// (p = r + beta p with the neighbour's r), so the copies stay bit-identical;
// the only data crossing CTAs per iteration is each band's first and last
// row of r, published before the second reduction and read after it
// (double-buffered by iteration parity).
constexpr int kTileThreads = 512;
// default band-local Chebyshev preconditioner of the on-chip path
constexpr int kPolyDegree = 5;
constexpr double kPolyRatio = 30.0;

struct TileArgs {
	float* xbuf;           // [3][C][2][ny]: band edge rows of r (two iteration
	                       // parities), then of r after a residual replacement
	int rows_max;
	MgArgs mg;             // the multigrid preconditioner (mg.nlev > 0)
	DctArgs dct;           // the spectral preconditioner (dct.on)
	int df;                // spectral: x, b and the refinement residuals in
	                       // double-float (FP32 pipe), the coefficients being
	                       // exact in FP32
};

__device__ __forceinline__ int band_lo(int c, int C, int nx) {
	return (int)((long)c * nx / C);
}

struct TileOut {
	int iters, updates, done;
	double resid;
	double xmean;   // fused: the mean of the final x (for the epilogue)
};

// NC columns per thread, RM rows per band at most.
template<int NC, int RM>
__device__ void tile_solve(const GridSpace& sp, const StencilOp<double>& op,
		const Vecs<double>& v, const MixedArgs& m, const TileArgs& ta,
		const SolveCtl& sc, bool mean, double normb, const GridCtl& gc,
		int& bank, TileOut& to, double bmean = 0.0) {
	extern __shared__ __align__(16) float smem[];
	__shared__ double s_sc[4];
	__shared__ double s_xm;
	const int C = gridDim.x, c = blockIdx.x, T = blockDim.x, tid = threadIdx.x;
	const int nx = sp.nx, ny = sp.ny, gl = sp.gl, P = sp.P;
	const int r0 = band_lo(c, C, nx), r1 = band_lo(c + 1, C, nx);
	const int rows = r1 - r0;
	const int np = (ta.rows_max + 2) * ny + 2;
	const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
	const int la = sp.last_addr();
	const double ncell = (double)sp.count();
	float* p = smem;                // p[1 + (lr + 1) * ny + j], lr = -1 .. rows
	float* rhal = p + np;           // halo rows of r: [0, ny) above, [ny, 2ny) below
	float* rs = rhal + 2 * ny;      // the band's r, rs[lr * ny + j]
	float* axs = rs + ta.rows_max * ny;   // x-face coefficients of faces r0 .. r1
	float* ays = axs + ta.rows_max + 1;
	float* dd = ays + ny + 1;       // the band's diagonal, dd[lr * ny + j]
	// preconditioned: z = M r with its halo rows from the neighbours (in
	// rhal); the Chebyshev directions, two buffers in the layout of p with
	// zero halo rows (one read, one written per step)
	const int K = m.pdeg;
	const MgArgs& mg = ta.mg;
	const bool use_mg = mg.nlev > 0;
	const DctArgs& dc = ta.dct;
	const bool use_dct = dc.on != 0;
	float* zs = (K > 0 || use_mg || use_dct) ? dd + ta.rows_max * ny : rs;
	// spectral: the FFT buffer after zs at an even float offset (8 bytes),
	// then the column phase's spectrum (B columns x nx, real)
	const int zs_end = (int)(zs - smem) + ta.rows_max * ny;
	float2* dbuf = reinterpret_cast<float2*>(smem + ((zs_end + 1) & ~1));
	float* dspec = reinterpret_cast<float*>(dbuf + ta.dct.fb);
	float* dsa = zs + ta.rows_max * ny;    // dsa[1 + (lr + 1) * ny + j]
	float* dsb = dsa + np;
	// multigrid (K == 0 then): the corrected fine values of the band and its
	// halo rows in the place of dsa, then the shared-memory coarse levels
	float* mgc = dsa;
	float* mgsm = mgc + np;
	const bool up = c > 0, down = c < C - 1;
	const size_t edge = (size_t)2 * C * ny;   // one edge region
	float* rbuf = ta.xbuf + 2 * edge;         // r edges
	int par = 0;                              // q edges: xbuf + par * edge
	for (int t = tid; t < np; t += T) p[t] = 0.f;
	if (K > 0)
		for (int t = tid; t < 2 * np; t += T) dsa[t] = 0.f;
	for (int t = tid; t < ny; t += T) { rhal[t] = 0.f; rhal[ny + t] = 0.f; }
	for (int t = tid; t < rows * ny; t += T) {
		const int lr = t / ny, j = t - lr * ny;
		dd[t] = m.op32.D[(r0 + lr + gl) * P + j + gl];
	}
	for (int t = tid; t <= rows; t += T) axs[t] = m.op32.ax[r0 + t];
	for (int t = tid; t <= ny; t += T) ays[t] = m.op32.ay[t];
	float x[RM][NC], q[RM][NC];
#pragma unroll
	for (int lr = 0; lr < RM; ++lr)
#pragma unroll
		for (int k = 0; k < NC; ++k) x[lr][k] = q[lr][k] = 0.f;
	__syncthreads();
	// the y-face coefficients of the thread's columns, for the whole solve
	float ayl[NC], ayr[NC];
#pragma unroll
	for (int k = 0; k < NC; ++k) {
		const int j = tid + k * T;
		ayl[k] = j < ny ? ays[j] : 0.f;
		ayr[k] = j < ny ? ays[j + 1] : 0.f;
	}
	// r (FP32) = (r64 - mean) * scale0 with scale0 fixed for the whole solve
	double scale0 = 1.0, rn0 = 1.0;
	float rrn = 0.f;   // (r, r) of the current FP32 residual
	double nrmb = normb;   // ||b|| (fused: from the first residual's reduction)
	float rr_band = 0.f;   // (r, r) of the band's newest FP32 residual
	to.xmean = 0.0;

	auto publish_r = [&]() {
		float* pub = rbuf + (size_t)(2 * c) * ny;
#pragma unroll
		for (int k = 0; k < NC; ++k) {
			const int j = tid + k * T;
			if (j < ny && rows > 0) {
				pub[j] = zs[j];
				pub[ny + j] = zs[(rows - 1) * ny + j];
			}
		}
	};
	// z = M r: K steps of the Chebyshev iteration for A_band z = r from
	// z = 0, A_band the band's operator with zero halo rows (a symmetric
	// positive definite block-diagonal M with no exchange between CTAs).
	// One pass per step: the stencil of the previous direction (read from
	// one buffer) updates the local residual (registers, in q) and gives
	// the next direction (written to the other buffer), so a step needs one
	// block barrier. Returns (r, z) and (r, r) of the band in g.
	auto precond = [&](float (&g)[2]) {
		g[0] = g[1] = 0.f;
		const float bmax = 2.f, amin = 2.f / m.pratio;
		const float th = 0.5f * (bmax + amin), de = 0.5f * (bmax - amin);
		const float sig = th / de;
		float rho = 1.f / sig;
		const float ith = 1.f / th;
		float* dcur = dsa;
		float* dnxt = dsb;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int cc = lr * ny + j;
					const float rv = rs[cc];
					const float dv = __fdividef(rv * ith, dd[cc]);
					dcur[1 + (lr + 1) * ny + j] = dv;
					zs[cc] = dv;
					q[lr][k] = rv;
				}
			}
		__syncthreads();
		for (int step = 1; step < K; ++step) {
			const float rn = 1.f / (2.f * sig - rho);
			const float c1 = rn * rho, c2f = 2.f * rn / de;
#pragma unroll
			for (int lr = 0; lr < RM; ++lr) {
				const float ax0 = axs[lr], ax1 = axs[lr + 1];
#pragma unroll
				for (int k = 0; k < NC; ++k) {
					const int j = tid + k * T;
					if (lr < rows && j < ny) {
						const int cc = lr * ny + j, pk = 1 + (lr + 1) * ny + j;
						const float dc = dcur[pk];
						float vv = dd[cc] * dc;
						vv = fmaf(ax0, dcur[pk - ny], vv);
						vv = fmaf(ax1, dcur[pk + ny], vv);
						vv = fmaf(ayl[k], dcur[pk - 1], vv);
						vv = fmaf(ayr[k], dcur[pk + 1], vv);
						const float rkv = q[lr][k] - vv;
						q[lr][k] = rkv;
						const float dv = fmaf(c1, dc, __fdividef(c2f * rkv, dd[cc]));
						dnxt[pk] = dv;
						zs[cc] += dv;
					}
				}
			}
			__syncthreads();
			float* t = dcur;
			dcur = dnxt;
			dnxt = t;
			rho = rn;
		}
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int cc = lr * ny + j;
					const float rv = rs[cc];
					g[0] = fmaf(rv, zs[cc], g[0]);
					g[1] = fmaf(rv, rv, g[1]);
				}
			}
	};
	// z = M r with M one multigrid V-cycle (mg.cuh); (r, z) and (r, r) of
	// the band in g. Every CTA passes the same grid barriers.
	auto precond_mg = [&](float (&g)[2]) -> bool {
		const float w = mg.omega, cx = mg.cx, cy = mg.cy;
		const LdL2 gld;
		const LdRo ro;
		const MgLevel& L0 = mg.lev[0];
		// level 0's diagonal is the band's own (dd); its reciprocal rounds
		// like the host-built L0.iD used outside the band
		auto r0at = [&](int i, int j) -> float {
			const int lr = i - r0;
			return (lr >= 0 && lr < rows) ? rs[lr * ny + j] : ldcg(L0.R + i * ny + j);
		};
		auto id0at = [&](int i, int j) -> float {
			const int lr = i - r0;
			return (lr >= 0 && lr < rows) ? __frcp_rn(dd[lr * ny + j]) : __ldg(L0.iD + i * ny + j);
		};
		// level 0: R0 = r of the band, for the neighbours
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) __stcg(L0.R + (r0 + lr) * ny + j, rs[lr * ny + j]);
			}
		if (!grid_sync(gc)) return false;
		// S0 = r - A0 (w iD r) on the band (the pre-smoothed correction is
		// recomputed from r wherever it is needed, never stored)
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int i = r0 + lr;
					const float rk = rs[lr * ny + j];
					const float dk = dd[lr * ny + j];
					float v = dk * (w * rk * __frcp_rn(dk));
					if (i > 0) v = fmaf(cx, w * r0at(i - 1, j) * id0at(i - 1, j), v);
					if (i < nx - 1) v = fmaf(cx, w * r0at(i + 1, j) * id0at(i + 1, j), v);
					if (j > 0) v = fmaf(cy, w * rs[lr * ny + j - 1] * __frcp_rn(dd[lr * ny + j - 1]), v);
					if (j < ny - 1) v = fmaf(cy, w * rs[lr * ny + j + 1] * __frcp_rn(dd[lr * ny + j + 1]), v);
					__stcg(L0.S + i * ny + j, rk - v);
				}
			}
		if (!grid_sync(gc)) return false;
		const int gt = c * T + tid, G = C * T;
		for (int l = 1; l < mg.nlev; ++l) {
			const MgLevel& F = mg.lev[l - 1];
			const MgLevel& L = mg.lev[l];
			const int n = L.nx * L.ny;
			mg_pass<4>(gt, G, n, [&](int k) {
				const int I = k / L.ny, J = k - I * L.ny;
				return mg_restrict(gld, F.S, I, J, F.nx, F.ny);
			}, [&](int k, float v) { __stcg(L.R + k, v); });
			if (!grid_sync(gc)) return false;
			mg_pass<4>(gt, G, n, [&](int k) {
				const int I = k / L.ny, J = k - I * L.ny;
				return mg_resid(ro, gld, L.R, L.D, L.iD, I, J, L.nx, L.ny, cx, cy, w);
			}, [&](int k, float v) { __stcg(L.S + k, v); });
			if (!grid_sync(gc)) return false;
		}
		if (c == 0) mg_coarse(mg, mgsm);
		if (!grid_sync(gc)) return false;
		for (int l = mg.nlev - 1; l >= 1; --l) {
			const MgLevel& L = mg.lev[l];
			const MgLevel& Cl = mg.lev[l + 1];
			mg_pass<2>(gt, G, L.nx * L.ny, [&](int k) {
				const int I = k / L.ny, J = k - I * L.ny;
				return mg_post(ro, gld, gld, L.R, Cl.Zp, L.D, L.iD, I, J, L.nx, L.ny, cx, cy, w);
			}, [&](int k, float v) { __stcg(L.Zp + k, v); });
			if (!grid_sync(gc)) return false;
		}
		// level 0: c = w iD r + P z1 on the band and its halo rows, then the
		// post-smoothed z of the band
		const MgLevel& L1 = mg.lev[1];
		mg_pass<4>(tid, T, (rows + 2) * ny, [&](int t) {
			const int lr = t / ny - 1, j = t - (lr + 1) * ny;
			const int i = r0 + lr;
			return (i >= 0 && i < nx)
					? fmaf(w * r0at(i, j), id0at(i, j), mg_prolong(gld, L1.Zp, i, j, L1.nx, L1.ny))
					: 0.f;
		}, [&](int t, float v) { mgc[t] = v; });
		__syncthreads();
		g[0] = g[1] = 0.f;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int i = r0 + lr, cc = lr * ny + j, pk = (lr + 1) * ny + j;
					const float cv = mgc[pk];
					const float d = dd[cc];
					float ac = d * cv;
					if (i > 0) ac = fmaf(cx, mgc[pk - ny], ac);
					if (i < nx - 1) ac = fmaf(cx, mgc[pk + ny], ac);
					if (j > 0) ac = fmaf(cy, mgc[pk - 1], ac);
					if (j < ny - 1) ac = fmaf(cy, mgc[pk + 1], ac);
					const float rv = rs[cc];
					const float z = fmaf(w * (rv - ac), __frcp_rn(d), cv);
					zs[cc] = z;
					g[0] = fmaf(rv, z, g[0]);
					g[1] = fmaf(rv, rv, g[1]);
				}
			}
		return true;
	};
	// z = M r with M = A^-1 through the separable transforms (dct.cuh):
	// the band's rows along y, a grid barrier, this CTA's block of columns
	// along x with the division by the eigenvalues and back, a grid barrier,
	// the band's rows back along y, each z value handed to out(row, col, z).
	auto dct_apply = [&](auto out) -> bool {
		float* G = dc.G;
		// the transform reads every cell of the band's r, which the callers
		// wrote thread by thread
		__syncthreads();
		dct_forward<false>(dbuf, rows, dc.ly, dc.twy, dc.ey, dc.fy != 0,
				[&](int sq, int n) { return rs[sq * ny + n]; },
				[&](int sq, int k, float val) { __stcg(G + (size_t)(r0 + sq) * ny + k, val); });
		if (!grid_sync(gc)) return false;
		const int l0 = band_lo(c, C, ny), B = band_lo(c + 1, C, ny) - l0;
		const int nxc = 1 << dc.lx;
		// the scaled spectrum stays in shared memory between the two passes
		dct_forward<true>(dbuf, B, dc.lx, dc.twx, dc.ex, dc.fx != 0,
				[&](int sq, int n) { return ldcg(G + (size_t)n * ny + l0 + sq); },
				[&](int sq, int k, float val) {
					const float lam = __ldg(dc.lamx + k) + __ldg(dc.lamy + l0 + sq);
					dspec[sq * (nxc + 1) + k] = lam > 0.f ? val / lam : 0.f;
				});
		dct_inverse<true>(dbuf, B, dc.lx, dc.twx, dc.ex, dc.fx != 0,
				[&](int sq, int k) { return dspec[sq * (nxc + 1) + k]; },
				[&](int sq, int n, float val) { __stcg(G + (size_t)n * ny + l0 + sq, val); });
		if (!grid_sync(gc)) return false;
		dct_inverse<false>(dbuf, rows, dc.ly, dc.twy, dc.ey, dc.fy != 0,
				[&](int sq, int k) { return ldcg(G + (size_t)(r0 + sq) * ny + k); },
				out);
		return true;
	};
	// the spectral preconditioner of the CG: z into zs, (r, z) and (r, r) of
	// the band in g
	auto precond_dct = [&](float (&g)[2]) -> bool {
		if (!dct_apply([&](int sq, int n, float val) { zs[sq * ny + n] = val; })) return false;
		g[0] = g[1] = 0.f;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int cc = lr * ny + j;
					const float rv = rs[cc];
					g[0] = fmaf(rv, zs[cc], g[0]);
					g[1] = fmaf(rv, rv, g[1]);
				}
			}
		return true;
	};
	// the preconditioner in use: spectral, multigrid, the band-local
	// polynomial, or none (z = r)
	auto apply_m = [&](float (&g)[2]) -> bool {
		if (use_dct) return precond_dct(g);
		if (use_mg) return precond_mg(g);
		if (K > 0) precond(g);
		return true;
	};
	// the neighbours' edge rows of region `src` into the halo rows of z.
	// Thread t writes entries t and ny + t, the same mapping every reader of
	// rhal uses, so no barrier is needed between the write and the reads.
	auto read_rh = [&](const float* src) {
		for (int t = tid; t < ny; t += T) {
			if (up) rhal[t] = ldcg(src + (size_t)(2 * (c - 1) + 1) * ny + t);
			if (down) rhal[ny + t] = ldcg(src + (size_t)(2 * (c + 1)) * ny + t);
		}
	};
	// FP64 residual of the band (x64 complete on entry) and its norms; unless
	// it meets the tolerance, the scaled FP32 residual into rs (the residual
	// is kept in FP32, so the scaling costs no FP64 operation). Tags
	// (std::integral_constant, so that optional terms are compiled in or out
	// rather than issued predicated):
	// fb: the first call of the spectral path, whose prologue leaves b
	//   uncentred: b's mean bmean is taken off here and ||b|| summed, in
	//   place of two separate passes;
	// sx: the sum of x rides along for the epilogue's mean removal;
	// sp: the spectral path, whose M ignores the mean of r (the lambda = 0
	//   mode maps to 0), so no sum of r; its scale is ||r|| itself.
	// The reference's nrm2 leaves the last element out: on the spectral path
	// its square is dropped in the loop (a zero factor), otherwise taken
	// off once by the thread that holds it.
	auto resid64 = [&](auto fbt, auto sxt, auto spt, bool first) -> bool {
		constexpr bool fb = decltype(fbt)::value;
		constexpr bool sx = decltype(sxt)::value;
		constexpr bool spc = decltype(spt)::value;
		// spectral: (r, r) without the last, [sum x], [(b, b) without the
		// last]; else: (r, r), sum r, the last r^2
		constexpr int NV = spc ? 1 + (sx ? 1 : 0) + (fb ? 1 : 0) : 3;
		constexpr int IX = 1, IB = sx ? 2 : 1;
		double sums[NV];
#pragma unroll
		for (int m = 0; m < NV; ++m) sums[m] = 0.0;
		double rla = 0.0;
		float* r32 = reinterpret_cast<float*>(v.r);
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int kk = (r0 + lr) * ny + j;
					const int a = (r0 + lr + gl) * P + j + gl;
					const bool last = a == la && !full;
					double bb = v.b[a];
					if (fb) {
						bb = bb - bmean;
						v.b[a] = bb;
						sums[IB] = fma(bb, last ? 0.0 : bb, sums[IB]);
					}
					if (sx) sums[IX] += ldcg(v.x + a);
					const double rv = bb - op.apply(v.x, kk, a);
					r32[a] = (float)rv;
					if (spc) {
						sums[0] = fma(rv, last ? 0.0 : rv, sums[0]);
					} else {
						sums[0] = fma(rv, rv, sums[0]);
						sums[1] += rv;
						if (last) rla = rv;
					}
				}
			}
		if (!spc) sums[2] = rla * rla;
		if (!grid_allreduce_w0<NV>(sums, gc, bank)) return false;
		if (tid == 0) {
			if (fb) {
				const double nb = sqrt(fmax(sums[IB], 0.0));
				s_sc[3] = nb == 0.0 ? 1.0 : nb;
			}
			const double nrm = fb ? s_sc[3] : nrmb;
			if (spc) {
				s_sc[0] = sqrt(fmax(sums[0], 0.0)) / nrm;
				s_sc[1] = 0.0;
				s_sc[2] = sqrt(fmax(sums[0], 0.0));
			} else {
				const double mr = mean ? sums[1] / ncell : 0.0;
				s_sc[0] = sqrt(fmax(sums[0] - sums[2], 0.0)) / nrm;
				s_sc[1] = mr;
				s_sc[2] = sqrt(mean ? fmax(sums[0] - sums[1] * mr, 0.0) : sums[0]);
			}
			s_xm = sx ? sums[IX] / ncell : 0.0;
		}
		__syncthreads();
		if (fb) nrmb = s_sc[3];
		to.resid = s_sc[0];
		to.xmean = s_xm;
		// converged: the caller stops, no FP32 residual or preconditioner
		if (to.resid <= sc.tol) return true;
		if (first) {
			rn0 = s_sc[2];
			scale0 = rn0 > 0.0 ? 1.0 / rn0 : 1.0;
		}
		const float mr = (float)s_sc[1], sc32 = (float)scale0;
		float rr = 0.f;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int a = (r0 + lr + gl) * P + j + gl;
					const float rv = spc ? r32[a] * sc32 : (r32[a] - mr) * sc32;
					rs[lr * ny + j] = rv;
					rr = fmaf(rv, rv, rr);
				}
			}
		rr_band = rr;
		return true;
	};
	// The spectral path's residual in double-float (ta.df: x and b as hi + lo
	// float pairs in the p and q vectors' memory, the coefficients exact in
	// FP32): b - A x with TwoSum / TwoProd on the FP32 pipe, the FP32
	// residual the pair's high part. fb (the first call): b centred (bmean)
	// and the squares summed in FP64; later calls sum the squares of r
	// scaled by 1 / rn0 in FP32 (so they stay in range). The last element's
	// square is dropped (the reference's nrm2); the sum of x (double-float,
	// for the epilogue) rides along.
	float2* xdf = reinterpret_cast<float2*>(v.p);
	float2* bdf = reinterpret_cast<float2*>(v.q);
	auto resid_df = [&](auto fbt) -> bool {
		constexpr bool fb = decltype(fbt)::value;
		constexpr int NV = fb ? 3 : 2;   // (r, r), sum x, [(b, b)]
		const float2 nbm = df_neg(df_from_double(bmean));
		const float sc32 = (float)scale0;
		double q2d = 0.0, b2d = 0.0;
		float q2 = 0.f;
		float2 sxa = make_float2(0.f, 0.f);
		float* r32 = reinterpret_cast<float*>(v.r);
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int a = (r0 + lr + gl) * P + j + gl, cc = lr * ny + j;
					const bool last = a == la && !full;
					// L2 loads (ldcg): the neighbour bands' x was written by
					// other SMs, whose stores no L1 here sees
					float2 bb = ldcg(bdf + a);
					if (fb) {
						bb = df_add(bb, nbm);
						bdf[a] = bb;
						const double bd = f2d_bits(bb.x);
						b2d = fma(bd, last ? 0.0 : bd, b2d);
					}
					const float2 xc = ldcg(xdf + a);
					sxa = df_add(sxa, xc);
					float2 ax = df_mul_f(xc, dd[cc]);
					ax = df_add(ax, df_mul_f(ldcg(xdf + a - P), axs[lr]));
					ax = df_add(ax, df_mul_f(ldcg(xdf + a + P), axs[lr + 1]));
					ax = df_add(ax, df_mul_f(ldcg(xdf + a - 1), ayl[k]));
					ax = df_add(ax, df_mul_f(ldcg(xdf + a + 1), ayr[k]));
					const float rh = df_add(bb, df_neg(ax)).x;
					r32[a] = rh;
					if (fb) {
						const double rd = f2d_bits(rh);
						q2d = fma(rd, last ? 0.0 : rd, q2d);
					} else {
						const float rsc = __fmul_rn(rh, sc32);
						q2 = __fmaf_rn(rsc, last ? 0.f : rsc, q2);
					}
				}
			}
		double sums[NV];
		sums[0] = fb ? q2d : f2d_bits(q2);
		sums[1] = df_to_double(sxa);
		if (fb) sums[NV - 1] = b2d;
		if (!grid_allreduce_w0<NV>(sums, gc, bank)) return false;
		if (tid == 0) {
			if (fb) {
				const double nb = sqrt(fmax(sums[NV - 1], 0.0));
				s_sc[3] = nb == 0.0 ? 1.0 : nb;
			}
			const double nrm = fb ? s_sc[3] : nrmb;
			// later calls summed (r / rn0)^2
			const double rn = fb ? sqrt(fmax(sums[0], 0.0)) : sqrt(fmax(sums[0], 0.0)) * rn0;
			s_sc[0] = rn / nrm;
			s_sc[2] = rn;
			s_xm = sums[1] / ncell;
		}
		__syncthreads();
		if (fb) nrmb = s_sc[3];
		to.resid = s_sc[0];
		to.xmean = s_xm;
		if (to.resid <= sc.tol) return true;
		if (fb) {
			rn0 = s_sc[2];
			scale0 = rn0 > 0.0 ? 1.0 / rn0 : 1.0;
		}
		const float s32 = (float)scale0;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int a = (r0 + lr + gl) * P + j + gl;
					rs[lr * ny + j] = __fmul_rn(r32[a], s32);
				}
			}
		return true;
	};
	// resid64, then (unless converged) z = M r with the edges exchanged;
	// returns gamma = (r, z) and rrn = (r, r) of the new FP32 residual
	auto true_residual = [&](bool first, float& gamma) -> bool {
		if (!resid64(std::false_type{}, std::false_type{}, std::false_type{}, first)) return false;
		if (to.resid <= sc.tol) return true;
		// (r, z) and (r, r) of the band: z = r without a preconditioner
		float g[2] = { rr_band, rr_band };
		if (!apply_m(g)) return false;
		__syncthreads();
		publish_r();
		if (!grid_allreduce<float, 2>(g, gc, bank)) return false;
		read_rh(rbuf);
		gamma = g[0];
		rrn = g[1];
		return true;
	};
	// fold x (FP32, scaled) into x64 and clear it
	auto fold_x = [&]() {
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int a = (r0 + lr + gl) * P + j + gl;
					v.x[a] = fma(rn0, (double)x[lr][k], v.x[a]);
				}
				x[lr][k] = 0.f;
			}
	};

	to.iters = 0;
	to.updates = 0;
	to.done = 0;
	if (use_dct && ta.df) {
		// the same refinement with x, b and the residual in double-float
		if (!resid_df(std::true_type{})) return;
		const float2 rdf = df_from_double(rn0);
		int it = 0;
		while (!(to.resid <= sc.tol) && it < sc.max_iter) {
			if (!dct_apply([&](int sq, int n, float val) {
					const int a = (r0 + sq + gl) * P + n + gl;
					xdf[a] = df_add(ldcg(xdf + a), df_mul_f(rdf, val));
				}))
				return;
			++it;
			if (!grid_sync(gc)) return;
			if (!resid_df(std::false_type{})) return;
			++to.updates;
		}
		to.iters = it;
		to.done = to.resid <= sc.tol ? 1 : 0;
		return;
	}
	if (use_dct) {
		// Iterative refinement with M = A^-1 to FP32 rounding: x += rn0 M r
		// (r scaled by 1 / rn0), then the FP64 residual, until it meets the
		// tolerance. The CG step of the other preconditioners would take
		// alpha = 1 up to FP32 rounding here; it is left out, with its two
		// reductions and its halo exchange.
		// (every call here is fused: the sum of x always rides along)
		if (!resid64(std::true_type{}, std::true_type{}, std::true_type{}, true)) return;
		int it = 0;
		while (!(to.resid <= sc.tol) && it < sc.max_iter) {
			if (!dct_apply([&](int sq, int n, float val) {
					const int a = (r0 + sq + gl) * P + n + gl;
					v.x[a] = fma(rn0, (double)val, v.x[a]);
				}))
				return;
			++it;
			if (!grid_sync(gc)) return;
			if (!resid64(std::false_type{}, std::true_type{}, std::true_type{}, false)) return;
			++to.updates;
		}
		to.iters = it;
		to.done = to.resid <= sc.tol ? 1 : 0;
		return;
	}
	float gamma = 0.f;   // (r, z)
	if (!true_residual(true, gamma)) return;
	if (to.resid <= sc.tol) { to.done = 1; return; }
	float gamma_ref = gamma, gamma_old = 1.f;
	// an update when (r, z) (the residual's squared norm in the
	// preconditioner's metric, (r, r) without one) has dropped by inner_tol^2
	// (inner_tol capped at 1e-2 from below), and at least every kStall
	// iterations: FP32 CG cannot drive its recursive residual much further
	// before it stops tracking the true one
	const double it_tol = fmax(m.inner_tol, 1e-2);
	const float drop = (float)(it_tol * it_tol);
	constexpr int kStall = 1000;
	int since = 0;
	// iterated-residual level at which the FP64 residual is worth checking
	const double tol_scaled = sc.tol * nrmb * scale0;
	const float near = (float)(0.25 * tol_scaled * tol_scaled);
	int it = 0;
	bool first = true;
	while (it < sc.max_iter && gamma > 0.f) {
		const float beta = first ? 0.f : gamma / gamma_old;
		first = false;
		// p = z + beta p over the band and its halo rows
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int pk = 1 + (lr + 1) * ny + j;
					p[pk] = fmaf(beta, p[pk], zs[lr * ny + j]);
				}
			}
		for (int t = tid; t < ny; t += T) {
			if (up) p[1 + t] = fmaf(beta, p[1 + t], rhal[t]);
			if (down) {
				float* pp = p + 1 + (rows + 1) * ny + t;
				*pp = fmaf(beta, *pp, rhal[ny + t]);
			}
		}
		__syncthreads();
		// q = A p, (p, q)
		float pq[1] = { 0.f };
#pragma unroll
		for (int lr = 0; lr < RM; ++lr) {
			const float ax0 = axs[lr], ax1 = axs[lr + 1];
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int pk = 1 + (lr + 1) * ny + j;
					const float pc = p[pk];
					float vv = dd[lr * ny + j] * pc;
					vv = fmaf(ax0, p[pk - ny], vv);
					vv = fmaf(ax1, p[pk + ny], vv);
					vv = fmaf(ayl[k], p[pk - 1], vv);
					vv = fmaf(ayr[k], p[pk + 1], vv);
					q[lr][k] = vv;
					pq[0] = fmaf(pc, vv, pq[0]);
				}
			}
		}
		if (!grid_allreduce<float, 1>(pq, gc, bank)) return;
		const float alpha = gamma / pq[0];
		// x += alpha p, r -= alpha q; z = M r, (r, z), (r, r); z's band
		// edges published
		float rr = 0.f;
#pragma unroll
		for (int lr = 0; lr < RM; ++lr)
#pragma unroll
			for (int k = 0; k < NC; ++k) {
				const int j = tid + k * T;
				if (lr < rows && j < ny) {
					const int pk = 1 + (lr + 1) * ny + j;
					x[lr][k] = fmaf(alpha, p[pk], x[lr][k]);
					const float rv = fmaf(-alpha, q[lr][k], rs[lr * ny + j]);
					rs[lr * ny + j] = rv;
					rr = fmaf(rv, rv, rr);
				}
			}
		float gn[2] = { rr, rr };
		if (!apply_m(gn)) return;
		float* ebuf = ta.xbuf + (size_t)par * edge;
#pragma unroll
		for (int k = 0; k < NC; ++k) {
			const int j = tid + k * T;
			if (j < ny && rows > 0) {
				ebuf[(size_t)(2 * c) * ny + j] = zs[j];
				ebuf[(size_t)(2 * c + 1) * ny + j] = zs[(rows - 1) * ny + j];
			}
		}
		if (!grid_allreduce<float, 2>(gn, gc, bank)) return;
		read_rh(ebuf);
		par ^= 1;
		++it;
		++since;
		float gnew = gn[0];
		rrn = gn[1];
		if (gnew < drop * gamma_ref || rrn <= near || since >= kStall) {
			since = 0;
			// reliable update: fold x, replace r by the FP64 residual
			fold_x();
			if (!grid_sync(gc)) return;
			if (!true_residual(false, gnew)) return;
			++to.updates;
			if (to.resid <= sc.tol) { to.done = 1; break; }
			gamma_ref = gnew;
		}
		gamma_old = gamma;
		gamma = gnew;
	}
	to.iters = it;
	if (!to.done) {
		fold_x();
		if (!grid_sync(gc)) return;
	}
}

// The mixed solve with the Krylov state on chip (tile_solve), one call site
// per instantiation. Spectral path (fused): b of the CTA's band (the row
// constant's folds only at the boundary cells, which take the general form
// out of line) with x0, one reduction for b's mean (also the barrier that
// completes x0); tile_solve then centres b, sums ||b|| and takes the first
// residual in one pass, and returns x's mean from its last residual; the
// epilogue writes the band's phi. Other preconditioners: b and x0 over
// the grid, b centred, ||b|| (the reference's nrm2), and the mean of x
// after the solve.
template<int SRC, int NC, int RM>
__global__ void __launch_bounds__(kTileThreads, 1) k_poisson_mixed_tile(
		StencilOp<double> op, Vecs<double> v, RhsArgs ra, MixedArgs mx,
		TileArgs ta, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	const GridSpace& sp = op.sp;
	const bool fused = ta.dct.on != 0;
	const int C = gridDim.x, c = blockIdx.x, T = blockDim.x, tid = threadIdx.x;
	const int nx = sp.nx, ny = sp.ny, gl = sp.gl, P = sp.P;
	const int r0 = band_lo(c, C, nx), rows = band_lo(c + 1, C, nx) - r0;
	__shared__ double s_nb;
	double bm = 0.0, normb = 1.0;
	if (fused) {
		double s[1] = { 0 };
		// double-float: x and b as hi + lo float pairs in the p and q vectors'
		// memory, with a zero first ghost layer around x (the wall faces'
		// coefficients are 0, so the ghosts need only be finite)
		float2* xdf = reinterpret_cast<float2*>(v.p);
		float2* bdf = reinterpret_cast<float2*>(v.q);
		for (int t = tid; t < rows * ny; t += T) {
			const int lr = t / ny, j = t - lr * ny, i = r0 + lr;
			const int a = (i + gl) * P + j + gl;
			const bool in = i > 0 && i < nx - 1 && j > 0 && j < ny - 1;
			const double bb = in ? rhs_in<SRC>(sp, ra, i, j, a) : rhs_at_call<SRC>(sp, ra, i, j, a);
			if (ta.df) {
				bdf[a] = df_from_double(bb);
				xdf[a] = df_from_double(ra.phi[a]);
			} else {
				v.b[a] = bb;
				v.x[a] = ra.phi[a];
			}
			s[0] += bb;
		}
		if (ta.df) {
			const float2 z = make_float2(0.f, 0.f);
			for (int t = tid; t < 2 * rows; t += T) {
				const int i = r0 + t / 2, j = (t & 1) ? ny : -1;
				xdf[(i + gl) * P + j + gl] = z;
			}
			if (r0 == 0)
				for (int j = tid; j < ny; j += T) xdf[(gl - 1) * P + j + gl] = z;
			if (r0 + rows == nx)
				for (int j = tid; j < ny; j += T) xdf[(nx + gl) * P + j + gl] = z;
		}
		if (!grid_allreduce<double, 1>(s, gc, bank)) return;
		bm = ra.mean ? s[0] / (double)sp.count() : 0.0;
	} else {
		double s[1] = { 0 };
		KLOOP(sp) {
			int i, j;
			sp.ij(k, i, j);
			int a = sp.addr(k);
			double bb = rhs_at<SRC>(sp, ra, i, j, a);
			v.b[a] = bb;
			v.x[a] = ra.phi[a];
			s[0] += bb;
		}
		if (ra.mean) {
			if (!grid_allreduce<double, 1>(s, gc, bank)) return;
			double mm = s[0] / (double)sp.count();
			KLOOP(sp) { int a = sp.addr(k); v.b[a] = v.b[a] - mm; }
		}
		if (!grid_sync(gc)) return;
		const bool full = (sc.flags & CARPIO_GPU_FLAG_FULL_NRM2) || sp.count() == 1;
		const int la = sp.last_addr();
		double acc[1] = { 0 };
		KLOOP(sp) {
			int a = sp.addr(k);
			double bb = v.b[a];
			if (a != la || full) acc[0] = fma(bb, bb, acc[0]);
		}
		if (!grid_allreduce<double, 1>(acc, gc, bank)) return;
		if (threadIdx.x == 0) {
			double nb = sqrt(acc[0]);
			s_nb = nb == 0.0 ? 1.0 : nb;
		}
		__syncthreads();
		normb = s_nb;
	}
	TileOut to;
	tile_solve<NC, RM>(sp, op, v, mx, ta, sc, ra.mean != 0, normb, gc, bank, to, bm);
	if (read_err(gc)) {
		if (blockIdx.x == 0 && threadIdx.x == 0) sc.out->code = read_err(gc);
		return;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		sc.out->outer = to.updates;
		sc.out->inner = to.iters;
	}
	finish(sc, to.done ? 0 : 1, to.iters, to.resid, to.updates + 1);
	if (fused) {
		const double xm = ra.mean ? to.xmean : 0.0;
		const float2* xdf = reinterpret_cast<const float2*>(v.p);
		for (int t = tid; t < rows * ny; t += T) {
			const int lr = t / ny, j = t - lr * ny;
			const int a = (r0 + lr + gl) * P + j + gl;
			const double xv = ta.df ? df_to_double(ldcg(xdf + a)) : v.x[a];
			ra.phi[a] = ra.mean ? xv - xm : xv;
		}
		return;
	}
	double mx0 = 0.0;
	if (ra.mean) {
		double t[1] = { 0 };
		KLOOP(sp) { int a = sp.addr(k); t[0] += v.x[a]; }
		if (!grid_allreduce<double, 1>(t, gc, bank)) {
			if (blockIdx.x == 0 && threadIdx.x == 0) sc.out->code = read_err(gc);
			return;
		}
		mx0 = t[0] / (double)sp.count();
	}
	KLOOP(sp) { int a = sp.addr(k); ra.phi[a] = ra.mean ? v.x[a] - mx0 : v.x[a]; }
}

// b and x0 as vectors in the reference's numbering (x fastest: i + j nx),
// for the solvers that run on an assembled CSR matrix
template<int SRC>
__global__ void __launch_bounds__(kThreads) k_rhs_vec(GridSpace sp, RhsArgs ra,
		double* b, double* x) {
	KLOOP(sp) {
		int i, j;
		sp.ij(k, i, j);
		const int a = sp.addr(k);
		const int r = i + j * sp.nx;
		b[r] = rhs_at<SRC>(sp, ra, i, j, a);
		x[r] = ra.phi[a];
	}
}

template<int SRC>
const void* pick_kernel(int kind, int precision, bool nu) {
	if (nu) {
		if (precision == CARPIO_GPU_MIXED) return (const void*)k_poisson<SRC, 4, true>;
		switch (kind) {
		case CARPIO_GPU_CG: return (const void*)k_poisson<SRC, CARPIO_GPU_CG, true>;
		case CARPIO_GPU_JACOBI: return (const void*)k_poisson<SRC, CARPIO_GPU_JACOBI, true>;
		default: return (const void*)k_poisson<SRC, CARPIO_GPU_BICGSTAB, true>;
		}
	}
	if (precision == CARPIO_GPU_MIXED) return (const void*)k_poisson<SRC, 4, false>;
	switch (kind) {
	case CARPIO_GPU_CG: return (const void*)k_poisson<SRC, CARPIO_GPU_CG, false>;
	case CARPIO_GPU_JACOBI: return (const void*)k_poisson<SRC, CARPIO_GPU_JACOBI, false>;
	default: return (const void*)k_poisson<SRC, CARPIO_GPU_BICGSTAB, false>;
	}
}

bool same_bc(const carpio_gpu_bc& a, const carpio_gpu_bc& b) {
	return std::memcmp(&a, &b, sizeof a) == 0;
}

}  // namespace

namespace cg_host {

void grid_release(carpio_gpu_grid* g) {
	if (g->refs.fetch_sub(1) != 1) return;
	if (g->stream) cudaStreamSynchronize(g->stream);
	cudaFree(g->d_cx);
	cudaFree(g->d_sx);
	cudaFree(g->d_cy);
	cudaFree(g->d_sy);
	if (g->stream) cudaStreamDestroy(g->stream);
	delete g;
}

// Grid_::_set_uniform_grid (s_grid.hpp:372-395): centres and sizes of the
// n + 2 gl cells of one axis, ghosts included
void uniform_axis(int n, int gl, double lo, double hi, std::vector<double>& c,
		std::vector<double>& s) {
	int N = n + 2 * gl;
	double ds = (hi - lo) / n;
	s.assign(N, ds);
	c.assign(N, 0.0);
	double csum = 0.0, llg = 0.0;
	for (int i = 0; i < N; ++i) {
		c[i] = csum + 0.5 * s[i];
		csum += s[i];
	}
	for (int i = 0; i < gl; ++i) llg += s[i];
	double sh = lo - llg;
	for (int i = 0; i < N; ++i) c[i] += sh;
}

void stencil_host(int nx, int ny, int gl, int P, const std::vector<double>& cx,
		const std::vector<double>& sx, const std::vector<double>& cy,
		const std::vector<double>& sy, const carpio_gpu_bc& bc, double beta,
		std::vector<double>& D, std::vector<double>& ax, std::vector<double>& ay,
		std::vector<double>& fold, bool helm, double alpha, std::vector<double>* cf,
		const double* bfield) {
	auto CX = [&](int i) { return cx[i + gl]; };
	auto CY = [&](int j) { return cy[j + gl]; };
	auto SX = [&](int i) { return sx[i + gl]; };
	auto SY = [&](int j) { return sy[j + gl]; };
	const size_t NF = (size_t)(nx + 2 * gl) * P;
	if (cf) cf->assign(4 * NF, 0.0);
	// face value of a beta field (StencilPoisson_::_build_default_beta,
	// s_poisson.hpp:144-164): weights df_ = |half size - centre|
	// (Grid_::df_, s_grid.hpp:226-230) of the cell and of its neighbour on
	// the face's side, values of the cell and of its + neighbour (the
	// reference takes index.p(dim) for both faces)
	const int NJ = ny + 2 * gl;
	auto BF = [&](int i, int j) { return bfield[(size_t)(i + gl) * NJ + (j + gl)]; };
	auto DFX = [&](int i) { return std::fabs(SX(i) * 0.5 - CX(i)); };
	auto DFY = [&](int j) { return std::fabs(SY(j) * 0.5 - CY(j)); };
	auto betaf = [&](int i, int j, int dim, int ori) {
		if (!bfield) return beta;
		const double v = BF(i, j);
		const double df = dim == 0 ? DFX(i) : DFY(j);
		const double vo = dim == 0 ? BF(i + 1, j) : BF(i, j + 1);
		const int o = ori == 0 ? -1 : 1;
		const double dfo = dim == 0 ? DFX(i + o) : DFY(j + o);
		return (df * v + dfo * vo) / (df + dfo);
	};
	D.assign((size_t)(nx + 2 * gl) * P, 0.0);
	ax.assign(nx + 1, 0.0);
	ay.assign(ny + 1, 0.0);
	fold.assign(2 * (size_t)ny + 2 * (size_t)nx, 0.0);
	// ghost substitution of one boundary face (Ghost_::_substitute_ghost,
	// s_ghost.hpp:140-179): returns the centre increment, adds the constant
	auto ghost = [&](int seg, int i, int j, double coe, double& dcen,
			double& cst) {
		int a = seg < 2 ? 0 : 1;
		int gi = i, gj = j, oi = i, oj = j;
		if (seg == 0) gi = -1;
		if (seg == 1) gi = nx;
		if (seg == 2) gj = -1;
		if (seg == 3) gj = ny;
		double c0 = a == 0 ? CX(gi) : CY(gj);
		double c1 = a == 0 ? CX(oi) : CY(oj);
		double hs = (a == 0 ? SX(oi) : SY(oj)) * 0.5;
		double cf = (seg == 1 || seg == 3) ? c1 + hs : c1 - hs;
		double dl = std::fabs(c1 - c0);
		double d0 = std::fabs(cf - c0);
		double d1 = std::fabs(c1 - cf);
		double val = bc.value[seg];
		if (coe == 0) return;
		if (bc.type[seg] == 1) {
			dcen = dcen + -coe * d0 / d1;
			cst = cst + coe * dl * val / d1;
		} else {
			dcen = dcen + coe;
			cst = cst + -val * dl * coe;
		}
	};
	for (int j = 0; j < ny; ++j) {
		for (int i = 0; i < nx; ++i) {
			double axf = SY(j) * 1.0, ayf = 1.0 * SX(i);
			double cxp = (-betaf(i, j, 0, 1)) * axf / std::fabs(CX(i) - CX(i + 1));
			double cxm = (-betaf(i, j, 0, 0)) * axf / std::fabs(CX(i) - CX(i - 1));
			double cyp = (-betaf(i, j, 1, 1)) * ayf / std::fabs(CY(j) - CY(j + 1));
			double cym = (-betaf(i, j, 1, 0)) * ayf / std::fabs(CY(j) - CY(j - 1));
			double coec = 0;
			coec += -cxm;
			coec += -cxp;
			coec += -cym;
			coec += -cyp;
			if (helm) {
				// StencilHelmholtz_::coe_row: coec + (1 * sx * sy) alpha
				double v = 1.0;
				v *= SX(i);
				v *= SY(j);
				coec = coec + v * alpha;
			}
			// boundary constants accumulate per segment cell; for a corner
			// cell the x- fold and the y- fold land in different arrays and
			// are added in map order (x-, y-, y+, x+) on the device
			double cW = 0, cS = 0, cN = 0, cE = 0;
			if (i == 0) ghost(0, i, j, cxm, coec, cW);
			if (j == 0) ghost(2, i, j, cym, coec, cS);
			if (j == ny - 1) ghost(3, i, j, cyp, coec, cN);
			if (i == nx - 1) ghost(1, i, j, cxp, coec, cE);
			D[(size_t)(i + gl) * P + (j + gl)] = coec;
			if (i == 0) fold[j] = cW;
			if (i == nx - 1) fold[ny + j] = cE;
			if (j == 0) fold[2 * ny + i] = cS;
			if (j == ny - 1) fold[2 * ny + nx + i] = cN;
			if (j == 0) ax[i] = i == 0 ? 0.0 : cxm;
			if (j == 0 && i == nx - 1) ax[nx] = 0.0;
			if (i == 0) ay[j] = j == 0 ? 0.0 : cym;
			if (i == 0 && j == ny - 1) ay[ny] = 0.0;
			if (cf) {
				// the row's own coefficients; boundary faces are folded
				const size_t a = (size_t)(i + gl) * P + (j + gl);
				(*cf)[a] = i == 0 ? 0.0 : cxm;
				(*cf)[NF + a] = i == nx - 1 ? 0.0 : cxp;
				(*cf)[2 * NF + a] = j == 0 ? 0.0 : cym;
				(*cf)[3 * NF + a] = j == ny - 1 ? 0.0 : cyp;
			}
		}
	}
}

int stencil_prepare(carpio_gpu_grid* g, const carpio_gpu_bc& bc, double beta,
		StencilCoeffs& c, cudaStream_t s, bool helm, double alpha,
		const double* bfield) {
	// a beta field is read afresh every time (its contents are not tracked)
	if (!bfield && c.valid && c.bfield_free && same_bc(c.bc, bc) && c.beta == beta
			&& c.helm == helm && (!helm || c.alpha == alpha))
		return 0;
	const int gl = g->gl;
	bool uniform = !bfield;
	for (int i = 1; i < g->nx && uniform; ++i) uniform = g->sx[i + gl] == g->sx[gl];
	for (int j = 1; j < g->ny && uniform; ++j) uniform = g->sy[j + gl] == g->sy[gl];
	std::vector<double> bhost;
	if (bfield && is_device_ptr(bfield)) {
		bhost.resize((size_t)g->NI * g->NJ);
		CG_CK(cudaMemcpy(bhost.data(), bfield, sizeof(double) * bhost.size(),
				cudaMemcpyDeviceToHost));
		bfield = bhost.data();
	}
	std::vector<double> D, ax, ay, fold, cf;
	stencil_host(g->nx, g->ny, gl, g->P, g->cx, g->sx, g->cy, g->sy, bc, beta,
			D, ax, ay, fold, helm, alpha, uniform ? nullptr : &cf, bfield);
	std::vector<float> D32(D.size()), ax32(ax.size()), ay32(ay.size());
	for (size_t k = 0; k < D.size(); ++k) D32[k] = (float)D[k];
	for (size_t k = 0; k < ax.size(); ++k) ax32[k] = (float)ax[k];
	for (size_t k = 0; k < ay.size(); ++k) ay32[k] = (float)ay[k];
	int rc;
	if ((rc = to_device(c.D, D.data(), sizeof(double) * D.size(), s))) return rc;
	if ((rc = to_device(c.ax, ax.data(), sizeof(double) * ax.size(), s))) return rc;
	if ((rc = to_device(c.ay, ay.data(), sizeof(double) * ay.size(), s))) return rc;
	if ((rc = to_device(c.fold, fold.data(), sizeof(double) * fold.size(), s))) return rc;
	if ((rc = to_device(c.D32, D32.data(), sizeof(float) * D32.size(), s))) return rc;
	if ((rc = to_device(c.ax32, ax32.data(), sizeof(float) * ax32.size(), s))) return rc;
	if ((rc = to_device(c.ay32, ay32.data(), sizeof(float) * ay32.size(), s))) return rc;
	// a non-uniform grid or a beta field: every row's own four coefficients
	std::vector<float> cf32(cf.begin(), cf.end());
	if (!uniform) {
		if ((rc = to_device(c.cf, cf.data(), sizeof(double) * cf.size(), s))) return rc;
		if ((rc = to_device(c.cf32, cf32.data(), sizeof(float) * cf32.size(), s))) return rc;
	}
	// multigrid levels (uniform grids, no Helmholtz term): sizes halved
	// while both sides are even, down to a level of at most kMgGather cells
	c.mg_nlev = 0;
	c.mg_dims.clear();
	std::vector<float> mgd;
	if (uniform && !helm && g->nx >= 2 && g->ny >= 2) {
		c.mg_dims.push_back({ g->nx, g->ny });
		while ((int)c.mg_dims.size() < kMgMaxLev) {
			const int a = c.mg_dims.back().first, b = c.mg_dims.back().second;
			if ((a & 1) || (b & 1)) break;
			c.mg_dims.push_back({ a / 2, b / 2 });
		}
		for (size_t l = 1; l < c.mg_dims.size(); ++l)
			if ((long)c.mg_dims[l].first * c.mg_dims[l].second <= kMgGather) {
				c.mg_nlev = (int)l;
				break;
			}
		// the interior face coefficients (equal on every face of a uniform
		// grid up to the rounding of the centre distances)
		const double cxd = ax[g->nx / 2], cyd = ay[g->ny / 2];
		c.mg_cx = (float)cxd;
		c.mg_cy = (float)cyd;
		// each level's diagonal: every face contributes -c; a boundary face
		// folds like the fine grid's ghost substitution (Dirichlet: -2c in
		// all, Neumann: 0)
		// level 0 is the fine grid's own FP32 diagonal (the tile kernel's
		// band copy), the coarser ones follow the rule above; then every
		// level's reciprocal
		for (size_t l = 0; l < c.mg_dims.size(); ++l) {
			const auto& dm = c.mg_dims[l];
			for (int I = 0; I < dm.first; ++I)
				for (int J = 0; J < dm.second; ++J) {
					if (l == 0) {
						mgd.push_back(D32[(size_t)(I + gl) * g->P + (J + gl)]);
						continue;
					}
					double d = 0.0;
					d += I > 0 ? -cxd : (bc.type[0] == 1 ? -2.0 * cxd : 0.0);
					d += I < dm.first - 1 ? -cxd : (bc.type[1] == 1 ? -2.0 * cxd : 0.0);
					d += J > 0 ? -cyd : (bc.type[2] == 1 ? -2.0 * cyd : 0.0);
					d += J < dm.second - 1 ? -cyd : (bc.type[3] == 1 ? -2.0 * cyd : 0.0);
					mgd.push_back((float)d);
				}
		}
		const size_t nd = mgd.size();
		for (size_t k = 0; k < nd; ++k) mgd.push_back(mgd[k] > 0.f ? 1.0f / mgd[k] : 0.f);
		if (c.mg_nlev > 0 && (rc = to_device(c.mgD, mgd.data(), sizeof(float) * mgd.size(), s)))
			return rc;
	}
	// the spectral preconditioner: power-of-two sides, Neumann or Dirichlet
	// on both sides of each axis, and an operator that is the separable
	// five-point one (uniform interior faces, the diagonal folded as above)
	c.dct_ok = false;
	c.dct_df = false;
	auto pow2 = [](int n, int& lg) {
		lg = 0;
		while ((1 << lg) < n) ++lg;
		return n >= 2 && (1 << lg) == n && n <= 4096;
	};
	int lgx = 0, lgy = 0;
	if (uniform && !helm && pow2(g->nx, lgx) && pow2(g->ny, lgy) && bc.type[0] == bc.type[1]
			&& bc.type[2] == bc.type[3] && (bc.type[0] == 1 || bc.type[0] == 2)
			&& (bc.type[2] == 1 || bc.type[2] == 2)) {
		const int nx = g->nx, ny = g->ny;
		const double cxd = ax[nx / 2], cyd = ay[ny / 2];
		bool ok = cxd < 0.0 && cyd < 0.0;
		auto near = [](double a, double b) { return std::fabs(a - b) <= 1e-10 * std::fabs(b); };
		for (int i = 1; i < nx && ok; ++i) ok = near(ax[i], cxd);
		for (int j = 1; j < ny && ok; ++j) ok = near(ay[j], cyd);
		for (int i = 0; i < nx && ok; ++i)
			for (int j = 0; j < ny && ok; ++j) {
				double d = 0.0;
				d += i > 0 ? -cxd : (bc.type[0] == 1 ? -2.0 * cxd : 0.0);
				d += i < nx - 1 ? -cxd : (bc.type[1] == 1 ? -2.0 * cxd : 0.0);
				d += j > 0 ? -cyd : (bc.type[2] == 1 ? -2.0 * cyd : 0.0);
				d += j < ny - 1 ? -cyd : (bc.type[3] == 1 ? -2.0 * cyd : 0.0);
				ok = near(D[(size_t)(i + gl) * g->P + (j + gl)], d);
			}
		if (ok) {
			const double pi = 3.14159265358979323846;
			std::vector<float> t;
			auto lam = [&](int N, double cc, bool dir) {
				for (int m = 0; m < N; ++m) {
					const double th = pi * (dir ? N - m : m) / N;
					t.push_back((float)(-cc * (2.0 - 2.0 * std::cos(th))));
				}
			};
			auto cplx = [&](double a) {
				t.push_back((float)std::cos(a));
				t.push_back((float)std::sin(a));
			};
			lam(nx, cxd, bc.type[0] == 1);
			lam(ny, cyd, bc.type[2] == 1);
			for (int q = 0; q < nx / 2; ++q) cplx(-2.0 * pi * q / nx);
			for (int q = 0; q < ny / 2; ++q) cplx(-2.0 * pi * q / ny);
			for (int k = 0; k < nx; ++k) cplx(-pi * k / (2.0 * nx));
			for (int k = 0; k < ny; ++k) cplx(-pi * k / (2.0 * ny));
			if ((rc = to_device(c.dctT, t.data(), sizeof(float) * t.size(), s))) return rc;
			c.dct_ok = true;
			bool ex = true;
			auto f32 = [](double x) { return (double)(float)x == x && std::fabs(x) < 1e30; };
			for (int i = 0; i <= nx && ex; ++i) ex = f32(ax[i]);
			for (int j = 0; j <= ny && ex; ++j) ex = f32(ay[j]);
			for (int i = 0; i < nx && ex; ++i)
				for (int j = 0; j < ny && ex; ++j) ex = f32(D[(size_t)(i + gl) * g->P + (j + gl)]);
			c.dct_df = ex;
			c.dct_lx = lgx;
			c.dct_ly = lgy;
			c.dct_fx = bc.type[0] == 1;
			c.dct_fy = bc.type[2] == 1;
		}
	}
	CG_CK(cudaStreamSynchronize(s));  // host vectors go out of scope
	c.uniform = uniform;
	c.bfield_free = !bfield;
	c.bc = bc;
	c.beta = beta;
	c.helm = helm;
	c.alpha = alpha;
	c.valid = true;
	return 0;
}

// IC_CGS / IC_CG at the structure level (Solver_IC_CGS_, s_solver.hpp:
// 329-352, with the drop-in's mean removal): the CSR matrix assembled on the
// host from the stencil rows (x-fastest numbering, columns ascending), b
// from the device right-hand side, the algebra-level IC solver, x back into
// phi's normal cells. Synchronous (small systems: the IC solves are level
// scheduled).
static int ic_structured(carpio_gpu_grid* g, StencilCoeffs& c, int src_mode,
		const double* src_a, const double* src_b, double* phi,
		const carpio_gpu_solver_cfg& cfg, double* hist_dev, int hist_cap,
		cg_dev::SolveOut* out_dev, cudaStream_t s) {
	const int nx = g->nx, ny = g->ny, gl = g->gl, P = g->P;
	const int n = nx * ny;
	std::vector<double> D, ax, ay, fold, cf;
	stencil_host(nx, ny, gl, P, g->cx, g->sx, g->cy, g->sy, c.bc, c.beta, D, ax, ay,
			fold, c.helm, c.alpha, &cf, nullptr);
	const size_t NF = (size_t)g->NI * P;
	std::vector<uint32_t> rp(n + 1, 0), ci;
	std::vector<double> va;
	ci.reserve(5 * (size_t)n);
	va.reserve(5 * (size_t)n);
	for (int j = 0; j < ny; ++j)
		for (int i = 0; i < nx; ++i) {
			const int r = i + j * nx;
			const size_t a = (size_t)(i + gl) * P + (j + gl);
			auto put = [&](int col, double v) { ci.push_back((uint32_t)col); va.push_back(v); };
			if (j > 0) put(r - nx, cf[2 * NF + a]);
			if (i > 0) put(r - 1, cf[a]);
			put(r, D[a]);
			if (i < nx - 1) put(r + 1, cf[NF + a]);
			if (j < ny - 1) put(r + nx, cf[3 * NF + a]);
			rp[r + 1] = (uint32_t)ci.size();
		}
	DevBuf bx;
	int rc;
	if ((rc = bx.ensure(sizeof(double) * 2 * (size_t)n))) return rc;
	RhsArgs ra;
	ra.sx = g->d_sx;
	ra.sy = g->d_sy;
	ra.fold = c.fold.as<double>();
	ra.src_a = src_a;
	ra.src_b = src_b;
	rhs_set_p2(ra, g->sx, g->sy);
	ra.phi = phi;
	ra.mean = 0;
	ra.helm = c.helm ? 1 : 0;
	const GridSpace sp{ nx, ny, gl, P };
	const int nb = (int)std::min<long>(((long)n + kThreads - 1) / kThreads, 8L * sm_count());
	if (src_mode == SRC_DIV)
		k_rhs_vec<SRC_DIV><<<nb, kThreads, 0, s>>>(sp, ra, bx.as<double>(), bx.as<double>() + n);
	else
		k_rhs_vec<SRC_FIELD><<<nb, kThreads, 0, s>>>(sp, ra, bx.as<double>(), bx.as<double>() + n);
	CG_CK(cudaGetLastError());
	std::vector<double> b(n), x(n);
	CG_CK(cudaMemcpyAsync(b.data(), bx.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
	CG_CK(cudaMemcpyAsync(x.data(), bx.as<double>() + n, sizeof(double) * n,
			cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	// the drop-in's null-space removal: the mean in sequence, then a - m
	auto remove_mean = [&](std::vector<double>& v) {
		double m = 0;
		for (double e : v) m += e;
		m = m / double(v.size());
		for (double& e : v) e = e - m;
	};
	if (cfg.mean_removal) remove_mean(b);
	int it = cfg.max_iter;
	double tol = cfg.tol;
	int hl = 0;
	const int code = carpio_gpu_krylov_csr(cfg.kind, n, (int)ci.size(), rp.data(), ci.data(),
			va.data(), b.data(), x.data(), &it, &tol, hist_dev, hist_cap, &hl, cfg.flags);
	cg_dev::SolveOut o{};
	o.code = code;
	o.iters = it;
	o.tol = tol;
	o.hist_len = hl;
	if (code >= 0) {
		if (cfg.mean_removal) remove_mean(x);
		std::vector<double> f(NF);
		CG_CK(cudaMemcpy(f.data(), phi, sizeof(double) * NF, cudaMemcpyDeviceToHost));
		for (int j = 0; j < ny; ++j)
			for (int i = 0; i < nx; ++i) f[(size_t)(i + gl) * P + (j + gl)] = x[i + j * nx];
		CG_CK(cudaMemcpy(phi, f.data(), sizeof(double) * NF, cudaMemcpyHostToDevice));
	}
	CG_CK(cudaMemcpy(out_dev, &o, sizeof o, cudaMemcpyHostToDevice));
	return 0;
}

int poisson_launch(carpio_gpu_grid* g, StencilCoeffs& c, PoissonWs& w,
		int src_mode, const double* src_a, const double* src_b, double* phi,
		const carpio_gpu_solver_cfg& cfg, double* hist_dev, int hist_cap,
		cg_dev::SolveOut* out_dev, cudaStream_t s) {
	if (cfg.kind == CARPIO_GPU_IC_CGS || cfg.kind == CARPIO_GPU_IC_CG) {
		if (cfg.precision != CARPIO_GPU_FP64 || !c.bfield_free) return CARPIO_GPU_EINVAL;
		return ic_structured(g, c, src_mode, src_a, src_b, phi, cfg, hist_dev, hist_cap,
				out_dev, s);
	}
	const size_t NF = (size_t)g->NI * g->P;
	const bool mixed = cfg.precision == CARPIO_GPU_MIXED;
	// FP32 vectors: x r p q for the inner CG, 13 (all of Vecs) for the
	// inner BiCGSTAB
	const int nv64 = 13, nv32 = cfg.kind == CARPIO_GPU_CG ? 4 : 13;
	int rc;
	if (w.v64.bytes < sizeof(double) * NF * nv64) {
		if ((rc = w.v64.ensure(sizeof(double) * NF * nv64))) return rc;
		CG_CK(cudaMemsetAsync(w.v64.p, 0, w.v64.bytes, s));   // zero ghost rings
	}
	if (mixed && w.v32.bytes < sizeof(float) * NF * nv32) {
		if ((rc = w.v32.ensure(sizeof(float) * NF * nv32))) return rc;
		CG_CK(cudaMemsetAsync(w.v32.p, 0, w.v32.bytes, s));
	}
	const void* kern = src_mode == SRC_DIV ? pick_kernel<SRC_DIV>(cfg.kind, cfg.precision, !c.uniform)
	                                       : pick_kernel<SRC_FIELD>(cfg.kind, cfg.precision, !c.uniform);
	long n = (long)g->nx * g->ny;
	// at most two 256-thread blocks per SM: enough warps for the FP64 pipe,
	// few enough arrivals at each grid barrier
	int blocks = std::min(coop_blocks(kern, n, 2), 2 * sm_count());
	if ((rc = w.lw.ensure(blocks))) return rc;
	StencilOp<double> op;
	op.sp = GridSpace{ g->nx, g->ny, g->gl, g->P };
	op.D = c.D.as<double>();
	op.ax = c.ax.as<double>();
	op.ay = c.ay.as<double>();
	op.cf = c.uniform ? nullptr : c.cf.as<double>();
	op.cfs = (size_t)g->NI * g->P;
	Vecs<double> v;
	double* base = w.v64.as<double>();
	double** slots[nv64] = { &v.x, &v.b, &v.r, &v.p, &v.q, &v.z, &v.rt, &v.ph,
		&v.s, &v.sh, &v.t, &v.v, &v.d };
	for (int i = 0; i < nv64; ++i) *slots[i] = base + (size_t)i * NF;
	MixedArgs mx;
	mx.op32.sp = op.sp;
	mx.op32.D = c.D32.as<float>();
	mx.op32.ax = c.ax32.as<float>();
	mx.op32.ay = c.ay32.as<float>();
	mx.op32.cf = c.uniform ? nullptr : c.cf32.as<float>();
	mx.op32.cfs = (size_t)g->NI * g->P;
	std::memset(&mx.f, 0, sizeof mx.f);
	if (mixed) {
		float* fb = w.v32.as<float>();
		float** fs[13] = { &mx.f.x, &mx.f.r, &mx.f.p, &mx.f.q, &mx.f.b, &mx.f.z,
			&mx.f.rt, &mx.f.ph, &mx.f.s, &mx.f.sh, &mx.f.t, &mx.f.v, &mx.f.d };
		for (int i = 0; i < nv32; ++i) *fs[i] = fb + (size_t)i * NF;
	}
	mx.inner_tol = cfg.inner_tol > 0 ? cfg.inner_tol : 1e-4;
	mx.inner_max = cfg.inner_max_iter > 0 ? cfg.inner_max_iter : 1 << 30;
	mx.pdeg = 0;
	mx.pratio = 1.f;
	RhsArgs ra;
	ra.sx = g->d_sx;
	ra.sy = g->d_sy;
	ra.fold = c.fold.as<double>();
	ra.src_a = src_a;
	ra.src_b = src_b;
	rhs_set_p2(ra, g->sx, g->sy);
	ra.phi = phi;
	ra.mean = cfg.mean_removal ? 1 : 0;
	ra.helm = c.helm ? 1 : 0;
	SolveCtl sc;
	sc.kind = cfg.kind;
	sc.max_iter = cfg.max_iter;
	sc.tol = cfg.tol;
	sc.flags = cfg.flags;
	sc.hist = hist_dev;
	sc.hist_cap = hist_dev ? hist_cap : 0;
	sc.out = out_dev;
	// mixed solves whose bands fit the tile kernel run on chip
	// the on-chip kernel keeps one coefficient per face row / column: uniform
	// grids only (non-uniform ones run the global-memory FP32 inner CG)
	if (mixed && c.uniform && cfg.kind == CARPIO_GPU_CG && !(cfg.flags & CARPIO_GPU_FLAG_NO_TILE)) {
		const int C = std::min(sm_count(), g->nx);
		const int rows_max = (g->nx + C - 1) / C;
		const int nc = (g->ny + kTileThreads - 1) / kTileThreads;
		const void* tk = nullptr;
#define TILE_PICK(NC_, RM_)                                                         \
		if (!tk && nc <= NC_ && rows_max <= RM_)                                    \
			tk = src_mode == SRC_DIV ? (const void*)k_poisson_mixed_tile<SRC_DIV, NC_, RM_>      \
			                         : (const void*)k_poisson_mixed_tile<SRC_FIELD, NC_, RM_>;
		TILE_PICK(1, 4) TILE_PICK(1, 16) TILE_PICK(2, 8) TILE_PICK(4, 4)
#undef TILE_PICK
		int pdeg = cfg.poly_degree < 0 ? 0 : (cfg.poly_degree == 0 ? kPolyDegree : cfg.poly_degree);
		const size_t np = (size_t)(rows_max + 2) * g->ny + 2;
		const size_t base = sizeof(float) * (np + 2 * (size_t)g->ny + (size_t)rows_max * g->ny
				+ rows_max + 1 + g->ny + 1 + (size_t)rows_max * g->ny);
		TileArgs ta;
		std::memset(&ta, 0, sizeof ta);
		size_t smem = base;
		// the spectral preconditioner where asked for (or by default) and the
		// operator allows it: zs, then the FFT buffer of the band's rows or
		// of a CTA's block of columns, whichever is longer
		bool mg = false, spec = false;
		if ((cfg.precond == CARPIO_GPU_PRECOND_DEFAULT || cfg.precond == CARPIO_GPU_PRECOND_SPECTRAL)
				&& c.dct_ok) {
			const size_t zsn = (size_t)rows_max * g->ny;
			const size_t cmax = ((size_t)g->ny + C - 1) / C;
			// the FFT buffer: ceil(B / 2) sequences per pass (two real ones
			// share one), the column passes' sequences one element apart
			const size_t fb = std::max((zsn / g->ny + 1) / 2 * (size_t)g->ny,
					(cmax + 1) / 2 * ((size_t)g->nx + 1));
			const size_t ssmem = base + sizeof(float) * (zsn + 1) + sizeof(float2) * fb
					+ sizeof(float) * cmax * ((size_t)g->nx + 1);
			if (ssmem <= 220 * 1024) {
				if ((rc = w.dct.ensure(sizeof(float) * (size_t)g->nx * g->ny))) return rc;
				DctArgs& d = ta.dct;
				const float* tp = c.dctT.as<float>();
				const int nx = g->nx, ny = g->ny;
				d.on = 1;
				d.lx = c.dct_lx;
				d.ly = c.dct_ly;
				d.fx = c.dct_fx;
				d.fy = c.dct_fy;
				d.lamx = tp;
				d.lamy = tp + nx;
				const float2* cp = reinterpret_cast<const float2*>(tp + nx + ny);
				d.twx = cp;
				d.twy = cp + nx / 2;
				d.ex = cp + nx / 2 + ny / 2;
				d.ey = cp + nx / 2 + ny / 2 + nx;
				d.G = w.dct.as<float>();
				d.fb = (int)fb;
				ta.df = c.dct_df ? 1 : 0;
				smem = ssmem;
				pdeg = 0;
				spec = true;
			}
		}
		// the multigrid V-cycle where asked for and the grid allows it
		if (!spec && cfg.precond != CARPIO_GPU_PRECOND_CHEBYSHEV && c.mg_nlev > 0) {
			size_t coarse = 0, work = 0;
			const int ntot = (int)c.mg_dims.size();
			for (int l = c.mg_nlev; l < ntot; ++l)
				coarse += 3 * (size_t)c.mg_dims[l].first * c.mg_dims[l].second;
			const size_t msmem = base + sizeof(float) * ((size_t)rows_max * g->ny + np + coarse);
			for (int l = 0; l <= c.mg_nlev; ++l)
				work += (l == 0 ? 2 : l < c.mg_nlev ? 3 : 1)
						* (size_t)c.mg_dims[l].first * c.mg_dims[l].second;
			if (msmem <= 220 * 1024) {
				if ((rc = w.mg.ensure(sizeof(float) * work))) return rc;
				MgArgs& m = ta.mg;
				m.nlev = c.mg_nlev;
				m.ntot = ntot;
				m.cx = c.mg_cx;
				m.cy = c.mg_cy;
				m.omega = 0.8f;
				size_t nd = 0;
				for (int l = 0; l < ntot; ++l) nd += (size_t)c.mg_dims[l].first * c.mg_dims[l].second;
				const float* dp = c.mgD.as<float>();
				float* wp = w.mg.as<float>();
				for (int l = 0; l < ntot; ++l) {
					const size_t n = (size_t)c.mg_dims[l].first * c.mg_dims[l].second;
					MgLevel& L = m.lev[l];
					L.nx = c.mg_dims[l].first;
					L.ny = c.mg_dims[l].second;
					L.D = dp;
					L.iD = dp + nd;
					dp += n;
					if (l == 0) {
						L.R = wp; L.S = wp + n;
						wp += 2 * n;
					} else if (l < c.mg_nlev) {
						L.R = wp; L.S = wp + n; L.Zp = wp + 2 * n;
						wp += 3 * n;
					} else if (l == c.mg_nlev) {
						L.Zp = wp;
						wp += n;
					}
				}
				smem = msmem;
				pdeg = 0;
				mg = true;
			}
		}
		if (pdeg > 0) smem += sizeof(float) * ((size_t)rows_max * g->ny + 2 * np);
		mx.pdeg = pdeg;
		mx.pratio = (float)(cfg.poly_ratio > 1.0 ? cfg.poly_ratio : kPolyRatio);
		if (tk && smem <= 220 * 1024) {
			CG_CK(cudaFuncSetAttribute(tk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
			int per_sm = 0;
			CG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tk, kTileThreads, smem));
			if (per_sm >= 1) {
				if ((rc = w.lw.ensure(C))) return rc;
				if ((rc = w.xbuf.ensure(sizeof(float) * 6 * (size_t)C * g->ny))) return rc;
				ta.xbuf = w.xbuf.as<float>();
				ta.rows_max = rows_max;
				// the polynomial-preconditioned FP32 CG stops tracking its
				// residual sooner: replace it after a 1e-1 reduction; with
				// the V-cycle each iteration gains about a digit, so after
				// 1e-2 (the smallest step allowed on chip)
				mx.inner_tol = cfg.inner_tol > 0 ? cfg.inner_tol
				                                 : ((mg || spec) ? 1e-2 : pdeg > 0 ? 1e-1 : 3e-2);
				GridCtl gc = make_gridctl(w.lw);
				CG_CK(cudaMemsetAsync(w.lw.ctl.p, 0, sizeof(Ctl), s));
				CG_CK(cudaMemsetAsync(out_dev, 0, sizeof(cg_dev::SolveOut), s));
				void* args[] = { &op, &v, &ra, &mx, &ta, &sc, &gc };
				CG_CK(cudaLaunchCooperativeKernel(tk, C, kTileThreads, args, smem, s));
				return 0;
			}
		}
	}
	GridCtl gc = make_gridctl(w.lw);
	CG_CK(cudaMemsetAsync(w.lw.ctl.p, 0, sizeof(Ctl), s));
	CG_CK(cudaMemsetAsync(out_dev, 0, sizeof(cg_dev::SolveOut), s));
	void* args[] = { &op, &v, &ra, &mx, &sc, &gc };
	CG_CK(cudaLaunchCooperativeKernel(kern, blocks, kThreads, args, 0, s));
	return 0;
}

}  // namespace cg_host

// ------------------------------------------------------------------ C ABI --
extern "C" {

}  // extern "C"

namespace cg_host {

// Centres and sizes of the n + 2 gl cells of an axis given the normal cells'
// sizes (Grid_::_set_non_uniform_grid, s_grid.hpp:397-434): ghosts take the
// size of the nearest normal cell; centres are running sums shifted so the
// first normal cell starts at lo.
void sized_axis(int n, int gl, double lo, const double* cs, std::vector<double>& c,
		std::vector<double>& s) {
	const int N = n + 2 * gl;
	s.assign(N, 0.0);
	c.assign(N, 0.0);
	for (int i = 0; i < N; ++i) s[i] = i < gl ? cs[0] : (i - gl >= n ? cs[n - 1] : cs[i - gl]);
	double csum = 0.0, llg = 0.0;
	for (int i = 0; i < N; ++i) {
		c[i] = csum + 0.5 * s[i];
		csum += s[i];
	}
	for (int i = 0; i < gl; ++i) llg += s[i];
	const double sh = lo - llg;
	for (int i = 0; i < N; ++i) c[i] += sh;
}

// A grid handle around host-built axes: stream and device copies.
static int grid_from_axes(int nx, int ny, int gl, std::vector<double>&& cx,
		std::vector<double>&& sx, std::vector<double>&& cy, std::vector<double>&& sy,
		carpio_gpu_grid** out) {
	carpio_gpu_grid* g = new carpio_gpu_grid();
	g->nx = nx;
	g->ny = ny;
	g->gl = gl;
	g->NI = nx + 2 * gl;
	g->NJ = ny + 2 * gl;
	g->P = (g->NJ + 31) / 32 * 32;
	g->cx = std::move(cx);
	g->sx = std::move(sx);
	g->cy = std::move(cy);
	g->sy = std::move(sy);
	cudaGetDevice(&g->device);
	auto fail = [&](int code) {
		carpio_gpu_grid_destroy(g);
		return code;
	};
	if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	double** dp[4] = { &g->d_cx, &g->d_sx, &g->d_cy, &g->d_sy };
	std::vector<double>* hp[4] = { &g->cx, &g->sx, &g->cy, &g->sy };
	for (int k = 0; k < 4; ++k) {
		if (cudaMalloc((void**)dp[k], sizeof(double) * hp[k]->size()) != cudaSuccess) {
			cudaGetLastError();
			return fail(CARPIO_GPU_ENOMEM);
		}
		if (cudaMemcpy(*dp[k], hp[k]->data(), sizeof(double) * hp[k]->size(),
				cudaMemcpyHostToDevice) != cudaSuccess) {
			note_cuda_error(cudaGetLastError());
			return fail(CARPIO_GPU_ECUDA);
		}
	}
	*out = g;
	return 0;
}

}  // namespace cg_host

extern "C" {

int carpio_gpu_grid_create_uniform(int nx, int ny, int gl, double xmin,
		double xmax, double ymin, double ymax, carpio_gpu_grid** out) {
	using namespace cg_host;
	if (!out || nx < 1 || ny < 1 || gl < 1 || gl > 8 || !(xmax > xmin)
			|| !(ymax > ymin) || (long)nx * ny > (1L << 30))
		return CARPIO_GPU_EINVAL;
	*out = nullptr;
	std::vector<double> cx, sx, cy, sy;
	uniform_axis(nx, gl, xmin, xmax, cx, sx);
	uniform_axis(ny, gl, ymin, ymax, cy, sy);
	return grid_from_axes(nx, ny, gl, std::move(cx), std::move(sx), std::move(cy),
			std::move(sy), out);
}

int carpio_gpu_grid_create(int nx, int ny, int gl, double xmin, double ymin,
		const double* csx, const double* csy, carpio_gpu_grid** out) {
	using namespace cg_host;
	if (!out || !csx || !csy || nx < 1 || ny < 1 || gl < 1 || gl > 8
			|| (long)nx * ny > (1L << 30))
		return CARPIO_GPU_EINVAL;
	for (int i = 0; i < nx; ++i)
		if (!(csx[i] > 0.0) || !std::isfinite(csx[i])) return CARPIO_GPU_EINVAL;
	for (int j = 0; j < ny; ++j)
		if (!(csy[j] > 0.0) || !std::isfinite(csy[j])) return CARPIO_GPU_EINVAL;
	*out = nullptr;
	std::vector<double> cx, sx, cy, sy;
	sized_axis(nx, gl, xmin, csx, cx, sx);
	sized_axis(ny, gl, ymin, csy, cy, sy);
	return grid_from_axes(nx, ny, gl, std::move(cx), std::move(sx), std::move(cy),
			std::move(sy), out);
}

int carpio_gpu_output_scalar(const carpio_gpu_grid* g, const char* filename,
		const double* field) {
	using namespace cg_host;
	if (!g || !filename || !field) return CARPIO_GPU_EINVAL;
	const size_t n = (size_t)g->NI * g->NJ;
	std::vector<double> host;
	const double* f = field;
	if (is_device_ptr(field)) {
		host.resize(n);
		if (cudaMemcpy(host.data(), field, sizeof(double) * n, cudaMemcpyDeviceToHost)
				!= cudaSuccess) {
			note_cuda_error(cudaGetLastError());
			return CARPIO_GPU_ECUDA;
		}
		f = host.data();
	}
	FILE* fp = std::fopen(filename, "w");
	if (!fp) return CARPIO_GPU_EIO;
	const int gl = g->gl;
	bool ok = std::fprintf(fp, "## Size : %ld\n## Dim : 2\n## NX :  %d\n## NY :  %d\n",
			(long)g->nx * g->ny, g->nx, g->ny) > 0;
	for (int j = 0; j < g->ny && ok; ++j)
		for (int i = 0; i < g->nx && ok; ++i)
			ok = std::fprintf(fp, "%10.6e, %10.6e, %10.6e, %10.6e\n", g->cx[i + gl],
					g->cy[j + gl], 0.0, f[(size_t)(i + gl) * g->NJ + (j + gl)]) > 0;
	ok = (std::fclose(fp) == 0) && ok;
	return ok ? 0 : CARPIO_GPU_EIO;
}

int carpio_gpu_grid_destroy(carpio_gpu_grid* g) {
	if (!g) return CARPIO_GPU_EINVAL;
	cg_host::grid_release(g);
	return 0;
}

int carpio_gpu_grid_coords(const carpio_gpu_grid* g, double* cx, double* sx,
		double* cy, double* sy) {
	if (!g) return CARPIO_GPU_EINVAL;
	if (cx) std::memcpy(cx, g->cx.data(), sizeof(double) * g->cx.size());
	if (sx) std::memcpy(sx, g->sx.data(), sizeof(double) * g->sx.size());
	if (cy) std::memcpy(cy, g->cy.data(), sizeof(double) * g->cy.size());
	if (sy) std::memcpy(sy, g->sy.data(), sizeof(double) * g->sy.size());
	return 0;
}

}  // extern "C"

// Poisson_::run for a set_depend'ed field; helm: the StencilHelmholtz_
// variant (Poisson_ with an alpha term, s_poisson.hpp:343-347, 577-590)
static int structured_solve(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		bool helm, double alpha, double beta, const double* bfield, const double* source,
		double* phi, const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats) {
	using namespace cg_host;
	if (!g || !bc || !source || !phi || !cfg || cfg->max_iter < 0
			|| cfg->kind < 0 || cfg->kind > CARPIO_GPU_IC_CG || hist_cap < 0
			|| (hist_cap > 0 && !resid_hist) || !(beta == beta) || !(alpha == alpha))
		return CARPIO_GPU_EINVAL;
	// FP32 inner iterations: CG, Dia_BiCGSTAB and BiCGSTAB
	if (cfg->precision == CARPIO_GPU_MIXED && cfg->kind != CARPIO_GPU_CG
			&& cfg->kind != CARPIO_GPU_DIA_BICGSTAB && cfg->kind != CARPIO_GPU_BICGSTAB)
		return CARPIO_GPU_EINVAL;
	for (int k = 0; k < 4; ++k)
		if (bc->type[k] != 1 && bc->type[k] != 2) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(g->mu);
	cudaStream_t s = g->stream;
	int rc;
	if ((rc = stencil_prepare(g, *bc, beta, g->coeffs, s, helm, alpha, bfield))) return rc;
	PoissonWs& w = g->pws;
	const size_t NF = (size_t)g->NI * g->P;
	if ((rc = w.src.ensure(sizeof(double) * NF))) return rc;
	if ((rc = w.phi.ensure(sizeof(double) * NF))) return rc;
	if ((rc = w.out.ensure(sizeof(cg_dev::SolveOut)))) return rc;
	if ((rc = w.hist.ensure(sizeof(double) * (size_t)(hist_cap > 0 ? hist_cap : 1)))) return rc;
	const size_t wb = sizeof(double) * g->NJ, pb = sizeof(double) * g->P;
	CG_CK(cudaMemcpy2DAsync(w.src.p, pb, source, wb, wb, g->NI, cudaMemcpyDefault, s));
	CG_CK(cudaMemcpy2DAsync(w.phi.p, pb, phi, wb, wb, g->NI, cudaMemcpyDefault, s));
	cudaEvent_t e0, e1;
	CG_CK(cudaEventCreate(&e0));
	CG_CK(cudaEventCreate(&e1));
	CG_CK(cudaEventRecord(e0, s));
	rc = poisson_launch(g, g->coeffs, w, SRC_FIELD, w.src.as<double>(), nullptr,
			w.phi.as<double>(), *cfg, hist_cap > 0 ? w.hist.as<double>() : nullptr,
			hist_cap, w.out.as<cg_dev::SolveOut>(), s);
	if (rc) {
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		return rc;
	}
	CG_CK(cudaEventRecord(e1, s));
	cg_dev::SolveOut o;
	CG_CK(cudaMemcpyAsync(&o, w.out.p, sizeof o, cudaMemcpyDeviceToHost, s));
	Ctl ctl{};
	// the IC kinds run on the algebra-level workspace: no grid control block
	if (cfg->kind != CARPIO_GPU_IC_CGS && cfg->kind != CARPIO_GPU_IC_CG)
		CG_CK(cudaMemcpyAsync(&ctl, w.lw.ctl.p, sizeof ctl, cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	float ms = 0;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	int code = ctl.err ? ctl.err : o.code;
	if (code >= 0) {
		CG_CK(cudaMemcpy2DAsync(phi, wb, w.phi.p, pb, wb, g->NI, cudaMemcpyDefault, s));
		int keep = std::min(o.hist_len, hist_cap);
		if (keep > 0)
			CG_CK(cudaMemcpyAsync(resid_hist, w.hist.p, sizeof(double) * keep,
					cudaMemcpyDefault, s));
		CG_CK(cudaStreamSynchronize(s));
	}
	if (stats) {
		stats->code = code;
		stats->iters = o.iters;
		stats->tol_out = o.tol;
		stats->outer_iters = o.outer;
		stats->hist_len = o.hist_len;
		stats->ms = ms;
	}
	return code;
}

extern "C" {

int carpio_gpu_poisson_solve(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double beta, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats) {
	return structured_solve(g, bc, false, 0.0, beta, nullptr, source, phi, cfg, resid_hist,
			hist_cap, stats);
}

int carpio_gpu_poisson_solve_beta(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		const double* beta_field, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats) {
	if (!beta_field) return CARPIO_GPU_EINVAL;
	return structured_solve(g, bc, false, 0.0, 1.0, beta_field, source, phi, cfg,
			resid_hist, hist_cap, stats);
}

int carpio_gpu_helmholtz_solve(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double alpha, double beta, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats) {
	return structured_solve(g, bc, true, alpha, beta, nullptr, source, phi, cfg, resid_hist,
			hist_cap, stats);
}

}  // extern "C"
