// Batched Poisson solves with the multigrid-preconditioned CG: one CTA per
// problem, problems taken largest first from a queue by the CTAs of one
// persistent launch (plain launch, no clusters, capturable in a CUDA graph).
//
// Each problem is solved like carpio_gpu_poisson_solve's MIXED path with the
// V-cycle of mg.cuh as the FP32 CG's preconditioner: b from the source with
// the reference's row constants, mean removal of b, FP32 CG with reliable
// updates (the FP64 residual b - A x replaces r whenever (r, z) has dropped
// by inner_tol squared), the stopping test on the FP64 residual with the
// reference's nrm2, mean removal of x. All of a problem's vectors live in
// global memory (its FP64 fields in the batch's arena, FP32 vectors and the
// level hierarchy in a per-problem scratch region); a CTA needs only block
// barriers, so no CTA ever waits on another.
//
// Every level's diagonal comes from the problem's five FP32 constants (the
// interior value and what each side's ghost fold adds): coarsening keeps the
// face coefficients and the folds of a uniform grid, so the same constants
// describe every level.
#include "batch_dev.cuh"
#include "mg.cuh"

namespace cg_batch {

namespace {

using namespace cg_dev;

constexpr int kMgBatchMaxLev = 16;
constexpr int kMgSweeps = 20;   // damped Jacobi sweeps on the coarsest level

struct Lvl {
	int nx, ny;
	float *R, *S, *Zp;
};

// the diagonal of cell (I, J) of a level of nx x ny cells
__device__ __forceinline__ float diag_at(const BatchProb& pr, int I, int J, int nx, int ny) {
	float d = pr.d0;
	d += I == 0 ? pr.dw : 0.f;
	d += I == nx - 1 ? pr.de : 0.f;
	d += J == 0 ? pr.ds : 0.f;
	d += J == ny - 1 ? pr.dn : 0.f;
	return d;
}

// (A z)(I, J) with the level's diagonal
__device__ __forceinline__ float apply32(const BatchProb& pr, const float* z, int I, int J,
		int nx, int ny) {
	const int k = I * ny + J;
	float v = diag_at(pr, I, J, nx, ny) * z[k];
	if (I > 0) v = fmaf(pr.cx, z[k - ny], v);
	if (I < nx - 1) v = fmaf(pr.cx, z[k + ny], v);
	if (J > 0) v = fmaf(pr.cy, z[k - 1], v);
	if (J < ny - 1) v = fmaf(pr.cy, z[k + 1], v);
	return v;
}

// the pre-smoothed correction w D^-1 r at (I, J) (recomputed, never stored)
__device__ __forceinline__ float pre_at(const BatchProb& pr, const float* r, int I, int J,
		int nx, int ny, float w) {
	return w * r[I * ny + J] * __frcp_rn(diag_at(pr, I, J, nx, ny));
}

// corrected value c = w D^-1 r + P zc at (i, j)
__device__ __forceinline__ float corr_at(const BatchProb& pr, const float* r, const float* zc,
		int i, int j, int nx, int ny, float w) {
	const LdSm sl;
	return pre_at(pr, r, i, j, nx, ny, w) + mg_prolong(sl, zc, i, j, nx >> 1, ny >> 1);
}

// z = M r, one V(1,1)-cycle over the levels of lv (level 0's R is r, its
// final correction goes to z); block barriers between the passes
__device__ void vcycle(const BatchProb& pr, const Lvl* lv, int ntot, const float* r,
		float* z, float w) {
	const int T = blockDim.x, tid = threadIdx.x;
	const LdSm sl;
	// down: s = r - A (w D^-1 r), then the next level's r = P^T s
	for (int l = 0; l < ntot - 1; ++l) {
		const Lvl& L = lv[l];
		const float* rl = l == 0 ? r : L.R;
		const int n = L.nx * L.ny;
		mg_pass<4>(tid, T, n, [&](int k) {
			const int I = k / L.ny, J = k - I * L.ny;
			float v = diag_at(pr, I, J, L.nx, L.ny) * pre_at(pr, rl, I, J, L.nx, L.ny, w);
			if (I > 0) v = fmaf(pr.cx, pre_at(pr, rl, I - 1, J, L.nx, L.ny, w), v);
			if (I < L.nx - 1) v = fmaf(pr.cx, pre_at(pr, rl, I + 1, J, L.nx, L.ny, w), v);
			if (J > 0) v = fmaf(pr.cy, pre_at(pr, rl, I, J - 1, L.nx, L.ny, w), v);
			if (J < L.ny - 1) v = fmaf(pr.cy, pre_at(pr, rl, I, J + 1, L.nx, L.ny, w), v);
			return rl[k] - v;
		}, [&](int k, float v) { L.S[k] = v; });
		__syncthreads();
		const Lvl& C = lv[l + 1];
		mg_pass<4>(tid, T, C.nx * C.ny, [&](int k) {
			const int I = k / C.ny, J = k - I * C.ny;
			return mg_restrict(sl, L.S, I, J, L.nx, L.ny);
		}, [&](int k, float v) { C.R[k] = v; });
		__syncthreads();
	}
	// coarsest: damped Jacobi sweeps from zero (exact for one cell)
	{
		const Lvl& L = lv[ntot - 1];
		const int n = L.nx * L.ny;
		const float* rl = ntot == 1 ? r : L.R;
		float* zl = ntot == 1 ? z : L.Zp;
		for (int k = tid; k < n; k += T) {
			const int I = k / L.ny, J = k - I * L.ny;
			const float d = diag_at(pr, I, J, L.nx, L.ny);
			zl[k] = d > 0.f ? (n == 1 ? rl[k] : w * rl[k]) * __frcp_rn(d) : 0.f;
		}
		__syncthreads();
		if (n > 1) {
			for (int sweep = 1; sweep < kMgSweeps; ++sweep) {
				for (int k = tid; k < n; k += T) {
					const int I = k / L.ny, J = k - I * L.ny;
					const float d = diag_at(pr, I, J, L.nx, L.ny);
					L.S[k] = d > 0.f
							? fmaf(w * (rl[k] - apply32(pr, zl, I, J, L.nx, L.ny)), __frcp_rn(d), zl[k])
							: 0.f;
				}
				__syncthreads();
				for (int k = tid; k < n; k += T) zl[k] = L.S[k];
				__syncthreads();
			}
		}
	}
	// up: z_l = c + w D^-1 (r - A c), c = w D^-1 r + P z_{l+1}
	for (int l = ntot - 2; l >= 0; --l) {
		const Lvl& L = lv[l];
		const float* rl = l == 0 ? r : L.R;
		float* zl = l == 0 ? z : L.Zp;
		const float* zc = lv[l + 1].Zp;
		mg_pass<2>(tid, T, L.nx * L.ny, [&](int k) {
			const int I = k / L.ny, J = k - I * L.ny;
			const float c = corr_at(pr, rl, zc, I, J, L.nx, L.ny, w);
			float ac = diag_at(pr, I, J, L.nx, L.ny) * c;
			if (I > 0) ac = fmaf(pr.cx, corr_at(pr, rl, zc, I - 1, J, L.nx, L.ny, w), ac);
			if (I < L.nx - 1) ac = fmaf(pr.cx, corr_at(pr, rl, zc, I + 1, J, L.nx, L.ny, w), ac);
			if (J > 0) ac = fmaf(pr.cy, corr_at(pr, rl, zc, I, J - 1, L.nx, L.ny, w), ac);
			if (J < L.ny - 1) ac = fmaf(pr.cy, corr_at(pr, rl, zc, I, J + 1, L.nx, L.ny, w), ac);
			return fmaf(w * (rl[k] - ac), __frcp_rn(diag_at(pr, I, J, L.nx, L.ny)), c);
		}, [&](int k, float v) { zl[k] = v; });
		__syncthreads();
	}
}

// block sums with a plain fixed-order tree (every thread gets the sums)
template<class R, int NV>
__device__ __forceinline__ void bsum(R (&v)[NV]) { block_sum<R, NV>(v); }

// One problem on this CTA. Returns false when the launch must stop (error
// word set or deadline passed).
__device__ bool solve_one(const BatchArgs& a, const BatchProb& pr, int pi, float* w32,
		const Watch& wt) {
	__shared__ int s_stop;
	const int T = blockDim.x, tid = threadIdx.x;
	const int nx = pr.nx, ny = pr.ny, P = ny + 2, n = nx * ny;
	const long long off = pr.cell;
	double* x64 = a.phi + off;
	double* b64 = a.b + off;
	double* r64 = a.r + off;
	const double* D = a.D + off;
	const double* ax = a.ax + pr.axo;
	const double* ay = a.ay + pr.ayo;
	const double nall = (double)n;
	const unsigned long long t_start = globaltimer();
	auto gaddr = [&](int k) { const int i = k / ny; return (i + 1) * P + (k - i * ny) + 1; };
	auto counted = [&](int k) { return pr.full || k != n - 1; };
	// FP32 vectors and the level hierarchy
	float* xe = w32;
	float* r = xe + n;
	float* p = r + n;
	float* q = p + n;
	float* z = q + n;
	Lvl lv[kMgBatchMaxLev];
	int ntot = 0;
	{
		float* h = z + n;
		int lx = nx, ly = ny;
		for (;;) {
			Lvl& L = lv[ntot++];
			L.nx = lx;
			L.ny = ly;
			L.R = h;
			L.S = h + (size_t)lx * ly;
			L.Zp = h + 2 * (size_t)lx * ly;
			h += 3 * (size_t)lx * ly;
			if ((lx & 1) || (ly & 1) || ntot == kMgBatchMaxLev) break;
			lx >>= 1;
			ly >>= 1;
		}
	}
	const float w = 0.8f;

	// b with the reference's row constants, its mean removed, its norm
	GridSpace sp{ nx, ny, 1, P };
	RhsArgs ra;
	ra.sx = a.sx + pr.sxo;
	ra.sy = a.sy + pr.syo;
	ra.fold = a.fold + pr.foldo;
	ra.src_a = a.src + off;
	ra.src_b = nullptr;
	ra.phi = x64;
	ra.mean = pr.mean;
	double s1[1] = { 0.0 };
	for (int k = tid; k < n; k += T) {
		const int i = k / ny, j = k - i * ny, ad = gaddr(k);
		const double bb = rhs_at<cg_host::SRC_FIELD>(sp, ra, i, j, ad);
		b64[ad] = bb;
		s1[0] += bb;
	}
	bsum<double, 1>(s1);
	if (pr.mean) {
		const double mb = s1[0] / nall;
		for (int k = tid; k < n; k += T) { const int ad = gaddr(k); b64[ad] = b64[ad] - mb; }
		__syncthreads();
	}
	double nb[1] = { 0.0 };
	for (int k = tid; k < n; k += T) {
		const double bb = b64[gaddr(k)];
		if (counted(k)) nb[0] = fma(bb, bb, nb[0]);
	}
	bsum<double, 1>(nb);
	double normb = sqrt(nb[0]);
	if (normb == 0.0) normb = 1.0;
	for (int k = tid; k < n; k += T) { xe[k] = 0.f; p[k] = 0.f; }
	__syncthreads();

	double scale0 = 1.0, rn0 = 1.0, resid = 0.0;
	// FP64 residual into r (FP32, mean removed, scaled by the first
	// residual's norm), then z = M r; returns (r, z) and (r, r)
	auto true_residual = [&](bool first, float& gz, float& gr) {
		double sums[3] = { 0.0, 0.0, 0.0 };
		for (int k = tid; k < n; k += T) {
			const int i = k / ny, j = k - i * ny, ad = gaddr(k);
			const double rv = b64[ad] - apply64(D, ax, ay, x64, P, i, j, ad);
			r64[ad] = rv;
			if (counted(k)) sums[0] = fma(rv, rv, sums[0]);
			sums[1] += rv;
			sums[2] = fma(rv, rv, sums[2]);
		}
		bsum<double, 3>(sums);
		resid = sqrt(sums[0]) / normb;
		const double mr = pr.mean ? sums[1] / nall : 0.0;
		if (first) {
			rn0 = sqrt(pr.mean ? fmax(sums[2] - sums[1] * mr, 0.0) : sums[2]);
			scale0 = rn0 > 0.0 ? 1.0 / rn0 : 1.0;
		}
		for (int k = tid; k < n; k += T) r[k] = (float)((r64[gaddr(k)] - mr) * scale0);
		__syncthreads();
		vcycle(pr, lv, ntot, r, z, w);
		float g[2] = { 0.f, 0.f };
		for (int k = tid; k < n; k += T) {
			g[0] = fmaf(r[k], z[k], g[0]);
			g[1] = fmaf(r[k], r[k], g[1]);
		}
		bsum<float, 2>(g);
		gz = g[0];
		gr = g[1];
	};
	auto fold_x = [&]() {
		for (int k = tid; k < n; k += T) {
			const int ad = gaddr(k);
			x64[ad] = fma(rn0, (double)xe[k], x64[ad]);
			xe[k] = 0.f;
		}
		__syncthreads();
	};

	float gamma = 0.f, rrn = 0.f;
	true_residual(true, gamma, rrn);
	bool done = resid <= pr.tol;
	int it = 0, updates = 0, since = 0;
	const double it_tol = fmax(a.inner_tol, 1e-2);
	const float drop = (float)(it_tol * it_tol);
	const double tol_scaled = pr.tol * normb * scale0;
	const float near = (float)(0.25 * tol_scaled * tol_scaled);
	float gamma_ref = gamma, gamma_old = 1.f;
	bool first = true;
	bool stop = false;
	while (!done && it < pr.max_iter && gamma > 0.f) {
		const float beta = first ? 0.f : gamma / gamma_old;
		first = false;
		for (int k = tid; k < n; k += T) p[k] = fmaf(beta, p[k], z[k]);
		__syncthreads();
		float pq[1] = { 0.f };
		mg_pass<4>(tid, T, n, [&](int k) {
			const int I = k / ny, J = k - I * ny;
			return apply32(pr, p, I, J, nx, ny);
		}, [&](int k, float v) { q[k] = v; pq[0] = fmaf(p[k], v, pq[0]); });
		bsum<float, 1>(pq);
		const float alpha = gamma / pq[0];
		for (int k = tid; k < n; k += T) {
			xe[k] = fmaf(alpha, p[k], xe[k]);
			r[k] = fmaf(-alpha, q[k], r[k]);
		}
		__syncthreads();
		vcycle(pr, lv, ntot, r, z, w);
		float g[2] = { 0.f, 0.f };
		for (int k = tid; k < n; k += T) {
			g[0] = fmaf(r[k], z[k], g[0]);
			g[1] = fmaf(r[k], r[k], g[1]);
		}
		bsum<float, 2>(g);
		++it;
		++since;
		float gnew = g[0];
		rrn = g[1];
		if (gnew < drop * gamma_ref || rrn <= near || since >= kStallIters) {
			since = 0;
			fold_x();
			true_residual(false, gnew, rrn);
			++updates;
			if (resid <= pr.tol) { done = true; break; }
			gamma_ref = gnew;
		}
		gamma_old = gamma;
		gamma = gnew;
		// the launch's error word and deadline, every 32 iterations
		if ((it & 31) == 0) {
			if (tid == 0) {
				int st = *(volatile int*)wt.err != 0 ? 1 : 0;
				if (!st && globaltimer() > wt.deadline) {
					watch_fail(wt, CARPIO_GPU_ETIMEOUT);
					st = 1;
				}
				s_stop = st;
			}
			__syncthreads();
			if (s_stop) { stop = true; break; }
		}
	}
	if (stop) return false;
	if (!done) fold_x();
	if (pr.mean) {
		double sx1[1] = { 0.0 };
		for (int k = tid; k < n; k += T) sx1[0] += x64[gaddr(k)];
		bsum<double, 1>(sx1);
		const double mx = sx1[0] / nall;
		for (int k = tid; k < n; k += T) { const int ad = gaddr(k); x64[ad] = x64[ad] - mx; }
	}
	if (tid == 0) {
		BatchRes o;
		o.code = done ? 0 : 1;
		o.iters = it;
		o.updates = updates;
		o.ran = 1;
		o.resid = resid;
		o.ms = (double)(globaltimer() - t_start) * 1e-6;
		a.res[pi] = o;
	}
	__syncthreads();
	return true;
}

template<int T>
__global__ void __launch_bounds__(T) k_batch_mg(BatchArgs a) {
	__shared__ int s_pi;
	const Watch w{ &a.ctl->err, a.ctl->wait_ns, globaltimer() + a.ctl->solve_ns };
	for (;;) {
		if (threadIdx.x == 0) {
			int pi = -1;
			if (*(volatile int*)&a.ctl->err == 0) {
				const unsigned qn = atomicAdd(a.queue, 1u);
				if (qn < (unsigned)a.count) pi = a.order[qn];
			}
			s_pi = pi;
		}
		__syncthreads();
		const int pi = s_pi;
		__syncthreads();
		if (pi < 0) break;
		const BatchProb pr = a.prob[pi];
		if (!solve_one(a, pr, pi, a.w32 + a.w32off[pi], w)) break;
	}
}

}  // namespace

const void* kernel_mg(int T) {
	if (T == 256) return (const void*)k_batch_mg<256>;
	if (T == 512) return (const void*)k_batch_mg<512>;
	if (T == 1024) return (const void*)k_batch_mg<1024>;
	return nullptr;
}

// FP32 scratch of one problem in floats: five vectors and three per level
long long mg_scratch_floats(int nx, int ny) {
	long long f = 5LL * nx * ny;
	int lx = nx, ly = ny, nl = 0;
	for (;;) {
		f += 3LL * lx * ly;
		++nl;
		if ((lx & 1) || (ly & 1) || nl == kMgBatchMaxLev) break;
		lx >>= 1;
		ly >>= 1;
	}
	return (f + 63) / 64 * 64;
}

}  // namespace cg_batch
