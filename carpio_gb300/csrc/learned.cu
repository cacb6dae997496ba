// Poisson solves preconditioned by the learned U-Net: flexible conjugate
// gradients (FCG(m), Notay 2000) in FP64 whose preconditioner is the network
// followed by damped Jacobi sweeps,
//
//   M(r) = S^nu( s * net(r / s) ),   s = rms(r),
//   S(z) = z + omega D^-1 (r - A z)  (mean removed for all-Neumann systems),
//
// with the network applied in BF16/FP32 on the tensor cores. The first
// direction is the network's answer to the initial residual, i.e. the network
// is also the warm start (the first step takes its optimal multiple). Every
// FCG direction is A-orthogonalised against the m previous ones, so the
// iteration tolerates a preconditioner that is not a fixed linear map. When
// the recursively updated residual reaches the tolerance the true residual
// b - A x is formed in FP64 and is the judge; if it has not dropped by 10 %
// over `stall` iterations (or a direction fails), the solve finishes with the
// plain MIXED CG from the current iterate.
//
// Reductions go to per-block partials that the host adds in block order, so
// results do not depend on scheduling.
#include "internal.hpp"
#include "poisson_rhs.cuh"

#include <cmath>
#include <vector>


namespace {

using namespace cg_dev;
constexpr int kLT = 256;

#define LLOOP(n) for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < (n); k += gridDim.x * blockDim.x)

// Device scalars of the iteration (doubles): [0, 8) reductions, 8 alpha,
// 9 failure flag, [16, 24) (p, q) of the ring slots, [24, 28) beta.
enum { S_RED = 0, S_ALPHA = 8, S_FAIL = 9, S_PQ = 16, S_BETA = 24 };

template<int NV>
__device__ __forceinline__ void block_partials(double (&v)[NV], double* part) {
	__shared__ double s[NV][kLT / 32];
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		double x = v[m];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		if ((threadIdx.x & 31) == 0) s[m][threadIdx.x >> 5] = x;
	}
	__syncthreads();
	if (threadIdx.x < NV) {
		double x = 0;
		for (int w = 0; w < kLT / 32; ++w) x += s[threadIdx.x][w];
		part[(size_t)blockIdx.x * NV + threadIdx.x] = x;
	}
}

template<int SRC>
__global__ void __launch_bounds__(kLT) k_rhs(GridSpace sp, RhsArgs ra, double* b, double* x,
		double* part) {
	double v[1] = { 0 };
	LLOOP(sp.count()) {
		int i, j;
		sp.ij(k, i, j);
		const int a = sp.addr(k);
		const double bb = rhs_at<SRC>(sp, ra, i, j, a);
		b[a] = bb;
		x[a] = ra.phi[a];
		v[0] += bb;
	}
	block_partials<1>(v, part);
}

__global__ void __launch_bounds__(kLT) k_shift(GridSpace sp, double* f, double m) {
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		f[a] -= m;
	}
}

// r = b - A x; partials: nrm2 quirk sum, full sum of squares, sum
__global__ void __launch_bounds__(kLT) k_resid(StencilOp<double> op, const double* b,
		const double* x, double* r, int full, double* part) {
	const GridSpace& sp = op.sp;
	const int la = sp.last_addr();
	double v[3] = { 0, 0, 0 };
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		const double rv = b[a] - op.apply(x, k, a);
		r[a] = rv;
		if (a != la || full) v[0] = fma(rv, rv, v[0]);
		v[1] = fma(rv, rv, v[1]);
		v[2] += rv;
	}
	block_partials<3>(v, part);
}

// q = A p; partials: (p, q), (p, r)
__global__ void __launch_bounds__(kLT) k_apply_dots(StencilOp<double> op, const double* p,
		const double* r, double* q, double* part) {
	const GridSpace& sp = op.sp;
	double v[2] = { 0, 0 };
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		const double qv = op.apply(p, k, a);
		q[a] = qv;
		v[0] = fma(p[a], qv, v[0]);
		v[1] = fma(p[a], r[a], v[1]);
	}
	block_partials<2>(v, part);
}

// x += alpha p, r -= alpha q (alpha from the device scalars); partials of
// the new residual: nrm2 quirk, full squares, sum
__global__ void __launch_bounds__(kLT) k_step(GridSpace sp, const double* sc, const double* p,
		const double* q, double* x, double* r, int full, double* part) {
	const double alpha = sc[S_ALPHA];
	const int la = sp.last_addr();
	double v[3] = { 0, 0, 0 };
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		x[a] = fma(alpha, p[a], x[a]);
		const double rv = fma(-alpha, q[a], r[a]);
		r[a] = rv;
		if (a != la || full) v[0] = fma(rv, rv, v[0]);
		v[1] = fma(rv, rv, v[1]);
		v[2] += rv;
	}
	block_partials<3>(v, part);
}

// network input: r / s as a dense [nx][ny] FP32 field
__global__ void __launch_bounds__(kLT) k_pack(GridSpace sp, const double* r, double inv_s,
		float* out) {
	LLOOP(sp.count()) out[k] = (float)(r[sp.addr(k)] * inv_s);
}

// z = s * network output; partial: sum z
__global__ void __launch_bounds__(kLT) k_unpack(GridSpace sp, const float* in, double s,
		double* z, double* part) {
	double v[1] = { 0 };
	LLOOP(sp.count()) {
		const double zv = s * (double)in[k];
		z[sp.addr(k)] = zv;
		v[0] += zv;
	}
	block_partials<1>(v, part);
}

// one damped Jacobi sweep zo = z + omega (r - A z) / D (minus the mean m of
// z); partial: sum zo
__global__ void __launch_bounds__(kLT) k_jacobi(StencilOp<double> op, const double* r,
		const double* z, double zmean, double omega, double* zo, double* part) {
	const GridSpace& sp = op.sp;
	double v[1] = { 0 };
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		const double az = op.apply(z, k, a);   // A (z - m) = A z for the Neumann system
		const double zv = (z[a] - zmean) + omega * (r[a] - az) / op.D[a];
		zo[a] = zv;
		v[0] += zv;
	}
	block_partials<1>(v, part);
}

// the FCG ring of previous directions, by value
struct Ring {
	const double* p[4];
	const double* q[4];
	int slot[4];   // their slots in the (p, q) curvature ring
	int n;
};

// partials of (z, q_j) for the ring's directions
template<int NJ>
__global__ void __launch_bounds__(kLT) k_dots_zq(GridSpace sp, const double* z, Ring rg,
		double* part) {
	double v[NJ];
#pragma unroll
	for (int j = 0; j < NJ; ++j) v[j] = 0;
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		const double zv = z[a];
#pragma unroll
		for (int j = 0; j < NJ; ++j) v[j] = fma(zv, rg.q[j][a], v[j]);
	}
	block_partials<NJ>(v, part);
}

// sums of NV per-block partials in block order (one thread per value)
template<int NV>
__global__ void k_reduce(const double* part, int nb, double* sc) {
	const int m = threadIdx.x;
	if (m >= NV) return;
	double x = 0;
	for (int b = 0; b < nb; ++b) x += part[(size_t)b * NV + m];
	sc[S_RED + m] = x;
}

// beta_j = (z, q_j) / (p_j, q_j)
__global__ void k_beta(double* sc, Ring rg) {
	const int j = threadIdx.x;
	if (j < rg.n) sc[S_BETA + j] = sc[S_RED + j] / sc[S_PQ + rg.slot[j]];
}

// p = z - sum_j beta_j p_j
__global__ void __launch_bounds__(kLT) k_combine(GridSpace sp, const double* z, Ring rg,
		const double* sc, double* p) {
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		double pv = z[a];
		for (int j = 0; j < rg.n; ++j) pv = fma(-sc[S_BETA + j], rg.p[j][a], pv);
		p[a] = pv;
	}
}

// alpha = (p, r) / (p, q); (p, q) kept for the ring; a failed direction
// (no positive curvature) sets the flag and alpha 0
__global__ void k_alpha(double* sc, int slot) {
	const double ppq = sc[S_RED], ppr = sc[S_RED + 1];
	const bool ok = ppq > 0 && isfinite(ppr) && isfinite(ppq);
	sc[S_ALPHA] = ok ? ppr / ppq : 0.0;
	sc[S_FAIL] = ok ? 0.0 : 1.0;
	sc[S_PQ + slot] = ok ? ppq : 1.0;
}

__global__ void __launch_bounds__(kLT) k_sum(GridSpace sp, const double* f, double* part) {
	double v[1] = { 0 };
	LLOOP(sp.count()) v[0] += f[sp.addr(k)];
	block_partials<1>(v, part);
}

// phi's normal cells = x - m
__global__ void __launch_bounds__(kLT) k_store(GridSpace sp, const double* x, double m,
		double* phi) {
	LLOOP(sp.count()) {
		const int a = sp.addr(k);
		phi[a] = x[a] - m;
	}
}

}  // namespace

namespace cg_host {

namespace {

using cg_dev::SolveOut;

struct Sums {
	LearnedWs& w;
	cudaStream_t s;
	// add the per-block partials of NV values in block order
	int read(int nv, double* out) {
		const size_t n = (size_t)w.nblk * nv;
		if (w.hpart.size() < n) w.hpart.resize(n);
		CG_CK(cudaMemcpyAsync(w.hpart.data(), w.part.p, sizeof(double) * n,
				cudaMemcpyDeviceToHost, s));
		CG_CK(cudaStreamSynchronize(s));
		for (int m = 0; m < nv; ++m) out[m] = 0;
		for (int b = 0; b < w.nblk; ++b)
			for (int m = 0; m < nv; ++m) out[m] += w.hpart[(size_t)b * nv + m];
		return 0;
	}
};

}  // namespace

bool learned_shape_ok(int nx, int ny) {
	// the network's tiles: multiples of 8, at least 16 cells, whole 128-pixel
	// tiles of rows at the coarsest level
	if (nx < 16 || ny < 16 || nx % 8 || ny % 8) return false;
	const int h3 = nx / 8, w3 = ny / 8;
	const int bw = std::min(w3, 128), bh = std::min(h3, 128 / bw);
	return bw * bh == 128 && w3 % bw == 0 && h3 % bh == 0;
}

int learned_solve(carpio_gpu_grid* g, StencilCoeffs& c, PoissonWs& pws, LearnedWs& w,
		int src_mode, const double* src_a, const double* src_b, double* phi,
		const carpio_gpu_solver_cfg& cfg, carpio_gpu_unet* net,
		const carpio_gpu_learned_cfg& lc, SolveOut& out, cudaStream_t s,
		std::vector<double>* hist_out) {
	const int nx = g->nx, ny = g->ny;
	const size_t NF = (size_t)g->NI * g->P;
	const long n = (long)nx * ny;
	const int m = std::max(1, std::min(4, lc.memory));
	const int nfield = 6 + 2 * (m + 1);   // x b r z zt t, p/q ring
	int rc;
	if (w.f64.bytes < sizeof(double) * NF * nfield) {
		if ((rc = w.f64.ensure(sizeof(double) * NF * nfield))) return rc;
		CG_CK(cudaMemsetAsync(w.f64.p, 0, w.f64.bytes, s));   // zero ghost rings
	}
	if ((rc = w.f32.ensure(sizeof(float) * 2 * (size_t)n))) return rc;
	w.nblk = 2 * sm_count();
	if ((rc = w.part.ensure(sizeof(double) * 4 * (size_t)w.nblk))) return rc;

	double* F = w.f64.as<double>();
	double *x = F, *b = F + NF, *r = F + 2 * NF, *z = F + 3 * NF, *zt = F + 4 * NF;
	double* P[5];
	double* Q[5];
	for (int j = 0; j <= m; ++j) {
		P[j] = F + (6 + 2 * j) * NF;
		Q[j] = F + (7 + 2 * j) * NF;
	}
	float* x32 = w.f32.as<float>();
	float* z32 = x32 + n;
	double* part = w.part.as<double>();
	const int nb = w.nblk;
	Sums sums{ w, s };
	StencilOp<double> op;
	op.sp = GridSpace{ nx, ny, g->gl, g->P };
	op.D = c.D.as<double>();
	op.ax = c.ax.as<double>();
	op.ay = c.ay.as<double>();
	// the network was trained on uniform grids and the kernels here apply
	// the uniform operator
	if (!c.uniform) return CARPIO_GPU_EINVAL;
	const GridSpace sp = op.sp;
	const bool mean = cfg.mean_removal != 0;
	const int full = (cfg.flags & CARPIO_GPU_FLAG_FULL_NRM2) || n == 1 ? 1 : 0;
	const bool use_net = lc.use_net && net && learned_shape_ok(nx, ny);
	double v[4];

	// b, x0, mean removal of b, ||b||
	RhsArgs ra;
	ra.sx = g->d_sx;
	ra.sy = g->d_sy;
	ra.fold = c.fold.as<double>();
	ra.src_a = src_a;
	ra.src_b = src_b;
	rhs_set_p2(ra, g->sx, g->sy);
	ra.phi = phi;
	ra.mean = mean ? 1 : 0;
	if (src_mode == SRC_DIV) k_rhs<SRC_DIV><<<nb, kLT, 0, s>>>(sp, ra, b, x, part);
	else k_rhs<SRC_FIELD><<<nb, kLT, 0, s>>>(sp, ra, b, x, part);
	CG_CK(cudaGetLastError());
	if ((rc = sums.read(1, v))) return rc;
	if (mean) k_shift<<<nb, kLT, 0, s>>>(sp, b, v[0] / (double)n);
	// ||b|| with the reference's nrm2 (b - A 0)
	CG_CK(cudaMemsetAsync(zt, 0, sizeof(double) * NF, s));
	k_resid<<<nb, kLT, 0, s>>>(op, b, zt, r, full, part);
	if ((rc = sums.read(3, v))) return rc;
	double normb = std::sqrt(v[0]);
	if (normb == 0.0) normb = 1.0;
	k_resid<<<nb, kLT, 0, s>>>(op, b, x, r, full, part);
	if ((rc = sums.read(3, v))) return rc;
	double resid = std::sqrt(v[0]) / normb, rr = v[1];
	std::vector<double> hist{ resid };
	const int stall = lc.stall > 0 ? lc.stall : 20;
	const double omega = lc.omega > 0 ? lc.omega : 0.8;
	const int nu = std::max(0, lc.smooth);
	int nring = 0, head = 0, it = 0, fallback_iters = 0, code = 1;
	bool done = resid <= cfg.tol, stalled = false;
	double best = resid;
	int best_it = 0;
	if ((rc = w.sc.ensure(sizeof(double) * 32))) return rc;
	double* sc = w.sc.as<double>();
	CG_CK(cudaMemsetAsync(sc, 0, sizeof(double) * 32, s));
	std::vector<int> slot_of(m + 1, 0);
	while (!done && it < cfg.max_iter) {
		// z = M(r). A constant added to z changes neither A z nor, for the
		// consistent all-Neumann system, any inner product the iteration
		// uses, so the mean is removed from x once at the end. The network
		// is positively homogeneous, so the scale s only keeps its input in
		// range.
		if (use_net) {
			const double scl = std::sqrt(rr / (double)n);
			if (!(scl > 0)) break;
			k_pack<<<nb, kLT, 0, s>>>(sp, r, 1.0 / scl, x32);
			CG_CK(cudaGetLastError());
			if ((rc = unet_forward_async(net, 1, nx, ny, x32, z32, s))) return rc;
			k_unpack<<<nb, kLT, 0, s>>>(sp, z32, scl, z, part);
		} else {
			CG_CK(cudaMemsetAsync(z, 0, sizeof(double) * NF, s));
		}
		for (int k = 0; k < nu; ++k) {
			k_jacobi<<<nb, kLT, 0, s>>>(op, r, z, 0.0, omega, zt, part);
			std::swap(z, zt);
		}
		// p = z - sum_j (z, q_j) / (p_j, q_j) p_j over the ring (scalars stay
		// on the device)
		double* pnew = P[head];
		double* qnew = Q[head];
		Ring rg;
		rg.n = nring;
		for (int j = 0; j < 4; ++j) {
			const int id = j < nring ? (head + m + 1 - nring + j) % (m + 1) : head;
			rg.p[j] = P[id];
			rg.q[j] = Q[id];
			rg.slot[j] = id;
		}
		if (nring > 0) {
			switch (nring) {
			case 1: k_dots_zq<1><<<nb, kLT, 0, s>>>(sp, z, rg, part); k_reduce<1><<<1, 32, 0, s>>>(part, nb, sc); break;
			case 2: k_dots_zq<2><<<nb, kLT, 0, s>>>(sp, z, rg, part); k_reduce<2><<<1, 32, 0, s>>>(part, nb, sc); break;
			case 3: k_dots_zq<3><<<nb, kLT, 0, s>>>(sp, z, rg, part); k_reduce<3><<<1, 32, 0, s>>>(part, nb, sc); break;
			default: k_dots_zq<4><<<nb, kLT, 0, s>>>(sp, z, rg, part); k_reduce<4><<<1, 32, 0, s>>>(part, nb, sc); break;
			}
			k_beta<<<1, 32, 0, s>>>(sc, rg);
			k_combine<<<nb, kLT, 0, s>>>(sp, z, rg, sc, pnew);
		} else {
			CG_CK(cudaMemcpyAsync(pnew, z, sizeof(double) * NF, cudaMemcpyDeviceToDevice, s));
		}
		k_apply_dots<<<nb, kLT, 0, s>>>(op, pnew, r, qnew, part);
		k_reduce<2><<<1, 32, 0, s>>>(part, nb, sc);
		k_alpha<<<1, 1, 0, s>>>(sc, head);
		k_step<<<nb, kLT, 0, s>>>(sp, sc, pnew, qnew, x, r, full, part);
		k_reduce<3><<<1, 32, 0, s>>>(part, nb, sc);
		CG_CK(cudaGetLastError());
		// one host read per iteration: the new residual, the failure flag
		// and the network's device-side error flag
		double hs[10];
		int nerr = 0;
		CG_CK(cudaMemcpyAsync(hs, sc, sizeof(double) * 10, cudaMemcpyDeviceToHost, s));
		if (use_net)
			CG_CK(cudaMemcpyAsync(&nerr, unet_err_flag(net), sizeof(int),
					cudaMemcpyDeviceToHost, s));
		CG_CK(cudaStreamSynchronize(s));
		if (nerr) return unet_take_err(net);
		if (hs[S_FAIL] != 0.0) { stalled = true; break; }
		rr = hs[S_RED + 1];
		head = (head + 1) % (m + 1);
		nring = std::min(nring + 1, m);
		++it;
		double rec = std::sqrt(hs[S_RED]) / normb;
		if (rec <= cfg.tol) {
			// the true residual judges; a miss restarts from it
			k_resid<<<nb, kLT, 0, s>>>(op, b, x, r, full, part);
			if ((rc = sums.read(3, v))) return rc;
			rec = std::sqrt(v[0]) / normb;
			rr = v[1];
			nring = 0;
			if (rec <= cfg.tol) done = true;
		}
		resid = rec;
		hist.push_back(rec);
		// stalled: no new low (by 1 %) for `stall` iterations
		if (rec < 0.99 * best) {
			best = rec;
			best_it = it;
		} else if (!done && it - best_it >= stall) {
			stalled = true;
			break;
		}
	}
	if (hist_out) *hist_out = hist;
	if (done) code = 0;
	if (!done) {
		k_resid<<<nb, kLT, 0, s>>>(op, b, x, r, full, part);
		if ((rc = sums.read(3, v))) return rc;
		resid = std::sqrt(v[0]) / normb;
	}
	// x -> phi's normal cells (mean removed for the all-Neumann system)
	double xm = 0;
	if (mean) {
		k_sum<<<nb, kLT, 0, s>>>(sp, x, part);
		if ((rc = sums.read(1, v))) return rc;
		xm = v[0] / (double)n;
	}
	k_store<<<nb, kLT, 0, s>>>(sp, x, xm, phi);
	CG_CK(cudaGetLastError());
	out.code = code;
	out.iters = it;
	out.tol = resid;
	out.hist_len = (int)hist.size();
	out.outer = it;
	out.inner = 0;
	if (!done && stalled && lc.fallback) {
		// the plain MIXED CG from the current iterate
		carpio_gpu_solver_cfg fc = cfg;
		fc.kind = CARPIO_GPU_CG;
		fc.precision = CARPIO_GPU_MIXED;
		fc.max_iter = std::max(0, cfg.max_iter - it);
		if ((rc = pws.out.ensure(sizeof(SolveOut)))) return rc;
		if ((rc = poisson_launch(g, c, pws, src_mode, src_a, src_b, phi, fc, nullptr, 0,
				pws.out.as<SolveOut>(), s)))
			return rc;
		SolveOut fo;
		Ctl ctl;
		CG_CK(cudaMemcpyAsync(&fo, pws.out.p, sizeof fo, cudaMemcpyDeviceToHost, s));
		CG_CK(cudaMemcpyAsync(&ctl, pws.lw.ctl.p, sizeof ctl, cudaMemcpyDeviceToHost, s));
		CG_CK(cudaStreamSynchronize(s));
		if (ctl.err) return ctl.err;
		out.code = fo.code;
		out.iters = it + fo.iters;
		out.tol = fo.tol;
		out.hist_len = (int)hist.size() + fo.hist_len;
		out.inner = fo.iters;
	}
	return 0;
}

}  // namespace cg_host

extern "C" int carpio_gpu_poisson_solve_learned(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double beta, const double* source, double* phi, const carpio_gpu_solver_cfg* cfg,
		carpio_gpu_unet* net, const carpio_gpu_learned_cfg* lc, double* resid_hist,
		int hist_cap, carpio_gpu_solver_stats* stats) {
	using namespace cg_host;
	if (!g || !bc || !source || !phi || !cfg || !lc || cfg->max_iter < 0 || hist_cap < 0
			|| (hist_cap > 0 && !resid_hist)
			|| cfg->kind != CARPIO_GPU_CG || !(beta == beta) || (lc->use_net && !net)
			|| (lc->use_net && !learned_shape_ok(g->nx, g->ny)))
		return CARPIO_GPU_EINVAL;
	for (int k = 0; k < 4; ++k)
		if (bc->type[k] != 1 && bc->type[k] != 2) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(g->mu);
	cudaStream_t s = g->stream;
	int rc;
	if ((rc = stencil_prepare(g, *bc, beta, g->coeffs, s))) return rc;
	PoissonWs& w = g->pws;
	const size_t NF = (size_t)g->NI * g->P;
	if ((rc = w.src.ensure(sizeof(double) * NF))) return rc;
	if ((rc = w.phi.ensure(sizeof(double) * NF))) return rc;
	const size_t wb = sizeof(double) * g->NJ, pb = sizeof(double) * g->P;
	CG_CK(cudaMemcpy2DAsync(w.src.p, pb, source, wb, wb, g->NI, cudaMemcpyDefault, s));
	CG_CK(cudaMemcpy2DAsync(w.phi.p, pb, phi, wb, wb, g->NI, cudaMemcpyDefault, s));
	cudaEvent_t e0, e1;
	CG_CK(cudaEventCreate(&e0));
	CG_CK(cudaEventCreate(&e1));
	CG_CK(cudaEventRecord(e0, s));
	cg_dev::SolveOut o;
	std::vector<double> hist;
	rc = learned_solve(g, g->coeffs, w, g->lws, SRC_FIELD, w.src.as<double>(), nullptr,
			w.phi.as<double>(), *cfg, net, *lc, o, s, &hist);
	for (int k = 0; k < hist_cap && k < (int)hist.size(); ++k) resid_hist[k] = hist[k];
	cudaEventRecord(e1, s);
	cudaStreamSynchronize(s);
	float ms = 0;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (rc) return rc;
	CG_CK(cudaMemcpy2DAsync(phi, wb, w.phi.p, pb, wb, g->NI, cudaMemcpyDefault, s));
	CG_CK(cudaStreamSynchronize(s));
	if (stats) {
		stats->code = o.code;
		stats->iters = o.iters;
		stats->tol_out = o.tol;
		stats->outer_iters = o.outer;
		stats->hist_len = o.hist_len;
		stats->ms = ms;
	}
	return o.code;
}
