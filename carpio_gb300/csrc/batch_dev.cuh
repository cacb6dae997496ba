// Device side of the batched structure-level Poisson solves: many independent Poisson_::run()
// problems (s_poisson.hpp:320-420) of uneven sizes in one persistent launch
// of thread-block clusters, captured once into a CUDA graph and replayed.
//
// Each problem is solved like carpio_gpu_poisson_solve's on-chip MIXED CG
// (poisson.cu): b from the source with the reference's row constants, mean
// removal of b, FP32 CG with reliable updates (the FP64 residual b - A x
// replaces r whenever the FP32 residual has dropped by inner_tol), the
// stopping test on the FP64 residual with the reference's nrm2, mean removal
// of x.
//
// A problem is owned by a team of t = 1, 2, 4, 8 or 16 CTAs of one cluster,
// each CTA a band of x-rows. The band's FP32 state is on chip: p (with one
// halo row above and below, and a zero pad column) and the FP32 iterate in
// shared memory, r and q in registers; the FP32 diagonal is formed from five
// per-problem constants (uniform grids fold the same ghost terms into every
// cell of a side). Team reductions and
// the two halo rows cross CTAs through distributed shared memory
// (cluster.cuh); FP64 fields stay in global memory and are touched only at
// reliable updates. The host planner gives every cluster one team size, cuts
// it into 16 / t slots and spreads the problems over the slots largest first
// (LPT); the autotuner times launch configurations on the caller's data.
#pragma once

#include "internal.hpp"
#include "poisson_rhs.cuh"
#include "cluster.cuh"

namespace cg_batch {

using namespace cg_dev;

constexpr int kCellsPerCta = 16384;   // on-chip capacity of one CTA
constexpr int kStallIters = 1000;     // reliable update at least this often
constexpr int kMaxQ = 8;             // quads (4 cells) per thread at most

struct BatchProb {
	int nx, ny, team, kc;   // kc: quads per thread the kernel is instantiated for
	int mean, full, max_iter, pad;
	long long cell;         // offset of the problem's fields in the field arenas
	long long axo, ayo, sxo, syo, foldo;
	double tol;
	float cx, cy;           // FP32 interior face coefficients
	float d0;               // FP32 diagonal of an interior cell
	float dw, de, ds, dn;   // what the ghost folds of segments x-, x+, y-, y+
	                        // add to the diagonal of the cells along them
	float pad2;
};

struct BatchRes {           // per problem, written by the team's member 0
	int code, iters, updates, ran;
	double resid;
	double ms;
};

// Limits and error word of one launch; the host writes the limits before
// every launch (also before a graph replay), so a captured graph follows the
// current watchdog.
struct BatchCtl {
	int err;
	int pad;
	unsigned long long wait_ns, solve_ns;
};

struct BatchArgs {
	BatchCtl* ctl;
	const BatchProb* prob;
	const int* cl_team;     // team size of each cluster
	const int* slot_ptr;    // [clusters * kMaxTeam + 1]
	const int* slot_list;
	const double* src;
	double* phi;
	double* b;
	double* r;
	const double* D;
	const double* ax;
	const double* ay;
	const double* sx;
	const double* sy;
	const double* fold;
	BatchRes* res;
	double inner_tol;
	// the one-CTA-per-problem multigrid kernel (batch_mg.cu): the queue
	// counter, the problems largest first, FP32 scratch and its offsets
	unsigned* queue;
	const int* order;
	int count;
	float* w32;
	const long long* w32off;
};

__device__ __forceinline__ int band_of(int m, int t, int nx) {
	return (int)((long)m * nx / t);
}

// Cells are handled four at a time along y ("quads", float4 in shared
// memory), which divides the index arithmetic and the shared-memory
// instructions by four. A band row holds qpr = ceil(ny / 4) quads; when ny is
// not a multiple of 4 the last quad of a row has dead lanes, kept at zero.
// Thread tid's quads are u = tid + k T, k < KQ, walked with the (row, quad)
// pair advanced incrementally.
struct QuadWalk {
	int li0, q0, dq, dr;
	__device__ __forceinline__ void init(int tid, int T, int qpr) {
		li0 = tid / qpr;
		q0 = tid - li0 * qpr;
		dq = T / qpr;
		dr = T - dq * qpr;
	}
};

// Every thread visits exactly KQ quads, so the unrolled bodies are free of
// branches and the compiler can overlap their shared-memory loads. A visit
// past the band's last quad is made on a clamped copy (the last row) with
// valid = false: its loads are harmless, and the body sends its stores to a
// scratch slot and leaves it out of the sums. The start values pass through
// an empty asm so that the (row, quad) sequence is recomputed in every walk
// instead of keeping KQ of each live across the whole solve.
template<int KQ, class F>
__device__ __forceinline__ void walk(const QuadWalk& qw, int rows, int qpr, F&& f) {
	int li = qw.li0, jq = qw.q0;
	asm volatile("" : "+r"(li), "+r"(jq));
#pragma unroll
	for (int k = 0; k < KQ; ++k) {
		const bool valid = li < rows;
		f(k, valid ? li : rows - 1, jq, valid);
		li += qw.dq;
		jq += qw.dr;
		const bool wrap = jq >= qpr;
		jq = wrap ? jq - qpr : jq;
		li = wrap ? li + 1 : li;
	}
}

__device__ __forceinline__ float4 f4fma(float a, float4 x, float4 y) {
	return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
}
__device__ __forceinline__ float4 ld_cluster_f4(uint32_t a) {
	float4 v;
	asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
			: "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a) : "memory");
	return v;
}
__device__ __forceinline__ float& f4at(float4& v, int e) {
	return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w;
}

// FP64 operator row (StencilOp::apply with the cell's row and column known)
__device__ __forceinline__ double apply64(const double* D, const double* ax,
		const double* ay, const double* x, int P, int i, int j, int a) {
	double c = D[a] * ldcg(x + a);
	c = fma(ax[i], ldcg(x + a - P), c);
	c = fma(ax[i + 1], ldcg(x + a + P), c);
	c = fma(ay[j], ldcg(x + a - 1), c);
	c = fma(ay[j + 1], ldcg(x + a + 1), c);
	return c;
}

// One problem on one team; every member runs it on its band. All control
// decisions come from team-reduced values, so the members take the same path
// and make the same sequence of team reductions.
template<int T, int KQ>
__device__ __noinline__ bool team_solve(const BatchArgs& a, const BatchProb& prob,
		int pi, Team& team, const Watch& w) {
	// declared here, not passed in, so the compiler addresses it as shared
	// memory (32-bit shared-window addresses rather than generic pointers)
	extern __shared__ __align__(16) float smem[];
	__shared__ int s_stop;
	Team tm = team;
	const BatchProb pr = prob;
	const int tid = threadIdx.x;
	const int nx = pr.nx, ny = pr.ny, t = (int)tm.t, m = (int)tm.m;
	const int r0 = band_of(m, t, nx), rows = band_of(m + 1, t, nx) - r0;
	// the shared-memory layout follows the team's largest band, so every
	// member's arrays (re in particular) sit at the same offsets
	const int rm = (nx + t - 1) / t;
	const int qpr = (ny + 3) >> 2, ny4 = qpr * 4;
	const int W = ny4 + 4, W4 = W >> 2, P = ny + 2;
	const bool ragged = ny4 != ny;
	const bool up = m > 0, down = m + 1 < t;
	const double nall = (double)nx * (double)ny;
	const int last_li = m == t - 1 ? rows - 1 : -1;   // row of cell (nx-1, ny-1)
	// p: rows -1 .. rows, pitch W (ny4 cells and a zero pad quad)
	float* pe = smem;
	float4* pe4 = reinterpret_cast<float4*>(pe);
	float4* xs4 = pe4 + (rm + 2) * W4;     // FP32 iterate of the band
	float4* re4 = xs4 + rm * qpr;          // r's first and last row
	float4* junk = re4 + 2 * qpr + tid;    // target of the stores of invalid visits
	const long long off = pr.cell;
	double* x64 = a.phi + off;
	double* b64 = a.b + off;
	double* r64 = a.r + off;
	const double* D = a.D + off;
	const double* ax = a.ax + pr.axo;
	const double* ay = a.ay + pr.ayo;
	const unsigned long long t_start = globaltimer();
	QuadWalk qw;
	qw.init(tid, T, qpr);
	auto counted = [&](int li, int j) { return pr.full || !(li == last_li && j == ny - 1); };
	auto gaddr = [&](int li, int j) { return (r0 + li + 1) * P + j + 1; };
	// the live cells of a quad, one FP64 visit each (the rare passes)
	auto cells = [&](auto&& g) {
		walk<KQ>(qw, rows, qpr, [&](int k, int li, int jq, bool v) {
#pragma unroll
			for (int e = 0; e < 4; ++e) {
				const int j = jq * 4 + e;
				g(k, e, li, j < ny ? j : ny - 1, v && j < ny);
			}
		});
	};

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
	cells([&](int, int, int li, int j, bool v) {
		const int i = r0 + li, ad = gaddr(li, j);
		const double bb = rhs_at<cg_host::SRC_FIELD>(sp, ra, i, j, ad);
		if (v) b64[ad] = bb;
		s1[0] += v ? bb : 0.0;
	});
	if (pr.mean) {
		if (!team_allreduce<double, 1>(s1, tm, w)) return false;
		const double mb = s1[0] / nall;
		cells([&](int, int, int li, int j, bool v) {
			const int ad = gaddr(li, j);
			const double bb = b64[ad] - mb;
			if (v) b64[ad] = bb;
		});
	}
	double nb[1] = { 0.0 };
	cells([&](int, int, int li, int j, bool v) {
		const double bb = b64[gaddr(li, j)];
		nb[0] = (v && counted(li, j)) ? fma(bb, bb, nb[0]) : nb[0];
	});
	if (!team_allreduce<double, 1>(nb, tm, w)) return false;
	double normb = sqrt(nb[0]);
	if (normb == 0.0) normb = 1.0;

	// on-chip state
	for (int q = tid; q < (rm + 2) * W4 + rm * qpr + 2 * qpr; q += T)
		pe4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
	__syncthreads();
	float4 r[KQ], q[KQ];
#pragma unroll
	for (int k = 0; k < KQ; ++k) r[k] = q[k] = make_float4(0.f, 0.f, 0.f, 0.f);
	double scale0 = 1.0, rn0 = 1.0, resid = 0.0;

	// FP64 residual of the band into r (FP32, mean removed, scaled by the
	// first residual's norm); returns its FP32 (r, r)
	auto true_residual = [&](bool first, float& gamma) -> bool {
		double sums[3] = { 0.0, 0.0, 0.0 };
		cells([&](int, int, int li, int j, bool v) {
			const int i = r0 + li, ad = gaddr(li, j);
			const double rv = b64[ad] - apply64(D, ax, ay, x64, P, i, j, ad);
			if (v) r64[ad] = rv;
			sums[0] = (v && counted(li, j)) ? fma(rv, rv, sums[0]) : sums[0];
			sums[1] += v ? rv : 0.0;
			sums[2] = v ? fma(rv, rv, sums[2]) : sums[2];
		});
		if (!team_allreduce<double, 3>(sums, tm, w)) return false;
		resid = sqrt(sums[0]) / normb;
		const double mr = pr.mean ? sums[1] / nall : 0.0;
		if (first) {
			rn0 = sqrt(pr.mean ? fmax(sums[2] - sums[1] * mr, 0.0) : sums[2]);
			scale0 = rn0 > 0.0 ? 1.0 / rn0 : 1.0;
		}
		float g[1] = { 0.f };
		cells([&](int k, int e, int li, int j, bool v) {
			const float rv = v ? (float)((r64[gaddr(li, j)] - mr) * scale0) : 0.f;
			f4at(r[k], e) = rv;
			g[0] = fmaf(rv, rv, g[0]);
		});
		walk<KQ>(qw, rows, qpr, [&](int k, int li, int jq, bool v) {
			if (v && li == 0) re4[jq] = r[k];
			if (v && li == rows - 1) re4[qpr + jq] = r[k];
		});
		if (!team_allreduce<float, 1>(g, tm, w)) return false;
		gamma = g[0];
		return true;
	};
	// x += alpha p
	auto add_p = [&](float alpha) {
		walk<KQ>(qw, rows, qpr, [&](int, int li, int jq, bool v) {
			float4* xp = v ? xs4 + li * qpr + jq : junk;
			*xp = f4fma(alpha, pe4[(li + 1) * W4 + jq], *xp);
		});
	};
	// the FP32 iterate into the FP64 solution
	auto fold_x = [&]() {
		walk<KQ>(qw, rows, qpr, [&](int, int li, int jq, bool v) {
			float4 xv = xs4[li * qpr + jq];
#pragma unroll
			for (int e = 0; e < 4; ++e) {
				const int j = jq * 4 + e;
				if (v && j < ny) {
					const int ad = gaddr(li, j);
					x64[ad] = fma(rn0, (double)f4at(xv, e), x64[ad]);
				}
			}
			if (v) xs4[li * qpr + jq] = make_float4(0.f, 0.f, 0.f, 0.f);
		});
		__threadfence();
	};
	auto team_sync = [&]() -> bool {
		double z[1] = { 0.0 };
		return team_allreduce<double, 1>(z, tm, w);
	};

	float gamma = 0.f;
	if (!true_residual(true, gamma)) return false;
	bool done = resid <= pr.tol;
	int it = 0, updates = 0, since = 0;
	const double it_tol = fmax(a.inner_tol, 1e-2);
	const float drop = (float)(it_tol * it_tol);
	const double tol_scaled = pr.tol * normb * scale0;
	const float near = (float)(0.25 * tol_scaled * tol_scaled);
	float gamma_ref = gamma, gamma_old = 1.f;
	bool first = true;
	const uint32_t re_addr = smem_u32(re4);
	const float cx = pr.cx, cy = pr.cy;
	while (!done && it < pr.max_iter && gamma > 0.f) {
		const float beta = first ? 0.f : gamma / gamma_old;
		first = false;
		// p = r + beta p over the band; the halo rows get the same FMA on the
		// neighbours' edge rows of r, so they equal the neighbours' own p
		walk<KQ>(qw, rows, qpr, [&](int k, int li, int jq, bool v) {
			const int s = (li + 1) * W4 + jq;
			*(v ? pe4 + s : junk) = f4fma(beta, pe4[s], r[k]);
		});
		if (up || down) {
			for (int c = tid; c < qpr; c += T) {
				if (up) {
					float4* h = pe4 + c;
					*h = f4fma(beta, *h, ld_cluster_f4(dsmem_map(re_addr + 16u * (qpr + c), tm.lo + m - 1)));
				}
				if (down) {
					float4* h = pe4 + (rows + 1) * W4 + c;
					*h = f4fma(beta, *h, ld_cluster_f4(dsmem_map(re_addr + 16u * c, tm.lo + m + 1)));
				}
			}
		}
		__syncthreads();
		// q = A p, (p, q); the diagonal from the problem's constants
		float pq[1] = { 0.f };
		walk<KQ>(qw, rows, qpr, [&](int k, int li, int jq, bool v) {
			const int i = r0 + li, s = (li + 1) * W4 + jq;
			const float4 pc = pe4[s], pu = pe4[s - W4], pd = pe4[s + W4];
			const float pl = pe[4 * s - 1], pr4 = pe[4 * s + 4];
			float drow = pr.d0;
			drow += i == 0 ? pr.dw : 0.f;
			drow += i == nx - 1 ? pr.de : 0.f;
			const int j0 = jq * 4;
			float4 d = make_float4(drow, drow, drow, drow);
			d.x += j0 == 0 ? pr.ds : 0.f;
			d.x += j0 == ny - 1 ? pr.dn : 0.f;
			d.y += j0 + 1 == ny - 1 ? pr.dn : 0.f;
			d.z += j0 + 2 == ny - 1 ? pr.dn : 0.f;
			d.w += j0 + 3 == ny - 1 ? pr.dn : 0.f;
			float4 o;
			o.x = fmaf(cy, pc.y, fmaf(cy, pl, fmaf(cx, pd.x, fmaf(cx, pu.x, d.x * pc.x))));
			o.y = fmaf(cy, pc.z, fmaf(cy, pc.x, fmaf(cx, pd.y, fmaf(cx, pu.y, d.y * pc.y))));
			o.z = fmaf(cy, pc.w, fmaf(cy, pc.y, fmaf(cx, pd.z, fmaf(cx, pu.z, d.z * pc.z))));
			o.w = fmaf(cy, pr4, fmaf(cy, pc.z, fmaf(cx, pd.w, fmaf(cx, pu.w, d.w * pc.w))));
			q[k] = o;
			float dot = pc.x * o.x;
			dot = fmaf(pc.y, o.y, dot);
			dot = fmaf(pc.z, o.z, dot);
			dot = fmaf(pc.w, o.w, dot);
			pq[0] += v ? dot : 0.f;
		});
		if (!team_allreduce<float, 1>(pq, tm, w)) return false;
		const float alpha = gamma / pq[0];
		// r -= alpha q, (r, r), the band's edge rows of r; x += alpha p runs
		// while the partials of (r, r) travel
		float gn[1] = { 0.f };
		walk<KQ>(qw, rows, qpr, [&](int k, int li, int jq, bool v) {
			float4 rv = f4fma(-alpha, q[k], r[k]);
			if (ragged) {
				// dead lanes of a row's last quad stay zero
				const int j0 = jq * 4;
				rv.y = j0 + 1 < ny ? rv.y : 0.f;
				rv.z = j0 + 2 < ny ? rv.z : 0.f;
				rv.w = j0 + 3 < ny ? rv.w : 0.f;
			}
			rv = v ? rv : make_float4(0.f, 0.f, 0.f, 0.f);
			r[k] = rv;
			float g = rv.x * rv.x;
			g = fmaf(rv.y, rv.y, g);
			g = fmaf(rv.z, rv.z, g);
			g = fmaf(rv.w, rv.w, g);
			gn[0] += g;
			if (v && li == 0) re4[jq] = rv;
			if (v && li == rows - 1) re4[qpr + jq] = rv;
		});
		team_post<float, 1>(gn, tm);
		add_p(alpha);
		if (!team_wait<float, 1>(gn, tm, w)) return false;
		++it;
		++since;
		float gnew = gn[0];
		if (gnew < drop * gamma_ref || gnew <= near || since >= kStallIters) {
			since = 0;
			fold_x();
			if (!team_sync()) return false;
			if (!true_residual(false, gnew)) return false;
			++updates;
			if (resid <= pr.tol) {
				done = true;
				break;
			}
			gamma_ref = gnew;
		}
		gamma_old = gamma;
		gamma = gnew;
		// the launch's error word and deadline, every 256 iterations (a team
		// whose reductions never have to wait would not see them otherwise);
		// a member that stops here leaves its team mates waiting for it,
		// and they stop at their next poll of the error word
		if ((it & 255) == 0) {
			if (tid == 0) {
				int st = *(volatile int*)w.err != 0 ? 1 : 0;
				if (!st && globaltimer() > w.deadline) {
					watch_fail(w, CARPIO_GPU_ETIMEOUT);
					st = 1;
				}
				s_stop = st;
			}
			__syncthreads();
			if (s_stop) return false;
		}
	}
	if (!done) {
		fold_x();
		if (!team_sync()) return false;
	}
	if (pr.mean) {
		double sx1[1] = { 0.0 };
		cells([&](int, int, int li, int j, bool v) {
			sx1[0] += v ? x64[gaddr(li, j)] : 0.0;
		});
		if (!team_allreduce<double, 1>(sx1, tm, w)) return false;
		const double mx = sx1[0] / nall;
		cells([&](int, int, int li, int j, bool v) {
			const int ad = gaddr(li, j);
			const double xv = x64[ad] - mx;
			if (v) x64[ad] = xv;
		});
	}
	if (m == 0 && tid == 0) {
		BatchRes o;
		o.code = done ? 0 : 1;
		o.iters = it;
		o.updates = updates;
		o.ran = 1;
		o.resid = resid;
		o.ms = (double)(globaltimer() - t_start) * 1e-6;
		a.res[pi] = o;
	}
	__syncthreads();   // the next problem reuses the shared memory
	team = tm;
	return true;
}

template<int T, int K>
__device__ __forceinline__ bool dispatch(int kc, const BatchArgs& a,
		const BatchProb& pr, int pi, Team& tm, const Watch& w) {
	if constexpr (K > kMaxQ) {
		watch_fail(w, CARPIO_GPU_EINVAL);
		return false;
	} else {
		if (kc == K) return team_solve<T, K>(a, pr, pi, tm, w);
		return dispatch<T, K * 2>(kc, a, pr, pi, tm, w);
	}
}

template<int T>
__global__ void __launch_bounds__(T, 1) k_batch(BatchArgs a) {
	__shared__ __align__(8) uint64_t s_bar[2];
	__shared__ double s_slot[2 * kTeamNV * kMaxTeam];
	__shared__ int s_go;
	const unsigned cr = cluster_rank(), cid = cluster_index();
	const int t = a.cl_team[cid];
	Team tm;
	tm.t = (unsigned)t;
	tm.m = cr % (unsigned)t;
	tm.lo = cr - tm.m;
	tm.bar = s_bar;
	tm.slot = s_slot;
	tm.par = 0;
	tm.bank = 0;
	if (threadIdx.x == 0) {
		mbar_init(&s_bar[0], (unsigned)t);
		mbar_init(&s_bar[1], (unsigned)t);
		fence_mbar_init_cluster();
	}
	__syncthreads();
	// every mbarrier of the cluster is initialised before any remote arrive
	cluster_barrier();
	const Watch w{ &a.ctl->err, a.ctl->wait_ns, globaltimer() + a.ctl->solve_ns };
	const int slot = (int)cid * kMaxTeam + (int)(cr / (unsigned)t);
	for (int q = a.slot_ptr[slot]; q < a.slot_ptr[slot + 1]; ++q) {
		if (threadIdx.x == 0) s_go = *(volatile int*)&a.ctl->err == 0;
		__syncthreads();
		const bool go = s_go != 0;
		__syncthreads();
		if (!go) break;
		const int pi = a.slot_list[q];
		const BatchProb pr = a.prob[pi];
		if (!dispatch<T, 1>(pr.kc, a, pr, pi, tm, w)) break;
	}
	// no CTA leaves while a team mate may still address its shared memory
	cluster_barrier();
}

}  // namespace cg_batch
