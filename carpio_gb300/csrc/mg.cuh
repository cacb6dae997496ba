// Geometric multigrid V-cycle as the preconditioner of the on-chip FP32 CG
// (k_poisson_mixed_tile): z = M r with M one V(1,1)-cycle, FP32.
//
// Levels: level 0 is the fine grid; level l + 1 halves both sides of level
// l while both are even (cell-centred coarsening, each coarse cell the union
// of 2 x 2 fine cells) and stops at an odd side or at one cell. Every level
// has the 5-point operator of the volume-scaled Laplacian: the interior face
// coefficients cx, cy of the fine grid (the same on every level, as the
// ratio of face area to centre distance does not change under coarsening),
// zero on boundary faces, and a diagonal D_l built on the host with the
// fine grid's boundary folding (a Dirichlet face doubles its coefficient, a
// Neumann face cancels it).
//
// The smoother scales by a stored reciprocal of D (the same on both sides of
// the cycle, so M stays symmetric) and the pre-smoothed z = w D^-1 r is never
// stored: every pass that needs it recomputes it from r.
//
// One cycle: pre-smoothing z = w D^-1 r (damped Jacobi from zero), the
// residual s = r - A z, restriction r_c = P^T s, the cycle on the coarse
// level, prolongation c = z + P z_c, post-smoothing z = c + w D^-1 (r - A c).
// P is the bilinear interpolation of cell-centred grids (weights 3/4, 1/4
// per axis; at a boundary the missing coarse neighbour is replaced by the
// cell itself) and R = P^T, so M is symmetric and positive (semi-)definite
// and plain CG stays valid. The coarsest level is solved with a fixed number
// of damped Jacobi sweeps from zero (exactly, z = r / D, for one cell; zero
// for the one-cell all-Neumann level, whose D is 0).
//
// Distribution: the largest levels (more than kMgGather cells) live in global
// memory (L2-resident at these sizes) and every thread of the cooperative
// grid takes cells of each level in turn, with a grid barrier between the
// passes that read neighbours; the remaining levels run in one CTA's shared
// memory with block barriers while the other CTAs wait at one grid barrier.
#pragma once

#include "krylov.cuh"

namespace cg_dev {

constexpr int kMgMaxLev = 16;
constexpr int kMgGather = 1024;     // levels of at most this many cells: one CTA
constexpr int kMgCoarseSweeps = 20; // damped Jacobi sweeps on the coarsest level

struct MgLevel {
	int nx, ny;
	float* R;          // right-hand side of the level (level 0: the fine r)
	float* S;          // residual after pre-smoothing
	float* Zp;         // the level's final correction (after post-smoothing)
	const float* D;    // diagonal, nx * ny
	const float* iD;   // its reciprocal (0 where D is 0): the smoother's scaling
};

struct MgArgs {
	int nlev;          // levels 0 .. nlev-1 in global memory (0: no multigrid)
	int ntot;          // levels nlev .. ntot-1 in one CTA's shared memory
	float cx, cy;      // interior face coefficients (negative)
	float omega;       // damped Jacobi weight
	MgLevel lev[kMgMaxLev];
};

// bilinear prolongation weight of coarse index I for fine index i along an
// axis of nc coarse cells (with the boundary clamp), as a function of i
__device__ __forceinline__ void mg_parents(int i, int nc, int& I0, int& I1, float& w0,
		float& w1) {
	I0 = i >> 1;
	I1 = (i & 1) ? I0 + 1 : I0 - 1;
	if (I1 < 0 || I1 >= nc) { I1 = I0; w0 = 1.f; w1 = 0.f; }
	else { w0 = 0.75f; w1 = 0.25f; }
}

// restriction weights: the fine indices 2I-1 .. 2I+2 that carry coarse index I
// in P, with their weights (P^T), along an axis of nc coarse cells
__device__ __forceinline__ float mg_rw(int I, int nc, int t) {
	// t = 0: i = 2I-1, 1: 2I, 2: 2I+1, 3: 2I+2
	switch (t) {
	case 0: return I >= 1 ? 0.25f : 0.f;
	case 1: return I == 0 ? 1.f : 0.75f;
	case 2: return I == nc - 1 ? 1.f : 0.75f;
	default: return I <= nc - 2 ? 0.25f : 0.f;
	}
}

// y = (A z)(I, J) on a level stored compactly (row-major, y fastest), with
// `ld` the loader (global L2 or shared memory)
template<class Ld>
__device__ __forceinline__ float mg_apply(const Ld& ld, const float* z, const float* D,
		int I, int J, int nx, int ny, float cx, float cy) {
	const int k = I * ny + J;
	float v = ld(D, k) * ld(z, k);
	if (I > 0) v = fmaf(cx, ld(z, k - ny), v);
	if (I < nx - 1) v = fmaf(cx, ld(z, k + ny), v);
	if (J > 0) v = fmaf(cy, ld(z, k - 1), v);
	if (J < ny - 1) v = fmaf(cy, ld(z, k + 1), v);
	return v;
}

// (P^T s)(I, J): s on the fine level (nxf x nyf), (I, J) on the coarse one
template<class Ld>
__device__ __forceinline__ float mg_restrict(const Ld& ld, const float* s, int I, int J,
		int nxf, int nyf) {
	const int nxc = nxf >> 1, nyc = nyf >> 1;
	float acc = 0.f;
#pragma unroll
	for (int a = 0; a < 4; ++a) {
		const float wa = mg_rw(I, nxc, a);
		if (wa == 0.f) continue;
		const int i = 2 * I - 1 + a;
		float row = 0.f;
#pragma unroll
		for (int b = 0; b < 4; ++b) {
			const float wb = mg_rw(J, nyc, b);
			if (wb == 0.f) continue;
			row = fmaf(wb, ld(s, i * nyf + 2 * J - 1 + b), row);
		}
		acc = fmaf(wa, row, acc);
	}
	return acc;
}

// (P zc)(i, j): zc on the coarse level (nxc x nyc), (i, j) on the fine one
template<class Ld>
__device__ __forceinline__ float mg_prolong(const Ld& ld, const float* zc, int i, int j,
		int nxc, int nyc) {
	int I0, I1, J0, J1;
	float a0, a1, b0, b1;
	mg_parents(i, nxc, I0, I1, a0, a1);
	mg_parents(j, nyc, J0, J1, b0, b1);
	float v = a0 * (b0 * ld(zc, I0 * nyc + J0) + b1 * ld(zc, I0 * nyc + J1));
	return fmaf(a1, b0 * ld(zc, I1 * nyc + J0) + b1 * ld(zc, I1 * nyc + J1), v);
}

// the corrected value c = w iD r + P zc at fine cell (i, j) (the
// pre-smoothed correction from r, plus the coarse correction); lc reads the
// constants (iD), lr reads r, lz reads zc
template<class Lc, class Lr, class Lz>
__device__ __forceinline__ float mg_corrected(const Lc& lc, const Lr& lr, const Lz& lz,
		const float* r, const float* iD, const float* zc, int i, int j, int nyf, int nxc,
		int nyc, float w) {
	const int k = i * nyf + j;
	return fmaf(w * lr(r, k), lc(iD, k), mg_prolong(lz, zc, i, j, nxc, nyc));
}

// post-smoothing at (I, J) of a level: c at the cell and its neighbours,
// then c + w iD (r - A c)
template<class Lc, class Lr, class Lz>
__device__ __forceinline__ float mg_post(const Lc& lc, const Lr& lr, const Lz& lz,
		const float* r, const float* zc, const float* D, const float* iD, int I, int J,
		int nx, int ny, float cx, float cy, float w) {
	const int nxc = nx >> 1, nyc = ny >> 1;
	const float c = mg_corrected(lc, lr, lz, r, iD, zc, I, J, ny, nxc, nyc, w);
	const int k = I * ny + J;
	float ac = lc(D, k) * c;
	if (I > 0) ac = fmaf(cx, mg_corrected(lc, lr, lz, r, iD, zc, I - 1, J, ny, nxc, nyc, w), ac);
	if (I < nx - 1) ac = fmaf(cx, mg_corrected(lc, lr, lz, r, iD, zc, I + 1, J, ny, nxc, nyc, w), ac);
	if (J > 0) ac = fmaf(cy, mg_corrected(lc, lr, lz, r, iD, zc, I, J - 1, ny, nxc, nyc, w), ac);
	if (J < ny - 1) ac = fmaf(cy, mg_corrected(lc, lr, lz, r, iD, zc, I, J + 1, ny, nxc, nyc, w), ac);
	return fmaf(w * (lr(r, k) - ac), lc(iD, k), c);
}

// s = r - A (w iD r) at (I, J): the residual after pre-smoothing, with the
// pre-smoothed correction recomputed from r. ld reads D and iD, lr reads r.
template<class Ld, class Lr>
__device__ __forceinline__ float mg_resid(const Ld& ld, const Lr& lr, const float* r,
		const float* D, const float* iD, int I, int J, int nx, int ny, float cx, float cy,
		float w) {
	const int k = I * ny + J;
	const float rk = lr(r, k);
	float v = ld(D, k) * (w * rk * ld(iD, k));
	if (I > 0) v = fmaf(cx, w * lr(r, k - ny) * ld(iD, k - ny), v);
	if (I < nx - 1) v = fmaf(cx, w * lr(r, k + ny) * ld(iD, k + ny), v);
	if (J > 0) v = fmaf(cy, w * lr(r, k - 1) * ld(iD, k - 1), v);
	if (J < ny - 1) v = fmaf(cy, w * lr(r, k + 1) * ld(iD, k + 1), v);
	return rk - v;
}

struct LdL2 {   // data written by other CTAs of the launch
	__device__ __forceinline__ float operator()(const float* p, int k) const { return ldcg(p + k); }
};
struct LdSm {   // this CTA's shared memory (plain loads)
	__device__ __forceinline__ float operator()(const float* p, int k) const { return p[k]; }
};
struct LdRo {   // read-only data of the launch (the diagonals)
	__device__ __forceinline__ float operator()(const float* p, int k) const { return __ldg(p + k); }
};

// a distributed pass: every thread of the grid takes cells gt, gt + G, ...
// of a level, CH at a time, and computes all CH values before storing any,
// so the loads of the CH cells are in flight together
template<int CH, class Fn, class St>
__device__ __forceinline__ void mg_pass(int gt, int G, int n, Fn&& fn, St&& st) {
	for (int k0 = gt; k0 < n; k0 += CH * G) {
		float val[CH];
#pragma unroll
		for (int u = 0; u < CH; ++u) {
			const int k = k0 + u * G;
			val[u] = k < n ? fn(k) : 0.f;
		}
#pragma unroll
		for (int u = 0; u < CH; ++u) {
			const int k = k0 + u * G;
			if (k < n) st(k, val[u]);
		}
	}
}

// The levels nlev .. ntot-1 in this CTA's shared memory (called by one CTA):
// r of level nlev from S of level nlev - 1, the cycle, and level nlev's final
// correction into lev[nlev].Zp. sm: 3 * (cells of levels nlev .. ntot-1)
// floats (r, z, s of each level).
__device__ inline void mg_coarse(const MgArgs& mg, float* sm) {
	const int T = blockDim.x, tid = threadIdx.x;
	const LdSm sl;
	const LdRo ro;
	const LdL2 gl;
	// r, z, s of level l at base(l), base(l) + n, base(l) + 2 n
	auto base = [&](int l) {
		float* q = sm;
		for (int m = mg.nlev; m < l; ++m) q += 3 * mg.lev[m].nx * mg.lev[m].ny;
		return q;
	};
	const float w = mg.omega, cx = mg.cx, cy = mg.cy;
	// r of the first shared level from the distributed level above it
	{
		const MgLevel& f = mg.lev[mg.nlev - 1];
		const MgLevel& c = mg.lev[mg.nlev];
		float* r = base(mg.nlev);
		mg_pass<4>(tid, T, c.nx * c.ny, [&](int k) {
			const int I = k / c.ny, J = k - I * c.ny;
			return mg_restrict(gl, f.S, I, J, f.nx, f.ny);
		}, [&](int k, float v) { r[k] = v; });
	}
	__syncthreads();
	// down: s = r - A (w iD r), then r of the next level
	for (int l = mg.nlev; l < mg.ntot - 1; ++l) {
		const MgLevel& L = mg.lev[l];
		const int n = L.nx * L.ny;
		float* r = base(l);
		float* s = r + 2 * n;
		for (int k = tid; k < n; k += T) {
			const int I = k / L.ny, J = k - I * L.ny;
			s[k] = mg_resid(ro, sl, r, L.D, L.iD, I, J, L.nx, L.ny, cx, cy, w);
		}
		__syncthreads();
		const MgLevel& C = mg.lev[l + 1];
		float* rc = base(l + 1);
		for (int k = tid; k < C.nx * C.ny; k += T) {
			const int I = k / C.ny, J = k - I * C.ny;
			rc[k] = mg_restrict(sl, s, I, J, L.nx, L.ny);
		}
		__syncthreads();
	}
	// coarsest: damped Jacobi sweeps from zero (one cell: exact)
	{
		const int l = mg.ntot - 1;
		const MgLevel& L = mg.lev[l];
		const int n = L.nx * L.ny;
		float* r = base(l);
		float* z = r + n;
		float* s = r + 2 * n;
		for (int k = tid; k < n; k += T) {
			const float id = __ldg(L.iD + k);
			z[k] = (n == 1 ? r[k] : w * r[k]) * id;
		}
		__syncthreads();
		if (n > 1) {
			for (int sweep = 1; sweep < kMgCoarseSweeps; ++sweep) {
				for (int k = tid; k < n; k += T) {
					const int I = k / L.ny, J = k - I * L.ny;
					s[k] = fmaf(w * (r[k] - mg_apply(sl, z, L.D, I, J, L.nx, L.ny, cx, cy)),
							__ldg(L.iD + k), z[k]);
				}
				__syncthreads();
				for (int k = tid; k < n; k += T) z[k] = s[k];
				__syncthreads();
			}
		}
	}
	// up: the post-smoothed correction into z (this level's z is not read
	// by the pass: c is recomputed from r and the coarser z)
	for (int l = mg.ntot - 2; l >= mg.nlev; --l) {
		const MgLevel& L = mg.lev[l];
		const MgLevel& C = mg.lev[l + 1];
		const int n = L.nx * L.ny;
		float* r = base(l);
		float* z = r + n;
		const float* zc = base(l + 1) + C.nx * C.ny;
		for (int k = tid; k < n; k += T) {
			const int I = k / L.ny, J = k - I * L.ny;
			z[k] = mg_post(ro, sl, sl, r, zc, L.D, L.iD, I, J, L.nx, L.ny, cx, cy, w);
		}
		__syncthreads();
	}
	const MgLevel& L = mg.lev[mg.nlev];
	const float* z = base(mg.nlev) + L.nx * L.ny;
	for (int k = tid; k < L.nx * L.ny; k += T) __stcg(L.Zp + k, z[k]);
}

}  // namespace cg_dev
