// Explicit projection step of NS_explicit_ (lib/structure/s_ns_explicit.hpp:
// 118-229) on the GPU, plus the single Operation_ operators.
//
// This file is compiled with --fmad=false: every expression below rounds
// exactly like the reference's C++ (no contraction), and divisions and sqrt
// are IEEE round-to-nearest, so the operators reproduce the reference's
// doubles bit for bit. The projection's Krylov solve lives in poisson.cu.
//
// Fields are the reference's full arrays (ghosts included) in the device
// layout of the grid: cell (i, j), i, j in normal-cell coordinates, at
// (i + gl) * P + (j + gl).
#include "internal.hpp"
#include "bits.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

using namespace cg_dev;

constexpr double kSmall = 1e-10;  // SMALL, lib/type_define.hpp

struct Geo {
	int nx, ny, gl, P, NI, NJ;
	const double *cx, *sx, *cy, *sy;   // incl. ghosts
	// p2: every cell size along x is hx and along y hy, both powers of two,
	// and every centre distance (ghosts included) is exactly hx or hy; then
	// dividing by one of those lengths (or by twice or half of one) equals
	// multiplying by its reciprocal bit for bit (both round the same exact
	// real number), and the P2 kernels below do that
	int p2;
	double hx, hy, ihx, ihy;
	int kx, ky;   // p2: ihx = 2^kx, ihy = 2^ky
	__device__ __forceinline__ int at(int i, int j) const { return (i + gl) * P + (j + gl); }
	__device__ __forceinline__ double CX(int i) const { return cx[i + gl]; }
	__device__ __forceinline__ double CY(int j) const { return cy[j + gl]; }
	__device__ __forceinline__ double SX(int i) const { return sx[i + gl]; }
	__device__ __forceinline__ double SY(int j) const { return sy[j + gl]; }
};

struct BcDev {
	int type[4];
	double value[4];
	// optional boundary value per ghost cell (a field in the grid's layout),
	// for boundary conditions given as functions; null: value[segment]
	const double* gv;
};

__host__ __device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

// GB300 issues one FP64 instruction per warp every 64 cycles, so the
// helpers below replace FP64 operations by integer ones where the result is
// the same bits.

// x / d rounded to nearest, for a divisor fixed per launch, with y =
// RN(1 / d): q = RN(x y) is within one ulp of x / d, r = x - d q is exact
// by the FMA, and RN(q + r y) = RN(x / d) (Markstein, IBM J. Res. Dev.
// 34(1), 1990: correction of a faithful quotient with the correctly
// rounded reciprocal). Valid without under- or overflow: `on` is set on
// the host for |d| within 2^+-100, and x here within 2^+-800; zeros,
// subnormals, infinities and NaNs divide.
struct FixedDiv {
	double d, y;
	int on;
};

inline FixedDiv make_fixed_div(double d) {
	FixedDiv f;
	f.d = d;
	f.y = 1.0 / d;
	int ex = 0;
	const double m = std::frexp(std::fabs(d), &ex);
	f.on = std::isfinite(d) && m != 0.0 && ex >= -100 && ex <= 100 ? 1 : 0;
	return f;
}

__device__ __noinline__ double div_slow(double x, double d) {
	return __ddiv_rn(x, d);
}

// r + |r| by the bits: +0 for finite r <= 0, 2r (the exponent field + 1)
// for normal r > 0 below 2^1023; subnormals, infinities and NaNs by the FPU
__device__ __noinline__ double r_plus_abs_slow(double r) {
	return __dadd_rn(r, fabs(r));
}

__device__ __forceinline__ double r_plus_abs(double r) {
	unsigned lo, hi;
	split_bits(r, lo, hi);
	const int e = (int)((hi >> 20) & 0x7ffu);
	if (e < 2047 && ((hi >> 31) != 0u || (hi | lo) == 0u)) return join_bits(0u, 0u);
	if ((hi >> 31) == 0u && e >= 1 && e <= 2045) return join_bits(lo, hi + (1u << 20));
	return r_plus_abs_slow(r);
}

__device__ __forceinline__ double fixed_div(double x, const FixedDiv& f) {
	const int e = exp_field(x);
	if (f.on && e >= 1023 - 800 && e <= 1023 + 800) {
		const double q = __dmul_rn(x, f.y);
		const double r = __fma_rn(-f.d, q, x);
		return __fma_rn(r, f.y, q);
	}
	return div_slow(x, f.d);
}

// ------------------------------------------------------------ ghost fill --
// Value Equation_::apply_bc (s_equation.hpp:340-378) gives ghost (i, j) when
// its source cell (oi, oj) holds `src`.
__device__ __forceinline__ double ghost_value(const Geo& g, const BcDev& bc,
		int i, int j, double src, int& oi, int& oj) {
	int seg, a;
	oi = i;
	oj = j;
	if (i < 0 || i >= g.nx) { a = 0; seg = i < 0 ? 0 : 1; oi = i < 0 ? 0 : g.nx - 1; }
	else { a = 1; seg = j < 0 ? 2 : 3; oj = j < 0 ? 0 : g.ny - 1; }
	double val = bc.gv ? bc.gv[g.at(i, j)] : bc.value[seg];
	double cgh = a == 0 ? g.CX(i) : g.CY(j);
	double co = a == 0 ? g.CX(oi) : g.CY(oj);
	if (bc.type[seg] == 1) {
		double hs = (a == 0 ? g.SX(oi) : g.SY(oj)) * 0.5;
		double cf = (seg == 1 || seg == 3) ? co + hs : co - hs;
		double u = (cgh - cf) / (co - cf);
		return (val * (1.0 - u)) + (src * u);
	}
	double dl = fabs(cgh - co);
	return src - val * dl;
}

// source cell of a ghost without evaluating it
__device__ __forceinline__ void ghost_src(const Geo& g, int i, int j, int& oi, int& oj) {
	oi = i;
	oj = j;
	if (i < 0 || i >= g.nx) oi = i < 0 ? 0 : g.nx - 1;
	else oj = j < 0 ? 0 : g.ny - 1;
}

// One block per field. The reference visits ghosts in IJK order (x fastest)
// and writes in place, so a corner ghost (x and y out of range) reads the
// y-ghost of the first/last normal column of its row: the old value for the
// low-x corners (visited first), the new one for the high-x corners. Phase 1
// captures the old values the low-x corners need; phase 2 writes everything.
struct BcFields {
	double* f[2];
	BcDev bc[2];
};

// the fill of one field by one block; s_old holds 2 gl^2 doubles
__device__ void bc_fill(const Geo& g, double* f, const BcDev& bc, double* s_old) {
	const int gl = g.gl, nx = g.nx, ny = g.ny;
	const int NI = g.NI, NJ = g.NJ;
	const int ncorner = 2 * gl * gl;     // low-x corners: I < gl, J < gl or J >= NJ-gl
	for (int t = threadIdx.x; t < ncorner; t += blockDim.x) {
		int r = t / gl, c = t - r * gl;   // r: ghost row 0..2gl-1, c: ghost column
		int J = r < gl ? r : NJ - 2 * gl + r;
		int i = c - gl, j = J - gl;
		int oi, oj;
		ghost_src(g, i, j, oi, oj);
		s_old[t] = f[g.at(oi, oj)];
	}
	__syncthreads();
	// walk the ghost frame: rows J < gl and J >= NJ-gl fully, columns I < gl
	// and I >= NI-gl for the other rows
	const int frame_rows = 2 * gl;
	const long n_rows = (long)frame_rows * NI;
	const long n_cols = (long)(NJ - 2 * gl) * 2 * gl;
	for (long t = threadIdx.x; t < n_rows + n_cols; t += blockDim.x) {
		int I, J;
		if (t < n_rows) {
			int r = (int)(t / NI);
			I = (int)(t - (long)r * NI);
			J = r < gl ? r : NJ - 2 * gl + r;
		} else {
			long u = t - n_rows;
			int r = (int)(u / (2 * gl));
			int c = (int)(u - (long)r * 2 * gl);
			J = gl + r;
			I = c < gl ? c : NI - 2 * gl + c;
		}
		int i = I - gl, j = J - gl;
		int oi, oj;
		ghost_src(g, i, j, oi, oj);
		double src;
		bool xg = i < 0 || i >= nx, yg = j < 0 || j >= ny;
		if (xg && yg) {
			if (i < 0) {
				int r = J < gl ? J : J - (NJ - 2 * gl);
				src = s_old[r * gl + I];
			} else {
				// the y-ghost (nx-1, j) as this same call has just written it
				int oi2, oj2;
				ghost_src(g, oi, oj, oi2, oj2);
				src = ghost_value(g, bc, oi, oj, f[g.at(oi2, oj2)], oi2, oj2);
			}
		} else {
			src = f[g.at(oi, oj)];
		}
		f[(long)I * g.P + J] = ghost_value(g, bc, i, j, src, oi, oj);
	}
}

// The same fill spread over blocks (blockIdx.y: the field). The cells with
// an order dependency -- the corner ghosts and the y-ghosts of column i = 0
// whose old values the low-x corners read -- go to block 0, which captures
// the old values first; every other ghost reads only normal cells, so blocks
// 1.. fill the rest of the frame in any order.
__device__ void bc_fill_ordered(const Geo& g, double* f, const BcDev& bc, double* s_old) {
	const int gl = g.gl, nx = g.nx;
	const int NI = g.NI, NJ = g.NJ;
	const int ncorner = 2 * gl * gl;
	for (int t = threadIdx.x; t < ncorner; t += blockDim.x) {
		int r = t / gl, c = t - r * gl;
		int J = r < gl ? r : NJ - 2 * gl + r;
		int i = c - gl, j = J - gl;
		int oi, oj;
		ghost_src(g, i, j, oi, oj);
		s_old[t] = f[g.at(oi, oj)];
	}
	__syncthreads();
	// the frame rows' cells with I < gl + 1 or I >= NI - gl: 2 gl rows of
	// 2 gl + 1 cells
	const int per_row = 2 * gl + 1;
	for (int t = threadIdx.x; t < 2 * gl * per_row; t += blockDim.x) {
		const int r = t / per_row, c = t - r * per_row;
		const int J = r < gl ? r : NJ - 2 * gl + r;
		const int I = c <= gl ? c : NI - 2 * gl - 1 + c;
		int i = I - gl, j = J - gl;
		int oi, oj;
		ghost_src(g, i, j, oi, oj);
		double src;
		if (i < 0) {
			src = s_old[r * gl + I];
		} else if (i >= nx) {
			int oi2, oj2;
			ghost_src(g, oi, oj, oi2, oj2);
			src = ghost_value(g, bc, oi, oj, f[g.at(oi2, oj2)], oi2, oj2);
		} else {
			src = f[g.at(oi, oj)];
		}
		f[(long)I * g.P + J] = ghost_value(g, bc, i, j, src, oi, oj);
	}
}

__device__ void bc_fill_rest(const Geo& g, double* f, const BcDev& bc, int part, int nparts) {
	const int gl = g.gl;
	const int NI = g.NI, NJ = g.NJ;
	const long row_cells = NI - 2 * gl - 1;           // I in [gl + 1, NI - gl)
	const long n_rows = 2L * gl * row_cells;
	const long n_cols = 2L * gl * (NJ - 2 * gl);     // I < gl or >= NI - gl, J in [gl, NJ - gl)
	for (long t = part * (long)blockDim.x + threadIdx.x; t < n_rows + n_cols;
			t += (long)nparts * blockDim.x) {
		int I, J;
		if (t < n_rows) {
			const int r = (int)(t / row_cells);
			I = gl + 1 + (int)(t - r * row_cells);
			J = r < gl ? r : NJ - 2 * gl + r;
		} else {
			const long u = t - n_rows;
			const int r = (int)(u / (2 * gl));
			const int c = (int)(u - (long)r * 2 * gl);
			J = gl + r;
			I = c < gl ? c : NI - 2 * gl + c;
		}
		int i = I - gl, j = J - gl;
		int oi, oj;
		ghost_src(g, i, j, oi, oj);
		f[(long)I * g.P + J] = ghost_value(g, bc, i, j, f[g.at(oi, oj)], oi, oj);
	}
}

__global__ void __launch_bounds__(256) k_apply_bc(Geo g, BcFields bf) {
	extern __shared__ double s_old[];   // [2 * gl (rows) * gl (cols)]
	const int fi = blockIdx.y;
	if (blockIdx.x == 0) bc_fill_ordered(g, bf.f[fi], bf.bc[fi], s_old);
	else bc_fill_rest(g, bf.f[fi], bf.bc[fi], blockIdx.x - 1, gridDim.x - 1);
}

// ------------------------------------------------------ advection schemes --
// s_operation.hpp:313-628 (+ minmod, src/calculation/advection.hpp:1079-1081)
__device__ __forceinline__ double limiter(int sch, double r, double R) {
	switch (sch) {
	case CARPIO_GPU_VANLEER: return 0.5 * R * (r + fabs(r)) / (R - 1 + r);
	case CARPIO_GPU_SUPERBEE: return smax(smax(0.0, smin(R * r, 1.0)), smin(r, R));
	case CARPIO_GPU_WAHYD:
		if (r <= 1.0) return 0.5 * R * (r + fabs(r)) / (R - 1 + r);
		return smin((r + R * r * fabs(r)) / (R + r * r), R);
	case CARPIO_GPU_QUICK: return 0.75 * r + 0.25;
	case CARPIO_GPU_CUI: return 2.0 / 3.0 * r + 1.0 / 3.0;
	case CARPIO_GPU_UPWIND2: return r;
	case CARPIO_GPU_MINMOD: return smax(0.0, smin(1.0, r));
	}
	return 0.0;
}

// The stencil ratio of a TVD face on a P2 grid, ((a 2h) / b) / (2h) with the
// reciprocal of 2h: both scalings are exact while a 2h and the quotients
// stay normal, and then the value is RN(a / b). The exponent fields are
// checked with a margin of 100 (|log2 2h| <= 91 on a P2 grid); a zero a
// gives the same signed zero (or NaN) either way, an infinite quotient the
// same infinity; anything else takes the reference's three operations.
__device__ __noinline__ double tvd_ratio_slow(double a, double b, double h2, double ih2) {
	return __dmul_rn(__ddiv_rn(__dmul_rn(a, h2), b), ih2);
}

__device__ __forceinline__ double tvd_ratio(double a, double b, double h2, double ih2) {
	const double r = __ddiv_rn(a, b);
	const int ea = exp_field(a), er = exp_field(r);
	const bool a0 = is_zero_bits(a);
	if (a0 || (ea >= 100 && ea <= 1947 && ((er >= 100 && er <= 1947) || er == 2047)))
		return r;
	return tvd_ratio_slow(a, b, h2, ih2);
}

// The TVD schemes (upwind2, van Leer, superbee, WAHYD, QUICK, CUI) build
// each face value from an upwind-biased stencil of three cells; the others
// (upwind1, center, center4) are single expressions.
template<int SCH>
constexpr bool kTvdScheme = SCH != CARPIO_GPU_UPWIND1 && SCH != CARPIO_GPU_CENTER
		&& SCH != CARPIO_GPU_CENTER4;

// One face value of a TVD scheme at cell (i, j) along axis D (0 x, 1 y):
// `plus` the face at +1/2 (fp), else the face at -1/2 (fm), the stencil
// chosen by the sign of the cell's velocity veo. P2: the grid's lengths are
// the powers of two of Geo::p2, so the divisions by them are
// multiplications by exact reciprocals (the same bits); the divisions by
// data stay. The field may sit in another array than the faces (a tile in
// shared memory, a lane's registers): f at index fa with stride fst along
// the axis; the faces at the grid's index of (i, j).
// The face value from its three stencil cells at offsets D_, C_, U_
// (downwind, central, upwind) of cell (i, j) along axis D.
template<int SCH, int D, bool P2>
__device__ __forceinline__ double tvd_value(const Geo& g, const double* f, int fa,
		int fst, int i, int j, int D_, int C_, int U_) {
#define F(k) f[fa + (k) * fst]
#define S(k) (D == 0 ? g.SX(i + (k)) : g.SY(j + (k)))
	if (P2) {
		// every S is h: R = 2h / h = 2, the sums are 2h
		const double h = D == 0 ? g.hx : g.hy;
		const double ih = D == 0 ? g.ihx : g.ihy;
		const double h2 = h + h, ih2 = 0.5 * ih;
		const double R = 2.0;
		const double dc = F(D_) - F(C_);
		const double r = tvd_ratio(F(C_) - F(U_), dc + kSmall, h2, ih2);
		// van Leer's 0.5 R (r + |r|) / (R - 1 + r) is (r + |r|) / (1 + r)
		// at R = 2 (0.5 R = 1 exactly)
		const double lim = SCH == CARPIO_GPU_VANLEER ? r_plus_abs(r) / (1.0 + r)
		                                             : limiter(SCH, r, R);
		return F(C_) + mul_p2(lim, -1, 0.5) * dc;
	}
	const double R = (S(D_) + S(C_)) / S(C_);
	const double r = (F(C_) - F(U_)) * (S(D_) + S(C_)) / (F(D_) - F(C_) + kSmall) / (S(C_) + S(U_));
	return F(C_) + limiter(SCH, r, R) / R * (F(D_) - F(C_));
#undef F
#undef S
}

// The stencil orientation of a cell from its velocity veo = (x + y) * 0.5:
// 1 (veo >= 0), -1 (veo < 0), 0 (NaN: every offset 0), from s = x + y by
// its bits: the halving keeps the sign and turns only -2^-1074 into -0
// (round to nearest even), which orients like a positive value
__device__ __forceinline__ int tvd_orient_sum(double s) {
	unsigned lo, hi;
	split_bits(s, lo, hi);
	const unsigned mag = hi & 0x7fffffffu;
	if (mag > 0x7ff00000u || (mag == 0x7ff00000u && lo != 0u)) return 0;   // NaN
	if ((hi >> 31) == 0u) return 1;
	return (mag == 0u && lo <= 1u) ? 1 : -1;
}

// the +1/2 face of a cell in its own frame: the same value as the -1/2
// face of the next cell with the same orientation (the same three cells)
// The stencil offsets are chosen first and the face evaluated once: with
// one tvd_value per orientation the compiler may predicate them, and a
// predicated-off FP64 instruction still takes its issue slot.
template<int SCH, int D, bool P2>
__device__ __forceinline__ double tvd_plus(const Geo& g, const double* f, int fa,
		int fst, int i, int j, int o) {
	// o > 0: (1, 0, -1); o < 0: (0, 1, 2); o == 0: (0, 0, 0)
	const int d_ = o > 0 ? 1 : 0, c_ = o < 0 ? 1 : 0, u_ = o > 0 ? -1 : (o < 0 ? 2 : 0);
	return tvd_value<SCH, D, P2>(g, f, fa, fst, i, j, d_, c_, u_);
}

template<int SCH, int D, bool P2>
__device__ __forceinline__ double tvd_half(const Geo& g, const double* face,
		const double* f, int fa, int fst, int i, int j, bool plus) {
	const int st = D == 0 ? g.P : 1;
	const int a = g.at(i, j);
	// veo = (face[a] + face[a - st]) * 0.5
	const int o = tvd_orient_sum(face[a] + face[a - st]);
	if (plus) return tvd_plus<SCH, D, P2>(g, f, fa, fst, i, j, o);
	// the -1/2 face: o > 0: (0, -1, -2); o < 0: (-1, 0, 1); o == 0: (0, 0, 0)
	const int d_ = o < 0 ? -1 : 0, c_ = o > 0 ? -1 : 0, u_ = o > 0 ? -2 : (o < 0 ? 1 : 0);
	return tvd_value<SCH, D, P2>(g, f, fa, fst, i, j, d_, c_, u_);
}

// The stencil offsets (D, C, U) from frame cell c of the face between c and
// c + 1 for the orientation o of the cell that owns it: the same cells
// whether that is c (own, the +1/2 face) or c + 1 (the -1/2 face), except
// for o == 0 (NaN velocity), whose stencil is the owning cell alone.
__device__ __forceinline__ void face_offsets(int o, bool own, int& d_, int& c_, int& u_) {
	if (o > 0) { d_ = 1; c_ = 0; u_ = -1; }
	else if (o < 0) { d_ = 0; c_ = 1; u_ = 2; }
	else { d_ = c_ = u_ = own ? 0 : 1; }
}

// the -1/2 face of cell c + 1 where it differs from the +1/2 face of c (the
// orientations differ): out of line, so that the common path carries one
// face evaluation
template<int SCH, int D, bool P2>
__device__ __noinline__ double tvd_face_next(const Geo& g, const double* f, int fa,
		int fst, int i, int j, int o) {
	int d_, c_, u_;
	face_offsets(o, false, d_, c_, u_);
	return tvd_value<SCH, D, P2>(g, f, fa, fst, i, j, d_, c_, u_);
}

// the TVD axis term from its two face values: (u+ fp - u- fm) / S(0)
template<int D, bool P2>
__device__ __forceinline__ double tvd_combine(const Geo& g, const double* face,
		int i, int j, double fp, double fm) {
	const int st = D == 0 ? g.P : 1;
	const int a = g.at(i, j);
	const double fa0 = face[a], fam = face[a - st];
	if (P2) return mul_p2(fa0 * fp - fam * fm, D == 0 ? g.kx : g.ky, D == 0 ? g.ihx : g.ihy);
	return (fa0 * fp - fam * fm) / (D == 0 ? g.SX(i) : g.SY(j));
}

// one axis of VdotNabla at cell (i, j); D = 0 x, 1 y (field addressing as
// tvd_half)
template<int SCH, int D, bool P2 = false>
__device__ __forceinline__ double adv_axis_at(const Geo& g, const double* face,
		const double* f, int fa, int fst, int i, int j) {
	if constexpr (kTvdScheme<SCH>) {
		const double fp = tvd_half<SCH, D, P2>(g, face, f, fa, fst, i, j, true);
		const double fm = tvd_half<SCH, D, P2>(g, face, f, fa, fst, i, j, false);
		return tvd_combine<D, P2>(g, face, i, j, fp, fm);
	}
	const int st = D == 0 ? g.P : 1;
	const int a = g.at(i, j);
#define F(k) f[fa + (k) * fst]
#define C(k) (D == 0 ? g.CX(i + (k)) : g.CY(j + (k)))
	const double fa0 = face[a], fam = face[a - st];
	const double veo = (fa0 + fam) * 0.5;
	if (SCH == CARPIO_GPU_UPWIND1) {
		if (veo > 0.0) return veo * (F(0) - F(-1)) / (C(0) - C(-1));
		if (veo < 0.0) return veo * (F(1) - F(0)) / (C(1) - C(0));
		return 0.0;
	} else if (SCH == CARPIO_GPU_CENTER) {
		return veo * (F(1) - F(-1)) / (C(1) - C(-1));
	}
	double din = (F(1) - F(-1)) / (C(1) - C(-1));
	double dout = (F(2) - F(-2)) / (C(2) - C(-2));
	return (4.0 * din - dout) / 3.0;
#undef F
#undef C
}

template<int SCH, int D, bool P2 = false>
__device__ __forceinline__ double adv_axis(const Geo& g, const double* face,
		const double* f, int i, int j) {
	return adv_axis_at<SCH, D, P2>(g, face, f, g.at(i, j), D == 0 ? g.P : 1, i, j);
}

template<int SCH, bool P2 = false>
__device__ __forceinline__ double adv_cell(const Geo& g, const double* uf,
		const double* vf, const double* f, int i, int j) {
	double a0 = adv_axis<SCH, 0, P2>(g, uf, f, i, j);
	double a1 = adv_axis<SCH, 1, P2>(g, vf, f, i, j);
	double s = 0.0;
	s += a0;
	s += a1;
	return s;
}

// NablaMuNabla(Vt mu, ...) (s_operation.hpp:664-688). MU1: mu is 1.0, and
// mu * x is x (the same bits)
template<bool P2 = false, bool MU1 = false>
__device__ __forceinline__ double diffusion(const Geo& g, double mu,
		const double* f, int i, int j) {
	const int a = g.at(i, j);
	double t0, t1;
	if (P2) {
		// centre distances and sizes are hx, hy: multiply by 1 / h
#define MUX(x) (MU1 ? (x) : mu * (x))
		{
			double dm = mul_p2(MUX(f[a] - f[a - g.P]), g.kx, g.ihx);
			double dp = mul_p2(MUX(f[a + g.P] - f[a]), g.kx, g.ihx);
			t0 = mul_p2(dp - dm, g.kx, g.ihx);
		}
		{
			double dm = mul_p2(MUX(f[a] - f[a - 1]), g.ky, g.ihy);
			double dp = mul_p2(MUX(f[a + 1] - f[a]), g.ky, g.ihy);
			t1 = mul_p2(dp - dm, g.ky, g.ihy);
		}
#undef MUX
		// res = 0; res += t0; res += t1
		return plus_zero(t0 + t1);
	}
	{
		double dm = mu * (f[a] - f[a - g.P]) / (g.CX(i) - g.CX(i - 1));
		double dp = mu * (f[a + g.P] - f[a]) / (g.CX(i + 1) - g.CX(i));
		t0 = (dp - dm) / g.SX(i);
	}
	{
		double dm = mu * (f[a] - f[a - 1]) / (g.CY(j) - g.CY(j - 1));
		double dp = mu * (f[a + 1] - f[a]) / (g.CY(j + 1) - g.CY(j));
		t1 = (dp - dm) / g.SY(j);
	}
	double res = 0.0;
	res += t0;
	res += t1;
	return res;
}

// NablaMuNabla(const Scalar& mu, ...) (s_operation.hpp:630-662): face mu
// from the cell and its neighbour weighted by the half sizes
__device__ __forceinline__ double diffusion_var(const Geo& g, const double* mu,
		const double* f, int i, int j) {
	const int a = g.at(i, j);
	double t[2];
#pragma unroll
	for (int d = 0; d < 2; ++d) {
		const int st = d == 0 ? g.P : 1;
		const double hs = (d == 0 ? g.SX(i) : g.SY(j)) * 0.5;
		const double hsp = (d == 0 ? g.SX(i + 1) : g.SY(j + 1)) * 0.5;
		const double hsm = (d == 0 ? g.SX(i - 1) : g.SY(j - 1)) * 0.5;
		const double c = d == 0 ? g.CX(i) : g.CY(j);
		const double cp = d == 0 ? g.CX(i + 1) : g.CY(j + 1);
		const double cm = d == 0 ? g.CX(i - 1) : g.CY(j - 1);
		const double mufp = (hs * mu[a + st] + hsp * mu[a]) / (hsp + hs);
		const double mufm = (hs * mu[a - st] + hsm * mu[a]) / (hsm + hs);
		const double dp = mufp * (f[a + st] - f[a]) / (cp - c);
		const double dm = mufm * (f[a] - f[a - st]) / (c - cm);
		t[d] = (dp - dm) / (d == 0 ? g.SX(i) : g.SY(j));
	}
	double res = 0.0;
	res += t[0];
	res += t[1];
	return res;
}

// ------------------------------------------------ stand-alone advection --
// Advection_::run_one_step (s_advection.hpp:185-212) `steps` times: the
// ghosts of phi refilled, then every normal cell updated in place in Ijk
// order (x fastest), phi - dt * VdotNabla, so cell (i, j) reads the new
// values of (i-1, j), (i-2, j), (i, j-1), (i, j-2) and the old values of
// the cells after it. Every scheme's stencil is the axis cross of radius 2:
// no cell reads a cell of its own anti-diagonal i + j = L, each reads only
// lower diagonals (already swept) and higher ones (not yet), so sweeping
// the diagonals in order, the cells of one in parallel, gives the values
// of the sequential loop. A diagonal holds at most min(nx, ny) cells: one
// block runs every step, with a block barrier between diagonals.
template<int SCH, bool P2 = false>
__global__ void __launch_bounds__(1024) k_advect(Geo g, double* phi, BcDev bc,
		const double* uf, const double* vf, double dt, int steps) {
	extern __shared__ double s_old[];
	const int nx = g.nx, ny = g.ny;
	for (int st = 0; st < steps; ++st) {
		bc_fill(g, phi, bc, s_old);
		__syncthreads();
		for (int L = 0; L <= nx + ny - 2; ++L) {
			const int i0 = L - (ny - 1) > 0 ? L - (ny - 1) : 0;
			const int i1 = L < nx - 1 ? L : nx - 1;
			for (int i = i0 + (int)threadIdx.x; i <= i1; i += blockDim.x) {
				const int j = L - i;
				const double adv = adv_cell<SCH, P2>(g, uf, vf, phi, i, j);
				const int a = g.at(i, j);
				const double phin = phi[a];
				phi[a] = phin - dt * adv;
			}
			__syncthreads();
		}
	}
}

// The sweep as pipelined bands: block b owns rows [b R, b R + R) and sweeps
// its own anti-diagonals (local level l: cells (b R + k, l - k)). Its first
// rows read the new values of the two rows above, which the band above
// writes at its levels R - 1 + l and R - 2 + l, so block b starts level l
// once the band above has published R + l finished levels; the same chain
// keeps the band below from overwriting (i + 1, j), (i + 2, j) before they
// are read. No grid barrier per diagonal: one progress word per band
// (release store / acquire poll, bounded by the watchdog), and two grid
// barriers per step around block 0's ghost refill.
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
	asm volatile("st.release.gpu.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

template<int SCH, bool P2 = false>
__global__ void __launch_bounds__(kThreads) k_advect_band(Geo g, double* phi, BcDev bc,
		const double* uf, const double* vf, double dt, int steps, int R,
		unsigned* prog, GridCtl gc) {
	extern __shared__ double s_old[];
	__shared__ int s_ok;
	gc.start();
	const int nx = g.nx, ny = g.ny, b = blockIdx.x;
	const int r0 = b * R;
	const int rb = min(R, nx - r0);                  // rows of this band
	const int rp = b > 0 ? R : 0;                     // rows of the band above
	const unsigned T = (unsigned)(R + ny);            // > any band's levels per step
	for (int st = 0; st < steps; ++st) {
		if (b == 0) bc_fill(g, phi, bc, s_old);
		if (!grid_sync(gc)) return;
		const unsigned base = (unsigned)st * T;
		const int nl = rb + ny - 1;
		const int nlp = rp + ny - 1;
		for (int l = 0; l < nl; ++l) {
			if (b > 0) {
				const unsigned need = base + (unsigned)min(rp + l, nlp);
				if (threadIdx.x == 0) {
					int ok = 1;
					unsigned polls = 0;
					unsigned long long t0 = 0;
					while (ld_acquire_gpu(&prog[b - 1]) < need) {
						if ((++polls & 63u) == 0) {
							if (*(volatile int*)gc.err) { ok = 0; break; }
							const unsigned long long t = globaltimer();
							if (t0 == 0) t0 = t;
							if (t - t0 > gc.wait_ns || t > gc.deadline) {
								set_err(gc, CARPIO_GPU_ETIMEOUT);
								ok = 0;
								break;
							}
						}
					}
					s_ok = ok;
				}
				// the acquire poll plus the block barrier order this band's
				// loads after the band above's writes (no full fence needed)
				__syncthreads();
				if (!s_ok) return;
			}
			for (int k = threadIdx.x; k < rb; k += blockDim.x) {
				const int j = l - k;
				if (j >= 0 && j < ny) {
					const int i = r0 + k;
					const double adv = adv_cell<SCH, P2>(g, uf, vf, phi, i, j);
					const int a = g.at(i, j);
					const double phin = phi[a];
					phi[a] = phin - dt * adv;
				}
			}
			// the block barrier orders every thread's writes before thread 0's
			// release store (release is cumulative over what it has observed)
			__syncthreads();
			if (threadIdx.x == 0) st_release_gpu(&prog[b], base + (unsigned)l + 1u);
		}
		if (!grid_sync(gc)) return;
	}
}

// Row-pipelined sweep: lane l < RPW of band b owns grid row i = RPW b + l and walks
// its columns j in order, one step behind lane l - 1, so that at every step
// the lanes of a warp hold one anti-diagonal of the in-place sweep. A cell
// reads, as the reference's loop does, the new values of (i-1, j), (i-2, j),
// (i, j-1), (i, j-2) and the old values of (i+1, j), (i+2, j), (i, j+1),
// (i, j+2): the rows above come from lanes l - 1 and l - 2 (their last two
// results, by shuffle), the own row's new values are the lane's last two
// results, and the old values come from a three-cell window that each lane
// keeps of its own row ahead of its column (lanes l + 1 and l + 2, by
// shuffle). There is no barrier per diagonal. Only the two rows across a
// band edge go through memory: the next band's first lanes read the two
// rows above from L2 once this band's last lane has published its column
// (release/acquire progress word, every kAdvPub columns), and this band's
// last lanes read the two old rows below before they publish. A band is
// one warp (RPW rows, lanes beyond RPW idle); NW bands share a block.
constexpr int kAdvPub = 8;          // columns per progress publication
constexpr int kAdvRows = 32;        // rows per band (one warp)
constexpr int kAdvBands = 1;        // bands per block

// NF = 4 (TVD schemes): four warps per band, warp q computing one of the
// cell's four face values (x at +1/2 and -1/2, y at +1/2 and -1/2) on its
// own SMSP -- a warp issues one FP64 instruction per 64 cycles, so a face's
// ~50 instead of a cell's ~200 per step -- with identical lane state in all
// four; the faces meet in shared memory behind one barrier of the band's
// warps per step (double-buffered by step parity), every warp combines
// them, and warp 0 alone stores and publishes.
template<int SCH, bool P2, int RPW, int NW, int NF>
__global__ void __launch_bounds__(NW * NF * 32, 1) k_advect_rows(Geo g, double* phi,
		BcDev bc, const double* uf, const double* vf, double dt, int steps,
		unsigned* prog, GridCtl gc) {
	static_assert(RPW >= 4 && RPW <= 32, "band rows");
	static_assert(NF == 1 || (NF == 4 && kTvdScheme<SCH> && NW == 1), "face split");
	__shared__ double scr[NW * NF][10][32];        // a lane's two stencils, [k][lane]
	__shared__ double sfc[2][NW][NF][32];          // face values by step parity
	__shared__ double s_old[32];
	// the per-step barrier counts NF warps per band: any other block size
	// is refused before the first barrier (uniform over the grid)
	if (blockDim.x != NW * NF * 32) {
		if (threadIdx.x == 0 && blockIdx.x == 0) set_err(gc, CARPIO_GPU_EINVAL);
		return;
	}
	gc.start();
	const int wq = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int warp = wq / NF, q = wq - warp * NF;  // band in the block, face
	const int nx = g.nx, ny = g.ny, gl = g.gl;
	const int nb = (nx + RPW - 1) / RPW;
	const int band = blockIdx.x * NW + warp;
	const int i0 = band * RPW;
	// idle lanes get a row outside the ghost ring: `at` gives them 0
	const int i = lane < RPW ? i0 + lane : -4 * (gl + 1);
	const bool act = lane < RPW && band < nb && i < nx;   // the lane computes cells
	constexpr int LB = RPW - 1;                   // the band's last lane
	double* F = &scr[wq][0][0];
	// phi at (r, c) inside the ghost ring, else 0 (never used)
	auto at = [&](int r, int c) -> double {
		return (r >= -gl && r < nx + gl && c >= -gl && c < ny + gl) ? ldcg(phi + g.at(r, c)) : 0.0;
	};
	for (int st = 0; st < steps; ++st) {
		if (!grid_sync(gc)) return;
		if (blockIdx.x == 0) {
			bc_fill(g, phi, bc, s_old);
			for (int t = threadIdx.x; t < nb; t += blockDim.x) prog[t] = 0u;
		}
		if (!grid_sync(gc)) return;
		if (band >= nb) continue;
		const bool upper = band > 0;                  // rows above from band - 1
		const bool lower = band + 1 < nb;             // band + 1 reads this band
		// own row: the last two new values (the ghosts left of column 0
		// before the first cell) and the old window at columns t .. t + 3
		double res1 = at(i, -1), res2 = at(i, -2);
		const int tz = -lane;                         // column at step 0
		double o0 = at(i, tz), o1 = at(i, tz + 1), o2 = at(i, tz + 2), o3 = at(i, tz + 3);
		// rows i0 - 1, i0 - 2 at column s (lane 0) and i0 - 1 at s - 1
		double aC = 0.0, bC = 0.0, aP = 0.0, aN = 0.0, bN = 0.0;
		// rows i0 + RPW, i0 + RPW + 1 (old) at columns s - LB (and i0 + RPW
		// at s - LB + 1), for the last two lanes
		double cC = 0.0, cN = 0.0, dC = 0.0, cNN = 0.0, dN = 0.0;
		unsigned have = 0;
		bool ok = true;
		// lane 0: wait until band - 1 has published `need` columns
		auto wait_up = [&](unsigned need) {
			if (!upper || have >= need || !ok) return;
			unsigned polls = 0;
			unsigned long long t0 = 0;
			for (;;) {
				have = ld_acquire_gpu(&prog[band - 1]);
				if (have >= need) return;
				if ((++polls & 63u) == 0) {
					if (*(volatile int*)gc.err) { ok = false; return; }
					const unsigned long long tt = globaltimer();
					if (t0 == 0) t0 = tt;
					if (tt - t0 > gc.wait_ns || tt > gc.deadline) {
						set_err(gc, CARPIO_GPU_ETIMEOUT);
						ok = false;
						return;
					}
				}
			}
		};
		if (lane == 0) {
			wait_up(1u);
			aC = at(i0 - 1, 0);
			bC = at(i0 - 2, 0);
			aP = at(i0 - 1, -1);
			if (ny > 1) {
				wait_up(2u);
				aN = at(i0 - 1, 1);
				bN = at(i0 - 2, 1);
			}
		}
		if (lane == LB) {
			cC = at(i0 + RPW, -LB);
			cN = at(i0 + RPW, -LB + 1);
			dC = at(i0 + RPW + 1, -LB);
			cNN = at(i0 + RPW, -LB + 2);
			dN = at(i0 + RPW + 1, -LB + 1);
		}
		for (int s = 0; s < ny + LB; ++s) {
			const int t = s - lane;                   // this lane's column
			const bool on = act && t >= 0 && t < ny;
			// new values of the rows above at column t, old values below
			double up1 = __shfl_up_sync(0xffffffffu, res1, 1);
			double up2 = __shfl_up_sync(0xffffffffu, res2, 2);
			double dn1 = __shfl_down_sync(0xffffffffu, o1, 1);
			double dn2 = __shfl_down_sync(0xffffffffu, o2, 2);
			const double aPl = __shfl_sync(0xffffffffu, aP, 0);
			const double cNl = __shfl_sync(0xffffffffu, cN, LB);
			if (lane == 0) { up1 = aC; up2 = bC; }
			if (lane == 1) up2 = aPl;
			if (lane == LB - 1) dn2 = cNl;
			if (lane == LB) { dn1 = cC; dn2 = dC; }
			if (on && (t & 7) == 0 && t + 16 < ny) {
				// the face velocities' next lines into L1 (read-only here)
				const int ap = g.at(i, t + 16);
				asm volatile("prefetch.global.L1 [%0];" :: "l"(uf + ap));
				asm volatile("prefetch.global.L1 [%0];" :: "l"(uf + ap - g.P));
				asm volatile("prefetch.global.L1 [%0];" :: "l"(vf + ap));
			}
			double a0 = 0.0, a1 = 0.0;   // the two axis terms
			if (on) {
				F[0 * 32 + lane] = up2;
				F[1 * 32 + lane] = up1;
				F[2 * 32 + lane] = o0;
				F[3 * 32 + lane] = dn1;
				F[4 * 32 + lane] = dn2;
				F[5 * 32 + lane] = res2;
				F[6 * 32 + lane] = res1;
				F[7 * 32 + lane] = o0;
				F[8 * 32 + lane] = o1;
				F[9 * 32 + lane] = o2;
				const int fa = 2 * 32 + lane;
				if constexpr (NF == 4) {
					double fv;
					switch (q) {
					case 0: fv = tvd_half<SCH, 0, P2>(g, uf, F, fa, 32, i, t, true); break;
					case 1: fv = tvd_half<SCH, 0, P2>(g, uf, F, fa, 32, i, t, false); break;
					case 2: fv = tvd_half<SCH, 1, P2>(g, vf, F + 5 * 32, fa, 32, i, t, true); break;
					default: fv = tvd_half<SCH, 1, P2>(g, vf, F + 5 * 32, fa, 32, i, t, false); break;
					}
					sfc[s & 1][warp][q][lane] = fv;
				} else {
					a0 = adv_axis_at<SCH, 0, P2>(g, uf, F, fa, 32, i, t);
					a1 = adv_axis_at<SCH, 1, P2>(g, vf, F + 5 * 32, fa, 32, i, t);
				}
			}
			if constexpr (NF == 4) {
				// every warp of the band, every step
				asm volatile("bar.sync %0, %1;" :: "r"(1 + warp), "r"(NF * 32) : "memory");
			}
			if (on) {
				if constexpr (NF == 4) {
					const double (*fv)[32] = sfc[s & 1][warp];
					a0 = tvd_combine<0, P2>(g, uf, i, t, fv[0][lane], fv[1][lane]);
					a1 = tvd_combine<1, P2>(g, vf, i, t, fv[2][lane], fv[3][lane]);
				}
				double adv = 0.0;
				adv += a0;
				adv += a1;
				const double nv = o0 - dt * adv;
				if (q == 0) phi[g.at(i, t)] = nv;
				res2 = res1;
				res1 = nv;
			} else if (t >= ny) {
				res2 = res1;                          // past the row end: keep the last two
			}
			// advance the window (old values of the own row, loaded ahead)
			o0 = o1;
			o1 = o2;
			o2 = o3;
			o3 = at(i, t + 4);
			// lane 0: the rows above at columns s + 1 (ready) and s + 2 (loaded)
			if (lane == 0) {
				aP = aC;
				aC = aN;
				bC = bN;
				if (s + 2 < ny) {
					wait_up((unsigned)(s + 3));
					aN = at(i0 - 1, s + 2);
					bN = at(i0 - 2, s + 2);
				}
			}
			// the last lane: the old rows below at columns s - LB + 1 and
			// s - LB + 2 for the next steps
			if (lane == LB) {
				cC = cN;
				cN = cNN;
				dC = dN;
				cNN = at(i0 + RPW, s - LB + 3);
				dN = at(i0 + RPW + 1, s - LB + 2);
			}
			// publish the last lane's progress (the lane before is one ahead)
			const int tl = s - LB;
			if (q == 0 && lower && tl >= 0 && tl < ny && ((tl + 1) % kAdvPub == 0 || tl == ny - 1)) {
				if (lane == LB - 1 || lane == LB) __threadfence();
				__syncwarp();
				if (lane == LB) st_release_gpu(&prog[band], (unsigned)(tl + 1));
			}
		}
		// lane 0 may have stopped on an error: the grid barrier returns it
	}
}

// ------------------------------------------------------------- NS kernels --
struct StepScalars {
	double dt;                // current time step (Time_::_dt)
	double t;                 // current time
	unsigned long long maxmag_bits;   // max |u_c|^2 of this step (as bits)
	unsigned done;            // blocks finished with the max reduction
	unsigned step;            // current step
};

struct DtRule {
	double cfl, diff_number, diff_coef;
	double mins, minx, miny;  // Grid_::min_size() and per axis
};

// NS_::restrict_time (s_ns.hpp:146-169): max_magnitude over the normal cells,
// then the last block updates dt (it can only shrink).
__global__ void __launch_bounds__(kThreads) k_restrict_time(Geo g,
		const double* u, const double* v, StepScalars* ss, DtRule rule,
		double* step_dt, int st) {
	double m = 0.0;
	const long n = (long)g.nx * g.ny;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int a = g.at(i, j);
		double s = 0;
		s += u[a] * u[a];
		s += v[a] * v[a];
		// max sqrt(s) = sqrt(max s): a correctly rounded sqrt is monotone,
		// so one sqrt of the largest square gives the same bits
		m = smax(m, s);
	}
	m = block_max(m);
	__shared__ bool last;
	if (threadIdx.x == 0) {
		atomicMax(&ss->maxmag_bits, (unsigned long long)__double_as_longlong(m));
		__threadfence();
		last = atomicAdd(&ss->done, 1u) == gridDim.x - 1;
	}
	__syncthreads();
	if (last && threadIdx.x == 0) {
		__threadfence();
		double maxmag = sqrt(__longlong_as_double((long long)atomicAdd(&ss->maxmag_bits, 0ull)));
		double rdt = rule.cfl * rule.mins / maxmag;
		double dt = ss->dt;
		double rdt2 = dt;
		if (rule.diff_number < 100) {
			double den = 0.0;
			den += 1.0 / (rule.minx * rule.minx);
			den += 1.0 / (rule.miny * rule.miny);
			rdt2 = rule.diff_number / rule.diff_coef / den;
		}
		if (dt > smin(rdt, rdt2)) dt = smin(rdt, rdt2);
		ss->dt = dt;
		ss->maxmag_bits = 0ull;
		ss->done = 0u;
		if (step_dt) step_dt[st] = dt;
	}
}

// VectorCenter_::max_magnitude (s_vector.hpp:89-103) alone
__global__ void __launch_bounds__(kThreads) k_maxmag(Geo g, const double* u,
		const double* v, unsigned long long* out) {
	double m = 0.0;
	const long n = (long)g.nx * g.ny;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int a = g.at(i, j);
		double s = 0;
		s += u[a] * u[a];
		s += v[a] * v[a];
		m = smax(m, sqrt(s));
	}
	m = block_max(m);
	if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// u* = u + dt (-adv + diff / rho) for both components
// (NS_explicit_::_veo_star_center, s_ns_explicit.hpp:173-229)
template<int SCH, bool P2 = false>
__global__ void __launch_bounds__(kThreads) k_predictor(Geo g, const double* u,
		const double* v, const double* uf, const double* vf, double* us,
		double* vs, const StepScalars* ss, double rho, double mu, const double* muf) {
	const double dt = ss->dt;
	const long n = (long)g.nx * g.ny;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int a = g.at(i, j);
		// __diffusion_term (s_ns_explicit.hpp:235-241): the mu field when the
		// uniform mu was unset
		{
			double adv = adv_cell<SCH, P2>(g, uf, vf, u, i, j);
			double dif = muf ? diffusion_var(g, muf, u, i, j) : diffusion<P2>(g, mu, u, i, j);
			double src = 0;
			us[a] = (-adv + (dif + src) / rho) * dt + u[a];
		}
		{
			double adv = adv_cell<SCH, P2>(g, uf, vf, v, i, j);
			double dif = muf ? diffusion_var(g, muf, v, i, j) : diffusion<P2>(g, mu, v, i, j);
			double src = 0;
			vs[a] = (-adv + (dif + src) / rho) * dt + v[a];
		}
	}
}

// The predictor for the TVD schemes, by tiles of kPredTI x kPredTJ cells:
// a face's value depends only on the face and the upwind orientation, so
// the +1/2 face of a cell and the -1/2 face of the next cell are the same
// bits whenever the two cells' velocities have the same sign. Each tile
// stages the component with two halo cells in shared memory, evaluates
// every face it needs once per orientation its cells ask for (once where
// they agree, the usual case), then combines them per cell exactly as
// adv_cell does. The per-cell arithmetic is k_predictor's.
constexpr int kPredTI = 8, kPredTJ = 64, kPredThreads = 512;

// DIFF: 0 the mu field muf, 1 the uniform mu, 2 the uniform mu 1.0.
template<int SCH, bool P2, int DIFF>
__global__ void __launch_bounds__(kPredThreads) k_predictor_tiles(Geo g, const double* u,
		const double* v, const double* uf, const double* vf, double* us,
		double* vs, const StepScalars* ss, FixedDiv rho, double mu, const double* muf) {
	constexpr int TI = kPredTI, TJ = kPredTJ, SJ = TJ + 4;
	__shared__ double tile[(TI + 4) * SJ];   // the component, two halo cells
	__shared__ double fpx[TI * TJ], fmx[TI * TJ], fpy[TI * TJ], fmy[TI * TJ];
	__shared__ signed char ox[TI * TJ], oy[TI * TJ];   // the cells' orientations
	const double dt = ss->dt;
	const int i0 = blockIdx.y * TI, j0 = blockIdx.x * TJ;
	const int ti = min(TI, g.nx - i0), tj = min(TJ, g.ny - j0);
	const int tid = threadIdx.x, T = blockDim.x;
	for (int q = tid; q < ti * tj; q += T) {
		const int li = q / tj, lj = q - li * tj;
		const int a = g.at(i0 + li, j0 + lj);
		ox[li * TJ + lj] = (signed char)tvd_orient_sum(uf[a] + uf[a - g.P]);
		oy[li * TJ + lj] = (signed char)tvd_orient_sum(vf[a] + vf[a - 1]);
	}
	const int nxf = (ti + 1) * tj, nyf = ti * (tj + 1);
	for (int comp = 0; comp < 2; ++comp) {
		const double* f = comp == 0 ? u : v;
		__syncthreads();   // the previous component's readers are done
		for (int q = tid; q < (ti + 4) * (tj + 4); q += T) {
			const int li = q / (tj + 4), lj = q - li * (tj + 4);
			tile[li * SJ + lj] = f[g.at(i0 + li - 2, j0 + lj - 2)];
		}
		__syncthreads();
		for (int q = tid; q < nxf + nyf; q += T) {
			if (q < nxf) {
				// x face between local rows r and r + 1, frame cell r
				const int r = q / tj - 1, lj = q - (r + 1) * tj;
				const bool L = r >= 0, R = r + 1 < ti;
				const int oL = L ? ox[r * TJ + lj] : 0, oR = R ? ox[(r + 1) * TJ + lj] : 0;
				const int fa = (r + 2) * SJ + (lj + 2), i = i0 + r, j = j0 + lj;
				const bool shared = L && R && oL == oR && oL != 0;
				int d_, c_, u_;
				face_offsets(L ? oL : oR, L, d_, c_, u_);
				const double val = tvd_value<SCH, 0, P2>(g, tile, fa, SJ, i, j, d_, c_, u_);
				if (L) fpx[r * TJ + lj] = val;
				if (R && (shared || !L)) fmx[(r + 1) * TJ + lj] = val;
				if (L && R && !shared)
					fmx[(r + 1) * TJ + lj] = tvd_face_next<SCH, 0, P2>(g, tile, fa, SJ, i, j, oR);
			} else {
				// y face between local columns c and c + 1, frame cell c
				const int qq = q - nxf;
				const int li = qq / (tj + 1), c = qq - li * (tj + 1) - 1;
				const bool L = c >= 0, R = c + 1 < tj;
				const int oL = L ? oy[li * TJ + c] : 0, oR = R ? oy[li * TJ + c + 1] : 0;
				const int fa = (li + 2) * SJ + (c + 2), i = i0 + li, j = j0 + c;
				const bool shared = L && R && oL == oR && oL != 0;
				int d_, c_, u_;
				face_offsets(L ? oL : oR, L, d_, c_, u_);
				const double val = tvd_value<SCH, 1, P2>(g, tile, fa, 1, i, j, d_, c_, u_);
				if (L) fpy[li * TJ + c] = val;
				if (R && (shared || !L)) fmy[li * TJ + c + 1] = val;
				if (L && R && !shared)
					fmy[li * TJ + c + 1] = tvd_face_next<SCH, 1, P2>(g, tile, fa, 1, i, j, oR);
			}
		}
		__syncthreads();
		double* out = comp == 0 ? us : vs;
		for (int q = tid; q < ti * tj; q += T) {
			const int li = q / tj, lj = q - li * tj;
			const int i = i0 + li, j = j0 + lj, a = g.at(i, j), e = li * TJ + lj;
			const double a0 = tvd_combine<0, P2>(g, uf, i, j, fpx[e], fmx[e]);
			const double a1 = tvd_combine<1, P2>(g, vf, i, j, fpy[e], fmy[e]);
			// adv = 0; adv += a0; adv += a1
			const double adv = plus_zero(a0 + a1);
			const double dif = DIFF == 0 ? diffusion_var(g, muf, f, i, j)
			                             : diffusion<P2, DIFF == 2>(g, mu, f, i, j);
			// (dif + src) / rho with src = 0
			out[a] = (-adv + fixed_div(plus_zero(dif), rho)) * dt + f[a];
		}
	}
}

// Operation_::InterpolateC2F(VecC, VecF) (s_operation.hpp:166-187). The
// low wall faces (i = 0: the x face at -1/2, j = 0: the y face) come after
// the main loop, not inside it: a branch there gets predicated, and its
// FP64 instructions then take issue slots in every cell.
template<int PM = -1>
__global__ void __launch_bounds__(kThreads) k_c2f(Geo g, const double* u,
		const double* v, double* fx, double* fy) {
	const bool p2 = PM == 1 || (PM < 0 && g.p2);
	const long n = (long)g.nx * g.ny;
	const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long stride = (long)gridDim.x * blockDim.x;
	// Geo::p2: every half size is h / 2 = 2^(-k - 1) and (hs + hs') = h, so
	// both products and the division are exponent moves (mul_p2)
	const double hsx = g.hx * 0.5, hsy = g.hy * 0.5;
	for (long k = t0; k < n; k += stride) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int a = g.at(i, j);
		if (p2) {
			fx[a] = mul_p2(mul_p2(u[a + g.P], -g.kx - 1, hsx) + mul_p2(u[a], -g.kx - 1, hsx),
					g.kx, g.ihx);
			fy[a] = mul_p2(mul_p2(v[a + 1], -g.ky - 1, hsy) + mul_p2(v[a], -g.ky - 1, hsy),
					g.ky, g.ihy);
			continue;
		}
		double vc = u[a];
		double hs = g.SX(i) * 0.5, hsp = g.SX(i + 1) * 0.5;
		fx[a] = (u[a + g.P] * hs + vc * hsp) / (hs + hsp);
		vc = v[a];
		hs = g.SY(j) * 0.5;
		hsp = g.SY(j + 1) * 0.5;
		fy[a] = (v[a + 1] * hs + vc * hsp) / (hs + hsp);
	}
	for (long k = t0; k < (long)g.ny + g.nx; k += stride) {
		if (k < g.ny) {
			const int j = (int)k, a = g.at(0, j);
			const double vc = u[a];
			const double hs = g.SX(0) * 0.5, hsm = g.SX(-1) * 0.5;
			fx[a - g.P] = p2 ? (u[a - g.P] * hs + vc * hsm) * g.ihx
			                 : (u[a - g.P] * hs + vc * hsm) / (hs + hsm);
		} else {
			const int i = (int)(k - g.ny), a = g.at(i, 0);
			const double vc = v[a];
			const double hs = g.SY(0) * 0.5, hsm = g.SY(-1) * 0.5;
			fy[a - 1] = p2 ? (v[a - 1] * hs + vc * hsm) * g.ihy
			               : (v[a - 1] * hs + vc * hsm) / (hs + hsm);
		}
	}
}

// face gradient of Operation_::Grad (s_operation.hpp:46-72) at x face (i, j)
// (between i and i+1; i = -1 is the low wall face, computed from cell 0)
// (with Geo::p2 the centre distance is +-h: multiply by +-1/h)
// PM: 1 a P2 grid, 0 not, -1 read Geo::p2 (the compile-time forms keep the
// other branch's divisions out of the FP64 pipe). gx_in / gy_in: the
// interior faces (i >= 0, j >= 0).
// (the multiplications by +-1/h as exponent moves, mul_p2; x * -s is
// -(x * s))
template<int PM = -1>
__device__ __forceinline__ double gx_in(const Geo& g, const double* phi, int i, int j) {
	if (PM == 1 || (PM < 0 && g.p2))
		return mul_p2(phi[g.at(i + 1, j)] - phi[g.at(i, j)], g.kx, g.ihx);
	return (phi[g.at(i + 1, j)] - phi[g.at(i, j)]) / (g.CX(i + 1) - g.CX(i));
}
template<int PM = -1>
__device__ __forceinline__ double gy_in(const Geo& g, const double* phi, int i, int j) {
	if (PM == 1 || (PM < 0 && g.p2))
		return mul_p2(phi[g.at(i, j + 1)] - phi[g.at(i, j)], g.ky, g.ihy);
	return (phi[g.at(i, j + 1)] - phi[g.at(i, j)]) / (g.CY(j + 1) - g.CY(j));
}
template<int PM = -1>
__device__ __forceinline__ double gx_at(const Geo& g, const double* phi, int i, int j) {
	if (i >= 0) return gx_in<PM>(g, phi, i, j);
	if (PM == 1 || (PM < 0 && g.p2))
		return neg_bits(mul_p2(phi[g.at(-1, j)] - phi[g.at(0, j)], g.kx, g.ihx));
	return (phi[g.at(-1, j)] - phi[g.at(0, j)]) / (g.CX(-1) - g.CX(0));
}
template<int PM = -1>
__device__ __forceinline__ double gy_at(const Geo& g, const double* phi, int i, int j) {
	if (j >= 0) return gy_in<PM>(g, phi, i, j);
	if (PM == 1 || (PM < 0 && g.p2))
		return neg_bits(mul_p2(phi[g.at(i, -1)] - phi[g.at(i, 0)], g.ky, g.ihy));
	return (phi[g.at(i, -1)] - phi[g.at(i, 0)]) / (g.CY(-1) - g.CY(0));
}

// The end of run_one_step (s_ns_explicit.hpp:140-153) over every array
// element: gradphi = Grad(phi); p = phi, p *= 1/dt on normal cells;
// uf = us_f - gradphi; u = us - InterpolateF2C(gradphi). The cells with
// i >= 1 and j >= 1 (every face gradient they read an interior one) run
// first without a branch; the rest of the array (ghost frame, row 0,
// column 0) after them in the general form, so that no predicated branch
// costs FP64 issue slots in the bulk.
template<int PM = -1>
__global__ void __launch_bounds__(kThreads) k_correct(Geo g, const double* phi,
		const double* us, const double* vs, const double* usf,
		const double* vsf, double* u, double* v, double* uf, double* vf,
		double* p, const StepScalars* ss) {
	const double inv = 1.0 / ss->dt;
	const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
	const long stride = (long)gridDim.x * blockDim.x;
	const int mx = g.nx - 1, my = g.ny - 1;
	const long nin = (long)mx * my;
	for (long k = t0; k < nin; k += stride) {
		const int i = 1 + (int)(k / my), j = 1 + (int)(k - (long)(i - 1) * my);
		const int a = g.at(i, j);
		const double gx = gx_in<PM>(g, phi, i, j), gy = gy_in<PM>(g, phi, i, j);
		uf[a] = usf[a] - gx;
		vf[a] = vsf[a] - gy;
		const double gcx = mul_p2(gx + gx_in<PM>(g, phi, i - 1, j), -1, 0.5);
		const double gcy = mul_p2(gy + gy_in<PM>(g, phi, i, j - 1), -1, 0.5);
		u[a] = us[a] - gcx;
		v[a] = vs[a] - gcy;
		p[a] = phi[a] * inv;
	}
	// the rest: full rows I <= gl and I >= gl + nx, then in the rows between
	// the columns J <= gl and J >= gl + ny
	const int gl = g.gl, NJ = g.NJ;
	const int top = gl + 1, bot = g.NI - gl - g.nx, left = gl + 1, right = NJ - gl - g.ny;
	const long full = (long)(top + bot) * NJ;
	const int W = left + right;
	const long rest = full + (long)mx * W;
	for (long k = t0; k < rest; k += stride) {
		int I, J;
		if (k < full) {
			const int r = (int)(k / NJ);
			J = (int)(k - (long)r * NJ);
			I = r < top ? r : gl + g.nx + (r - top);
		} else {
			const long t = k - full;
			const int m = (int)(t / W), c = (int)(t - (long)m * W);
			I = gl + 1 + m;
			J = c < left ? c : gl + g.ny + (c - left);
		}
		int i = I - g.gl, j = J - g.gl;
		int a = I * g.P + J;
		bool jin = j >= 0 && j < g.ny, iin = i >= 0 && i < g.nx;
		double gx = (jin && i >= -1 && i < g.nx) ? gx_at<PM>(g, phi, i, j) : 0.0;
		double gy = (iin && j >= -1 && j < g.ny) ? gy_at<PM>(g, phi, i, j) : 0.0;
		uf[a] = usf[a] - gx;
		vf[a] = vsf[a] - gy;
		double gcx = 0.0, gcy = 0.0;
		if (iin && jin) {
			gcx = (gx + gx_at<PM>(g, phi, i - 1, j)) * 0.5;
			gcy = (gy + gy_at<PM>(g, phi, i, j - 1)) * 0.5;
		}
		u[a] = us[a] - gcx;
		v[a] = vs[a] - gcy;
		p[a] = (iin && jin) ? phi[a] * inv : phi[a];
	}
}

// ------------------------------------------------------------- NS_kim_ --
// NS_kim_::_veo_star_center (s_ns_kim.hpp:188-242): the right-hand side of
// each component's Helmholtz predictor, over the normal cells,
//   adv = 1.5 adv(uf, u) - 0.5 adv(umf, um)   (adv(uf, u) alone on step 0)
//   scr = (adv - (0.5 NablaMuNabla(mu, u) + 0) / rho) dt - u
// um, umf: the velocities copied at the start of the step (before the
// ghost fill of u), as run_one_step does.
template<int SCH>
__global__ void __launch_bounds__(kThreads) k_kim_source(Geo g, const double* u,
		const double* v, const double* uf, const double* vf, const double* um,
		const double* vm, const double* umf, const double* vmf, double* xs,
		double* ys, const StepScalars* ss, double rho, double mu, int first) {
	const double dt = ss->dt;
	const long n = (long)g.nx * g.ny;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int a = g.at(i, j);
#pragma unroll
		for (int d = 0; d < 2; ++d) {
			const double* s = d == 0 ? u : v;
			const double* sm = d == 0 ? um : vm;
			double advn = adv_cell<SCH>(g, uf, vf, s, i, j);
			double dif = diffusion(g, mu, s, i, j);
			double src = 0.0;
			double veos;
			if (first) {
				veos = (advn - (0.5 * dif + src) / rho) * dt - s[a];
			} else {
				double advnm1 = adv_cell<SCH>(g, umf, vmf, sm, i, j);
				double adv = 1.5 * advn - 0.5 * advnm1;
				veos = (adv - (0.5 * dif + src) / rho) * dt - s[a];
			}
			(d == 0 ? xs : ys)[a] = veos;
		}
	}
}

// The end of NS_kim_::run_one_step (s_ns_kim.hpp:160-187) over every array
// element: as k_correct, with p = phi / dt - NablaMuNabla(mu, phi) 0.5 / rho
// on the normal cells, and the corrected velocities also written back into
// the star fields (the reference corrects them in place and copies).
__global__ void __launch_bounds__(kThreads) k_kim_correct(Geo g, const double* phi,
		double* us, double* vs, double* usf, double* vsf, double* u, double* v,
		double* uf, double* vf, double* p, const StepScalars* ss, double rho,
		double mu) {
	const double inv = 1.0 / ss->dt;
	const double c = 0.5 / rho;
	const long n = (long)g.NI * g.NJ;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int I = (int)(k / g.NJ), J = (int)(k - (long)I * g.NJ);
		int i = I - g.gl, j = J - g.gl;
		int a = I * g.P + J;
		bool jin = j >= 0 && j < g.ny, iin = i >= 0 && i < g.nx;
		double gx = (jin && i >= -1 && i < g.nx) ? gx_at(g, phi, i, j) : 0.0;
		double gy = (iin && j >= -1 && j < g.ny) ? gy_at(g, phi, i, j) : 0.0;
		double pv = phi[a];
		if (iin && jin) {
			pv = pv * inv;
			double lap = diffusion(g, mu, phi, i, j);
			lap = lap * c;
			pv = pv - lap;
		}
		p[a] = pv;
		double ufn = usf[a] - gx, vfn = vsf[a] - gy;
		double gcx = 0.0, gcy = 0.0;
		if (iin && jin) {
			gcx = (gx + gx_at(g, phi, i - 1, j)) * 0.5;
			gcy = (gy + gy_at(g, phi, i, j - 1)) * 0.5;
		}
		double un = us[a] - gcx, vn = vs[a] - gcy;
		usf[a] = ufn;
		vsf[a] = vfn;
		uf[a] = ufn;
		vf[a] = vfn;
		us[a] = un;
		vs[a] = vn;
		u[a] = un;
		v[a] = vn;
	}
}

// ----------------------------------------------------- single operators --
__global__ void k_op(Geo g, int which, int sch, double coef, const double* a,
		const double* b, const double* c, double* o1, double* o2) {
	const long n = (long)g.nx * g.ny;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		int i = (int)(k / g.ny), j = (int)(k - (long)i * g.ny);
		int x = g.at(i, j);
		switch (which) {
		case 0:
			o1[x] = gx_at(g, a, i, j);
			if (i == 0) o1[x - g.P] = gx_at(g, a, -1, j);
			o2[x] = gy_at(g, a, i, j);
			if (j == 0) o2[x - 1] = gy_at(g, a, i, -1);
			break;
		case 1: {
			double d = 0;
			d += (a[x] - a[x - g.P]) / g.SX(i);
			d += (b[x] - b[x - 1]) / g.SY(j);
			o1[x] = d;
			break;
		}
		case 2:
			o1[x] = (a[x] + a[x - g.P]) * 0.5;
			o2[x] = (b[x] + b[x - 1]) * 0.5;
			break;
		case 4: {
			double r = 0;
			switch (sch) {
#define CASE(S) case S: r = adv_cell<S>(g, a, b, c, i, j); break;
			CASE(CARPIO_GPU_UPWIND1) CASE(CARPIO_GPU_CENTER) CASE(CARPIO_GPU_CENTER4)
			CASE(CARPIO_GPU_UPWIND2) CASE(CARPIO_GPU_VANLEER) CASE(CARPIO_GPU_SUPERBEE)
			CASE(CARPIO_GPU_WAHYD) CASE(CARPIO_GPU_QUICK) CASE(CARPIO_GPU_CUI)
			CASE(CARPIO_GPU_MINMOD)
#undef CASE
			}
			o1[x] = r;
			break;
		}
		case 5:
			o1[x] = diffusion(g, coef, c, i, j);
			break;
		case 8:
			o1[x] = diffusion_var(g, a, c, i, j);
			break;
		}
	}
}

// ---------------------------------------------------------------- host --
Geo make_geo(const carpio_gpu_grid* g) {
	Geo e;
	e.nx = g->nx;
	e.ny = g->ny;
	e.gl = g->gl;
	e.P = g->P;
	e.NI = g->NI;
	e.NJ = g->NJ;
	e.cx = g->d_cx;
	e.sx = g->d_sx;
	e.cy = g->d_cy;
	e.sy = g->d_sy;
	// the power-of-two case (Geo::p2), checked on the host copies of the axes;
	// h within 2^+-90, so that scaling by 2h never leaves the exponent range
	// that tvd_ratio's shortcut checks
	auto pow2 = [](double h) {
		int ex = 0;
		return h > 0 && std::frexp(h, &ex) == 0.5 && ex >= -90 && ex <= 90;
	};
	auto axis_ok = [&](const std::vector<double>& c, const std::vector<double>& sz, double h) {
		if (!pow2(h)) return false;
		for (size_t k = 0; k < sz.size(); ++k)
			if (sz[k] != h) return false;
		for (size_t k = 0; k + 1 < c.size(); ++k)
			if (c[k + 1] - c[k] != h) return false;
		return true;
	};
	e.hx = g->sx.empty() ? 0.0 : g->sx[0];
	e.hy = g->sy.empty() ? 0.0 : g->sy[0];
	e.p2 = axis_ok(g->cx, g->sx, e.hx) && axis_ok(g->cy, g->sy, e.hy) ? 1 : 0;
	e.ihx = e.p2 ? 1.0 / e.hx : 0.0;
	e.ihy = e.p2 ? 1.0 / e.hy : 0.0;
	int ex = 0;
	e.kx = e.p2 ? (std::frexp(e.ihx, &ex), ex - 1) : 0;
	e.ky = e.p2 ? (std::frexp(e.ihy, &ex), ex - 1) : 0;
	return e;
}

BcDev to_dev(const carpio_gpu_bc& b, const double* gv = nullptr) {
	BcDev d;
	for (int k = 0; k < 4; ++k) {
		d.type[k] = b.type[k];
		d.value[k] = b.value[k];
	}
	d.gv = gv;
	return d;
}

int grid_blocks(long n) {
	long b = (n + kThreads - 1) / kThreads;
	long cap = (long)cg_host::sm_count() * 8;
	return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t launch_bc(const Geo& geo, double* f0, const carpio_gpu_bc& b0,
		double* f1, const carpio_gpu_bc* b1, cudaStream_t s,
		const double* gv0 = nullptr, const double* gv1 = nullptr) {
	BcFields bf;
	bf.f[0] = f0;
	bf.bc[0] = to_dev(b0, gv0);
	bf.f[1] = f1;
	bf.bc[1] = b1 ? to_dev(*b1, gv1) : bf.bc[0];
	size_t smem = sizeof(double) * 2 * geo.gl * geo.gl;
	const long rest = 2L * geo.gl * (geo.NI - 2 * geo.gl - 1) + 2L * geo.gl * (geo.NJ - 2 * geo.gl);
	const int parts = (int)std::max(1L, std::min(64L, (rest + 255) / 256));
	k_apply_bc<<<dim3(1 + parts, b1 ? 2 : 1), 256, smem, s>>>(geo, bf);
	return cudaGetLastError();
}

template<int SCH>
cudaError_t launch_pred(const Geo& geo, int blocks, cudaStream_t s,
		const double* u, const double* v, const double* uf, const double* vf,
		double* us, double* vs, const StepScalars* ss, double rho, double mu,
		const double* muf) {
	if (kTvdScheme<SCH> && geo.gl >= 2) {
		// the face-sharing tiles (k_predictor_tiles, whose stencils reach
		// two cells into the ghost ring); `blocks` sizes the one-cell-per-
		// thread kernel of the other cases
		const dim3 grid((geo.ny + kPredTJ - 1) / kPredTJ, (geo.nx + kPredTI - 1) / kPredTI);
		const FixedDiv rd = make_fixed_div(rho);
		const int diff = muf ? 0 : (mu == 1.0 ? 2 : 1);
#define PT(P, D) k_predictor_tiles<SCH, P, D><<<grid, kPredThreads, 0, s>>>(geo, u, v, uf, vf, \
		us, vs, ss, rd, mu, muf)
		if (geo.p2) {
			if (diff == 0) PT(true, 0);
			else if (diff == 1) PT(true, 1);
			else PT(true, 2);
		} else {
			if (diff == 0) PT(false, 0);
			else PT(false, 1);
		}
#undef PT
		return cudaGetLastError();
	}
	if (geo.p2)
		k_predictor<SCH, true><<<blocks, kThreads, 0, s>>>(geo, u, v, uf, vf, us, vs, ss, rho, mu, muf);
	else
		k_predictor<SCH, false><<<blocks, kThreads, 0, s>>>(geo, u, v, uf, vf, us, vs, ss, rho, mu, muf);
	return cudaGetLastError();
}

cudaError_t launch_predictor(int sch, const Geo& geo, int blocks, cudaStream_t s,
		const double* u, const double* v, const double* uf, const double* vf,
		double* us, double* vs, const StepScalars* ss, double rho, double mu,
		const double* muf) {
	switch (sch) {
#define CASE(S) case S: return launch_pred<S>(geo, blocks, s, u, v, uf, vf, us, vs, ss, rho, \
		mu, muf);
	CASE(CARPIO_GPU_UPWIND1) CASE(CARPIO_GPU_CENTER) CASE(CARPIO_GPU_CENTER4)
	CASE(CARPIO_GPU_UPWIND2) CASE(CARPIO_GPU_VANLEER) CASE(CARPIO_GPU_SUPERBEE)
	CASE(CARPIO_GPU_WAHYD) CASE(CARPIO_GPU_QUICK) CASE(CARPIO_GPU_CUI)
	CASE(CARPIO_GPU_MINMOD)
#undef CASE
	}
	return cudaErrorInvalidValue;
}

template<int SCH>
cudaError_t launch_kim_src(const Geo& geo, int blocks, cudaStream_t s, const double* u,
		const double* v, const double* uf, const double* vf, const double* um,
		const double* vm, const double* umf, const double* vmf, double* xs,
		double* ys, const StepScalars* ss, double rho, double mu, int first) {
	k_kim_source<SCH><<<blocks, kThreads, 0, s>>>(geo, u, v, uf, vf, um, vm, umf, vmf,
			xs, ys, ss, rho, mu, first);
	return cudaGetLastError();
}

cudaError_t launch_kim_source(int sch, const Geo& geo, int blocks, cudaStream_t s,
		const double* u, const double* v, const double* uf, const double* vf,
		const double* um, const double* vm, const double* umf, const double* vmf,
		double* xs, double* ys, const StepScalars* ss, double rho, double mu, int first) {
	switch (sch) {
#define CASE(S) case S: return launch_kim_src<S>(geo, blocks, s, u, v, uf, vf, um, vm, \
		umf, vmf, xs, ys, ss, rho, mu, first);
	CASE(CARPIO_GPU_UPWIND1) CASE(CARPIO_GPU_CENTER) CASE(CARPIO_GPU_CENTER4)
	CASE(CARPIO_GPU_UPWIND2) CASE(CARPIO_GPU_VANLEER) CASE(CARPIO_GPU_SUPERBEE)
	CASE(CARPIO_GPU_WAHYD) CASE(CARPIO_GPU_QUICK) CASE(CARPIO_GPU_CUI)
	CASE(CARPIO_GPU_MINMOD)
#undef CASE
	}
	return cudaErrorInvalidValue;
}

template<int S>
const void* advect_band_kernel(bool p2) {
	return p2 ? (const void*)k_advect_band<S, true> : (const void*)k_advect_band<S, false>;
}

const void* pick_advect_band(int sch, bool p2) {
	switch (sch) {
	case CARPIO_GPU_UPWIND1: return advect_band_kernel<CARPIO_GPU_UPWIND1>(p2);
	case CARPIO_GPU_CENTER: return advect_band_kernel<CARPIO_GPU_CENTER>(p2);
	case CARPIO_GPU_CENTER4: return advect_band_kernel<CARPIO_GPU_CENTER4>(p2);
	case CARPIO_GPU_UPWIND2: return advect_band_kernel<CARPIO_GPU_UPWIND2>(p2);
	case CARPIO_GPU_VANLEER: return advect_band_kernel<CARPIO_GPU_VANLEER>(p2);
	case CARPIO_GPU_SUPERBEE: return advect_band_kernel<CARPIO_GPU_SUPERBEE>(p2);
	case CARPIO_GPU_WAHYD: return advect_band_kernel<CARPIO_GPU_WAHYD>(p2);
	case CARPIO_GPU_QUICK: return advect_band_kernel<CARPIO_GPU_QUICK>(p2);
	case CARPIO_GPU_CUI: return advect_band_kernel<CARPIO_GPU_CUI>(p2);
	}
	return nullptr;
}

// the row sweep's kernel for a scheme and its block size (threads)
template<int S>
const void* advect_rows_kernel(bool p2, int& threads) {
	constexpr int nf = kTvdScheme<S> ? 4 : 1;
	threads = kAdvBands * nf * 32;
	return p2 ? (const void*)k_advect_rows<S, true, kAdvRows, kAdvBands, nf>
	          : (const void*)k_advect_rows<S, false, kAdvRows, kAdvBands, nf>;
}

const void* pick_advect_rows(int sch, bool p2, int& threads) {
	switch (sch) {
	case CARPIO_GPU_UPWIND1: return advect_rows_kernel<CARPIO_GPU_UPWIND1>(p2, threads);
	case CARPIO_GPU_CENTER: return advect_rows_kernel<CARPIO_GPU_CENTER>(p2, threads);
	case CARPIO_GPU_CENTER4: return advect_rows_kernel<CARPIO_GPU_CENTER4>(p2, threads);
	case CARPIO_GPU_UPWIND2: return advect_rows_kernel<CARPIO_GPU_UPWIND2>(p2, threads);
	case CARPIO_GPU_VANLEER: return advect_rows_kernel<CARPIO_GPU_VANLEER>(p2, threads);
	case CARPIO_GPU_SUPERBEE: return advect_rows_kernel<CARPIO_GPU_SUPERBEE>(p2, threads);
	case CARPIO_GPU_WAHYD: return advect_rows_kernel<CARPIO_GPU_WAHYD>(p2, threads);
	case CARPIO_GPU_QUICK: return advect_rows_kernel<CARPIO_GPU_QUICK>(p2, threads);
	case CARPIO_GPU_CUI: return advect_rows_kernel<CARPIO_GPU_CUI>(p2, threads);
	}
	return nullptr;
}

cudaError_t launch_advect(int sch, const Geo& geo, cudaStream_t s, double* phi,
		const BcDev& bc, const double* uf, const double* vf, double dt, int steps) {
	const size_t smem = sizeof(double) * 2 * geo.gl * geo.gl;
	switch (sch) {
#define CASE(S) case S: \
		if (geo.p2) k_advect<S, true><<<1, 1024, smem, s>>>(geo, phi, bc, uf, vf, dt, steps); \
		else k_advect<S, false><<<1, 1024, smem, s>>>(geo, phi, bc, uf, vf, dt, steps); \
		return cudaGetLastError();
	CASE(CARPIO_GPU_UPWIND1) CASE(CARPIO_GPU_CENTER) CASE(CARPIO_GPU_CENTER4)
	CASE(CARPIO_GPU_UPWIND2) CASE(CARPIO_GPU_VANLEER) CASE(CARPIO_GPU_SUPERBEE)
	CASE(CARPIO_GPU_WAHYD) CASE(CARPIO_GPU_QUICK) CASE(CARPIO_GPU_CUI)
#undef CASE
	}
	return cudaErrorInvalidValue;
}

bool valid_bc(const carpio_gpu_bc& b) {
	for (int k = 0; k < 4; ++k)
		if (b.type[k] != 1 && b.type[k] != 2) return false;
	return true;
}

}  // namespace

struct carpio_gpu_ns {
	carpio_gpu_grid* g;
	carpio_gpu_ns_cfg cfg;
	cg_host::DevBuf fields;       // u v uf vf phi p us vs usf vsf
	double* f[10];
	cg_host::DevBuf stage;        // set_state: host fields, rows contiguous
	cg_host::DevBuf scal;         // StepScalars
	cg_host::DevBuf rec, rec_dt;  // per-step records
	cg_host::StencilCoeffs coeffs;
	cg_host::PoissonWs pws;
	cudaStream_t s;
	DtRule rule;
	double t_host = 0;
	// per-step events of the last run: [step start, solve start, solve end]
	std::vector<cudaEvent_t> ev;
	std::vector<cg_dev::SolveOut> last_rec;
	int last_steps = 0;
	// the projection with the learned preconditioner (carpio_gpu_ns_set_learned)
	carpio_gpu_unet* net = nullptr;
	carpio_gpu_learned_cfg lcfg{};
	bool learned = false;
	cg_host::LearnedWs lws;
	// NS_kim_ stepping (carpio_gpu_ns_set_stepper)
	int stepper = CARPIO_GPU_STEPPER_EXPLICIT;
	cg_host::DevBuf kim_fields;   // um vm umf vmf xscr yscr
	double* k[6] = {};
	cg_host::StencilCoeffs kim_coeffs;   // the predictor's Helmholtz rows
	cg_host::DevBuf kim_out;      // SolveOut of the predictor solves
	long steps_done = 0;          // Time_::current_step
	// a mu field in place of the uniform mu (carpio_gpu_ns_set_mu_field)
	cg_host::DevBuf muf;
	bool has_mu = false;
	~carpio_gpu_ns() {
		for (cudaEvent_t e : ev) cudaEventDestroy(e);
	}
};

extern "C" {

int carpio_gpu_ns_create(carpio_gpu_grid* g, const carpio_gpu_ns_cfg* cfg,
		double dt0, carpio_gpu_ns** out) {
	using namespace cg_host;
	if (!g || !cfg || !out || !(dt0 > 0) || g->gl < 2 || cfg->scheme < 0
			|| cfg->scheme > 9 || !valid_bc(cfg->bc_u) || !valid_bc(cfg->bc_v)
			|| !(cfg->rho != 0))
		return CARPIO_GPU_EINVAL;
	// the projection: CG (the drop-in) or Dia_BiCGSTAB / BiCGSTAB, in either
	// precision, or the shipped IC_CGS / IC_CG (FP64; solved synchronously
	// through the CSR layer)
	const int pk = cfg->projection.kind;
	const bool krylov = pk == CARPIO_GPU_CG || pk == CARPIO_GPU_DIA_BICGSTAB
			|| pk == CARPIO_GPU_BICGSTAB;
	if (!krylov && !((pk == CARPIO_GPU_IC_CGS || pk == CARPIO_GPU_IC_CG)
			&& cfg->projection.precision == CARPIO_GPU_FP64))
		return CARPIO_GPU_EINVAL;
	*out = nullptr;
	carpio_gpu_ns* ns = new carpio_gpu_ns();
	ns->g = g;
	g->refs.fetch_add(1);   // the grid outlives every NS handle built on it
	ns->cfg = *cfg;
	ns->s = g->stream;
	const size_t NF = (size_t)g->NI * g->P;
	if (ns->fields.ensure(sizeof(double) * NF * 10) || ns->scal.ensure(sizeof(StepScalars))) {
		delete ns;
		cg_host::grid_release(g);
		return CARPIO_GPU_ENOMEM;
	}
	for (int k = 0; k < 10; ++k) ns->f[k] = ns->fields.as<double>() + k * NF;
	StepScalars ss;
	std::memset(&ss, 0, sizeof ss);
	ss.dt = dt0;
	if (cudaMemsetAsync(ns->fields.p, 0, ns->fields.bytes, ns->s) != cudaSuccess
			|| cudaMemcpyAsync(ns->scal.p, &ss, sizeof ss, cudaMemcpyHostToDevice, ns->s) != cudaSuccess
			|| cudaStreamSynchronize(ns->s) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		delete ns;
		cg_host::grid_release(g);
		return CARPIO_GPU_ECUDA;
	}
	// Grid_::min_size (s_grid.hpp:173-185), cell sizes incl. ghosts
	double mx = 1.79769313486231570815e308, my = mx;
	for (double v : g->sx) mx = smin(mx, v);
	for (double v : g->sy) my = smin(my, v);
	ns->rule.cfl = cfg->cfl;
	ns->rule.diff_number = cfg->diff_number;
	ns->rule.diff_coef = cfg->diff_coef;
	ns->rule.minx = mx;
	ns->rule.miny = my;
	ns->rule.mins = smin(smin(1.79769313486231570815e308, mx), my);
	*out = ns;
	return 0;
}

int carpio_gpu_ns_destroy(carpio_gpu_ns* ns) {
	if (!ns) return CARPIO_GPU_EINVAL;
	cudaStreamSynchronize(ns->s);
	carpio_gpu_grid* g = ns->g;
	delete ns;
	cg_host::grid_release(g);
	return 0;
}

// set_state's staged fields: row-contiguous copies (NJ per row) into the
// fields at the device pitch P, one field per blockIdx.y
struct StageSet {
	const double* src[6];
	double* dst[6];
	int n;
};

__global__ void __launch_bounds__(kThreads) k_unstage(StageSet st, int NI, int NJ, int P) {
	const double* src = st.src[blockIdx.y];
	double* dst = st.dst[blockIdx.y];
	const long n = (long)NI * NJ;
	for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n;
			k += (long)gridDim.x * blockDim.x) {
		const int I = (int)(k / NJ), J = (int)(k - (long)I * NJ);
		dst[(long)I * P + J] = src[k];
	}
}

static int copy_field(carpio_gpu_grid* g, double* dst, const double* src,
		bool to_dev, cudaStream_t s) {
	const size_t wb = sizeof(double) * g->NJ, pb = sizeof(double) * g->P;
	if (to_dev) CG_CK(cudaMemcpy2DAsync(dst, pb, src, wb, wb, g->NI, cudaMemcpyDefault, s));
	else CG_CK(cudaMemcpy2DAsync(dst, wb, src, pb, wb, g->NI, cudaMemcpyDefault, s));
	return 0;
}

int carpio_gpu_ns_set_state(carpio_gpu_ns* ns, double dt, const double* u,
		const double* v, const double* uf, const double* vf,
		const double* phi, const double* p) {
	if (!ns || !(dt > 0)) return CARPIO_GPU_EINVAL;
	const double* in[6] = { u, v, uf, vf, phi, p };
	// host fields: one contiguous copy each into the staging buffer (the
	// pitched copy of the NI rows ran about 60 % slower over the host
	// link), then one kernel that lays the rows out at the device pitch;
	// device fields: the pitched device-to-device copy
	carpio_gpu_grid* g = ns->g;
	const size_t nf = (size_t)g->NI * g->NJ;
	StageSet st{};
	for (int k = 0; k < 6; ++k) {
		if (!in[k]) continue;
		if (cg_host::is_device_ptr(in[k])) {
			int rc = copy_field(g, ns->f[k], in[k], true, ns->s);
			if (rc) return rc;
			continue;
		}
		if (!ns->stage.p) {
			int rc = ns->stage.ensure(sizeof(double) * nf * 6);
			if (rc) return rc;
		}
		double* sk = ns->stage.as<double>() + (size_t)k * nf;
		CG_CK(cudaMemcpyAsync(sk, in[k], sizeof(double) * nf, cudaMemcpyHostToDevice, ns->s));
		st.src[st.n] = sk;
		st.dst[st.n] = ns->f[k];
		++st.n;
	}
	if (st.n > 0) {
		k_unstage<<<dim3(grid_blocks((long)nf), st.n), kThreads, 0, ns->s>>>(st, g->NI, g->NJ, g->P);
		CG_CK(cudaGetLastError());
	}
	CG_CK(cudaMemcpyAsync(&((StepScalars*)ns->scal.p)->dt, &dt, sizeof dt,
			cudaMemcpyHostToDevice, ns->s));
	CG_CK(cudaStreamSynchronize(ns->s));
	return 0;
}

int carpio_gpu_ns_get_state(carpio_gpu_ns* ns, double* dt, double* u,
		double* v, double* uf, double* vf, double* phi, double* p) {
	if (!ns) return CARPIO_GPU_EINVAL;
	double* out[6] = { u, v, uf, vf, phi, p };
	for (int k = 0; k < 6; ++k) {
		if (!out[k]) continue;
		int rc = copy_field(ns->g, out[k], ns->f[k], false, ns->s);
		if (rc) return rc;
	}
	if (dt)
		CG_CK(cudaMemcpyAsync(dt, &((StepScalars*)ns->scal.p)->dt, sizeof *dt,
				cudaMemcpyDeviceToHost, ns->s));
	CG_CK(cudaStreamSynchronize(ns->s));
	return 0;
}

int carpio_gpu_ns_run(carpio_gpu_ns* ns, int steps, double* step_dt,
		int* step_iters, double* step_resid) {
	using namespace cg_host;
	if (!ns || steps < 0) return CARPIO_GPU_EINVAL;
	if (steps == 0) return 0;
	carpio_gpu_grid* g = ns->g;
	cudaStream_t s = ns->s;
	int rc;
	carpio_gpu_bc bc_phi;
	for (int k = 0; k < 4; ++k) { bc_phi.type[k] = 2; bc_phi.value[k] = 0.0; }
	if ((rc = stencil_prepare(g, bc_phi, 1.0, ns->coeffs, s))) return rc;
	if ((rc = ns->rec.ensure(sizeof(cg_dev::SolveOut) * (size_t)steps))) return rc;
	if ((rc = ns->rec_dt.ensure(sizeof(double) * (size_t)steps))) return rc;
	const Geo geo = make_geo(g);
	double *u = ns->f[0], *v = ns->f[1], *uf = ns->f[2], *vf = ns->f[3],
		   *phi = ns->f[4], *p = ns->f[5], *us = ns->f[6], *vs = ns->f[7],
		   *usf = ns->f[8], *vsf = ns->f[9];
	StepScalars* ss = ns->scal.as<StepScalars>();
	const int nb = grid_blocks((long)g->nx * g->ny);
	const int nbf = grid_blocks((long)g->NI * g->NJ);
	const carpio_gpu_ns_cfg& c = ns->cfg;
	cg_dev::SolveOut* rec = ns->rec.as<cg_dev::SolveOut>();
	const size_t nev = 3 * (size_t)steps + 1;
	while (ns->ev.size() < nev) {
		cudaEvent_t e;
		CG_CK(cudaEventCreate(&e));
		ns->ev.push_back(e);
	}
	const bool kim = ns->stepper == CARPIO_GPU_STEPPER_KIM;
	carpio_gpu_solver_cfg jcfg{};
	cg_dev::SolveOut* kout = nullptr;
	if (kim) {
		// the predictor's Poisson_ (s_ns_kim.hpp:104, 232-235): Helmholtz rows
		// with alpha 1 and uniform beta dt 0.5 / rho, its own (default,
		// Neumann 0) boundary conditions for "phi", the default solver
		// Solver_Jacobi_ with max_iter 1000 and tolerance 1e-4 (s_solver.hpp:73-74)
		double dt;
		CG_CK(cudaMemcpyAsync(&dt, &ss->dt, sizeof dt, cudaMemcpyDeviceToHost, s));
		CG_CK(cudaStreamSynchronize(s));
		const double smu = dt * 0.5 / c.rho;
		carpio_gpu_bc bc_n;
		for (int k = 0; k < 4; ++k) { bc_n.type[k] = 2; bc_n.value[k] = 0.0; }
		if ((rc = stencil_prepare(g, bc_n, smu, ns->kim_coeffs, s, true, 1.0))) return rc;
		if ((rc = ns->kim_out.ensure(2 * sizeof(cg_dev::SolveOut)))) return rc;
		kout = ns->kim_out.as<cg_dev::SolveOut>();
		jcfg.kind = CARPIO_GPU_JACOBI;
		jcfg.precision = CARPIO_GPU_FP64;
		jcfg.max_iter = 1000;
		jcfg.tol = 1e-4;
	}
	const size_t fbytes = sizeof(double) * (size_t)g->NI * g->P;
	for (int st = 0; st < steps; ++st) {
		CG_CK(cudaEventRecord(ns->ev[3 * st], s));
		if (kim) {
			// NS_kim_::run_one_step (s_ns_kim.hpp:125-187): no restrict_time
			double* um = ns->k[0];
			double* vm = ns->k[1];
			double* umf = ns->k[2];
			double* vmf = ns->k[3];
			double* xs = ns->k[4];
			double* ys = ns->k[5];
			CG_CK(cudaMemcpyAsync(ns->rec_dt.as<double>() + st, &ss->dt, sizeof(double),
					cudaMemcpyDeviceToDevice, s));
			CG_CK(cudaMemcpyAsync(um, u, fbytes, cudaMemcpyDeviceToDevice, s));
			CG_CK(cudaMemcpyAsync(vm, v, fbytes, cudaMemcpyDeviceToDevice, s));
			CG_CK(cudaMemcpyAsync(umf, uf, fbytes, cudaMemcpyDeviceToDevice, s));
			CG_CK(cudaMemcpyAsync(vmf, vf, fbytes, cudaMemcpyDeviceToDevice, s));
			CG_CK(launch_bc(geo, u, c.bc_u, v, &c.bc_v, s));
			CG_CK(launch_kim_source(c.scheme, geo, nb, s, u, v, uf, vf, um, vm, umf, vmf,
					xs, ys, ss, c.rho, c.mu, ns->steps_done == 0 ? 1 : 0));
			if ((rc = poisson_launch(g, ns->kim_coeffs, ns->pws, SRC_FIELD, xs, nullptr, us,
					jcfg, nullptr, 0, kout, s)))
				return rc;
			if ((rc = poisson_launch(g, ns->kim_coeffs, ns->pws, SRC_FIELD, ys, nullptr, vs,
					jcfg, nullptr, 0, kout + 1, s)))
				return rc;
			CG_CK(launch_bc(geo, us, c.bc_u, vs, &c.bc_v, s));
			k_c2f<<<nb, kThreads, 0, s>>>(geo, us, vs, usf, vsf);
			CG_CK(cudaGetLastError());
			CG_CK(cudaEventRecord(ns->ev[3 * st + 1], s));
			if ((rc = poisson_launch(g, ns->coeffs, ns->pws, SRC_DIV, usf, vsf, phi,
					c.projection, nullptr, 0, rec + st, s)))
				return rc;
			CG_CK(cudaEventRecord(ns->ev[3 * st + 2], s));
			CG_CK(launch_bc(geo, phi, bc_phi, nullptr, nullptr, s));
			k_kim_correct<<<nbf, kThreads, 0, s>>>(geo, phi, us, vs, usf, vsf, u, v, uf,
					vf, p, ss, c.rho, c.mu);
			CG_CK(cudaGetLastError());
			++ns->steps_done;
			continue;
		}
		k_restrict_time<<<nb, kThreads, 0, s>>>(geo, u, v, ss, ns->rule,
				ns->rec_dt.as<double>(), st);
		CG_CK(cudaGetLastError());
		CG_CK(launch_bc(geo, u, c.bc_u, v, &c.bc_v, s));
		CG_CK(launch_predictor(c.scheme, geo, nb, s, u, v, uf, vf, us, vs, ss, c.rho, c.mu,
				ns->has_mu ? ns->muf.as<double>() : nullptr));
		CG_CK(launch_bc(geo, us, c.bc_u, vs, &c.bc_v, s));
		if (geo.p2) k_c2f<1><<<nb, kThreads, 0, s>>>(geo, us, vs, usf, vsf);
		else k_c2f<0><<<nb, kThreads, 0, s>>>(geo, us, vs, usf, vsf);
		CG_CK(cudaGetLastError());
		CG_CK(cudaEventRecord(ns->ev[3 * st + 1], s));
		if (ns->learned) {
			cg_dev::SolveOut o;
			if ((rc = learned_solve(g, ns->coeffs, ns->pws, ns->lws, SRC_DIV, usf, vsf, phi,
					c.projection, ns->net, ns->lcfg, o, s)))
				return rc;
			CG_CK(cudaMemcpyAsync(rec + st, &o, sizeof o, cudaMemcpyHostToDevice, s));
		} else if ((rc = poisson_launch(g, ns->coeffs, ns->pws, SRC_DIV, usf, vsf, phi,
				c.projection, nullptr, 0, rec + st, s))) {
			return rc;
		}
		CG_CK(cudaEventRecord(ns->ev[3 * st + 2], s));
		CG_CK(launch_bc(geo, phi, bc_phi, nullptr, nullptr, s));
		if (geo.p2)
			k_correct<1><<<nbf, kThreads, 0, s>>>(geo, phi, us, vs, usf, vsf, u, v, uf, vf, p, ss);
		else
			k_correct<0><<<nbf, kThreads, 0, s>>>(geo, phi, us, vs, usf, vsf, u, v, uf, vf, p, ss);
		CG_CK(cudaGetLastError());
		++ns->steps_done;
	}
	CG_CK(cudaEventRecord(ns->ev[3 * steps], s));
	std::vector<cg_dev::SolveOut> h(steps);
	std::vector<double> hdt(steps);
	CG_CK(cudaMemcpyAsync(h.data(), rec, sizeof(cg_dev::SolveOut) * steps,
			cudaMemcpyDeviceToHost, s));
	CG_CK(cudaMemcpyAsync(hdt.data(), ns->rec_dt.p, sizeof(double) * steps,
			cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	int first = 0;
	if (kim) {
		// the predictor's own result codes are not checked by the reference
		// (a Jacobi that reaches max_iter is kept); device errors are
		cg_dev::SolveOut ko[2];
		CG_CK(cudaMemcpy(ko, kout, sizeof ko, cudaMemcpyDeviceToHost));
		for (const cg_dev::SolveOut& o : ko)
			if (o.code < 0) return o.code;
	}
	for (int st = 0; st < steps; ++st) {
		if (step_dt) step_dt[st] = hdt[st];
		if (step_iters) step_iters[st] = h[st].iters;
		if (step_resid) step_resid[st] = h[st].tol;
		if (!first && h[st].code) first = h[st].code;
		ns->t_host += hdt[st];
	}
	ns->last_rec = h;
	ns->last_steps = steps;
	return first;
}

int carpio_gpu_ns_set_stepper(carpio_gpu_ns* ns, int stepper) {
	using namespace cg_host;
	if (!ns || (stepper != CARPIO_GPU_STEPPER_EXPLICIT && stepper != CARPIO_GPU_STEPPER_KIM))
		return CARPIO_GPU_EINVAL;
	if (stepper == CARPIO_GPU_STEPPER_KIM) {
		if (ns->learned || ns->has_mu) return CARPIO_GPU_EINVAL;
		carpio_gpu_grid* g = ns->g;
		const size_t fn = (size_t)g->NI * g->P;
		if (!ns->kim_fields.p) {
			int rc = ns->kim_fields.ensure(sizeof(double) * 6 * fn);
			if (rc) return rc;
			CG_CK(cudaMemsetAsync(ns->kim_fields.p, 0, ns->kim_fields.bytes, ns->s));
			CG_CK(cudaStreamSynchronize(ns->s));
		}
		for (int k = 0; k < 6; ++k) ns->k[k] = ns->kim_fields.as<double>() + k * fn;
	}
	ns->stepper = stepper;
	return 0;
}

int carpio_gpu_ns_set_mu_field(carpio_gpu_ns* ns, const double* mu) {
	if (!ns || ns->stepper != CARPIO_GPU_STEPPER_EXPLICIT) return CARPIO_GPU_EINVAL;
	if (!mu) {
		ns->has_mu = false;
		return 0;
	}
	carpio_gpu_grid* g = ns->g;
	int rc;
	if ((rc = ns->muf.ensure(sizeof(double) * (size_t)g->NI * g->P))) return rc;
	if ((rc = copy_field(g, ns->muf.as<double>(), mu, true, ns->s))) return rc;
	CG_CK(cudaStreamSynchronize(ns->s));
	ns->has_mu = true;
	return 0;
}

int carpio_gpu_ns_set_learned(carpio_gpu_ns* ns, carpio_gpu_unet* net,
		const carpio_gpu_learned_cfg* lc) {
	using namespace cg_host;
	if (!ns) return CARPIO_GPU_EINVAL;
	if (!net && (!lc || lc->use_net)) {
		ns->learned = false;
		ns->net = nullptr;
		return 0;
	}
	if (!lc || (lc->use_net && (!net || !learned_shape_ok(ns->g->nx, ns->g->ny))))
		return CARPIO_GPU_EINVAL;
	ns->net = net;
	ns->lcfg = *lc;
	ns->learned = true;
	return 0;
}

int carpio_gpu_ns_profile(carpio_gpu_ns* ns, int cap, int* n,
		double* solve_ms, double* step_ms, int* inner_iters, int* outer_iters) {
	if (!ns || cap < 0) return CARPIO_GPU_EINVAL;
	int m = ns->last_steps < cap ? ns->last_steps : cap;
	if (n) *n = ns->last_steps;
	for (int st = 0; st < m; ++st) {
		float a = 0, b = 0;
		CG_CK(cudaEventElapsedTime(&a, ns->ev[3 * st + 1], ns->ev[3 * st + 2]));
		CG_CK(cudaEventElapsedTime(&b, ns->ev[3 * st], ns->ev[3 * st + 3]));
		if (solve_ms) solve_ms[st] = a;
		if (step_ms) step_ms[st] = b;
		const cg_dev::SolveOut& o = ns->last_rec[st];
		// learned: all iterations (flexible CG + fallback) and the flexible
		// CG's alone; mixed: FP32 iterations and FP64 refinements
		bool mixed = ns->cfg.projection.precision == CARPIO_GPU_MIXED;
		if (inner_iters) inner_iters[st] = ns->learned ? o.iters : mixed ? o.inner : o.iters;
		if (outer_iters) outer_iters[st] = (ns->learned || mixed) ? o.outer : 0;
	}
	return 0;
}

int carpio_gpu_operator(carpio_gpu_grid* g, int which, int scheme,
		double coef, const carpio_gpu_bc* bc, const double* a,
		const double* b, const double* c, double* out1, double* out2,
		double* scalar) {
	using namespace cg_host;
	if (!g || which < 0 || which > 9) return CARPIO_GPU_EINVAL;
	if (which == 8 && (!a || !c)) return CARPIO_GPU_EINVAL;
	if ((which == 4 || which == 9) && (scheme < 0 || scheme > 9 || g->gl < (scheme >= 2 ? 2 : 1)))
		return CARPIO_GPU_EINVAL;
	if (which == 9 && (!a || !b || !c || !out1)) return CARPIO_GPU_EINVAL;
	if (which == 6 && (!bc || !valid_bc(*bc) || !out1)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(g->mu);
	cudaStream_t s = g->stream;
	const size_t NF = (size_t)g->NI * g->P;
	DevBuf buf;
	int rc;
	if ((rc = buf.ensure(sizeof(double) * NF * 5))) return rc;
	double* d[5];
	for (int k = 0; k < 5; ++k) d[k] = buf.as<double>() + k * NF;
	CG_CK(cudaMemsetAsync(buf.p, 0, buf.bytes, s));
	const double* in[3] = { a, b, c };
	for (int k = 0; k < 3; ++k)
		if (in[k] && (rc = copy_field(g, d[k], in[k], true, s))) return rc;
	if (which == 3) {  // C2F writes into the caller's face arrays
		if (out1 && (rc = copy_field(g, d[3], out1, true, s))) return rc;
		if (out2 && (rc = copy_field(g, d[4], out2, true, s))) return rc;
	}
	if (which == 6 && (rc = copy_field(g, d[3], out1, true, s))) return rc;
	const Geo geo = make_geo(g);
	const int nb = grid_blocks((long)g->nx * g->ny);
	if (which == 3) {
		k_c2f<<<nb, kThreads, 0, s>>>(geo, d[0], d[1], d[3], d[4]);
	} else if (which == 6) {
		CG_CK(launch_bc(geo, d[3], *bc, nullptr, nullptr, s));
	} else if (which == 7) {
		DevBuf mb;
		if ((rc = mb.ensure(sizeof(unsigned long long)))) return rc;
		CG_CK(cudaMemsetAsync(mb.p, 0, sizeof(unsigned long long), s));
		k_maxmag<<<nb, kThreads, 0, s>>>(geo, d[0], d[1], mb.as<unsigned long long>());
		CG_CK(cudaGetLastError());
		unsigned long long bits = 0;
		CG_CK(cudaMemcpyAsync(&bits, mb.p, sizeof bits, cudaMemcpyDeviceToHost, s));
		CG_CK(cudaStreamSynchronize(s));
		double mxm;
		std::memcpy(&mxm, &bits, sizeof mxm);
		if (scalar) *scalar = mxm;
		return 0;
	} else if (which == 9) {
		// the projection step's predictor on one field, dt = 1, rho from
		// *scalar (default 1): the kernel of the step itself (both
		// components of it given the field)
		const double rho = scalar && *scalar != 0.0 ? *scalar : 1.0;
		StepScalars hs{};
		hs.dt = 1.0;
		DevBuf sb;
		if ((rc = sb.ensure(sizeof(StepScalars)))) return rc;
		CG_CK(cudaMemcpyAsync(sb.p, &hs, sizeof hs, cudaMemcpyHostToDevice, s));
		CG_CK(launch_predictor(scheme, geo, nb, s, d[2], d[2], d[0], d[1], d[3], d[4],
				sb.as<StepScalars>(), rho, coef, nullptr));
		CG_CK(cudaStreamSynchronize(s));
	} else {
		k_op<<<nb, kThreads, 0, s>>>(geo, which, scheme, coef, d[0], d[1], d[2], d[3], d[4]);
	}
	CG_CK(cudaGetLastError());
	if (out1 && (rc = copy_field(g, out1, d[3], false, s))) return rc;
	if (out2 && which != 1 && which != 4 && which != 5 && which != 6 && which != 8 && which != 9
			&& (rc = copy_field(g, out2, d[4], false, s)))
		return rc;
	CG_CK(cudaStreamSynchronize(s));
	return 0;
}

}  // extern "C"

// ----------------------------------------------- stand-alone Advection_ --
struct carpio_gpu_advection {
	carpio_gpu_grid* g;
	cg_host::LaunchWs lw;     // control words of the band sweep
	cg_host::DevBuf prog;     // its progress word per band
	cg_host::DevBuf fields;   // u v uf vf phi, then the ghost values of u v phi
	double* f[8];
	carpio_gpu_bc bc[3];      // u v phi
	bool has_gv[3] = {};
	int scheme = CARPIO_GPU_UPWIND1;   // Advection_::_default_setup
	bool ready = false;                // initial() done
	cudaStream_t s;
};

extern "C" {

int carpio_gpu_advection_create(carpio_gpu_grid* g, carpio_gpu_advection** out) {
	using namespace cg_host;
	if (!g || !out) return CARPIO_GPU_EINVAL;
	*out = nullptr;
	carpio_gpu_advection* a = new carpio_gpu_advection();
	a->g = g;
	g->refs.fetch_add(1);
	a->s = g->stream;
	for (int k = 0; k < 3; ++k)
		for (int sg = 0; sg < 4; ++sg) {   // BoundaryIndex's default: Neumann 0
			a->bc[k].type[sg] = 2;
			a->bc[k].value[sg] = 0.0;
		}
	const size_t NF = (size_t)g->NI * g->P;
	if (a->fields.ensure(sizeof(double) * NF * 8)) {
		delete a;
		grid_release(g);
		return CARPIO_GPU_ENOMEM;
	}
	for (int k = 0; k < 8; ++k) a->f[k] = a->fields.as<double>() + k * NF;
	if (cudaMemsetAsync(a->fields.p, 0, a->fields.bytes, a->s) != cudaSuccess
			|| cudaStreamSynchronize(a->s) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		delete a;
		grid_release(g);
		return CARPIO_GPU_ECUDA;
	}
	*out = a;
	return 0;
}

int carpio_gpu_advection_destroy(carpio_gpu_advection* a) {
	if (!a) return CARPIO_GPU_EINVAL;
	cudaStreamSynchronize(a->s);
	carpio_gpu_grid* g = a->g;
	delete a;
	cg_host::grid_release(g);
	return 0;
}

int carpio_gpu_advection_set_scheme(carpio_gpu_advection* a, int scheme) {
	// set_advection_scheme (s_advection.hpp:140-183): the nine names it
	// knows; the radius-2 stencils need two ghost layers
	if (!a || scheme < CARPIO_GPU_UPWIND1 || scheme > CARPIO_GPU_CUI) return CARPIO_GPU_EINVAL;
	if (a->g->gl < (scheme >= CARPIO_GPU_CENTER4 ? 2 : 1)) return CARPIO_GPU_EINVAL;
	a->scheme = scheme;
	return 0;
}

int carpio_gpu_advection_set_bc(carpio_gpu_advection* a, int field,
		const carpio_gpu_bc* bc, const double* ghost_values) {
	if (!a || field < 0 || field > 2 || !bc || !valid_bc(*bc)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(a->g->mu);
	a->bc[field] = *bc;
	a->has_gv[field] = ghost_values != nullptr;
	if (ghost_values) {
		int rc = copy_field(a->g, a->f[5 + field], ghost_values, true, a->s);
		if (rc) return rc;
		CG_CK(cudaStreamSynchronize(a->s));
	}
	return 0;
}

int carpio_gpu_advection_initial(carpio_gpu_advection* a, const double* u,
		const double* v, const double* phi) {
	using namespace cg_host;
	if (!a) return CARPIO_GPU_EINVAL;
	carpio_gpu_grid* g = a->g;
	std::lock_guard<std::mutex> lock(g->mu);
	const size_t NF = (size_t)g->NI * g->P;
	const double* in[3] = { u, v, phi };
	double* dst[3] = { a->f[0], a->f[1], a->f[4] };
	int rc;
	for (int k = 0; k < 3; ++k) {
		if (in[k]) {
			if ((rc = copy_field(g, dst[k], in[k], true, a->s))) return rc;
		} else {
			CG_CK(cudaMemsetAsync(dst[k], 0, sizeof(double) * NF, a->s));
		}
	}
	// initial() (s_advection.hpp:101-135): ghosts of the cell velocities,
	// then the face velocities (new, zeroed face fields) by InterpolateC2F
	const Geo geo = make_geo(g);
	CG_CK(launch_bc(geo, a->f[0], a->bc[0], a->f[1], &a->bc[1], a->s,
			a->has_gv[0] ? a->f[5] : nullptr, a->has_gv[1] ? a->f[6] : nullptr));
	CG_CK(cudaMemsetAsync(a->f[2], 0, sizeof(double) * NF * 2, a->s));
	k_c2f<<<grid_blocks((long)g->nx * g->ny), kThreads, 0, a->s>>>(geo, a->f[0], a->f[1],
			a->f[2], a->f[3]);
	CG_CK(cudaGetLastError());
	CG_CK(cudaStreamSynchronize(a->s));
	a->ready = true;
	return 0;
}

int carpio_gpu_advection_step(carpio_gpu_advection* a, double dt, int steps) {
	using namespace cg_host;
	if (!a || steps < 0 || !(dt == dt) || !a->ready) return CARPIO_GPU_EINVAL;
	if (steps == 0) return 0;
	carpio_gpu_grid* g = a->g;
	std::lock_guard<std::mutex> lock(g->mu);
	const Geo geo = make_geo(g);
	// run_one_step refills the velocities' ghosts too: nothing reads them,
	// but a second fill changes the corners (they read the y-ghosts the
	// first fill wrote), and every later fill repeats the second
	CG_CK(launch_bc(geo, a->f[0], a->bc[0], a->f[1], &a->bc[1], a->s,
			a->has_gv[0] ? a->f[5] : nullptr, a->has_gv[1] ? a->f[6] : nullptr));
	const BcDev bcp = to_dev(a->bc[2], a->has_gv[2] ? a->f[7] : nullptr);
	// one block while the diagonals are short (van Leer: ~20 FP64 divisions
	// a cell); longer ones go to the row-pipelined sweep (two ghost layers
	// or more), else to the pipelined bands of rows, one per SM, whose
	// diagonals cost ~20 us (a hand-off through L2 per diagonal)
	const double avg_diag = (double)g->nx * g->ny / (double)(g->nx + g->ny - 1);
	if (avg_diag < 64.0 || g->nx < 8) {
		CG_CK(launch_advect(a->scheme, geo, a->s, a->f[4], bcp, a->f[2], a->f[3], dt, steps));
		CG_CK(cudaStreamSynchronize(a->s));
		return 0;
	}
	if (g->gl >= 2) {
		// the row-pipelined sweep (k_advect_rows): one lane per grid row
		int threads = 0;
		const void* kr = pick_advect_rows(a->scheme, geo.p2 != 0, threads);
		if (!kr) return CARPIO_GPU_EINVAL;
		const int nb = (g->nx + kAdvRows - 1) / kAdvRows;
		const int blocks = (nb + kAdvBands - 1) / kAdvBands;
		int per_sm = 0;
		CG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kr, threads, 0));
		if ((long)per_sm * sm_count() < blocks) return CARPIO_GPU_EINVAL;
		int rc;
		if ((rc = a->lw.ensure(blocks))) return rc;
		if ((rc = a->prog.ensure(sizeof(unsigned) * (size_t)nb))) return rc;
		CG_CK(cudaMemsetAsync(a->lw.ctl.p, 0, sizeof(Ctl), a->s));
		GridCtl gc = make_gridctl(a->lw);
		double* phi = a->f[4];
		const double* uf = a->f[2];
		const double* vf = a->f[3];
		unsigned* prog = a->prog.as<unsigned>();
		Geo gg = geo;
		BcDev bb = bcp;
		void* args[] = { &gg, &phi, &bb, &uf, &vf, &dt, &steps, &prog, &gc };
		CG_CK(cudaLaunchCooperativeKernel(kr, blocks, threads, args, 0, a->s));
		CG_CK(cudaMemcpyAsync(a->lw.host_ctl, a->lw.ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, a->s));
		CG_CK(cudaStreamSynchronize(a->s));
		return a->lw.host_ctl->err;
	}
	const void* k = pick_advect_band(a->scheme, geo.p2 != 0);
	if (!k) return CARPIO_GPU_EINVAL;
	// bands of R rows, one block each, at most one per SM (all co-resident)
	const int maxb = std::min(coop_blocks(k, (long)g->nx * kThreads, 1), sm_count());
	int R = (g->nx + maxb - 1) / maxb;
	const int blocks = (g->nx + R - 1) / R;
	// progress words count levels over all steps: keep them below 2^32
	if ((double)(R + g->ny) * steps >= 4.0e9) return CARPIO_GPU_EINVAL;
	int rc;
	if ((rc = a->lw.ensure(blocks))) return rc;
	if ((rc = a->prog.ensure(sizeof(unsigned) * (size_t)blocks))) return rc;
	CG_CK(cudaMemsetAsync(a->lw.ctl.p, 0, sizeof(Ctl), a->s));
	CG_CK(cudaMemsetAsync(a->prog.p, 0, sizeof(unsigned) * (size_t)blocks, a->s));
	GridCtl gc = make_gridctl(a->lw);
	double* phi = a->f[4];
	const double* uf = a->f[2];
	const double* vf = a->f[3];
	unsigned* prog = a->prog.as<unsigned>();
	Geo gg = geo;
	BcDev bb = bcp;
	void* args[] = { &gg, &phi, &bb, &uf, &vf, &dt, &steps, &R, &prog, &gc };
	const size_t smem = sizeof(double) * 2 * geo.gl * geo.gl;
	CG_CK(cudaLaunchCooperativeKernel(k, blocks, kThreads, args, smem, a->s));
	CG_CK(cudaMemcpyAsync(a->lw.host_ctl, a->lw.ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, a->s));
	CG_CK(cudaStreamSynchronize(a->s));
	return a->lw.host_ctl->err;
}

int carpio_gpu_advection_get(carpio_gpu_advection* a, double* u, double* v,
		double* uf, double* vf, double* phi) {
	if (!a) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(a->g->mu);
	double* out[5] = { u, v, uf, vf, phi };
	for (int k = 0; k < 5; ++k) {
		if (!out[k]) continue;
		int rc = copy_field(a->g, out[k], a->f[k], false, a->s);
		if (rc) return rc;
	}
	CG_CK(cudaStreamSynchronize(a->s));
	return 0;
}

}  // extern "C"
