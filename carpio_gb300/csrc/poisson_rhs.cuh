// Right-hand side of the structure-level Poisson solve, shared by the single
// and the batched solvers.
#pragma once

#include "internal.hpp"
#include "bits.cuh"

#include <cmath>
#include <vector>

namespace cg_dev {

struct RhsArgs {
	const double* sx;      // cell sizes incl. ghosts (device)
	const double* sy;
	const double* fold;    // [ny | ny | nx | nx]: x-, x+, y-, y+
	const double* src_a;   // SRC_FIELD: source field; SRC_DIV: x-face field
	const double* src_b;   // SRC_DIV: y-face field
	double* phi;           // field: x0 in, solution out (normal cells)
	int mean;
	// Helmholtz stencil (StencilHelmholtz_::coe_row, s_poisson.hpp:240-258):
	// the source scales by the cell volume sx sy; StencilPoisson_::src
	// (:75-83) multiplies sx by itself (it indexes the size by `dim`)
	int helm = 0;
	// every cell size a power of two, the same along each axis: the divisions
	// of Div by them are multiplications by their exact reciprocals (the
	// same bits)
	int p2 = 0;
	double ihx = 0.0, ihy = 0.0;
};

// RhsArgs::p2 and its reciprocals from the host copies of the cell sizes
inline void rhs_set_p2(RhsArgs& ra, const std::vector<double>& sx,
		const std::vector<double>& sy) {
	auto uniform_pow2 = [](const std::vector<double>& s, double& inv) {
		if (s.empty()) return false;
		int ex = 0;
		if (!(s[0] > 0.0) || std::frexp(s[0], &ex) != 0.5) return false;
		for (double v : s)
			if (v != s[0]) return false;
		inv = 1.0 / s[0];
		return true;
	};
	double ix = 0.0, iy = 0.0;
	ra.p2 = uniform_pow2(sx, ix) && uniform_pow2(sy, iy) ? 1 : 0;
	ra.ihx = ra.p2 ? ix : 0.0;
	ra.ihy = ra.p2 ? iy : 0.0;
}

// Row constant of StencilPoisson_::coe_row + ghost folds, then b = -constant
// (trimmed to +0 when the constant is exactly zero, s_solver.hpp:110-127).
// Exact IEEE operations in the reference's order (no contraction).
template<int SRC>
__device__ __forceinline__ double rhs_at(const GridSpace& sp, const RhsArgs& ra,
		int i, int j, int a) {
	const int gl = sp.gl;
	double sxi = ra.sx[i + gl];
	double f;
	if (SRC == cg_host::SRC_FIELD) {
		f = ra.src_a[a];
	} else {
		// Operation_::Div(VecF) (s_operation.hpp:100-120)
		double d = 0.0;
		if (ra.p2) {
			d = __dadd_rn(d, __dmul_rn(__dsub_rn(ra.src_a[a], ra.src_a[a - sp.P]), ra.ihx));
			d = __dadd_rn(d, __dmul_rn(__dsub_rn(ra.src_b[a], ra.src_b[a - 1]), ra.ihy));
		} else {
			d = __dadd_rn(d, __ddiv_rn(__dsub_rn(ra.src_a[a], ra.src_a[a - sp.P]), sxi));
			d = __dadd_rn(d, __ddiv_rn(__dsub_rn(ra.src_b[a], ra.src_b[a - 1]), ra.sy[j + gl]));
		}
		f = d;
	}
	double val = __dmul_rn(__dmul_rn(1.0, sxi), ra.helm ? ra.sy[j + gl] : sxi);
	val = __dmul_rn(val, f);
	const int nx = sp.nx, ny = sp.ny;
	if (i == 0) val = __dadd_rn(val, ra.fold[j]);
	if (j == 0) val = __dadd_rn(val, ra.fold[2 * ny + i]);
	if (j == ny - 1) val = __dadd_rn(val, ra.fold[2 * ny + nx + i]);
	if (i == nx - 1) val = __dadd_rn(val, ra.fold[ny + j]);
	return val == 0.0 ? 0.0 : -val;
}

template<int SRC>
__device__ __noinline__ double rhs_at_call(GridSpace sp, RhsArgs ra, int i, int j, int a) {
	return rhs_at<SRC>(sp, ra, i, j, a);
}

// rhs_at of a cell with no ghost fold (0 < i < nx - 1, 0 < j < ny - 1) on a
// RhsArgs::p2 grid with the same bits in fewer FP64 operations (GB300 issues
// one FP64 instruction per warp every 64 cycles): 0 + t as a sign fix,
// 1.0 * sx as sx, the final negation as a sign flip. Other grids take
// rhs_at out of line (so that its divisions are never issued predicated).
template<int SRC>
__device__ __forceinline__ double rhs_in(const GridSpace& sp, const RhsArgs& ra,
		int i, int j, int a) {
	if (!ra.p2) return rhs_at_call<SRC>(sp, ra, i, j, a);
	const int gl = sp.gl;
	const double sxi = ra.sx[i + gl];
	double f;
	if (SRC == cg_host::SRC_FIELD) {
		f = ra.src_a[a];
	} else {
		const double t1 = __dmul_rn(__dsub_rn(ra.src_a[a], ra.src_a[a - sp.P]), ra.ihx);
		const double t2 = __dmul_rn(__dsub_rn(ra.src_b[a], ra.src_b[a - 1]), ra.ihy);
		// d = 0; d += t1; d += t2
		f = __dadd_rn(plus_zero(t1), t2);
	}
	const double val = __dmul_rn(__dmul_rn(sxi, ra.helm ? ra.sy[j + gl] : sxi), f);
	// val == 0 ? +0 : -val
	return neg_or_plus_zero(val);
}

}  // namespace cg_dev
