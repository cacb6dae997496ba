// Double-float arithmetic (a value as the unevaluated sum hi + lo of two
// floats, about 48 significant bits) on the FP32 pipe, for the refinement
// steps of the spectral solve: on GB300 an FP64 warp instruction costs 64
// cycles of its sub-partition and an FP32 one a cycle, so a residual
// b - A x in double-float is far cheaper than in FP64 and still resolves
// the 1e-8 .. 1e-12 relative residuals a refinement needs. Knuth's TwoSum
// and the FMA TwoProd (Dekker 1971; Hida, Li & Bailey 2001, the
// "double-double" library) with every operation an explicit _rn
// intrinsic, so that nothing is contracted. Conversions from and to FP64
// are integer work on the bits (bits.cuh), with out-of-line FP64 fallbacks
// for values outside float's normal range.
#pragma once

#include "bits.cuh"

namespace cg_dev {

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
	s = __fadd_rn(a, b);
	const float bp = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// s + e = a + b exactly when |a| >= |b| (or a == 0) (Dekker)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
	s = __fadd_rn(a, b);
	e = __fsub_rn(b, __fsub_rn(s, a));
}

// x + y, both double-float (two TwoSums, then renormalised)
__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
	float s, e, t, f;
	two_sum(x.x, y.x, s, e);
	two_sum(x.y, y.y, t, f);
	e = __fadd_rn(e, t);
	fast_two_sum(s, e, s, e);
	e = __fadd_rn(e, f);
	fast_two_sum(s, e, s, e);
	return make_float2(s, e);
}

__device__ __forceinline__ float2 df_neg(float2 x) {
	return make_float2(-x.x, -x.y);
}

// x * c for a float c (TwoProd by FMA for the high part)
__device__ __forceinline__ float2 df_mul_f(float2 x, float c) {
	const float p = __fmul_rn(x.x, c);
	const float e = __fmaf_rn(x.x, c, -p);
	const float q = __fmaf_rn(x.y, c, e);
	float s, t;
	fast_two_sum(p, q, s, t);
	return make_float2(s, t);
}

__device__ __noinline__ float2 df_from_double_slow(double d) {
	const float h = __double2float_rn(d);
	return make_float2(h, __double2float_rn(d - (double)h));
}

// d as hi + lo: hi the float of d's sign, exponent and leading 24 bits
// (truncated), lo the remaining 29 bits rounded to a float (an error below
// 2^-48 |d|); integer work where d lies within [2^-70, 2^91), so that
// both floats stay normal, the FP64 conversions otherwise (0 included)
__device__ __forceinline__ float2 df_from_double(double d) {
	unsigned lo, hi;
	split_bits(d, lo, hi);
	const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
	if (e < -70 || e > 90) return df_from_double_slow(d);
	const unsigned sign = hi & 0x80000000u;
	// the leading 24 bits: 1 implicit + 20 from hi + 3 from lo
	const unsigned m23 = ((hi & 0x000fffffu) << 3) | (lo >> 29);
	const float fh = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | m23);
	// the remaining 29 bits, worth m29 * 2^(e - 52)
	const unsigned m29 = lo & 0x1fffffffu;
	float fl = __uint2float_rn(m29);   // exact below 2^24, rounded above
	// times 2^(e - 52), an exponent move: fl's exponent field is 127 ..
	// 155 and e - 52 >= -122, so the result stays normal
	if (m29 != 0u) {
		const unsigned fb = __float_as_uint(fl);
		fl = __uint_as_float(sign | (fb + ((unsigned)(e - 52) << 23)));
	}
	return make_float2(fh, fl);
}

__device__ __noinline__ double f2d_slow(float f) {
	return (double)f;
}

// a float as a double by its bits (normal floats and zero; the FP64
// conversion otherwise)
__device__ __forceinline__ double f2d_bits(float f) {
	const unsigned b = __float_as_uint(f);
	const unsigned ef = (b >> 23) & 0xffu;
	if ((b << 1) == 0u) return join_bits(0u, b);   // +-0
	if (ef == 0u || ef == 0xffu) return f2d_slow(f);
	const unsigned hi = (b & 0x80000000u) | ((ef + 896u) << 20) | ((b & 0x007fffffu) >> 3);
	return join_bits((b & 7u) << 29, hi);
}

// hi + lo in FP64 (one add)
__device__ __forceinline__ double df_to_double(float2 x) {
	return f2d_bits(x.x) + f2d_bits(x.y);
}

}  // namespace cg_dev
