// Integer stand-ins for FP64 operations whose result is fixed by the bits
// (GB300 issues one FP64 instruction per warp every 64 cycles; an integer
// instruction issues every cycle). The double is split into its 32-bit
// halves by inline PTX, which the optimiser cannot turn back into
// floating-point compares or adds: a test such as (bits << 1) == 0 written
// on the 64-bit pattern came out as one FP64 instruction anyway.
#pragma once

#include <cuda_runtime.h>

namespace cg_dev {

__device__ __forceinline__ void split_bits(double x, unsigned& lo, unsigned& hi) {
	asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
}

__device__ __forceinline__ double join_bits(unsigned lo, unsigned hi) {
	double x;
	asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
	return x;
}

// biased exponent field (0: zero or subnormal, 2047: infinity or NaN)
__device__ __forceinline__ int exp_field(double x) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	return (int)((hi >> 20) & 0x7ffu);
}

// x is +0 or -0
__device__ __forceinline__ bool is_zero_bits(double x) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	return ((hi << 1) | lo) == 0u;
}

// 0.0 + x: x with -0 turned into +0
__device__ __forceinline__ double plus_zero(double x) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	return join_bits(lo, (hi == 0x80000000u && lo == 0u) ? 0u : hi);
}

// -x
__device__ __forceinline__ double neg_bits(double x) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	return join_bits(lo, hi ^ 0x80000000u);
}

// val == 0 ? +0 : -val
__device__ __forceinline__ double neg_or_plus_zero(double x) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	return ((hi << 1) | lo) == 0u ? join_bits(0u, 0u) : join_bits(lo, hi ^ 0x80000000u);
}

static __device__ __noinline__ double mul_p2_slow(double x, double s) {
	return __dmul_rn(x, s);
}

// x * s for s = 2^k: the exponent field moved by k where x and the product
// are normal, x itself where x is +-0 (the product's sign is x's);
// subnormals, infinities, NaNs and products outside the normal range take
// the FPU multiply, out of line. The same bits as x * s in every case.
__device__ __forceinline__ double mul_p2(double x, int k, double s) {
	unsigned lo, hi;
	split_bits(x, lo, hi);
	if (((hi << 1) | lo) == 0u) return x;
	const int e = (int)((hi >> 20) & 0x7ffu), en = e + k;
	if ((unsigned)(e - 1) < 2046u && (unsigned)(en - 1) < 2046u)
		return join_bits(lo, hi + ((unsigned)k << 20));
	return mul_p2_slow(x, s);
}

}  // namespace cg_dev
