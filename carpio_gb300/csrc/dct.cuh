// Spectral preconditioner of the on-chip FP32 CG: on a uniform grid with a
// uniform coefficient, and the same boundary type on both sides of each
// axis, the five-point operator (with the ghost substitution folded into its
// diagonal) is separable, A = cx L_x (x) I + cy I (x) L_y, and L is
// diagonalised by the DCT-II (Neumann: mirrored ghosts) or the DST-II
// (Dirichlet: antisymmetric ghosts). M^-1 = C^-1 diag(1 / lambda) C applies
// A^-1 up to FP32 rounding (lambda = 0, the all-Neumann mean, maps to 0).
//
// A length-N DCT-II is one N-point complex FFT of the reordered sequence
// (two real sequences share one complex FFT)
// v[n] = x[2n], v[N-1-n] = x[2n+1] followed by X[k] = Re(e^{-i pi k / 2N} V[k])
// (Makhoul 1980); its inverse runs the same steps backwards, and the DST-II
// is the DCT-II of (-1)^n x read in reverse order (the order reversal lives
// in the eigenvalue table). The FFT is an in-place radix-2 decimation in
// time on bit-reversed input in shared memory, three stages per pass in
// registers and one block barrier per pass, a batch of sequences at a time.
// Lengths are powers of two, N >= 2.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cg_dev {

constexpr int kDctBatch = 2;   // loads per thread in flight in the fill passes

struct DctArgs {
	int on;              // 1: the spectral preconditioner
	int lx, ly;          // log2 nx, log2 ny
	int fx, fy;          // 1: Dirichlet sides on the axis (sign flip)
	const float* lamx;   // [nx] eigenvalue parts, DCT index order
	const float* lamy;   // [ny]
	const float2* twx;   // FFT twiddles e^{-2 pi i t / nx}, t < nx / 2
	const float2* twy;
	const float2* ex;    // e^{-i pi k / (2 nx)}, k < nx
	const float2* ey;
	float* G;            // [nx][ny] spectral workspace (global memory, L2)
	int fb;              // float2 elements of the shared FFT buffer
};

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
	return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int bitrev(int m, int logN) {
	return (int)(__brev((unsigned)m) >> (32 - logN));
}

// Physical slot of element e of a sequence in the shared FFT buffer: the
// low five bits XORed with the next five, so that the bit-reversed scatter
// of the fill passes (consecutive m, addresses N/32 apart) lands on
// distinct banks. A permutation of every aligned block of 32 elements
// (and the identity below 32), applied to every access of the buffer.
__device__ __forceinline__ int dswz(int e) {
	return e ^ ((e >> 5) & 31);
}

// element m of the reordered sequence comes from x[src]
__device__ __forceinline__ int dct_src(int m, int N) {
	return m < (N >> 1) ? 2 * m : 2 * (N - 1 - m) + 1;
}

// K consecutive radix-2 stages s0 .. s0 + K - 1 of the in-place
// decimation in time, fused in registers: a thread loads the 2^K elements
// base + m h0 (h0 = 2^(s0 - 1)) of a group, runs the K stages' butterflies
// on them (the same operations, in the same order per element, as K
// separate stages) and stores them back. One block barrier per pass
// instead of one per stage, and each element read and written once per
// pass.
template<int K>
__device__ __forceinline__ void fft_pass(float2* buf, int B, int logN, int s0,
		const float2* tw, int NS) {
	constexpr int R = 1 << K;
	const int h0 = 1 << (s0 - 1);
	const int gps = 1 << (logN - K);   // groups per sequence
	const int ng = B * gps;
	for (int g = threadIdx.x; g < ng; g += blockDim.x) {
		const int seq = g >> (logN - K);
		const int w = g & (gps - 1);
		const int pos = w & (h0 - 1);
		const int base = ((w - pos) << K) + pos;
		float2* sb = buf + seq * NS;
		float2 v[R];
#pragma unroll
		for (int m = 0; m < R; ++m) v[m] = sb[dswz(base + m * h0)];
#pragma unroll
		for (int t = 0; t < K; ++t) {
			const int sh = logN - (s0 + t);
#pragma unroll
			for (int m = 0; m < R; ++m) {
				if (m & (1 << t)) continue;
				// the element's position within the stage's half-span
				const int pt = pos + (m & ((1 << t) - 1)) * h0;
				const float2 x = cmulf(__ldg(tw + (pt << sh)), v[m + (1 << t)]);
				const float2 a = v[m];
				v[m] = make_float2(a.x + x.x, a.y + x.y);
				v[m + (1 << t)] = make_float2(a.x - x.x, a.y - x.y);
			}
		}
#pragma unroll
		for (int m = 0; m < R; ++m) sb[dswz(base + m * h0)] = v[m];
	}
	__syncthreads();
}

// B sequences of N = 2^logN complex values in buf, NS apart (bit-reversed
// order) -> their DFTs in natural order: the logN radix-2 stages in passes
// of three (then two or one). Begins after the caller's barrier, ends with
// one.
__device__ __forceinline__ void fft_stages(float2* buf, int B, int logN, const float2* tw,
		int NS) {
	int s = 1;
	for (; logN - s + 1 >= 3; s += 3) fft_pass<3>(buf, B, logN, s, tw, NS);
	if (logN - s + 1 == 2) fft_pass<2>(buf, B, logN, s, tw, NS);
	else if (logN - s + 1 == 1) fft_pass<1>(buf, B, logN, s, tw, NS);
}

// Thread t of the block takes element m of sequence seq: seq-major
// (t = seq N + m) or, SM, seq-minor (t = m B + seq: neighbouring threads on
// neighbouring sequences, for sequences that are columns in memory).
template<bool SM>
__device__ __forceinline__ void dct_index(int t, int B, int logN, int& seq, int& m) {
	if (SM) {
		m = t / B;
		seq = t - m * B;
	} else {
		seq = t >> logN;
		m = t & ((1 << logN) - 1);
	}
}

// Forward transform of B real sequences: in(seq, n) -> out(seq, k, X[k]).
// `flip`: the DST through the DCT of (-1)^n x. Two real sequences share one
// complex FFT (z = v0 + i v1): V0[k] = (Z[k] + conj Z[N-k]) / 2 and
// V1[k] = (Z[k] - conj Z[N-k]) / 2i, so B sequences take ceil(B / 2) FFTs.
template<bool SM, class IN, class OUT>
__device__ __forceinline__ void dct_forward(float2* buf, int B, int logN, const float2* tw,
		const float2* E, bool flip, IN in, OUT out) {
	const int N = 1 << logN, P = (B + 1) >> 1, tot = P * N, T = blockDim.x;
	// sequences one element apart more than their length when neighbouring
	// threads take neighbouring sequences (SM): distinct banks
	const int NS = SM ? N + 1 : N;
	// kDctBatch elements per thread in flight before their stores
	for (int t0 = 0; t0 < tot; t0 += kDctBatch * T) {
		float2 val[kDctBatch];
		int pos[kDctBatch];
#pragma unroll
		for (int e = 0; e < kDctBatch; ++e) {
			const int t = t0 + e * T + threadIdx.x;
			pos[e] = -1;
			if (t < tot) {
				int p, m;
				dct_index<SM>(t, P, logN, p, m);
				const int n = dct_src(m, N);
				float x0 = in(2 * p, n);
				float x1 = 2 * p + 1 < B ? in(2 * p + 1, n) : 0.f;
				if (flip && (n & 1)) { x0 = -x0; x1 = -x1; }
				val[e] = make_float2(x0, x1);
				pos[e] = p * NS + dswz(bitrev(m, logN));
			}
		}
#pragma unroll
		for (int e = 0; e < kDctBatch; ++e)
			if (pos[e] >= 0) buf[pos[e]] = val[e];
	}
	__syncthreads();
	fft_stages(buf, P, logN, tw, NS);
	for (int t = threadIdx.x; t < tot; t += T) {
		int p, k;
		dct_index<SM>(t, P, logN, p, k);
		const float2 zk = buf[p * NS + dswz(k)];
		const float2 zn = buf[p * NS + dswz((N - k) & (N - 1))];
		const float2 e = __ldg(E + k);
		const float2 v0 = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
		out(2 * p, k, e.x * v0.x - e.y * v0.y);
		if (2 * p + 1 < B) {
			const float2 v1 = make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x));
			out(2 * p + 1, k, e.x * v1.x - e.y * v1.y);
		}
	}
	__syncthreads();
}

// Inverse of dct_forward: in(seq, k) = X[k] -> out(seq, n, x[n]). With
// Y[k] = e^{-i pi k / 2N} (X[k] + i X[N-k]) = conj(V[k]), the FFT of
// Y0 + i Y1 is N (v0 + i v1) (v0, v1 real): two sequences per FFT, no
// separation step.
template<bool SM, class IN, class OUT>
__device__ __forceinline__ void dct_inverse(float2* buf, int B, int logN, const float2* tw,
		const float2* E, bool flip, IN in, OUT out) {
	const int N = 1 << logN, P = (B + 1) >> 1, tot = P * N, T = blockDim.x;
	const int NS = SM ? N + 1 : N;
	for (int t0 = 0; t0 < tot; t0 += kDctBatch * T) {
		float2 val[kDctBatch];
		int pos[kDctBatch];
#pragma unroll
		for (int e = 0; e < kDctBatch; ++e) {
			const int t = t0 + e * T + threadIdx.x;
			pos[e] = -1;
			if (t < tot) {
				int p, k;
				dct_index<SM>(t, P, logN, p, k);
				const bool two = 2 * p + 1 < B;
				const float2 ek = __ldg(E + k);
				const float2 y0 = cmulf(ek, make_float2(in(2 * p, k), k > 0 ? in(2 * p, N - k) : 0.f));
				const float2 y1 = two ? cmulf(ek, make_float2(in(2 * p + 1, k),
				                                          k > 0 ? in(2 * p + 1, N - k) : 0.f))
				                      : make_float2(0.f, 0.f);
				val[e] = make_float2(y0.x - y1.y, y0.y + y1.x);
				pos[e] = p * NS + dswz(bitrev(k, logN));
			}
		}
#pragma unroll
		for (int e = 0; e < kDctBatch; ++e)
			if (pos[e] >= 0) buf[pos[e]] = val[e];
	}
	__syncthreads();
	fft_stages(buf, P, logN, tw, NS);
	const float invN = 1.f / (float)N;
	for (int t = threadIdx.x; t < tot; t += T) {
		int p, m;
		dct_index<SM>(t, P, logN, p, m);
		const int n = dct_src(m, N);
		const float2 w = buf[p * NS + dswz(m)];
		float v0 = w.x * invN, v1 = w.y * invN;
		if (flip && (n & 1)) { v0 = -v0; v1 = -v1; }
		out(2 * p, n, v0);
		if (2 * p + 1 < B) out(2 * p + 1, n, v1);
	}
	__syncthreads();
}

}  // namespace cg_dev
