// The learned preconditioner: a 4-level BF16 U-Net (32/64/128/256 channels,
// 3x3 convolutions, ReLU, 2x2 average pooling, nearest upsampling, skip
// connections by channel concatenation; ~1.94 M parameters) that maps a
// residual field to a correction field.
//
//   a0 = relu(conv_in(x))            1 -> 32      (CUDA cores)
//   s0 = relu(conv(a0))             32 -> 32      (tensor cores, nn_conv.cu)
//   a1 = relu(conv(pool(s0)))       32 -> 64,  s1 = relu(conv(a1)) 64 -> 64
//   a2 = relu(conv(pool(s1)))       64 -> 128, s2 = relu(conv(a2))
//   a3 = relu(conv(pool(s2)))      128 -> 256, b3 = relu(conv(a3))
//   c2 = relu(conv([up(b3), s2]))  384 -> 128, d2 = relu(conv(c2))
//   c1 = relu(conv([up(d2), s1]))  192 -> 64,  d1 = relu(conv(c1))
//   c0 = relu(conv([up(d1), s0]))   96 -> 32,  d0 = relu(conv(c0))
//   z  = conv1x1(d0)                32 -> 1       (CUDA cores)
//
// No biases: the map is positively homogeneous, net(s r) = s net(r) for
// s > 0. Activations are BF16 NHWC; the 13 3x3 layers run on the tensor
// cores forward and for the input gradients (the same convolution with the
// weights transposed and the taps flipped, ReLU masks fused into the
// epilogue); weight gradients are reduced on the CUDA cores in FP32 with a
// fixed order (deterministic); Adam keeps FP32 master weights.
#include "internal.hpp"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

namespace cg_host {
// prepared tensor-core convolutions (nn_conv.cu)
int conv_prepare_ext(void** handle, const void* in0, int cin0, const void* in1, int cin1,
		int n, int h, int w, const void* wt, int cout, int ntile, void* out0, int split,
		void* out1, const void* mask0, const void* mask1, int relu, int* err);
int conv_launch_ext(const void* handle, cudaStream_t s);
void conv_free_ext(void* handle);
}

namespace {

using bf16 = __nv_bfloat16;
constexpr int C0 = 32, C1 = 64, C2 = 128, C3 = 256;
constexpr int kT = 256;

// ------------------------------------------------------------ CUDA-core ops --
__global__ void k_conv_in(const float* __restrict__ x, const float* __restrict__ w,
		bf16* __restrict__ out, int n, int h, int wd) {
	__shared__ float sw[9 * C0];
	for (int i = threadIdx.x; i < 9 * C0; i += blockDim.x) sw[i] = w[i];
	__syncthreads();
	const long px = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (px >= (long)n * h * wd) return;
	const int xx = (int)(px % wd), yy = (int)((px / wd) % h);
	const long img = px / ((long)h * wd);
	float in[9];
#pragma unroll
	for (int t = 0; t < 9; ++t) {
		const int y2 = yy + t / 3 - 1, x2 = xx + t % 3 - 1;
		in[t] = (y2 >= 0 && y2 < h && x2 >= 0 && x2 < wd) ? x[(img * h + y2) * wd + x2] : 0.f;
	}
	uint4* o = reinterpret_cast<uint4*>(out + px * C0);
#pragma unroll
	for (int g = 0; g < C0 / 8; ++g) {
		float v[8];
#pragma unroll
		for (int c = 0; c < 8; ++c) {
			float acc = 0.f;
#pragma unroll
			for (int t = 0; t < 9; ++t) acc = fmaf(in[t], sw[t * C0 + g * 8 + c], acc);
			v[c] = fmaxf(acc, 0.f);
		}
		uint4 pk;
		__nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]), p1 = __floats2bfloat162_rn(v[2], v[3]);
		__nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]), p3 = __floats2bfloat162_rn(v[6], v[7]);
		pk.x = *reinterpret_cast<uint32_t*>(&p0);
		pk.y = *reinterpret_cast<uint32_t*>(&p1);
		pk.z = *reinterpret_cast<uint32_t*>(&p2);
		pk.w = *reinterpret_cast<uint32_t*>(&p3);
		o[g] = pk;
	}
}

__global__ void k_conv_out(const bf16* __restrict__ d0, const float* __restrict__ w,
		float* __restrict__ z, long npx) {
	const long px = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (px >= npx) return;
	const bf16* p = d0 + px * C0;
	float acc = 0.f;
#pragma unroll
	for (int c = 0; c < C0; ++c) acc = fmaf(__bfloat162float(p[c]), w[c], acc);
	z[px] = acc;
}

// 8 channels per thread; out [n][h/2][w/2][c]
__global__ void k_pool(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int h,
		int wd, int c) {
	const int cg = c / 8, ho = h / 2, wo = wd / 2;
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= (long)n * ho * wo * cg) return;
	const int g = (int)(i % cg);
	const long op = i / cg;
	const int ox = (int)(op % wo), oy = (int)((op / wo) % ho);
	const long img = op / ((long)ho * wo);
	float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
	for (int dy = 0; dy < 2; ++dy)
#pragma unroll
		for (int dx = 0; dx < 2; ++dx) {
			const long ip = (img * h + 2 * oy + dy) * wd + 2 * ox + dx;
			const uint4 v = *reinterpret_cast<const uint4*>(in + ip * c + g * 8);
			const bf16* b = reinterpret_cast<const bf16*>(&v);
#pragma unroll
			for (int k = 0; k < 8; ++k) acc[k] += __bfloat162float(b[k]);
		}
	bf16 r[8];
#pragma unroll
	for (int k = 0; k < 8; ++k) r[k] = __float2bfloat16_rn(0.25f * acc[k]);
	*reinterpret_cast<uint4*>(out + op * c + g * 8) = *reinterpret_cast<uint4*>(r);
}

// nearest upsampling: out [n][2h][2w][c] from in [n][h][w][c]
__global__ void k_up(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int h,
		int wd, int c) {
	const int cg = c / 8, H = 2 * h, W = 2 * wd;
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= (long)n * H * W * cg) return;
	const int g = (int)(i % cg);
	const long op = i / cg;
	const int ox = (int)(op % W), oy = (int)((op / W) % H);
	const long img = op / ((long)H * W);
	const long ip = (img * h + oy / 2) * wd + ox / 2;
	*reinterpret_cast<uint4*>(out + op * c + g * 8) =
			*reinterpret_cast<const uint4*>(in + ip * c + g * 8);
}

// gradient through the 1x1 output layer into d0's pre-activation
__global__ void k_conv_out_bwd(const float* __restrict__ dz, const bf16* __restrict__ d0,
		const float* __restrict__ w, bf16* __restrict__ g, long npx) {
	const long px = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (px >= npx) return;
	const float gz = dz[px];
#pragma unroll
	for (int c = 0; c < C0; ++c) {
		const float a = __bfloat162float(d0[px * C0 + c]);
		g[px * C0 + c] = __float2bfloat16_rn(a > 0.f ? w[c] * gz : 0.f);
	}
}

// g_low = (sum of the 4 children of g_up) where low > 0
__global__ void k_up_bwd(const bf16* __restrict__ gup, const bf16* __restrict__ low,
		bf16* __restrict__ g, int n, int h, int wd, int c) {
	const int cg = c / 8, W = 2 * wd;
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= (long)n * h * wd * cg) return;
	const int gi = (int)(i % cg);
	const long op = i / cg;
	const int ox = (int)(op % wd), oy = (int)((op / wd) % h);
	const long img = op / ((long)h * wd);
	float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
	for (int dy = 0; dy < 2; ++dy)
#pragma unroll
		for (int dx = 0; dx < 2; ++dx) {
			const long ip = (img * 2 * h + 2 * oy + dy) * W + 2 * ox + dx;
			const uint4 v = *reinterpret_cast<const uint4*>(gup + ip * c + gi * 8);
			const bf16* b = reinterpret_cast<const bf16*>(&v);
#pragma unroll
			for (int k = 0; k < 8; ++k) acc[k] += __bfloat162float(b[k]);
		}
	const uint4 lv = *reinterpret_cast<const uint4*>(low + op * c + gi * 8);
	const bf16* lb = reinterpret_cast<const bf16*>(&lv);
	bf16 r[8];
#pragma unroll
	for (int k = 0; k < 8; ++k)
		r[k] = __float2bfloat16_rn(__bfloat162float(lb[k]) > 0.f ? acc[k] : 0.f);
	*reinterpret_cast<uint4*>(g + op * c + gi * 8) = *reinterpret_cast<uint4*>(r);
}

// g_s = (g_pool / 4 spread over the 2x2 window + g_skip) where s > 0
__global__ void k_pool_bwd(const bf16* __restrict__ gp, const bf16* __restrict__ gskip,
		const bf16* __restrict__ s, bf16* __restrict__ g, int n, int h, int wd, int c) {
	const int cg = c / 8;
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= (long)n * h * wd * cg) return;
	const int gi = (int)(i % cg);
	const long op = i / cg;
	const int ox = (int)(op % wd), oy = (int)((op / wd) % h);
	const long img = op / ((long)h * wd);
	const long pp = (img * (h / 2) + oy / 2) * (wd / 2) + ox / 2;
	const uint4 a = *reinterpret_cast<const uint4*>(gp + pp * c + gi * 8);
	const uint4 b = *reinterpret_cast<const uint4*>(gskip + op * c + gi * 8);
	const uint4 m = *reinterpret_cast<const uint4*>(s + op * c + gi * 8);
	const bf16* ab = reinterpret_cast<const bf16*>(&a);
	const bf16* bb = reinterpret_cast<const bf16*>(&b);
	const bf16* mb = reinterpret_cast<const bf16*>(&m);
	bf16 r[8];
#pragma unroll
	for (int k = 0; k < 8; ++k) {
		const float v = 0.25f * __bfloat162float(ab[k]) + __bfloat162float(bb[k]);
		r[k] = __float2bfloat16_rn(__bfloat162float(mb[k]) > 0.f ? v : 0.f);
	}
	*reinterpret_cast<uint4*>(g + op * c + gi * 8) = *reinterpret_cast<uint4*>(r);
}

// Weight gradient of a 3x3 layer, partial over a block of pixels:
//   part[pb][tap][co][ci] = sum over pixels p of block pb of
//                           g[p][co] * x[p + offset(tap)][ci]
// x is the concatenation of x0 (cx0 channels) and x1 (cx1). One CTA: one
// tap, a 32 x 64 (co x ci) tile, 128 threads with 4 x 4 outputs each,
// pixels staged 32 at a time through shared memory.
constexpr int kDwCo = 32, kDwCi = 64, kDwP = 32;
__global__ void __launch_bounds__(128) k_dw(const bf16* __restrict__ g, int cg_,
		const bf16* __restrict__ x0, int cx0, const bf16* __restrict__ x1, int cx1,
		int n, int h, int wd, long px_per_block, float* __restrict__ part) {
	__shared__ float sg[kDwP][kDwCo + 1];
	__shared__ float sx[kDwP][kDwCi + 4];
	const int tap = blockIdx.y;
	const int cix = cx0 + cx1;
	const int tiles_ci = (cix + kDwCi - 1) / kDwCi;
	const int co0 = (blockIdx.z / tiles_ci) * kDwCo, ci0 = (blockIdx.z % tiles_ci) * kDwCi;
	const int dy = tap / 3 - 1, dx = tap % 3 - 1;
	const long npx = (long)n * h * wd;
	const long p0 = (long)blockIdx.x * px_per_block;
	const long p1 = p0 + px_per_block < npx ? p0 + px_per_block : npx;
	const int tco = threadIdx.x / 16, tci = threadIdx.x % 16;   // 8 x 16 threads
	float acc[4][4] = {};
	for (long pb = p0; pb < p1; pb += kDwP) {
		for (int i = threadIdx.x; i < kDwP * kDwCo; i += 128) {
			const int pp = i / kDwCo, c = i % kDwCo;
			const long p = pb + pp;
			sg[pp][c] = (p < p1 && co0 + c < cg_) ? __bfloat162float(g[p * cg_ + co0 + c]) : 0.f;
		}
		for (int i = threadIdx.x; i < kDwP * kDwCi; i += 128) {
			const int pp = i / kDwCi, c = i % kDwCi;
			const long p = pb + pp;
			float v = 0.f;
			const int ci = ci0 + c;
			if (p < p1 && ci < cix) {
				const int xx = (int)(p % wd) + dx, yy = (int)((p / wd) % h) + dy;
				if (xx >= 0 && xx < wd && yy >= 0 && yy < h) {
					const long q = (p / ((long)h * wd) * h + yy) * wd + xx;
					v = ci < cx0 ? __bfloat162float(x0[q * cx0 + ci])
					             : __bfloat162float(x1[q * cx1 + ci - cx0]);
				}
			}
			sx[pp][c] = v;
		}
		__syncthreads();
#pragma unroll 4
		for (int pp = 0; pp < kDwP; ++pp) {
			float a[4], b[4];
#pragma unroll
			for (int u = 0; u < 4; ++u) a[u] = sg[pp][tco * 4 + u];
#pragma unroll
			for (int u = 0; u < 4; ++u) b[u] = sx[pp][tci * 4 + u];
#pragma unroll
			for (int u = 0; u < 4; ++u)
#pragma unroll
				for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
		}
		__syncthreads();
	}
	float* dst = part + ((size_t)blockIdx.x * 9 + tap) * (size_t)cg_ * cix;
#pragma unroll
	for (int u = 0; u < 4; ++u)
#pragma unroll
		for (int v = 0; v < 4; ++v) {
			const int co = co0 + tco * 4 + u, ci = ci0 + tci * 4 + v;
			if (co < cg_ && ci < cix) dst[(size_t)co * cix + ci] = acc[u][v];
		}
}

// sum of nb partials in block order
__global__ void k_sum_parts(const float* __restrict__ part, int nb, long len,
		float* __restrict__ out) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= len) return;
	float s = 0.f;
	for (int b = 0; b < nb; ++b) s += part[(size_t)b * len + i];
	out[i] = s;
}

// weight gradient of the input layer (1 -> 32), partial per pixel block
__global__ void k_dw_in(const bf16* __restrict__ g, const float* __restrict__ x, int n,
		int h, int wd, long px_per_block, float* __restrict__ part) {
	// thread t < 288 owns (tap, channel)
	const int t = threadIdx.x;
	const long npx = (long)n * h * wd;
	const long p0 = (long)blockIdx.x * px_per_block;
	const long p1 = p0 + px_per_block < npx ? p0 + px_per_block : npx;
	const int tap = t / C0, c = t % C0;
	const int dy = tap / 3 - 1, dx = tap % 3 - 1;
	float acc = 0.f;
	if (t < 9 * C0) {
		for (long p = p0; p < p1; ++p) {
			const int xx = (int)(p % wd) + dx, yy = (int)((p / wd) % h) + dy;
			float xv = 0.f;
			if (xx >= 0 && xx < wd && yy >= 0 && yy < h)
				xv = x[(p / ((long)h * wd) * h + yy) * wd + xx];
			acc = fmaf(__bfloat162float(g[p * C0 + c]), xv, acc);
		}
		part[(size_t)blockIdx.x * 9 * C0 + t] = acc;
	}
}

// weight gradient of the output layer, partial per pixel block
__global__ void k_dw_out(const float* __restrict__ dz, const bf16* __restrict__ d0,
		long npx, long px_per_block, float* __restrict__ part) {
	__shared__ float red[kT / 32][C0];
	const long p0 = (long)blockIdx.x * px_per_block;
	const long p1 = p0 + px_per_block < npx ? p0 + px_per_block : npx;
	const int c = threadIdx.x % C0, lane8 = threadIdx.x / C0;   // 8 pixel lanes
	float acc = 0.f;
	for (long p = p0 + lane8; p < p1; p += kT / C0)
		acc = fmaf(__bfloat162float(d0[p * C0 + c]), dz[p], acc);
	red[lane8][c] = acc;
	__syncthreads();
	if (threadIdx.x < C0) {
		float s = 0.f;
		for (int k = 0; k < kT / C0; ++k) s += red[k][threadIdx.x];
		part[(size_t)blockIdx.x * C0 + threadIdx.x] = s;
	}
}

// transposed, tap-flipped BF16 weights for the input-gradient convolution:
// wt2[8 - tap][ci][co] = w[tap][co][ci]
__global__ void k_wt_flip(const float* __restrict__ w, bf16* __restrict__ wbf,
		bf16* __restrict__ wt2, int co, int ci) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= 9L * co * ci) return;
	const int c_i = (int)(i % ci);
	const int c_o = (int)((i / ci) % co);
	const int tap = (int)(i / ((long)ci * co));
	const bf16 v = __float2bfloat16_rn(w[i]);
	wbf[i] = v;
	wt2[((size_t)(8 - tap) * ci + c_i) * co + c_o] = v;
}

// relative squared error, per-block partial sums of (z - t)^2 and t^2
__global__ void k_loss_parts(const float* __restrict__ z, const float* __restrict__ t,
		long npx, double* __restrict__ part) {
	__shared__ double s[2][kT];
	double e = 0, q = 0;
	for (long i = (long)blockIdx.x * kT + threadIdx.x; i < npx; i += (long)gridDim.x * kT) {
		const double d = (double)z[i] - (double)t[i];
		e += d * d;
		q += (double)t[i] * (double)t[i];
	}
	s[0][threadIdx.x] = e;
	s[1][threadIdx.x] = q;
	__syncthreads();
	for (int o = kT / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			s[0][threadIdx.x] += s[0][threadIdx.x + o];
			s[1][threadIdx.x] += s[1][threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		part[2 * blockIdx.x] = s[0][0];
		part[2 * blockIdx.x + 1] = s[1][0];
	}
}

// (A f)[i][j] over one image: the all-Neumann 5-point operator with unit
// face coefficients (sum over the existing neighbours of f - f_nb)
__device__ __forceinline__ float neumann_apply(const float* __restrict__ f, long px, int h,
		int wd) {
	const int xx = (int)(px % wd), yy = (int)((px / wd) % h);
	const float c = f[px];
	float a = 0.f;
	if (xx > 0) a += c - f[px - 1];
	if (xx < wd - 1) a += c - f[px + 1];
	if (yy > 0) a += c - f[px - wd];
	if (yy < h - 1) a += c - f[px + wd];
	return a;
}

// energy-norm loss parts: (e, A e) with e = z - t (e kept in `e`), (t, A t)
__global__ void k_energy_parts(const float* __restrict__ e, const float* __restrict__ t,
		int n, int h, int wd, double* __restrict__ part) {
	__shared__ double s[2][kT];
	const long npx = (long)n * h * wd;
	double a = 0, b = 0;
	for (long i = (long)blockIdx.x * kT + threadIdx.x; i < npx; i += (long)gridDim.x * kT) {
		a += (double)e[i] * (double)neumann_apply(e, i, h, wd);
		b += (double)t[i] * (double)neumann_apply(t, i, h, wd);
	}
	s[0][threadIdx.x] = a;
	s[1][threadIdx.x] = b;
	__syncthreads();
	for (int o = kT / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			s[0][threadIdx.x] += s[0][threadIdx.x + o];
			s[1][threadIdx.x] += s[1][threadIdx.x + o];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		part[2 * blockIdx.x] = s[0][0];
		part[2 * blockIdx.x + 1] = s[1][0];
	}
}

__global__ void k_sub(const float* __restrict__ z, const float* __restrict__ t, long npx,
		float* __restrict__ e) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < npx) e[i] = z[i] - t[i];
}

// dz = scale * A e
__global__ void k_dz_energy(const float* __restrict__ e, const float* __restrict__ scale,
		int n, int h, int wd, float* __restrict__ dz) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < (long)n * h * wd) dz[i] = neumann_apply(e, i, h, wd) * *scale;
}

// loss = sum e / sum q, and the gradient scale 2 / sum q
__global__ void k_loss_final(const double* __restrict__ part, int nb, double* __restrict__ loss,
		float* __restrict__ scale) {
	double e = 0, q = 0;
	for (int b = 0; b < nb; ++b) {
		e += part[2 * b];
		q += part[2 * b + 1];
	}
	if (q <= 0) q = 1;
	*loss = e / q;
	*scale = (float)(2.0 / q);
}

__global__ void k_dz(const float* __restrict__ z, const float* __restrict__ t,
		const float* __restrict__ scale, long npx, float* __restrict__ dz) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < npx) dz[i] = (z[i] - t[i]) * *scale;
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g,
		float* __restrict__ m, float* __restrict__ v, long len, float lr, float b1, float b2,
		float eps, float c1, float c2) {
	const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= len) return;
	const float gi = g[i];
	const float mi = b1 * m[i] + (1.f - b1) * gi;
	const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
	m[i] = mi;
	v[i] = vi;
	w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

unsigned nblk(long n, int t = kT) { return (unsigned)((n + t - 1) / t); }

// --------------------------------------------------------------- the net --
struct Layer {
	int cin0, cin1, cout;   // 3x3 layer: input channels (second source for a concat)
	long off;               // offset of its weights in the flat parameter vector
};

// The 13 tensor-core layers in parameter order.
const Layer* layers() {
	static Layer L[13] = {
		{ C0, 0, C0, 0 },     // 0  s0 = conv(a0)
		{ C0, 0, C1, 0 },     // 1  a1 = conv(p0)
		{ C1, 0, C1, 0 },     // 2  s1 = conv(a1)
		{ C1, 0, C2, 0 },     // 3  a2 = conv(p1)
		{ C2, 0, C2, 0 },     // 4  s2 = conv(a2)
		{ C2, 0, C3, 0 },     // 5  a3 = conv(p2)
		{ C3, 0, C3, 0 },     // 6  b3 = conv(a3)
		{ C3, C2, C2, 0 },    // 7  c2 = conv([u2, s2])
		{ C2, 0, C2, 0 },     // 8  d2 = conv(c2)
		{ C2, C1, C1, 0 },    // 9  c1 = conv([u1, s1])
		{ C1, 0, C1, 0 },     // 10 d1 = conv(c1)
		{ C1, C0, C0, 0 },    // 11 c0 = conv([u0, s0])
		{ C0, 0, C0, 0 },     // 12 d0 = conv(c0)
	};
	static bool init = false;
	if (!init) {
		long off = 9 * C0;
		for (auto& l : L) {
			l.off = off;
			off += 9L * l.cout * (l.cin0 + l.cin1);
		}
		init = true;
	}
	return L;
}
long n_params() { return layers()[12].off + 9L * C0 * C0 + C0; }
long off_out() { return layers()[12].off + 9L * C0 * C0; }

struct Buf {
	void* p = nullptr;
	size_t bytes = 0;
	int ensure(size_t n) {
		if (n <= bytes) return 0;
		if (p) cudaFree(p);
		p = nullptr;
		bytes = 0;
		if (cudaMalloc(&p, n) != cudaSuccess) {
			cudaGetLastError();
			return CARPIO_GPU_ENOMEM;
		}
		bytes = n;
		return 0;
	}
	~Buf() { if (p) cudaFree(p); }
	template<class T> T* as() const { return static_cast<T*>(p); }
};

// Activations and gradients of one input shape, with the prepared
// tensor-core launches (tensor maps built once).
struct Shape {
	int n, h, w;
	// forward activations per level l (size h>>l): a, s, c, d, u, p
	Buf a[4], s[3], p[3], u[3], c[3], d[3], b3;
	// gradients
	Buf gA[4], gS[3], gP[3], gU[3], gC[3], gD[3], gB3, gSkip[3];
	Buf z, dz, lpart, part;
	std::vector<void*> fwd, bwd;   // conv launch handles
	~Shape() {
		for (void* h : fwd) cg_host::conv_free_ext(h);
		for (void* h : bwd) cg_host::conv_free_ext(h);
	}
};

}  // namespace

struct carpio_gpu_unet {
	std::vector<float> host_w;        // initial / last set parameters
	Buf w, g, m, v;                   // FP32 master weights, gradient, Adam moments
	Buf wbf, wt2;                     // BF16 forward and transposed weights
	Buf loss;                         // double
	Buf err;
	long step = 0;
	cudaStream_t s = nullptr;
	std::map<std::tuple<int, int, int>, std::unique_ptr<Shape>> shapes;
	cudaGraphExec_t fwd_graph = nullptr;
	std::tuple<int, int, int> fwd_graph_shape{ 0, 0, 0 };
	const float* fwd_graph_x = nullptr;
	float* fwd_graph_z = nullptr;
	std::mutex mu;
	~carpio_gpu_unet() {
		if (s) cudaStreamSynchronize(s);
		if (fwd_graph) cudaGraphExecDestroy(fwd_graph);
		shapes.clear();
		if (s) cudaStreamDestroy(s);
	}
};

namespace {

using cg_host::note_cuda_error;

size_t act_bytes(const Shape& S, int lvl, int c) {
	return sizeof(bf16) * (size_t)S.n * (S.h >> lvl) * (S.w >> lvl) * c;
}

bf16* W16(carpio_gpu_unet* u, int l) { return u->wbf.as<bf16>() + layers()[l].off; }
bf16* WT2(carpio_gpu_unet* u, int l) { return u->wt2.as<bf16>() + layers()[l].off; }

// allocate a shape's buffers and prepare its convolution launches
int shape_prepare(carpio_gpu_unet* u, Shape& S) {
	const int n = S.n, h = S.h, w = S.w;
	const int CH[4] = { C0, C1, C2, C3 };
	int rc;
	for (int l = 0; l < 4; ++l) {
		if ((rc = S.a[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.gA[l].ensure(act_bytes(S, l, CH[l])))) return rc;
	}
	if ((rc = S.b3.ensure(act_bytes(S, 3, C3)))) return rc;
	if ((rc = S.gB3.ensure(act_bytes(S, 3, C3)))) return rc;
	for (int l = 0; l < 3; ++l) {
		if ((rc = S.s[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.p[l].ensure(act_bytes(S, l + 1, CH[l])))) return rc;
		if ((rc = S.u[l].ensure(act_bytes(S, l, CH[l + 1])))) return rc;
		if ((rc = S.c[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.d[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.gS[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.gP[l].ensure(act_bytes(S, l + 1, CH[l])))) return rc;
		if ((rc = S.gU[l].ensure(act_bytes(S, l, CH[l + 1])))) return rc;
		if ((rc = S.gC[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.gD[l].ensure(act_bytes(S, l, CH[l])))) return rc;
		if ((rc = S.gSkip[l].ensure(act_bytes(S, l, CH[l])))) return rc;
	}
	const size_t npx = (size_t)n * h * w;
	if ((rc = S.z.ensure(sizeof(float) * npx))) return rc;
	if ((rc = S.dz.ensure(sizeof(float) * npx))) return rc;
	if ((rc = S.lpart.ensure(sizeof(double) * (2 * 1024 + 1)))) return rc;
	int* err = u->err.as<int>();
	auto prep = [&](std::vector<void*>& v, const void* i0, int c0, const void* i1, int c1,
			int lvl, const void* wt, int cout, void* o0, int split, void* o1,
			const void* m0, const void* m1, int relu) {
		void* hnd = nullptr;
		const int ntile = cout <= 256 ? cout : (cout % 256 == 0 ? 256 : 192);
		int r = cg_host::conv_prepare_ext(&hnd, i0, c0, i1, c1, n, h >> lvl, w >> lvl, wt, cout,
				ntile, o0, split, o1, m0, m1, relu, err);
		if (r) return r;
		v.push_back(hnd);
		return 0;
	};
	// forward, in execution order
	struct F { int layer, lvl; const void *i0, *i1; void* o; };
	const F fw[13] = {
		{ 0, 0, S.a[0].p, nullptr, S.s[0].p },
		{ 1, 1, S.p[0].p, nullptr, S.a[1].p },
		{ 2, 1, S.a[1].p, nullptr, S.s[1].p },
		{ 3, 2, S.p[1].p, nullptr, S.a[2].p },
		{ 4, 2, S.a[2].p, nullptr, S.s[2].p },
		{ 5, 3, S.p[2].p, nullptr, S.a[3].p },
		{ 6, 3, S.a[3].p, nullptr, S.b3.p },
		{ 7, 2, S.u[2].p, S.s[2].p, S.c[2].p },
		{ 8, 2, S.c[2].p, nullptr, S.d[2].p },
		{ 9, 1, S.u[1].p, S.s[1].p, S.c[1].p },
		{ 10, 1, S.c[1].p, nullptr, S.d[1].p },
		{ 11, 0, S.u[0].p, S.s[0].p, S.c[0].p },
		{ 12, 0, S.c[0].p, nullptr, S.d[0].p },
	};
	for (const F& f : fw) {
		const Layer& L = layers()[f.layer];
		if ((rc = prep(S.fwd, f.i0, L.cin0, f.i1, L.cin1, f.lvl, W16(u, f.layer), L.cout, f.o,
				L.cout, nullptr, nullptr, nullptr, 1))) return rc;
	}
	// backward input gradients, in execution order: (layer, level, g_in, out0,
	// split, out1, mask0)
	struct B { int layer, lvl; const void* gin; void* o0; void* o1; const void* mk; };
	const B bw[13] = {
		{ 12, 0, S.gD[0].p, S.gC[0].p, nullptr, S.c[0].p },
		{ 11, 0, S.gC[0].p, S.gU[0].p, S.gSkip[0].p, nullptr },
		{ 10, 1, S.gD[1].p, S.gC[1].p, nullptr, S.c[1].p },
		{ 9, 1, S.gC[1].p, S.gU[1].p, S.gSkip[1].p, nullptr },
		{ 8, 2, S.gD[2].p, S.gC[2].p, nullptr, S.c[2].p },
		{ 7, 2, S.gC[2].p, S.gU[2].p, S.gSkip[2].p, nullptr },
		{ 6, 3, S.gB3.p, S.gA[3].p, nullptr, S.a[3].p },
		{ 5, 3, S.gA[3].p, S.gP[2].p, nullptr, nullptr },
		{ 4, 2, S.gS[2].p, S.gA[2].p, nullptr, S.a[2].p },
		{ 3, 2, S.gA[2].p, S.gP[1].p, nullptr, nullptr },
		{ 2, 1, S.gS[1].p, S.gA[1].p, nullptr, S.a[1].p },
		{ 1, 1, S.gA[1].p, S.gP[0].p, nullptr, nullptr },
		{ 0, 0, S.gS[0].p, S.gA[0].p, nullptr, S.a[0].p },
	};
	for (const B& b : bw) {
		const Layer& L = layers()[b.layer];
		// the transposed layer reads cout channels and writes cin0 + cin1
		if ((rc = prep(S.bwd, b.gin, L.cout, nullptr, 0, b.lvl, WT2(u, b.layer),
				L.cin0 + L.cin1, b.o0, L.cin0, b.o1, b.mk, nullptr, 0))) return rc;
	}
	return 0;
}

Shape* get_shape(carpio_gpu_unet* u, int n, int h, int w, int* rc) {
	auto key = std::make_tuple(n, h, w);
	auto it = u->shapes.find(key);
	if (it != u->shapes.end()) return it->second.get();
	auto S = std::make_unique<Shape>();
	S->n = n;
	S->h = h;
	S->w = w;
	*rc = shape_prepare(u, *S);
	if (*rc) return nullptr;
	Shape* p = S.get();
	u->shapes[key] = std::move(S);
	return p;
}

#define NN_CK(expr) do { int _r = (expr); if (_r) return _r; } while (0)

int forward(carpio_gpu_unet* u, Shape& S, const float* x, float* z, cudaStream_t st) {
	const int n = S.n, h = S.h, w = S.w;
	const int CH[4] = { C0, C1, C2, C3 };
	const float* W = u->w.as<float>();
	const long np0 = (long)n * h * w;
	k_conv_in<<<nblk(np0), kT, 0, st>>>(x, W, S.a[0].as<bf16>(), n, h, w);
	int li = 0;
	auto conv = [&]() { return cg_host::conv_launch_ext(S.fwd[li++], st); };
	// encoder
	NN_CK(conv());   // s0
	for (int l = 0; l < 3; ++l) {
		const int hl = h >> l, wl = w >> l;
		k_pool<<<nblk((long)n * (hl / 2) * (wl / 2) * CH[l] / 8), kT, 0, st>>>(
				S.s[l].as<bf16>(), S.p[l].as<bf16>(), n, hl, wl, CH[l]);
		NN_CK(conv());   // a_{l+1}
		if (l < 2) NN_CK(conv());   // s_{l+1}
	}
	NN_CK(conv());   // b3
	// decoder
	for (int l = 2; l >= 0; --l) {
		const int hl = h >> l, wl = w >> l;
		const bf16* low = l == 2 ? S.b3.as<bf16>() : S.d[l + 1].as<bf16>();
		k_up<<<nblk((long)n * hl * wl * CH[l + 1] / 8), kT, 0, st>>>(
				low, S.u[l].as<bf16>(), n, hl / 2, wl / 2, CH[l + 1]);
		NN_CK(conv());   // c_l
		NN_CK(conv());   // d_l
	}
	k_conv_out<<<nblk(np0), kT, 0, st>>>(S.d[0].as<bf16>(), W + off_out(), z, np0);
	CG_CK(cudaGetLastError());
	return 0;
}

int dw_layer(carpio_gpu_unet* u, Shape& S, int layer, int lvl, const bf16* g,
		const bf16* x0, const bf16* x1, cudaStream_t st) {
	const Layer& L = layers()[layer];
	const int hl = S.h >> lvl, wl = S.w >> lvl;
	const long npx = (long)S.n * hl * wl;
	const int cix = L.cin0 + L.cin1;
	const int tiles = ((L.cout + kDwCo - 1) / kDwCo) * ((cix + kDwCi - 1) / kDwCi);
	// enough CTAs for the GPU; each block covers whole 32-pixel groups
	long nb = std::max(1L, 2048L / (9L * tiles));
	nb = std::min(nb, (npx + kDwP - 1) / kDwP);
	const long per = ((npx + nb - 1) / nb + kDwP - 1) / kDwP * kDwP;
	nb = (npx + per - 1) / per;
	const long len = 9L * L.cout * cix;
	NN_CK(S.part.ensure(sizeof(float) * (size_t)(nb * len)));
	k_dw<<<dim3((unsigned)nb, 9, (unsigned)tiles), 128, 0, st>>>(g, L.cout, x0, L.cin0, x1,
			L.cin1, S.n, hl, wl, per, S.part.as<float>());
	k_sum_parts<<<nblk(len), kT, 0, st>>>(S.part.as<float>(), (int)nb, len,
			u->g.as<float>() + L.off);
	CG_CK(cudaGetLastError());
	return 0;
}

// forward, loss, backward: gradient in u->g, loss in u->loss
int grad(carpio_gpu_unet* u, Shape& S, const float* x, const float* t, int loss_mode,
		cudaStream_t st) {
	const int n = S.n, h = S.h, w = S.w;
	const int CH[4] = { C0, C1, C2, C3 };
	const long np0 = (long)n * h * w;
	float* z = S.z.as<float>();
	NN_CK(forward(u, S, x, z, st));
	const int nbl = 1024;
	float* scale = reinterpret_cast<float*>(S.lpart.as<double>() + 2 * nbl);
	if (loss_mode == 1) {
		// energy norm: (e, A e) / (t, A t), dz = 2 A e / (t, A t)
		float* e = S.gD[0].as<float>();   // scratch: gD[0] is written later
		k_sub<<<nblk(np0), kT, 0, st>>>(z, t, np0, e);
		k_energy_parts<<<nbl, kT, 0, st>>>(e, t, n, h, w, S.lpart.as<double>());
		k_loss_final<<<1, 1, 0, st>>>(S.lpart.as<double>(), nbl, u->loss.as<double>(), scale);
		k_dz_energy<<<nblk(np0), kT, 0, st>>>(e, scale, n, h, w, S.dz.as<float>());
	} else {
		k_loss_parts<<<nbl, kT, 0, st>>>(z, t, np0, S.lpart.as<double>());
		k_loss_final<<<1, 1, 0, st>>>(S.lpart.as<double>(), nbl, u->loss.as<double>(), scale);
		k_dz<<<nblk(np0), kT, 0, st>>>(z, t, scale, np0, S.dz.as<float>());
	}
	const float* W = u->w.as<float>();
	float* G = u->g.as<float>();
	// output layer
	{
		long nb = std::min(1024L, (np0 + 4095) / 4096);
		const long per = (np0 + nb - 1) / nb;
		nb = (np0 + per - 1) / per;
		NN_CK(S.part.ensure(sizeof(float) * (size_t)(nb * C0)));
		k_dw_out<<<(unsigned)nb, kT, 0, st>>>(S.dz.as<float>(), S.d[0].as<bf16>(), np0, per,
				S.part.as<float>());
		k_sum_parts<<<1, C0, 0, st>>>(S.part.as<float>(), (int)nb, C0, G + off_out());
		k_conv_out_bwd<<<nblk(np0), kT, 0, st>>>(S.dz.as<float>(), S.d[0].as<bf16>(),
				W + off_out(), S.gD[0].as<bf16>(), np0);
	}
	int bi = 0;
	auto dxconv = [&]() { return cg_host::conv_launch_ext(S.bwd[bi++], st); };
	// decoder levels 0, 1, 2
	for (int l = 0; l < 3; ++l) {
		const int ld = 12 - 2 * l, lc = 11 - 2 * l;   // d_l and c_l layers
		NN_CK(dw_layer(u, S, ld, l, S.gD[l].as<bf16>(), S.c[l].as<bf16>(), nullptr, st));
		NN_CK(dxconv());   // gC[l] (masked by c_l)
		NN_CK(dw_layer(u, S, lc, l, S.gC[l].as<bf16>(), S.u[l].as<bf16>(), S.s[l].as<bf16>(), st));
		NN_CK(dxconv());   // gU[l], gSkip[l]
		const int hl = h >> l, wl = w >> l;
		const bf16* low = l == 2 ? S.b3.as<bf16>() : S.d[l + 1].as<bf16>();
		bf16* glow = l == 2 ? S.gB3.as<bf16>() : S.gD[l + 1].as<bf16>();
		k_up_bwd<<<nblk((long)n * (hl / 2) * (wl / 2) * CH[l + 1] / 8), kT, 0, st>>>(
				S.gU[l].as<bf16>(), low, glow, n, hl / 2, wl / 2, CH[l + 1]);
	}
	// bottleneck: b3 = conv(a3), a3 = conv(p2)
	NN_CK(dw_layer(u, S, 6, 3, S.gB3.as<bf16>(), S.a[3].as<bf16>(), nullptr, st));
	NN_CK(dxconv());   // gA[3] (masked by a3)
	NN_CK(dw_layer(u, S, 5, 3, S.gA[3].as<bf16>(), S.p[2].as<bf16>(), nullptr, st));
	NN_CK(dxconv());   // gP[2]
	// encoder levels 2, 1, 0
	for (int l = 2; l >= 0; --l) {
		const int hl = h >> l, wl = w >> l;
		k_pool_bwd<<<nblk((long)n * hl * wl * CH[l] / 8), kT, 0, st>>>(S.gP[l].as<bf16>(),
				S.gSkip[l].as<bf16>(), S.s[l].as<bf16>(), S.gS[l].as<bf16>(), n, hl, wl, CH[l]);
		const int ls = l == 0 ? 0 : 2 * l;        // s_l = conv(a_l)
		NN_CK(dw_layer(u, S, ls, l, S.gS[l].as<bf16>(), S.a[l].as<bf16>(), nullptr, st));
		NN_CK(dxconv());   // gA[l] (masked by a_l)
		if (l > 0) {
			const int la = 2 * l - 1;              // a_l = conv(p_{l-1})
			NN_CK(dw_layer(u, S, la, l, S.gA[l].as<bf16>(), S.p[l - 1].as<bf16>(), nullptr, st));
			NN_CK(dxconv());   // gP[l-1]
		}
	}
	// input layer
	{
		long nb = std::min(1024L, (np0 + 1023) / 1024);
		const long per = (np0 + nb - 1) / nb;
		nb = (np0 + per - 1) / per;
		NN_CK(S.part.ensure(sizeof(float) * (size_t)(nb * 9 * C0)));
		k_dw_in<<<(unsigned)nb, 9 * C0 + 32 - (9 * C0) % 32, 0, st>>>(S.gA[0].as<bf16>(), x, n,
				h, w, per, S.part.as<float>());
		k_sum_parts<<<nblk(9 * C0), kT, 0, st>>>(S.part.as<float>(), (int)nb, 9 * C0, G);
	}
	CG_CK(cudaGetLastError());
	return 0;
}

int refresh_bf16(carpio_gpu_unet* u, cudaStream_t st) {
	const float* W = u->w.as<float>();
	for (int l = 0; l < 13; ++l) {
		const Layer& L = layers()[l];
		const long len = 9L * L.cout * (L.cin0 + L.cin1);
		k_wt_flip<<<nblk(len), kT, 0, st>>>(W + L.off, W16(u, l), WT2(u, l), L.cout,
				L.cin0 + L.cin1);
	}
	CG_CK(cudaGetLastError());
	return 0;
}

// deterministic He-normal initialisation (splitmix64 + Box-Muller)
void init_params(std::vector<float>& p, uint64_t seed) {
	p.assign(n_params(), 0.f);
	uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
	auto next = [&]() {
		uint64_t z = (st += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		return z ^ (z >> 31);
	};
	auto normal = [&]() {
		const double u1 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
		const double u2 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
		return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
	};
	for (long i = 0; i < 9 * C0; ++i) p[i] = (float)(normal() * std::sqrt(2.0 / 9.0));
	for (int l = 0; l < 13; ++l) {
		const Layer& L = layers()[l];
		const double sd = std::sqrt(2.0 / (9.0 * (L.cin0 + L.cin1)));
		const long len = 9L * L.cout * (L.cin0 + L.cin1);
		for (long i = 0; i < len; ++i) p[L.off + i] = (float)(normal() * sd);
	}
	for (int c = 0; c < C0; ++c) p[off_out() + c] = (float)(normal() * std::sqrt(1.0 / C0));
}

bool shape_ok(int n, int h, int w) {
	if (n < 1 || h < 16 || w < 16 || h % 8 || w % 8) return false;
	// 128-pixel tiles at the coarsest level: whole rows or whole images
	const int h3 = h / 8, w3 = w / 8;
	const int bw = std::min(w3, 128), bh = std::min(h3, 128 / bw);
	const int bn = 128 / (bw * bh);
	return bw * bh * bn == 128 && w3 % bw == 0 && h3 % bh == 0 && n % bn == 0;
}

}  // namespace

extern "C" {

long carpio_gpu_unet_num_params(void) { return n_params(); }

int carpio_gpu_unet_create(uint64_t seed, carpio_gpu_unet** out) {
	if (!out) return CARPIO_GPU_EINVAL;
	*out = nullptr;
	auto* u = new carpio_gpu_unet();
	auto fail = [&](int code) { delete u; return code; };
	if (cudaStreamCreateWithFlags(&u->s, cudaStreamNonBlocking) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	const long np = n_params();
	int rc;
	if ((rc = u->w.ensure(sizeof(float) * np)) || (rc = u->g.ensure(sizeof(float) * np))
			|| (rc = u->m.ensure(sizeof(float) * np)) || (rc = u->v.ensure(sizeof(float) * np))
			|| (rc = u->wbf.ensure(sizeof(bf16) * np)) || (rc = u->wt2.ensure(sizeof(bf16) * np))
			|| (rc = u->loss.ensure(sizeof(double))) || (rc = u->err.ensure(sizeof(int))))
		return fail(rc);
	init_params(u->host_w, seed);
	if (cudaMemcpy(u->w.p, u->host_w.data(), sizeof(float) * np, cudaMemcpyHostToDevice)
			!= cudaSuccess || cudaMemset(u->m.p, 0, sizeof(float) * np) != cudaSuccess
			|| cudaMemset(u->v.p, 0, sizeof(float) * np) != cudaSuccess
			|| cudaMemset(u->g.p, 0, sizeof(float) * np) != cudaSuccess
			|| cudaMemset(u->err.p, 0, sizeof(int)) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	if ((rc = refresh_bf16(u, u->s))) return fail(rc);
	if (cudaStreamSynchronize(u->s) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	*out = u;
	return 0;
}

int carpio_gpu_unet_destroy(carpio_gpu_unet* u) {
	if (!u) return CARPIO_GPU_EINVAL;
	delete u;
	return 0;
}

int carpio_gpu_unet_get_params(carpio_gpu_unet* u, float* out) {
	if (!u || !out) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	CG_CK(cudaMemcpyAsync(out, u->w.p, sizeof(float) * n_params(), cudaMemcpyDefault, u->s));
	CG_CK(cudaStreamSynchronize(u->s));
	return 0;
}

int carpio_gpu_unet_set_params(carpio_gpu_unet* u, const float* in) {
	if (!u || !in) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	CG_CK(cudaMemcpyAsync(u->w.p, in, sizeof(float) * n_params(), cudaMemcpyDefault, u->s));
	CG_CK(cudaMemsetAsync(u->m.p, 0, sizeof(float) * n_params(), u->s));
	CG_CK(cudaMemsetAsync(u->v.p, 0, sizeof(float) * n_params(), u->s));
	u->step = 0;
	int rc = refresh_bf16(u, u->s);
	if (rc) return rc;
	CG_CK(cudaStreamSynchronize(u->s));
	return 0;
}

static int unet_err(carpio_gpu_unet* u) {
	int e = 0;
	CG_CK(cudaMemcpyAsync(&e, u->err.p, sizeof(int), cudaMemcpyDeviceToHost, u->s));
	CG_CK(cudaStreamSynchronize(u->s));
	if (e) {
		cudaMemsetAsync(u->err.p, 0, sizeof(int), u->s);
		cudaStreamSynchronize(u->s);
	}
	return e;
}

}  // extern "C"

namespace cg_host {
// The forward for the library's own solvers: stream-ordered on `st`, no
// host synchronisation and no pointer checks (the caller passes device
// buffers it owns); a device-side failure is left in the flag unet_err_flag
// points to, for the caller to read with its next synchronisation.
int unet_forward_async(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		float* z, cudaStream_t st) {
	if (!u || !x || !z || !shape_ok(n, h, w)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	int rc = 0;
	Shape* S = get_shape(u, n, h, w, &rc);
	if (!S) return rc;
	return forward(u, *S, x, z, st);
}

int* unet_err_flag(carpio_gpu_unet* u) { return u->err.as<int>(); }

int unet_take_err(carpio_gpu_unet* u) { return unet_err(u); }
}  // namespace cg_host

extern "C" {

int carpio_gpu_unet_forward(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		float* z, void* stream) {
	if (!u || !x || !z || !shape_ok(n, h, w)) return CARPIO_GPU_EINVAL;
	if (!cg_host::is_device_ptr(x) || !cg_host::is_device_ptr(z)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	int rc = 0;
	Shape* S = get_shape(u, n, h, w, &rc);
	if (!S) return rc;
	cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : u->s;
	if ((rc = forward(u, *S, x, z, st))) return rc;
	CG_CK(cudaStreamSynchronize(st));
	return unet_err(u);
}

int carpio_gpu_unet_grad(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		const float* t, int loss_mode, float* grad_out, double* loss) {
	if (!u || !x || !t || !shape_ok(n, h, w) || loss_mode < 0 || loss_mode > 1)
		return CARPIO_GPU_EINVAL;
	if (!cg_host::is_device_ptr(x) || !cg_host::is_device_ptr(t)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	int rc = 0;
	Shape* S = get_shape(u, n, h, w, &rc);
	if (!S) return rc;
	if ((rc = grad(u, *S, x, t, loss_mode, u->s))) return rc;
	if (grad_out)
		CG_CK(cudaMemcpyAsync(grad_out, u->g.p, sizeof(float) * n_params(), cudaMemcpyDefault, u->s));
	if (loss) CG_CK(cudaMemcpyAsync(loss, u->loss.p, sizeof(double), cudaMemcpyDefault, u->s));
	CG_CK(cudaStreamSynchronize(u->s));
	return unet_err(u);
}

int carpio_gpu_unet_train_step(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		const float* t, int loss_mode, float lr, double* loss) {
	if (!u || !x || !t || !shape_ok(n, h, w) || !(lr >= 0) || loss_mode < 0 || loss_mode > 1)
		return CARPIO_GPU_EINVAL;
	if (!cg_host::is_device_ptr(x) || !cg_host::is_device_ptr(t)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(u->mu);
	int rc = 0;
	Shape* S = get_shape(u, n, h, w, &rc);
	if (!S) return rc;
	cudaStream_t st = u->s;
	if ((rc = grad(u, *S, x, t, loss_mode, st))) return rc;
	++u->step;
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.f - std::pow(b1, (float)u->step), c2 = 1.f - std::pow(b2, (float)u->step);
	k_adam<<<nblk(n_params()), kT, 0, st>>>(u->w.as<float>(), u->g.as<float>(),
			u->m.as<float>(), u->v.as<float>(), n_params(), lr, b1, b2, 1e-8f, c1, c2);
	if ((rc = refresh_bf16(u, st))) return rc;
	if (loss) CG_CK(cudaMemcpyAsync(loss, u->loss.p, sizeof(double), cudaMemcpyDefault, st));
	CG_CK(cudaStreamSynchronize(st));
	return unet_err(u);
}

}  // extern "C"
