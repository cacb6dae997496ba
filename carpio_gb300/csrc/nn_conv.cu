// 3x3 convolution (stride 1, zero padding 1) of BF16 NHWC activations as an
// implicit GEMM on the fifth-generation tensor cores: the learned
// preconditioner's hot operator.
//
//   out[p][co] = sum over taps (dy, dx) and input channels ci of
//                in[p + (dy - 1, dx - 1)][ci] * wt[dy * 3 + dx][co][ci]
//
// One CTA computes a tile of 128 output pixels x ntile output channels. The
// K loop runs over the 9 taps and the input channels in chunks of 32 (one
// 64-byte row per pixel): warp 0 streams the A tile (128 pixels of the
// shifted input window; TMA zero-fills the padding outside the image) and
// the B tile (ntile weight rows) into a 4-stage shared-memory ring with
// 64-byte swizzle; one thread of warp 1 issues two tcgen05.mma (K = 16 each)
// per chunk into an FP32 accumulator in tensor memory; warps 2-5 read the
// accumulator back (tcgen05.ld, one 32-lane quadrant per warp), apply ReLU
// or a ReLU mask, round to BF16 and store. Two input tensors can be read as
// one (channel concatenation), and the output channels can be split between
// two tensors, which is what the backward pass of a concatenating layer
// needs. Every mbarrier wait is bounded; a launch that gives up records an
// error, waits (bounded) for its own copies and MMAs and frees its tensor
// memory.
#include "internal.hpp"
#include "tc.cuh"

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

namespace cg_nn {

using namespace cg_tc;

constexpr int kConvThreads = 192;
constexpr int kStages = 4;
constexpr int kTileM = 128;
constexpr int kKC = 32;
constexpr uint32_t kABytes = kTileM * kKC * 2;

struct ConvDims {
	int nsrc, cin0, cin1;
	int n, h, w;
	int bw, bh, bn;          // pixel tile bw x bh x bn = 128
	int ntile, cout, split;  // channels [0, split) -> out0, the rest -> out1
	int relu;
	__nv_bfloat16* out0;
	__nv_bfloat16* out1;
	const __nv_bfloat16* mask0;
	const __nv_bfloat16* mask1;
	int* err;
	unsigned long long wait_ns;
};

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
	__nv_bfloat162 v = __floats2bfloat162_rn(a, b);
	return *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(kConvThreads, 1) k_conv3x3(
		const __grid_constant__ CUtensorMap in0, const __grid_constant__ CUtensorMap in1,
		const __grid_constant__ CUtensorMap wt, const ConvDims d) {
	extern __shared__ __align__(1024) uint8_t smem_raw[];
	__shared__ __align__(8) uint64_t full[kStages], empty[kStages], accf;
	__shared__ uint32_t s_tmem;
	__shared__ int s_abort, s_issued, s_consumed;
	uint8_t* base = reinterpret_cast<uint8_t*>(
			(reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
	const uint32_t bbytes = (uint32_t)d.ntile * kKC * 2;
	const uint32_t stage_bytes = kABytes + ((bbytes + 1023u) & ~1023u);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

	const int tiles_w = d.w / d.bw, tiles_h = d.h / d.bh;
	int tt = blockIdx.x;
	const int tw = tt % tiles_w;
	tt /= tiles_w;
	const int th = tt % tiles_h;
	tt /= tiles_h;
	const int w0 = tw * d.bw, h0 = th * d.bh, n0 = tt * d.bn;
	const int co0 = blockIdx.y * d.ntile;
	const int nch0 = d.cin0 / kKC, nch = nch0 + (d.nsrc > 1 ? d.cin1 / kKC : 0);
	const int nk = 9 * nch;
	uint32_t ncols = 32;
	while (ncols < (uint32_t)d.ntile) ncols <<= 1;

	if (threadIdx.x == 0) {
		for (int s = 0; s < kStages; ++s) {
			mbar_init(smem_addr(&full[s]), 1);
			mbar_init(smem_addr(&empty[s]), 1);
		}
		mbar_init(smem_addr(&accf), 1);
		fence_mbar_init();
		s_abort = 0;
		s_issued = 0;
		s_consumed = 0;
		prefetch_tmap(&in0);
		if (d.nsrc > 1) prefetch_tmap(&in1);
		prefetch_tmap(&wt);
	}
	if (warp == 1) {
		tmem_alloc(smem_addr(&s_tmem), ncols);
		tmem_relinquish();
	}
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const uint32_t tmem = s_tmem;

	if (warp == 0) {
		if (lane == 0) {
			int k = 0;
			for (; k < nk; ++k) {
				const int s = k % kStages;
				const uint32_t round = (uint32_t)(k / kStages);
				if (!mbar_wait(smem_addr(&empty[s]), (round & 1u) ^ 1u, d.err, d.wait_ns)) {
					atomicCAS(d.err, 0, CARPIO_GPU_ETIMEOUT);
					s_abort = 1;
					break;
				}
				const int tap = k / nch, c = k - tap * nch;
				const int dy = tap / 3, dx = tap - dy * 3;
				const bool second = c >= nch0;
				const int ci = (second ? c - nch0 : c) * kKC;       // channel in its source
				const int cw = c * kKC;                              // channel in the weights
				const uint32_t a_dst = smem_addr(base + (size_t)s * stage_bytes);
				const uint32_t bar = smem_addr(&full[s]);
				mbar_arrive_expect_tx(bar, kABytes + bbytes);
				tma_load_4d(a_dst, second ? &in1 : &in0, ci, w0 + dx - 1, h0 + dy - 1, n0, bar);
				tma_load_3d(a_dst + kABytes, &wt, cw, co0, tap, bar);
			}
			s_issued = k;
		}
	} else if (warp == 1) {
		if (lane == 0) {
			const uint32_t idesc = idesc_bf16_f32(kTileM, d.ntile);
			int k = 0;
			for (; k < nk; ++k) {
				const int s = k % kStages;
				const uint32_t round = (uint32_t)(k / kStages);
				if (!mbar_wait(smem_addr(&full[s]), round & 1u, d.err, d.wait_ns)) {
					atomicCAS(d.err, 0, CARPIO_GPU_ETIMEOUT);
					s_abort = 1;
					break;
				}
				tc_fence_after();
				const uint32_t a = smem_addr(base + (size_t)s * stage_bytes), b = a + kABytes;
#pragma unroll
				for (int j = 0; j < 2; ++j) {
					const uint64_t ad = smem_desc(a + 32u * j, 16, 512, kSwizzle64);
					const uint64_t bd = smem_desc(b + 32u * j, 16, 512, kSwizzle64);
					mma_bf16(tmem, ad, bd, idesc, (k > 0 || j > 0) ? 1u : 0u);
				}
				// the stage is free once these MMAs have read it
				mma_commit(smem_addr(&empty[s]));
			}
			s_consumed = k;
			// the accumulator is complete (after a give-up: every issued MMA
			// has finished)
			mma_commit(smem_addr(&accf));
		}
	} else {
		const int q = warp & 3;
		const int m = q * 32 + lane;
		bool ok = mbar_wait(smem_addr(&accf), 0, d.err, d.wait_ns);
		ok = __all_sync(0xffffffffu, ok);
		tc_fence_after();
		// (after a give-up elsewhere the tile is stored partial; the launch's
		// error word says so)
		if (!ok) {
			if (lane == 0) atomicCAS(d.err, 0, CARPIO_GPU_ETIMEOUT);
		} else {
			const int pw = m % d.bw, ph = (m / d.bw) % d.bh, pn = m / (d.bw * d.bh);
			const long gp = ((long)(n0 + pn) * d.h + (h0 + ph)) * d.w + (w0 + pw);
			for (int c = 0; c < d.ntile; c += 32) {
				float v[32];
				tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c, v);
				const int co = co0 + c;
				const bool first = co < d.split;
				const int cdst = first ? d.split : d.cout - d.split;
				const int cl = first ? co : co - d.split;
				__nv_bfloat16* dst = (first ? d.out0 : d.out1) + gp * cdst + cl;
				const __nv_bfloat16* mk = first ? d.mask0 : d.mask1;
				if (d.relu) {
#pragma unroll
					for (int i = 0; i < 32; ++i) v[i] = fmaxf(v[i], 0.f);
				}
				if (mk) {
					const uint4* mv = reinterpret_cast<const uint4*>(mk + gp * cdst + cl);
#pragma unroll
					for (int u = 0; u < 4; ++u) {
						const uint4 w4 = mv[u];
						const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(&w4);
#pragma unroll
						for (int i = 0; i < 8; ++i)
							if (!(__bfloat162float(mb[i]) > 0.f)) v[u * 8 + i] = 0.f;
					}
				}
				uint4* o = reinterpret_cast<uint4*>(dst);
#pragma unroll
				for (int u = 0; u < 4; ++u) {
					uint4 pk;
					pk.x = pack_bf16(v[u * 8 + 0], v[u * 8 + 1]);
					pk.y = pack_bf16(v[u * 8 + 2], v[u * 8 + 3]);
					pk.z = pack_bf16(v[u * 8 + 4], v[u * 8 + 5]);
					pk.w = pack_bf16(v[u * 8 + 6], v[u * 8 + 7]);
					o[u] = pk;
				}
			}
		}
	}
	tc_fence_before();
	__syncthreads();
	// after a give-up, the copies and MMAs still in flight finish before the
	// CTA frees its tensor memory and leaves
	if (s_abort && threadIdx.x == 0) {
		for (int k = s_consumed; k < s_issued; ++k)
			mbar_wait_for(smem_addr(&full[k % kStages]), (uint32_t)(k / kStages) & 1u, d.wait_ns);
	}
	if (s_abort && threadIdx.x == 32) mbar_wait_for(smem_addr(&accf), 0, d.wait_ns);
	__syncthreads();
	if (warp == 1) {
		tc_fence_after();
		tmem_dealloc(tmem, ncols);
	}
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	if (!fn) {
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
				cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
	}
	return fn;
}

}  // namespace cg_nn

namespace cg_host {

using namespace cg_nn;

// activation tensor [n][h][w][c] (BF16), box of 32 channels x bw x bh x bn
int act_map(CUtensorMap* m, const void* p, int c, int w, int h, int n, int bw, int bh, int bn) {
	auto enc = encode_fn();
	if (!enc) return CARPIO_GPU_ECUDA;
	if (reinterpret_cast<uintptr_t>(p) % 16) return CARPIO_GPU_EINVAL;
	cuuint64_t dims[4] = { (cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n };
	cuuint64_t str[3] = { (cuuint64_t)c * 2, (cuuint64_t)w * c * 2, (cuuint64_t)h * w * c * 2 };
	cuuint32_t box[4] = { (cuuint32_t)kKC, (cuuint32_t)bw, (cuuint32_t)bh, (cuuint32_t)bn };
	cuuint32_t es[4] = { 1, 1, 1, 1 };
	CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(p), dims, str,
			box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
			CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS ? 0 : CARPIO_GPU_EINVAL;
}

// weights [9][cout][ci] (BF16), box of 32 input channels x ntile rows
int wt_map(CUtensorMap* m, const void* p, int ci, int cout, int ntile) {
	auto enc = encode_fn();
	if (!enc) return CARPIO_GPU_ECUDA;
	if (reinterpret_cast<uintptr_t>(p) % 16) return CARPIO_GPU_EINVAL;
	cuuint64_t dims[3] = { (cuuint64_t)ci, (cuuint64_t)cout, 9 };
	cuuint64_t str[2] = { (cuuint64_t)ci * 2, (cuuint64_t)cout * ci * 2 };
	cuuint32_t box[3] = { (cuuint32_t)kKC, (cuuint32_t)ntile, 1 };
	cuuint32_t es[3] = { 1, 1, 1 };
	CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(p), dims, str,
			box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
			CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	return r == CUDA_SUCCESS ? 0 : CARPIO_GPU_EINVAL;
}

// A prepared convolution launch (tensor maps built once, replayable).
struct ConvLaunch {
	CUtensorMap in0, in1, wt;
	ConvDims d;
	dim3 grid;
	size_t smem = 0;
};

int conv_prepare(ConvLaunch& L, const void* in0, int cin0, const void* in1, int cin1,
		int n, int h, int w, const void* wt, int cout, int ntile, void* out0, int split,
		void* out1, const void* mask0, const void* mask1, int relu, int* err) {
	if (!in0 || !wt || !out0 || n < 1 || h < 1 || w < 1 || cin0 < kKC || cin0 % kKC
			|| (in1 && (cin1 < kKC || cin1 % kKC)) || cout < 32 || ntile < 32
			|| ntile > 256 || ntile % 32 || cout % ntile || split < 0 || split > cout
			|| split % 32 || (split < cout && !out1) || !err)
		return CARPIO_GPU_EINVAL;
	const int bw = std::min(w, kTileM), bh = std::min(h, kTileM / bw);
	const int bn = kTileM / (bw * bh);
	if (bw * bh * bn != kTileM || w % bw || h % bh || n % bn) return CARPIO_GPU_EINVAL;
	for (const void* p : { (const void*)out0, (const void*)out1, mask0, mask1 })
		if (p && reinterpret_cast<uintptr_t>(p) % 16) return CARPIO_GPU_EINVAL;
	int rc;
	if ((rc = act_map(&L.in0, in0, cin0, w, h, n, bw, bh, bn))) return rc;
	if ((rc = act_map(&L.in1, in1 ? in1 : in0, in1 ? cin1 : cin0, w, h, n, bw, bh, bn))) return rc;
	if ((rc = wt_map(&L.wt, wt, cin0 + (in1 ? cin1 : 0), cout, ntile))) return rc;
	ConvDims& d = L.d;
	d.nsrc = in1 ? 2 : 1;
	d.cin0 = cin0;
	d.cin1 = in1 ? cin1 : 0;
	d.n = n;
	d.h = h;
	d.w = w;
	d.bw = bw;
	d.bh = bh;
	d.bn = bn;
	d.ntile = ntile;
	d.cout = cout;
	d.split = split;
	d.relu = relu;
	d.out0 = static_cast<__nv_bfloat16*>(out0);
	d.out1 = static_cast<__nv_bfloat16*>(out1);
	d.mask0 = static_cast<const __nv_bfloat16*>(mask0);
	d.mask1 = static_cast<const __nv_bfloat16*>(mask1);
	d.err = err;
	d.wait_ns = (unsigned long long)watchdog().wait_ms * 1000000ull;
	L.grid = dim3((unsigned)((long)n * h * w / kTileM), (unsigned)(cout / ntile));
	const uint32_t bbytes = (uint32_t)ntile * kKC * 2;
	L.smem = 1024 + (size_t)kStages * (kABytes + ((bbytes + 1023u) & ~1023u));
	static bool attr = false;
	if (!attr) {
		CG_CK(cudaFuncSetAttribute((const void*)k_conv3x3,
				cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
		attr = true;
	}
	return 0;
}

int conv_launch(const ConvLaunch& L, cudaStream_t s) {
	k_conv3x3<<<L.grid, kConvThreads, L.smem, s>>>(L.in0, L.in1, L.wt, L.d);
	CG_CK(cudaGetLastError());
	return 0;
}

// heap-held launches for the U-Net runner (nn.cu)
int conv_prepare_ext(void** handle, const void* in0, int cin0, const void* in1, int cin1,
		int n, int h, int w, const void* wt, int cout, int ntile, void* out0, int split,
		void* out1, const void* mask0, const void* mask1, int relu, int* err) {
	auto* L = new ConvLaunch();
	int rc = conv_prepare(*L, in0, cin0, in1, cin1, n, h, w, wt, cout, ntile, out0, split,
			out1, mask0, mask1, relu, err);
	if (rc) {
		delete L;
		return rc;
	}
	*handle = L;
	return 0;
}

int conv_launch_ext(const void* handle, cudaStream_t s) {
	return conv_launch(*static_cast<const ConvLaunch*>(handle), s);
}

void conv_free_ext(void* handle) { delete static_cast<ConvLaunch*>(handle); }

}  // namespace cg_host

extern "C" int carpio_gpu_nn_conv3x3(const void* in0, int cin0, const void* in1, int cin1,
		int n, int h, int w, const void* wt, int cout, void* out0, int split, void* out1,
		const void* mask0, const void* mask1, int relu, void* stream) {
	using namespace cg_host;
	static int* err = nullptr;
	if (!err) {
		CG_CK(cudaMalloc(&err, sizeof(int)));
		CG_CK(cudaMemset(err, 0, sizeof(int)));
	}
	if (!in0 || !wt || !out0 || !is_device_ptr(in0) || !is_device_ptr(wt) || !is_device_ptr(out0))
		return CARPIO_GPU_EINVAL;
	ConvLaunch L;
	int ntile = cout <= 256 ? cout : (cout % 256 == 0 ? 256 : (cout % 192 == 0 ? 192 : 128));
	int rc = conv_prepare(L, in0, cin0, in1, cin1, n, h, w, wt, cout, ntile, out0,
			split > 0 ? split : cout, out1, mask0, mask1, relu, err);
	if (rc) return rc;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	if ((rc = conv_launch(L, s))) return rc;
	int herr = 0;
	CG_CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	if (herr) {
		cudaMemset(err, 0, sizeof(int));
		return herr;
	}
	return 0;
}
