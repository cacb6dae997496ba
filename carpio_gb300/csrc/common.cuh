// Shared device infrastructure for the persistent Krylov kernels.
//
//  * GridCtl / grid_sync: a software grid barrier for kernels launched with
//    cudaLaunchCooperativeKernel (all blocks co-resident). Every wait is
//    bounded by a %globaltimer deadline; on expiry the kernel records
//    CARPIO_GPU_ETIMEOUT in the error word and every block leaves at its next
//    barrier. Nothing spins without a limit.
//  * block_sum / grid_allreduce: fixed-order warp-shuffle + shared-memory
//    trees, then a fixed-order sum of the per-block partials done redundantly
//    by every block, so each block holds the same bits and the result does not
//    depend on scheduling.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/carpio_gpu.h"

namespace cg_dev {

constexpr int kThreads = 256;            // threads per block of every solver
constexpr int kWarps = kThreads / 32;
constexpr int kMaxReduce = 6;            // values per grid all-reduce

__device__ __forceinline__ unsigned long long globaltimer() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// L2-coherent loads for data written by other blocks of the same launch
template<class T> __device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

struct GridCtl {
	unsigned* count;          // barrier word (arrivals + release bit)
	unsigned* gen;            // unused by the barrier; kept for layout
	int* err;                 // first error code (0 = none)
	double* partials;         // [2 banks][kMaxReduce][gridDim.x]
	unsigned long long wait_ns;   // bound of one barrier wait
	unsigned long long solve_ns;  // bound of the whole launch
	unsigned long long deadline;  // absolute %globaltimer bound, set by start()
	// each block stamps its own deadline when it starts
	__device__ __forceinline__ void start() { deadline = globaltimer() + solve_ns; }
};

__device__ __forceinline__ int read_err(const GridCtl& c) {
	return *(volatile int*)c.err;
}

__device__ __forceinline__ void set_err(const GridCtl& c, int code) {
	atomicCAS(c.err, 0, code);
}

// Returns false once any block has recorded an error (timeout included);
// callers then leave the kernel. All threads of the block get the same answer.
//
// One counter word carries both arrival and release: every block adds 1,
// block 0 adds 2^31 - (gridDim.x - 1), so the barrier's increments total
// exactly 2^31 and the word's top bit flips when the last block arrives. A
// block waits until the top bit differs from the value its own atomicAdd
// returned. No reset is needed between barriers and the critical path is one
// atomic plus one poll.
// ONE: the caller may launch a single block, and then the block barrier
// is the grid barrier (the solve deadline is checked by the all-reduces).
template<bool ONE = false>
__device__ __forceinline__ bool grid_sync(const GridCtl& c) {
	__shared__ int s_ok;
	if (ONE && gridDim.x == 1) {
		__syncthreads();
		return true;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
		__threadfence();
		const unsigned old = atomicAdd(c.count, inc);
		volatile unsigned* vc = c.count;
		unsigned long long t0 = 0;
		unsigned polls = 0;
		int ok = 1;
		while (((*vc ^ old) & 0x80000000u) == 0) {
			if ((++polls & 63u) == 0) {
				// an error recorded by any block ends the wait; a block
				// that gave up never arrives again, so the others see the
				// error here within 64 polls
				if (*(volatile int*)c.err) { ok = 0; break; }
				unsigned long long t = globaltimer();
				if (t0 == 0) t0 = t;
				if (t - t0 > c.wait_ns || t > c.deadline) {
					set_err(c, CARPIO_GPU_ETIMEOUT);
					ok = 0;
					break;
				}
			}
		}
		// the solve deadline also binds launches whose blocks never wait
		if (ok && blockIdx.x == 0 && globaltimer() > c.deadline) {
			set_err(c, CARPIO_GPU_ETIMEOUT);
			ok = 0;
		}
		__threadfence();
		s_ok = ok;
	}
	__syncthreads();
	return s_ok != 0;
}

// Sum of NV values over the block in a fixed tree; every thread gets it.
// Any block size that is a multiple of 32, up to 1024.
template<class R, int NV>
__device__ __forceinline__ void block_sum(R (&v)[NV]) {
	__shared__ R s_w[NV][32];
	__shared__ R s_out[NV];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nwarps = blockDim.x >> 5;
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		R x = v[m];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		if (lane == 0) s_w[m][warp] = x;
	}
	__syncthreads();
	if (warp == 0) {
#pragma unroll
		for (int m = 0; m < NV; ++m) {
			R x = lane < nwarps ? s_w[m][lane] : R(0);
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
			if (lane == 0) s_out[m] = x;
		}
	}
	__syncthreads();
#pragma unroll
	for (int m = 0; m < NV; ++m) v[m] = s_out[m];
	__syncthreads();
}

// Max of a non-negative value over the block (NaN never wins, matching
// std::max(max, v) with max first).
__device__ __forceinline__ double block_max(double v) {
	__shared__ double s_w[32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nwarps = blockDim.x >> 5;
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		double y = __shfl_down_sync(0xffffffffu, v, o);
		v = (v < y) ? y : v;
	}
	if (lane == 0) s_w[warp] = v;
	__syncthreads();
	if (warp == 0) {
		v = lane < nwarps ? s_w[lane] : 0.0;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			double y = __shfl_down_sync(0xffffffffu, v, o);
			v = (v < y) ? y : v;
		}
		if (lane == 0) s_w[0] = v;
	}
	__syncthreads();
	v = s_w[0];
	__syncthreads();
	return v;
}

// Block sum with one __syncthreads: warp trees, lane 0 of each warp writes
// its value into buffer `buf`, then every thread adds the warp values in the
// same fixed order. The caller guarantees that no thread still reads `buf`
// from an earlier call (grid_allreduce alternates the buffers and a grid
// barrier sits between two uses of the same one).
template<class R, int NV>
__device__ __forceinline__ void block_sum_light(R (&v)[NV], int buf) {
	__shared__ R s_w[2][NV][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nwarps = blockDim.x >> 5;
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		R x = v[m];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		if (lane == 0) s_w[buf][m][warp] = x;
	}
	__syncthreads();
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		R x = 0;
		for (int w = 0; w < nwarps; ++w) x += s_w[buf][m][w];
		v[m] = x;
	}
}

// The same sum for thread 0 alone (the other threads' v is left
// unspecified): the warp values added in the same fixed order by one thread
// instead of by every thread of the block -- FP64 adds cost a warp
// instruction each on the FP64 pipe, whose throughput bounds the kernels
// that reduce in FP64.
template<class R, int NV>
__device__ __forceinline__ void block_sum_to0(R (&v)[NV], int buf) {
	__shared__ R s_w0[2][NV][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nwarps = blockDim.x >> 5;
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		R x = v[m];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		if (lane == 0) s_w0[buf][m][warp] = x;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
#pragma unroll
		for (int m = 0; m < NV; ++m) {
			R x = 0;
			for (int w = 0; w < nwarps; ++w) x += s_w0[buf][m][w];
			v[m] = x;
		}
	}
}

__device__ __forceinline__ unsigned atom_add_release_gpu(unsigned* p, unsigned v) {
	unsigned old;
	asm volatile("atom.add.release.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
	return old;
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
	unsigned v;
	asm volatile("ld.acquire.gpu.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

// Grid-wide sum of NV values (R = double or float); every block ends with
// the same bits. `bank` alternates 0/1 on consecutive calls so a fast block
// never overwrites partials a slow block is still reading.
//
// Thread 0's side of a grid all-reduce: arrive (release atomic on the
// flip-bit word) and poll with acquire loads until every block has arrived,
// bounded by the watchdog. Returns 0 on error (recorded in c.err).
__device__ __forceinline__ int grid_arrive_wait(const GridCtl& c) {
	int ok = 1;
	const unsigned inc = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
	const unsigned old = atom_add_release_gpu(c.count, inc);
	unsigned long long t0 = 0;
	unsigned polls = 0;
	while (((ld_acquire_gpu(c.count) ^ old) & 0x80000000u) == 0) {
		if ((++polls & 63u) == 0) {
			if (*(volatile int*)c.err) { ok = 0; break; }
			unsigned long long t = globaltimer();
			if (t0 == 0) t0 = t;
			if (t - t0 > c.wait_ns || t > c.deadline) {
				set_err(c, CARPIO_GPU_ETIMEOUT);
				ok = 0;
				break;
			}
		}
	}
	if (ok && blockIdx.x == 0 && globaltimer() > c.deadline) {
		set_err(c, CARPIO_GPU_ETIMEOUT);
		ok = 0;
	}
	return ok;
}

// One __syncthreads gathers the block's value; then warp 0 alone arrives at
// the barrier (thread 0: release atomic on the flip-bit word, acquire polls
// bounded by the watchdog), reads the blocks' partials in a fixed order and
// reduces them; a second __syncthreads hands the result to the block. The
// first __syncthreads also orders every thread's earlier global writes before
// thread 0's release, so data published before the call is visible to every
// block after it. Returns false on error.
template<class R, int NV, bool ONE = false>
__device__ __forceinline__ bool grid_allreduce(R (&v)[NV], const GridCtl& c,
		int& bank) {
	__shared__ R s_res[2][NV];
	__shared__ int s_ok[2];
	if (ONE && gridDim.x == 1) {
		// one block: its sum is the grid's; only the solve deadline binds.
		// block_sum_light's barrier publishes the flag.
		if (threadIdx.x == 0) {
			const bool late = globaltimer() > c.deadline;
			if (late) set_err(c, CARPIO_GPU_ETIMEOUT);
			s_ok[bank] = late ? 0 : 1;
		}
		block_sum_light<R, NV>(v, 0);
		const bool ok1 = s_ok[bank] != 0;
		bank ^= 1;
		return ok1;
	}
	block_sum_to0<R, NV>(v, 0);
	double* part = c.partials + (size_t)bank * kMaxReduce * gridDim.x;
	const int lane = threadIdx.x & 31;
	if (threadIdx.x < 32) {
		int ok = 1;
		if (lane == 0) {
#pragma unroll
			for (int m = 0; m < NV; ++m) part[m * gridDim.x + blockIdx.x] = (double)v[m];
			ok = grid_arrive_wait(c);
		}
		__syncwarp();
		ok = __shfl_sync(0xffffffffu, ok, 0);
		if (ok) {
#pragma unroll
			for (int m = 0; m < NV; ++m) {
				R acc = 0;
#pragma unroll 4
				for (int b = lane; b < (int)gridDim.x; b += 32)
					acc += (R)ldcg(&part[m * gridDim.x + b]);
#pragma unroll
				for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
				if (lane == 0) s_res[bank][m] = acc;
			}
		}
		if (lane == 0) s_ok[bank] = ok;
	}
	__syncthreads();
#pragma unroll
	for (int m = 0; m < NV; ++m) v[m] = s_res[bank][m];
	const bool ok = s_ok[bank] != 0;
	bank ^= 1;
	return ok;
}

// grid_allreduce for FP64 values with the block's last stage in warp 0's
// shuffles instead of thread 0's serial loop over the warps: an FP64 warp
// instruction costs 64 cycles of its sub-partition, so the serial loop over
// 16 warps' sums took 16 x 64 cycles a value. Same protocol, fixed order.
template<int NV>
__device__ __forceinline__ bool grid_allreduce_w0(double (&v)[NV], const GridCtl& c,
		int& bank) {
	static_assert(NV >= 1 && NV <= kMaxReduce, "partials");
	__shared__ double s_w[NV][32];
	__shared__ double s_r[2][NV];
	__shared__ int s_ok[2];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int nw = blockDim.x >> 5;
#pragma unroll
	for (int m = 0; m < NV; ++m) {
		double x = v[m];
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
		if (lane == 0) s_w[m][warp] = x;
	}
	__syncthreads();
	if (warp == 0) {
		double* part = c.partials + (size_t)bank * kMaxReduce * gridDim.x;
		double bs[NV];
#pragma unroll
		for (int m = 0; m < NV; ++m) {
			double x = lane < nw ? s_w[m][lane] : 0.0;
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
			bs[m] = x;
		}
		int ok = 1;
		if (lane == 0) {
#pragma unroll
			for (int m = 0; m < NV; ++m) part[m * gridDim.x + blockIdx.x] = bs[m];
			ok = grid_arrive_wait(c);
		}
		__syncwarp();
		ok = __shfl_sync(0xffffffffu, ok, 0);
		if (ok) {
#pragma unroll
			for (int m = 0; m < NV; ++m) {
				double acc = 0.0;
				for (int b = lane; b < (int)gridDim.x; b += 32) acc += ldcg(&part[m * gridDim.x + b]);
#pragma unroll
				for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
				if (lane == 0) s_r[bank][m] = acc;
			}
		}
		if (lane == 0) s_ok[bank] = ok;
	}
	__syncthreads();
#pragma unroll
	for (int m = 0; m < NV; ++m) v[m] = s_r[bank][m];
	const bool ok = s_ok[bank] != 0;
	bank ^= 1;
	return ok;
}

// Scalars computed once per block by thread 0 and broadcast: FP64 division
// and sqrt are long sequences on this GPU, not worth repeating per thread.
struct Bcast {
	double* s;   // shared scratch of at least 8 doubles
	__device__ __forceinline__ bool lead() const { return threadIdx.x == 0; }
	__device__ __forceinline__ void sync() const { __syncthreads(); }
};

}  // namespace cg_dev
