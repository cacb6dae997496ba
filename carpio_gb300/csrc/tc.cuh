// Blackwell tensor-core and TMA primitives (inline PTX) for the learned
// preconditioner's convolutions: mbarriers, TMA tensor loads, tcgen05 MMA
// with FP32 accumulators in tensor memory, and the 64-bit shared-memory /
// 32-bit instruction descriptors of tcgen05.mma.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace cg_tc {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
	return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// ---------------------------------------------------------------- mbarrier --
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok) : "r"(bar), "r"(parity) : "memory");
	return ok != 0;
}
// Bounded wait: false after `limit_ns` or once *err is set (checked every
// 1024 polls).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
		const int* err, unsigned long long limit_ns) {
	unsigned polls = 0;
	unsigned long long t0 = 0;
	while (!mbar_try_wait(bar, parity)) {
		if ((++polls & 1023u) == 0) {
			if (*(volatile const int*)err) return false;
			const unsigned long long now = gtimer();
			if (t0 == 0) t0 = now;
			else if (now - t0 > limit_ns) return false;
		}
	}
	return true;
}

// Bounded wait on time alone (for draining work already in flight).
__device__ __forceinline__ bool mbar_wait_for(uint32_t bar, uint32_t parity,
		unsigned long long limit_ns) {
	unsigned polls = 0;
	unsigned long long t0 = 0;
	while (!mbar_try_wait(bar, parity)) {
		if ((++polls & 1023u) == 0) {
			const unsigned long long now = gtimer();
			if (t0 == 0) t0 = now;
			else if (now - t0 > limit_ns) return false;
		}
	}
	return true;
}

// --------------------------------------------------------------------- TMA --
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map,
		int c0, int c1, int c2, uint32_t bar) {
	asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
			" [%0], [%1, {%2, %3, %4}], [%5];"
			:: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2),
			   "r"(bar) : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map,
		int c0, int c1, int c2, int c3, uint32_t bar) {
	asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
			" [%0], [%1, {%2, %3, %4, %5}], [%6];"
			:: "r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2),
			   "r"(c3), "r"(bar) : "memory");
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
	asm volatile("prefetch.tensormap [%0];" :: "l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ----------------------------------------------------------------- tcgen05 --
// Shared-memory matrix descriptor (tcgen05 "matrix descriptor"): start
// address >> 4 in bits [0,14), leading-dimension byte offset >> 4 in
// [16,30), stride-dimension byte offset >> 4 in [32,46), the fixed value
// 0b001 in [46,49), base offset 0, swizzle mode in [61,64).
constexpr uint64_t kSwizzleNone = 0, kSwizzle128 = 2, kSwizzle64 = 4, kSwizzle32 = 6;
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo,
		uint64_t swizzle) {
	uint64_t d = 0;
	d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1 << 46;
	d |= swizzle << 61;
	return d;
}
// Instruction descriptor of tcgen05.mma.kind::f16: FP32 accumulator (bits
// [4,6) = 1), A and B BF16 (bits [7,10) and [10,13) = 1), both K-major
// (bits 15, 16 = 0), N >> 3 in [17,23), M >> 4 in [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17)
		| ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
			:: "r"(dst_smem), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
			:: "r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
		uint32_t idesc, uint32_t accumulate) {
	asm volatile("{\n\t.reg .pred p;\n\t"
			"setp.ne.b32 p, %4, 0;\n\t"
			"tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
			:: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}
// arrive on an mbarrier once every tcgen05.mma issued so far by this thread
// has completed
__device__ __forceinline__ void mma_commit(uint32_t bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
			:: "r"(bar) : "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
	uint32_t r[32];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
			"{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
			"%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
			: "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
			  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
			  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
			  "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
			  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
			  "=r"(r[30]), "=r"(r[31])
			: "r"(taddr) : "memory");
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace cg_tc
