// Thread-block-cluster primitives for the batched solver: distributed shared
// memory (DSMEM) addressing, mbarriers armed from remote CTAs, and a team
// all-reduce over a contiguous range of a cluster's CTAs.
//
// Every wait is a bounded poll (mbarrier.try_wait in a loop that checks the
// launch's error word and a %globaltimer limit). The only unbounded waits are
// the two hardware cluster barriers at the start and the end of a launch,
// which every CTA reaches because everything between them is bounded.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace cg_dev {

constexpr int kMaxTeam = 16;     // CTAs per cluster at most
constexpr int kTeamNV = 4;       // values per team all-reduce at most

__device__ __forceinline__ unsigned cluster_rank() {
	unsigned r;
	asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
	return r;
}
__device__ __forceinline__ unsigned cluster_index() {
	unsigned r;
	asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
	return r;
}
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
	return (uint32_t)__cvta_generic_to_shared(p);
}
// address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t dsmem_map(uint32_t a, unsigned rank) {
	uint32_t r;
	asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
	return r;
}
__device__ __forceinline__ void dsmem_st_f64(uint32_t a, double v) {
	asm volatile("st.shared::cluster.f64 [%0], %1;" :: "r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ float dsmem_ld_f32(uint32_t a) {
	float v;
	asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
	return v;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init_cluster() {
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// arrive (release, cluster scope) on an mbarrier of any CTA of the cluster
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t remote_bar) {
	asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];"
			:: "r"(remote_bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(const uint64_t* bar, unsigned parity) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
	return ok != 0;
}
// hardware barrier over all threads of all CTAs of the cluster
__device__ __forceinline__ void cluster_barrier() {
	asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
			"barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Limits of every wait of one launch.
struct Watch {
	int* err;
	unsigned long long wait_ns;
	unsigned long long deadline;   // absolute %globaltimer
};

__device__ __forceinline__ void watch_fail(const Watch& w, int code) {
	atomicCAS(w.err, 0, code);
}

// A team: CTAs [lo, lo + t) of one cluster, this CTA being member m. Each
// CTA owns two mbarriers (expected count t, one per bank) and a slot array
// [2 banks][kTeamNV][kMaxTeam] of doubles in its shared memory.
struct Team {
	unsigned lo, t, m;
	uint64_t* bar;
	double* slot;
	unsigned par;   // bit b: phase parity expected next on bar[b]
	int bank;
};

// Sum of NV values over the team; every thread of every member gets the same
// bits. Split in two so that independent work can run while the partials
// travel: team_post forms the block's value with a fixed warp tree, then lanes
// 0..t-1 of warp 0 store it into slot [bank][.][m] of member `lane` and arrive
// on that member's bar[bank] (release, cluster scope); team_wait has lane 0
// wait for the t arrivals on its own bar[bank] (acquire), add the member
// values in member order and hand the sums to the block. Consecutive
// reductions alternate banks, and a member cannot post the reduction after
// next before every member has finished reading this one, so one slot array
// per bank is enough. A team of one CTA reduces within the block (post does
// it all). Between post and wait the block must not start another reduction.
// team_wait returns false once the launch has failed (this or another CTA).
template<class R, int NV>
__device__ __forceinline__ void team_post(R (&v)[NV], Team& tm) {
	static_assert(NV <= kTeamNV, "team reduction: too many values");
	const int bank = tm.bank;
	// the block's partials alternate between two buffers: a team of one has
	// no second block barrier, and a warp that runs ahead into the next call
	// must not overwrite values a slower warp is still adding up
	block_sum_light<R, NV>(v, bank);
	if (tm.t == 1 || threadIdx.x >= 32) return;
	const int lane = threadIdx.x;
	if (lane < (int)tm.t) {
		const unsigned dst = tm.lo + lane;
		const uint32_t sa = dsmem_map(smem_u32(tm.slot + (bank * kTeamNV) * kMaxTeam + tm.m), dst);
#pragma unroll
		for (int k = 0; k < NV; ++k) dsmem_st_f64(sa + 8u * kMaxTeam * k, (double)v[k]);
		mbar_arrive_cluster(dsmem_map(smem_u32(tm.bar + bank), dst));
	}
}

template<class R, int NV>
__device__ __forceinline__ bool team_wait(R (&v)[NV], Team& tm, const Watch& w) {
	__shared__ R s_res[NV];
	__shared__ int s_ok;
	const int bank = tm.bank;
	tm.bank = bank ^ 1;
	if (tm.t == 1) return true;
	if (threadIdx.x == 0) {
		int ok = 1;
		const unsigned parity = (tm.par >> bank) & 1u;
		unsigned polls = 0;
		unsigned long long t0 = 0;
		while (!mbar_try_wait_cluster(tm.bar + bank, parity)) {
			if ((++polls & 15u) == 0) {
				if (*(volatile int*)w.err) { ok = 0; break; }
				const unsigned long long now = globaltimer();
				if (t0 == 0) t0 = now;
				if (now - t0 > w.wait_ns || now > w.deadline) {
					watch_fail(w, CARPIO_GPU_ETIMEOUT);
					ok = 0;
					break;
				}
			}
		}
		// the thread that made the acquire reads the slots
		if (ok) {
#pragma unroll
			for (int k = 0; k < NV; ++k) {
				const double* sl = tm.slot + (bank * kTeamNV + k) * kMaxTeam;
				double acc = 0.0;
				for (unsigned q = 0; q < tm.t; ++q) acc += sl[q];
				s_res[k] = (R)acc;
			}
		}
		s_ok = ok;
	}
	__syncthreads();
#pragma unroll
	for (int k = 0; k < NV; ++k) v[k] = s_res[k];
	tm.par ^= 1u << bank;
	return s_ok != 0;
}

template<class R, int NV>
__device__ __forceinline__ bool team_allreduce(R (&v)[NV], Team& tm, const Watch& w) {
	team_post<R, NV>(v, tm);
	return team_wait<R, NV>(v, tm, w);
}

}  // namespace cg_dev
