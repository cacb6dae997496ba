// Library runtime: error strings, watchdog settings, device buffers and the
// cooperative-launch sizing shared by all entry points.
#include "internal.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace cg_host {

static thread_local cudaError_t g_last_cuda = cudaSuccess;

void note_cuda_error(cudaError_t e) {
	g_last_cuda = e;
	std::fprintf(stderr, "carpio_gpu: CUDA error %d (%s)\n", (int)e,
			cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
	if (!p) return false;
	cudaPointerAttributes a;
	cudaError_t e = cudaPointerGetAttributes(&a, p);
	if (e != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

Watchdog& watchdog() {
	static Watchdog w;
	return w;
}

int DevBuf::ensure(size_t n) {
	if (n <= bytes && p) return 0;
	release();
	if (n == 0) n = 16;
	cudaError_t e = cudaMalloc(&p, n);
	if (e != cudaSuccess) {
		cudaGetLastError();
		p = nullptr;
		bytes = 0;
		return CARPIO_GPU_ENOMEM;
	}
	bytes = n;
	return 0;
}

void DevBuf::release() {
	if (p) cudaFree(p);
	p = nullptr;
	bytes = 0;
}

int LaunchWs::ensure(int max_blocks) {
	int rc = ctl.ensure(sizeof(Ctl));
	if (rc) return rc;
	rc = partials.ensure(sizeof(double) * 2 * cg_dev::kMaxReduce * (size_t)max_blocks);
	if (rc) return rc;
	if (!host_ctl) {
		if (cudaMallocHost((void**)&host_ctl, sizeof(Ctl)) != cudaSuccess) {
			cudaGetLastError();
			host_ctl = nullptr;
			return CARPIO_GPU_ENOMEM;
		}
	}
	return 0;
}

LaunchWs::~LaunchWs() {
	if (host_ctl) cudaFreeHost(host_ctl);
}

int sm_count() {
	static int n = 0;
	if (!n) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
		if (n <= 0) n = 1;
	}
	return n;
}

int coop_blocks(const void* kernel, long nwork, int min_cells_per_thread) {
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel,
			cg_dev::kThreads, 0) != cudaSuccess || per_sm <= 0) {
		cudaGetLastError();
		per_sm = 1;
	}
	long maxb = (long)per_sm * sm_count();
	long want = (nwork + (long)cg_dev::kThreads * min_cells_per_thread - 1)
			/ ((long)cg_dev::kThreads * min_cells_per_thread);
	return (int)std::max(1L, std::min(maxb, want));
}

cg_dev::GridCtl make_gridctl(LaunchWs& ws) {
	cg_dev::GridCtl g;
	Ctl* c = ws.ctl.as<Ctl>();
	g.count = &c->count;
	g.gen = &c->gen;
	g.err = &c->err;
	g.partials = ws.partials.as<double>();
	g.wait_ns = (unsigned long long)watchdog().wait_ms * 1000000ull;
	g.solve_ns = (unsigned long long)watchdog().solve_ms * 1000000ull;
	g.deadline = 0;  // stamped by GridCtl::start() in the kernel
	return g;
}

int to_device(DevBuf& dst, const void* src, size_t bytes, cudaStream_t s) {
	int rc = dst.ensure(bytes);
	if (rc) return rc;
	if (bytes) CG_CK(cudaMemcpyAsync(dst.p, src, bytes, cudaMemcpyDefault, s));
	return 0;
}

}  // namespace cg_host

extern "C" {

const char* carpio_gpu_version(void) { return "carpio_gb300 0.1 (sm_103a)"; }

const char* carpio_gpu_strerror(int code) {
	switch (code) {
	case CARPIO_GPU_OK: return "converged";
	case CARPIO_GPU_MAXITER: return "reached max_iter";
	case CARPIO_GPU_BREAKDOWN_RHO: return "breakdown: rho == 0";
	case CARPIO_GPU_BREAKDOWN_OMEGA: return "breakdown: omega == 0";
	case CARPIO_GPU_EINVAL: return "invalid argument";
	case CARPIO_GPU_ECUDA: return "CUDA runtime error";
	case CARPIO_GPU_ENONFINITE: return "non-finite input";
	case CARPIO_GPU_EZERODIAG: return "zero diagonal (diagonal preconditioner failure)";
	case CARPIO_GPU_ETIMEOUT: return "device watchdog expired";
	case CARPIO_GPU_ENOMEM: return "device allocation failed";
	case CARPIO_GPU_EIO: return "file could not be written";
	}
	return "unknown code";
}

int carpio_gpu_set_watchdog(unsigned wait_ms, unsigned solve_ms) {
	if (wait_ms == 0 || solve_ms == 0) return CARPIO_GPU_EINVAL;
	cg_host::watchdog().wait_ms = wait_ms;
	cg_host::watchdog().solve_ms = solve_ms;
	return 0;
}

int carpio_gpu_device_count(void) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return n;
}

}  // extern "C"
