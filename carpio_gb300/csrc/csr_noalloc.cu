// carpio_gpu_krylov_csr_noalloc: the CSR Krylov solve of csr.cu for callers
// that must not allocate device memory during a solve.
//
// Who needs it: applications whose device memory is owned by a pool they do
// not control (a framework caching allocator that accounts every byte and
// fails at its cap when a library calls cudaMalloc behind its back), and
// long-running solvers that forbid allocation after start-up because
// cudaMalloc/cudaFree can synchronise the device and fragment memory in the
// middle of a time step. They pass device arrays they already own; this
// entry point calls no cudaMalloc, cudaFree or allocating library routine.
//
// Scratch: the solver's work vectors, control words and reduction partials
// live in one file-scope __device__ array of fixed size (below), which every
// GPU that loads the library holds until the process exits. Limits:
// n <= kNoallocMaxRows. Larger systems are rejected with CARPIO_GPU_EINVAL.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it for that
// device; make that first call before any stream capture begins.
//
// Sharing: all calls on a device use the same array and it keeps the last
// call's contents; the control words are cleared at the start of every call.
// Calls that overlap on the GPU (concurrent streams or host threads on the
// same device) race on the array and must be serialised by the caller.
#include "internal.hpp"

#include <mutex>

namespace {

using namespace cg_dev;

constexpr int kNoallocMaxRows = 32768;
constexpr int kNoallocMaxBlocks = 2048;
constexpr int kNoallocVecs = 11;   // r p q z rt ph s sh t v d

struct NoallocHead {
	cg_host::Ctl ctl;
	double pad[4];
};
constexpr size_t kHeadBytes = (sizeof(NoallocHead) + 255) / 256 * 256;
constexpr size_t kPartialBytes = sizeof(double) * 2 * kMaxReduce * kNoallocMaxBlocks;
constexpr size_t kVecBytes = sizeof(double) * (size_t)kNoallocVecs * kNoallocMaxRows;
constexpr size_t kScratchBytes = kHeadBytes + kPartialBytes + kVecBytes;

// ~3 MiB on every device that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

__global__ void __launch_bounds__(kThreads) k_csr_solve_noalloc(CsrOp op,
		FlatSpace sp, Vecs<double> v, SolveCtl sc, GridCtl gc) {
	gc.start();
	int bank = 0;
	krylov_run<double>(sp, op, v, sc, gc, bank);
}

std::mutex g_mu;
void* g_addr[64] = {};   // device address of the array, per device

int scratch_address(int dev, unsigned char** out) {
	if (dev < 0 || dev >= 64) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lock(g_mu);
	if (!g_addr[dev]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess || !p) {
			cg_host::note_cuda_error(e);
			return CARPIO_GPU_ECUDA;
		}
		g_addr[dev] = p;
	}
	*out = static_cast<unsigned char*>(g_addr[dev]);
	return 0;
}

// The rule on_this_device applies to cudaPointerGetAttributes' answer.
bool noalloc_pointer_ok(int type, int owner, int dev) {
	if (type == (int)cudaMemoryTypeManaged) return true;
	return type == (int)cudaMemoryTypeDevice && owner == dev;
}

// Device memory of the current device, or managed memory. Memory of another
// GPU is refused: without peer access the kernel would fault on it, and with
// peer access every load would cross the link.
bool on_this_device(const void* p, int dev) {
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return noalloc_pointer_ok((int)a.type, a.device, dev);
}

}  // namespace

extern "C" int carpio_gpu_krylov_csr_noalloc(int kind, int n, int nnz,
		const uint32_t* rowptr, const uint32_t* col, const double* val,
		const double* b, double* x, int* max_iter, double* tol,
		double* resid_hist, int hist_cap, int* hist_len, uint32_t flags,
		void* stream) {
	using namespace cg_host;
	if (n <= 0 || nnz < 0 || !rowptr || (!col && nnz) || (!val && nnz) || !b
			|| !x || !max_iter || !tol || kind < 0 || kind > 3)
		return CARPIO_GPU_EINVAL;
	if (n > kNoallocMaxRows) return CARPIO_GPU_EINVAL;   // beyond the static scratch
	if (hist_cap < 0 || (hist_cap > 0 && !resid_hist)) return CARPIO_GPU_EINVAL;
	int dev = 0;
	CG_CK(cudaGetDevice(&dev));
	// every array must already be memory this device can address directly:
	// nothing is staged here
	const void* ptrs[] = { rowptr, col, val, b, x };
	for (const void* p : ptrs)
		if (p && !on_this_device(p, dev)) return CARPIO_GPU_EINVAL;
	if (hist_cap > 0 && !on_this_device(resid_hist, dev)) return CARPIO_GPU_EINVAL;
	unsigned char* base = nullptr;
	int rc = scratch_address(dev, &base);
	if (rc) return rc;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	NoallocHead* head = reinterpret_cast<NoallocHead*>(base);
	double* partials = reinterpret_cast<double*>(base + kHeadBytes);
	double* vec = reinterpret_cast<double*>(base + kHeadBytes + kPartialBytes);
	Vecs<double> v;
	v.x = x;
	v.b = const_cast<double*>(b);
	double** slots[kNoallocVecs] = { &v.r, &v.p, &v.q, &v.z, &v.rt, &v.ph, &v.s,
		&v.sh, &v.t, &v.v, &v.d };
	for (int i = 0; i < kNoallocVecs; ++i) *slots[i] = vec + (size_t)i * kNoallocMaxRows;
	int blocks = coop_blocks((const void*)k_csr_solve_noalloc, n, 2);
	if (blocks > kNoallocMaxBlocks) blocks = kNoallocMaxBlocks;
	// clear the barrier/error words and the result of the previous call
	CG_CK(cudaMemsetAsync(&head->ctl, 0, sizeof(Ctl), s));
	CsrOp op{ rowptr, col, val };
	FlatSpace sp{ n };
	SolveCtl sc;
	sc.kind = kind;
	sc.max_iter = *max_iter;
	sc.tol = *tol;
	sc.flags = flags;
	sc.hist = hist_cap > 0 ? resid_hist : nullptr;
	sc.hist_cap = hist_cap;
	sc.out = &head->ctl.out;
	GridCtl gc;
	gc.count = &head->ctl.count;
	gc.gen = &head->ctl.gen;
	gc.err = &head->ctl.err;
	gc.partials = partials;
	gc.wait_ns = (unsigned long long)watchdog().wait_ms * 1000000ull;
	gc.solve_ns = (unsigned long long)watchdog().solve_ms * 1000000ull;
	gc.deadline = 0;
	void* args[] = { &op, &sp, &v, &sc, &gc };
	CG_CK(cudaLaunchCooperativeKernel((const void*)k_csr_solve_noalloc, blocks,
			kThreads, args, 0, s));
	Ctl c;
	CG_CK(cudaMemcpyAsync(&c, &head->ctl, sizeof c, cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	if (c.err) return c.err;
	if (c.out.code < 0) return c.out.code;
	*max_iter = c.out.iters;
	*tol = c.out.tol;
	if (hist_len) *hist_len = c.out.hist_len;
	return c.out.code;
}
