// Host-side internals shared by the translation units of libcarpio_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/carpio_gpu.h"
#include "krylov.cuh"

namespace cg_host {

#define CG_CK(expr)                                                          \
	do {                                                                     \
		cudaError_t _e = (expr);                                             \
		if (_e != cudaSuccess) { ::cg_host::note_cuda_error(_e); return CARPIO_GPU_ECUDA; } \
	} while (0)

void note_cuda_error(cudaError_t e);

// true if p is memory the device can address directly
bool is_device_ptr(const void* p);

struct Watchdog {
	unsigned wait_ms = 2000;
	unsigned solve_ms = 600000;
};
Watchdog& watchdog();

// Device-side control block of one persistent launch: barrier words, error
// word and the all-reduce partials; reset before every launch.
struct Ctl {
	unsigned count;
	unsigned gen;
	int err;
	int pad;
	cg_dev::SolveOut out;
};

// A growable device buffer.
struct DevBuf {
	void* p = nullptr;
	size_t bytes = 0;
	int ensure(size_t n);
	void release();
	~DevBuf() { release(); }
	template<class T> T* as() const { return static_cast<T*>(p); }
};

// Everything a persistent Krylov launch needs besides the problem data.
struct LaunchWs {
	DevBuf ctl;        // Ctl
	DevBuf partials;   // 2 * kMaxReduce * max_blocks doubles
	Ctl* host_ctl = nullptr;   // pinned mirror for the results
	int ensure(int max_blocks);
	~LaunchWs();
};

int sm_count();

// Number of blocks for a cooperative launch of `kernel` over `nwork` cells:
// enough blocks to give every thread a few cells, never more than can be
// co-resident.
int coop_blocks(const void* kernel, long nwork, int min_cells_per_thread);

cg_dev::GridCtl make_gridctl(LaunchWs& ws);

// Copy a host-or-device array into a device buffer (async on s).
int to_device(DevBuf& dst, const void* src, size_t bytes, cudaStream_t s);

}  // namespace cg_host

namespace cg_host {

// Matrix-free coefficients of StencilPoisson_ + GhostRegular_ for one
// (grid, bc, beta): D in the field layout, off-diagonal face coefficients
// ax[nx+1], ay[ny+1] (0 on boundary faces) and the boundary constants the
// ghost substitution adds to the row's constant (fold[0..3] = segments
// x-, x+, y-, y+; lengths ny, ny, nx, nx). FP32 copies for the mixed solver.
struct StencilCoeffs {
	bool valid = false;
	carpio_gpu_bc bc;
	double beta = 0;
	bool helm = false;            // StencilHelmholtz_: diagonal + sx sy alpha
	double alpha = 0;
	DevBuf D, ax, ay, fold, D32, ax32, ay32;
	bool uniform = true;          // rows described by ax / ay
	bool bfield_free = true;      // built without a beta field
	DevBuf cf, cf32;              // otherwise: per-cell coefficients x-, x+, y-, y+
	// multigrid preconditioner of the on-chip path (uniform grids without the
	// Helmholtz term): level sizes, the number of global-memory levels (0:
	// the grid does not coarsen far enough), the interior face coefficients
	// and every level's diagonal, concatenated
	std::vector<std::pair<int, int> > mg_dims;
	int mg_nlev = 0;
	float mg_cx = 0.f, mg_cy = 0.f;
	DevBuf mgD;
	// spectral preconditioner (separable operator, power-of-two sides, the
	// same boundary type on both sides of an axis): log2 of the sides, the
	// Dirichlet flags and the tables (eigenvalue parts [nx], [ny]; FFT
	// twiddles [nx/2], [ny/2]; DCT factors [nx], [ny] as float2), packed
	bool dct_ok = false;
	// the stencil's coefficients exact in FP32: the spectral path's refinement
	// residuals may run in double-float
	bool dct_df = false;
	int dct_lx = 0, dct_ly = 0, dct_fx = 0, dct_fy = 0;
	DevBuf dctT;
};

struct PoissonWs {
	LaunchWs lw;
	DevBuf v64, v32, src, phi, hist, out, xbuf;
	DevBuf mg;   // multigrid level vectors
	DevBuf dct;  // spectral workspace [nx][ny] (FP32)
};

// bfield: a variable beta (StencilPoisson_ with a beta field, face values
// by _build_default_beta, s_poisson.hpp:144-164), host or device, in the
// host field layout (nx + 2 gl) x (ny + 2 gl); null: the uniform beta
int stencil_prepare(carpio_gpu_grid* g, const carpio_gpu_bc& bc, double beta,
		StencilCoeffs& c, cudaStream_t s, bool helm = false, double alpha = 0.0,
		const double* bfield = nullptr);

// Centres and sizes of the n + 2 gl cells of one uniform axis.
void uniform_axis(int n, int gl, double lo, double hi, std::vector<double>& c,
		std::vector<double>& s);

// The coefficients above computed on the host from the axes (with ghosts):
// D in a layout of nx + 2 gl rows of pitch P, ax[nx+1], ay[ny+1], fold.
void stencil_host(int nx, int ny, int gl, int P, const std::vector<double>& cx,
		const std::vector<double>& sx, const std::vector<double>& cy,
		const std::vector<double>& sy, const carpio_gpu_bc& bc, double beta,
		std::vector<double>& D, std::vector<double>& ax, std::vector<double>& ay,
		std::vector<double>& fold, bool helm = false, double alpha = 0.0,
		std::vector<double>* cf = nullptr, const double* bfield = nullptr);

// Workspace of the learned-preconditioner solve (learned.cu).
struct LearnedWs {
	DevBuf f64, f32, part, sc;
	std::vector<double> hpart;
	int nblk = 0;
};

// Source of the right-hand side: a cell field, or the divergence of two face
// fields (Operation_::Div(VecF), s_operation.hpp:100-120) as the NS projection
// passes it.
enum { SRC_FIELD = 0, SRC_DIV = 1 };

// One persistent launch: b from the source, x from phi's normal cells,
// optional mean removal, the solve, optional mean removal, x back into phi.
// All pointers are device pointers; the result lands in *out_dev.
int poisson_launch(carpio_gpu_grid* g, StencilCoeffs& c, PoissonWs& w,
		int src_mode, const double* src_a, const double* src_b, double* phi,
		const carpio_gpu_solver_cfg& cfg, double* hist_dev, int hist_cap,
		cg_dev::SolveOut* out_dev, cudaStream_t s);

// FCG with the U-Net preconditioner (learned.cu): b from the source, x0 from
// phi, the solve, x (mean removed) back into phi; a stall finishes with the
// plain MIXED CG. All pointers are device pointers.
bool learned_shape_ok(int nx, int ny);
int learned_solve(carpio_gpu_grid* g, StencilCoeffs& c, PoissonWs& pws, LearnedWs& w,
		int src_mode, const double* src_a, const double* src_b, double* phi,
		const carpio_gpu_solver_cfg& cfg, carpio_gpu_unet* net,
		const carpio_gpu_learned_cfg& lc, cg_dev::SolveOut& out, cudaStream_t s,
		std::vector<double>* hist = nullptr);

// the U-Net forward for the library's own loops (nn.cu): stream-ordered,
// no host synchronisation; device-side failures land in *unet_err_flag(u),
// unet_take_err reads and clears it (synchronising the net's stream)
int unet_forward_async(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		float* z, cudaStream_t st);
int* unet_err_flag(carpio_gpu_unet* u);
int unet_take_err(carpio_gpu_unet* u);

}  // namespace cg_host

// Grid handle (defined here so poisson.cu and ns.cu share it).
struct carpio_gpu_grid {
	int nx, ny, gl;
	int NI, NJ;        // rows / columns incl. ghosts
	int P;             // device row pitch (doubles)
	std::vector<double> cx, sx, cy, sy;
	double *d_cx = nullptr, *d_sx = nullptr, *d_cy = nullptr, *d_sy = nullptr;
	cudaStream_t stream = nullptr;
	int device = 0;
	std::mutex mu;
	cg_host::StencilCoeffs coeffs;   // cache for carpio_gpu_poisson_solve
	cg_host::PoissonWs pws;
	cg_host::LearnedWs lws;
	// the caller's handle plus one per NS handle built on the grid; the grid
	// is freed when the last of them is released
	std::atomic<int> refs{ 1 };
};

namespace cg_host {
void grid_release(carpio_gpu_grid* g);
}

