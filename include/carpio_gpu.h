/*
 * carpio_gpu.h -- C ABI of the GB300 (sm_103a) projection hot path.
 *
 * Drop-in for the CPU path of hyperpower/carpios. Two layers, as the reference
 * has them:
 *
 *  1. Algebra level: the free-function Krylov solvers of
 *     lib/algebra/solver_matrix.hpp on a CSR matrix (MatrixSCR_,
 *     lib/algebra/matrix_SparCompRow.hpp:27-36), with the same in/out meaning
 *     of x, max_iter, tol and the residual list, and the same return codes.
 *  2. Structure level: the cell-centred 5-point Poisson solve behind
 *     structure::Solver_<2>::solve (lib/structure/s_solver.hpp:77-171, the
 *     seam Poisson_::solve calls, s_poisson.hpp:411-420) and the explicit
 *     projection step NS_explicit_::run_one_step
 *     (lib/structure/s_ns_explicit.hpp:118-229), matrix-free on the GPU.
 *
 * Only plain C types cross the boundary. Array arguments may be host or device
 * (CUDA) pointers; the library detects which. Fields use the reference's
 * SpaceT layout (lib/algebra/space.hpp:184-209): (nx+2gl) x (ny+2gl) doubles,
 * row I = x index incl. ghosts, column J = y index incl. ghosts, J contiguous.
 * Solver vectors (CSR layer) are plain length-n arrays.
 *
 * Errors are returned, never raised: no call exits or traps. Calls on one
 * handle are not thread-safe; separate handles are independent.
 */
#ifndef CARPIO_GPU_H
#define CARPIO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----- return codes ------------------------------------------------------
 * 0..3 are the reference's own solver codes (solver_matrix.hpp:264-745):
 * 0 converged, 1 reached max_iter, 2 rho breakdown, 3 omega breakdown.
 * Negative codes replace the reference's assert()/exit() paths. */
#define CARPIO_GPU_OK 0
#define CARPIO_GPU_MAXITER 1
#define CARPIO_GPU_BREAKDOWN_RHO 2
#define CARPIO_GPU_BREAKDOWN_OMEGA 3
#define CARPIO_GPU_EINVAL (-1)      /* bad argument */
#define CARPIO_GPU_ECUDA (-2)       /* CUDA runtime error */
#define CARPIO_GPU_ENONFINITE (-3)  /* NaN/Inf in an input */
#define CARPIO_GPU_EZERODIAG (-4)   /* DiaPre zero diagonal (preconditioner.hpp:223-227 exits) */
#define CARPIO_GPU_ETIMEOUT (-5)    /* device watchdog expired */
#define CARPIO_GPU_ENOMEM (-6)      /* device allocation failed */
#define CARPIO_GPU_EIO (-7)         /* file could not be written */

/* Krylov kinds, in the reference's order */
#define CARPIO_GPU_CG 0            /* carpio::CG            solver_matrix.hpp:264-316 */
#define CARPIO_GPU_JACOBI 1        /* carpio::Jacobi        solver_matrix.hpp:192-260 */
#define CARPIO_GPU_DIA_BICGSTAB 2  /* carpio::Dia_BiCGSTAB  solver_matrix.hpp:599-672 */
#define CARPIO_GPU_BICGSTAB 3      /* carpio::BiCGSTAB      solver_matrix.hpp:674-745 */
#define CARPIO_GPU_IC_CGS 4        /* carpio::IC_CGS        solver_matrix.hpp:376-438 (FP64) */
#define CARPIO_GPU_IC_CG 5         /* carpio::IC_CG         solver_matrix.hpp:318-374 (FP64) */

/* flags (bitwise OR). 0 = the reference's exact semantics. */
#define CARPIO_GPU_FLAG_FULL_NRM2 1u   /* use the full 2-norm instead of nrm2's
                                          drop-last-element (BLAS_Level1.hpp:569) */
#define CARPIO_GPU_FLAG_NO_TILE 2u     /* structure level, MIXED CG on a uniform
                                          grid: run the inner FP32 CG from global
                                          memory instead of the on-chip tile
                                          kernel; IC_CGS / IC_CG: level-scheduled
                                          triangular solves (IEEE divisions in the
                                          reference's order) instead of the
                                          five-point wavefront */
#define CARPIO_GPU_FLAG_MIXED 4u       /* CSR layer: the kind's iterations in FP32
                                          inside FP64 iterative refinement (CG,
                                          DIA_BICGSTAB, BICGSTAB; the stopping
                                          test the reference's, in FP64 on
                                          b - A x; max_iter out = FP32
                                          iterations, lresid = one FP64
                                          residual per refinement) */

/* ----- library ----------------------------------------------------------- */
const char* carpio_gpu_version(void);
const char* carpio_gpu_strerror(int code);
/* Bound on every device-side wait and on a whole solve (milliseconds);
 * on expiry the call returns CARPIO_GPU_ETIMEOUT. Defaults 2000 / 600000. */
int carpio_gpu_set_watchdog(unsigned wait_ms, unsigned solve_ms);
int carpio_gpu_device_count(void);

/* ----- 1. algebra level: CSR drop-in ---------------------------------------
 * Replaces   int CG(const MatrixSCR_<V>& A, ArrayListV<V>& x,
 *                   const ArrayListV<V>& b, int& max_iter, Float& tol,
 *                   std::list<Float>& lresid)
 * and Jacobi / Dia_BiCGSTAB / BiCGSTAB of the same shape
 * (lib/algebra/solver_matrix.hpp:193-198, 265-269, 600-606, 675-681).
 * rowptr[n+1], col[nnz] (0-based, unsigned 32-bit like St), val[nnz]: the
 * MatrixSCR_ arrays. x: in x0, out solution. max_iter, tol: in limits, out
 * iterations and reached residual, exactly as the reference writes them
 * (including its early exits that leave max_iter unchanged). resid_hist:
 * the lresid list, up to hist_cap entries; *hist_len gets its full length
 * (either may be NULL). Returns the reference's code or a negative error.
 * kind IC_CGS / IC_CG: ICPre's incomplete Cholesky factor of the upper
 * triangle (preconditioner.hpp:97-177) is built on the host in the
 * reference's order, the triangular solves run level by level on the GPU;
 * a row without a diagonal returns CARPIO_GPU_EZERODIAG (the reference
 * exits). */
int carpio_gpu_krylov_csr(int kind, int n, int nnz, const uint32_t* rowptr,
		const uint32_t* col, const double* val, const double* b, double* x,
		int* max_iter, double* tol, double* resid_hist, int hist_cap,
		int* hist_len, uint32_t flags);

/* Replaces   double Residual(const MatrixSCR_<V>& A, const ArrayListV<V>& x,
 *                             const ArrayListV<V>& b)
 * (lib/algebra/solver_matrix.hpp:583-597): *resid = nrm2(b - A x) / nrm2(b),
 * nrm2(b) taken as 1 when it is 0, nrm2 leaving out the last element as
 * the reference's does (CARPIO_GPU_FLAG_FULL_NRM2: all of them). b - A x is
 * formed row by row in the reference's order (bit-exact); the sums of
 * squares are fixed-order trees. Arrays host or device. */
int carpio_gpu_residual(int n, int nnz, const uint32_t* rowptr,
		const uint32_t* col, const double* val, const double* x, const double* b,
		uint32_t flags, double* resid);

/* The same solve for callers that cannot allocate device memory during a
 * solve (a framework that owns all device memory through its own pool, or a
 * time-stepping service that forbids cudaMalloc/cudaFree after start-up).
 * No counterpart in the reference. Kinds CG .. BICGSTAB only (the IC kinds
 * build their factor on the host and in device buffers: CARPIO_GPU_EINVAL).
 * All arrays must be memory of the current device (or managed memory) that
 * the caller owns; host memory and another GPU's memory give
 * CARPIO_GPU_EINVAL. The solver's scratch is a fixed ~3 MiB array compiled
 * into the library (held by every device that loads it) and n is limited to
 * 32768 rows (larger n: CARPIO_GPU_EINVAL). The first call on a device looks
 * up the array's address; make it before any stream capture begins. One
 * array serves every call on a device: calls that overlap on the GPU race
 * and must be serialised by the caller. `stream` is a cudaStream_t (NULL =
 * default); every call reads its result back and synchronises `stream`
 * before it returns. x is iterated in place: after a negative return it
 * holds a partial iterate, so a caller that needs x0 afterwards keeps a
 * copy (carpio_gpu_krylov_csr leaves x untouched on failure). */
int carpio_gpu_krylov_csr_noalloc(int kind, int n, int nnz,
		const uint32_t* rowptr, const uint32_t* col, const double* val,
		const double* b, double* x, int* max_iter, double* tol,
		double* resid_hist, int hist_cap, int* hist_len, uint32_t flags,
		void* stream);

/* ----- 2. structure level ------------------------------------------------ */
typedef struct carpio_gpu_grid carpio_gpu_grid;

/* Grid_<2>(min, max, n, gl) with uniform cells (lib/structure/s_grid.hpp:25-34,
 * 372-395). Centres are built by the same running sums, so they carry the
 * same rounding. gl >= 1 (>= 2 for TVD advection). */
int carpio_gpu_grid_create_uniform(int nx, int ny, int gl, double xmin,
		double xmax, double ymin, double ymax, carpio_gpu_grid** out);
/* Releases the caller's handle; the grid itself lives on while NS handles
 * created on it exist. */
int carpio_gpu_grid_destroy(carpio_gpu_grid* g);
/* cell centres / sizes incl. ghosts: cx, sx [nx+2gl], cy, sy [ny+2gl] (host) */
/* Grid_<2>(min, gl, csx, csy) (s_grid.hpp:35-48, 397-434): nx, ny normal
 * cells of the given sizes (host arrays of nx and ny positive values);
 * ghost cells take the size of the nearest normal cell. Every operator and
 * solver of the library works on it (coefficients from the axes); the
 * learned and batched paths take uniform grids only. */
int carpio_gpu_grid_create(int nx, int ny, int gl, double xmin, double ymin,
		const double* csx, const double* csy, carpio_gpu_grid** out);
/* structure::Output_Scalar (s_io_file.hpp:43-71): the text file the
 * reference's output events write ("## Size : N", "## Dim : 2",
 * "## NX :  nx", "## NY :  ny", then per normal cell, x fastest,
 * "x, y, z, value" in %10.6e with z = 0). field: the SpaceT layout with
 * ghosts ((nx+2gl) x (ny+2gl) doubles, y contiguous), host or device. */
int carpio_gpu_output_scalar(const carpio_gpu_grid* g, const char* filename,
		const double* field);
int carpio_gpu_grid_coords(const carpio_gpu_grid* g, double* cx, double* sx,
		double* cy, double* sy);

/* Boundary conditions of one field: BoundaryCondition type per segment
 * (1 = Dirichlet _BC1_, 2 = Neumann _BC2_; lib/structure/s_boundary.hpp:10-36)
 * and a constant value. Segments as GhostRegular_ numbers them
 * (s_ghost.hpp:210-232): 0 x-, 1 x+, 2 y-, 3 y+. The reference's default
 * (no BC registered) is Neumann 0. */
typedef struct {
	int type[4];
	double value[4];
} carpio_gpu_bc;

#define CARPIO_GPU_FP64 0
#define CARPIO_GPU_MIXED 1   /* FP32 inner CG / BiCGSTAB inside FP64 iterative
                                refinement */

typedef struct {
	int kind;          /* CARPIO_GPU_CG / JACOBI / DIA_BICGSTAB / BICGSTAB, or
	                      IC_CGS / IC_CG (FP64, no beta field: the stencil rows
	                      go to the CSR solver of section 1; synchronous) */
	int precision;     /* CARPIO_GPU_FP64 or CARPIO_GPU_MIXED (kinds CG,
	                      DIA_BICGSTAB and BICGSTAB: the inner iterations
	                      are the kind's own in FP32, the stopping test the
	                      reference's in FP64 on b - A x) */
	int max_iter;      /* Solver_::set_max_iter */
	double tol;        /* Solver_::set_tolerance (relative residual) */
	int mean_removal;  /* remove the mean of b and x (all-Neumann null space) */
	double inner_tol;  /* MIXED: residual reduction between two FP64 residual
	                      replacements (reliable updates; at most 1e-2 is used
	                      on chip); 0 = 1e-1 on chip with the Chebyshev
	                      preconditioner, 3e-2 on chip without it, 1e-4 on
	                      the global-memory path (BiCGSTAB kinds, non-uniform
	                      grids, CARPIO_GPU_FLAG_NO_TILE) */
	int inner_max_iter;/* MIXED, global-memory path: cap on one inner solve */
	uint32_t flags;    /* CARPIO_GPU_FLAG_* */
	int poly_degree;   /* MIXED, on-chip path: degree of the band-local
	                      Chebyshev preconditioner of the FP32 CG (each CTA's
	                      band with zero halo, so no exchange); 0 = default 5,
	                      < 0 = none (plain CG) */
	double poly_ratio; /* its eigenvalue interval [2 / ratio, 2] of D^-1 A;
	                      0 = 30 */
	int precond;       /* MIXED, on-chip path: preconditioner of the FP32 CG.
	                      CARPIO_GPU_PRECOND_MULTIGRID: one geometric-
	                      multigrid V(1,1)-cycle (damped Jacobi smoothing,
	                      bilinear prolongation, restriction its transpose)
	                      on grids whose sides halve down to at most 1024
	                      cells, without the Helmholtz term; other grids take
	                      the polynomial. CARPIO_GPU_PRECOND_CHEBYSHEV: the
	                      band-local polynomial above.
	                      CARPIO_GPU_PRECOND_SPECTRAL: M = A^-1 through the
	                      DCT-II / DST-II of both axes (FP32 FFTs on chip) on
	                      grids with power-of-two sides, a uniform
	                      coefficient and the same boundary type (Neumann or
	                      Dirichlet) on both sides of each axis; other grids
	                      as DEFAULT. CARPIO_GPU_PRECOND_DEFAULT (0): the
	                      spectral preconditioner where it applies, else the
	                      multigrid cycle where it applies, else the
	                      polynomial. */
} carpio_gpu_solver_cfg;

#define CARPIO_GPU_PRECOND_DEFAULT 0
#define CARPIO_GPU_PRECOND_CHEBYSHEV 1
#define CARPIO_GPU_PRECOND_MULTIGRID 2
#define CARPIO_GPU_PRECOND_SPECTRAL 3

typedef struct {
	int code;          /* solver code (0..3) or negative error */
	int iters;         /* the reference's max_iter out value (FP64); total
	                      inner iterations (MIXED) */
	double tol_out;    /* the reference's tol out value: relative residual */
	int outer_iters;   /* MIXED: refinement cycles */
	int hist_len;      /* length of the residual list */
	double ms;         /* device time of the solve (CUDA events) */
} carpio_gpu_solver_stats;

/* Poisson_::run() for a set_depend'ed field (s_poisson.hpp:320-420, 513-533):
 * assemble StencilPoisson_ (s_poisson.hpp:60-114) with GhostRegular_
 * substitution (s_ghost.hpp:140-179, 334-357) for uniform beta, copy phi's
 * normal cells to x (Solver_::_copy_to_x), solve, and write x back
 * (_copy_to_cs). source and phi are full fields with ghosts; phi's normal
 * cells are the initial guess and receive the solution, its ghosts are left
 * as they were (the reference does not touch them either). */
int carpio_gpu_poisson_solve(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double beta, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats);
/* Poisson_ with an alpha term (set_uniform_alpha, s_poisson.hpp:461-471):
 * the StencilHelmholtz_ rows (s_poisson.hpp:185-258), diagonal plus
 * sx sy alpha and the source scaled by sx sy; otherwise as
 * carpio_gpu_poisson_solve. */
/* Poisson_ with a beta field (set_depend with spbeta, s_poisson.hpp:513-533):
 * face values by StencilPoisson_::_build_default_beta (s_poisson.hpp:
 * 144-164), as the reference computes them (weights |half size - centre| of
 * the cell and its face-side neighbour, values of the cell and its +
 * neighbour), so the rows are not symmetric in general (use BiCGSTAB or
 * Jacobi). beta_field: full field with ghosts, host or device; the mixed
 * on-chip path is not used. Otherwise as carpio_gpu_poisson_solve. */
int carpio_gpu_poisson_solve_beta(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		const double* beta_field, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats);
int carpio_gpu_helmholtz_solve(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double alpha, double beta, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats);

/* Advection schemes of NS_::set_advection_scheme (s_ns.hpp:171-211), plus the
 * minmod limiter of src/calculation/advection.hpp:1079-1081 in the same TVD
 * framework (s_operation.hpp:549-596). */
#define CARPIO_GPU_UPWIND1 0
#define CARPIO_GPU_CENTER 1
#define CARPIO_GPU_CENTER4 2
#define CARPIO_GPU_UPWIND2 3
#define CARPIO_GPU_VANLEER 4
#define CARPIO_GPU_SUPERBEE 5
#define CARPIO_GPU_WAHYD 6
#define CARPIO_GPU_QUICK 7
#define CARPIO_GPU_CUI 8
#define CARPIO_GPU_MINMOD 9

typedef struct {
	double rho;          /* set_uniform_rho (NS_ s_ns.hpp:93-97) */
	double mu;           /* set_uniform_mu (s_ns.hpp:106-110) */
	double cfl;          /* set_CFL_number (s_ns.hpp:132-136) */
	double diff_number;  /* set_diffusion_number: value (>= 100 disables) */
	double diff_coef;    /*                         coefficient */
	int scheme;          /* CARPIO_GPU_UPWIND1 .. MINMOD */
	carpio_gpu_bc bc_u;  /* add_bc(0, seg, "u", ...) */
	carpio_gpu_bc bc_v;  /* add_bc(0, seg, "v", ...) */
	carpio_gpu_solver_cfg projection; /* set_projection_solver: CG (the
	                                     drop-in; mean removal is what makes
	                                     the all-Neumann projection solvable)
	                                     or the shipped IC_CGS / IC_CG (FP64,
	                                     usually without mean removal, as
	                                     Solver_IC_CGS_ does) */
} carpio_gpu_ns_cfg;

typedef struct carpio_gpu_ns carpio_gpu_ns;

/* NS_explicit_<2>(grid) + initial(): all fields zero, dt = dt0
 * (set_time(max_step, dt0), s_poisson.hpp/s_equation.hpp). */
int carpio_gpu_ns_create(carpio_gpu_grid* g, const carpio_gpu_ns_cfg* cfg,
		double dt0, carpio_gpu_ns** out);
int carpio_gpu_ns_destroy(carpio_gpu_ns* ns);
/* state: u, v (cell), uf, vf (face), phi, p (cell), all full fields with
 * ghosts; NULL leaves a field unchanged (set) or skips it (get). */
int carpio_gpu_ns_set_state(carpio_gpu_ns* ns, double dt, const double* u,
		const double* v, const double* uf, const double* vf,
		const double* phi, const double* p);
int carpio_gpu_ns_get_state(carpio_gpu_ns* ns, double* dt, double* u,
		double* v, double* uf, double* vf, double* phi, double* p);
/* `steps` passes of Equation_::run's loop body (s_equation.hpp:154-171):
 * run_one_step then Time_::advance. Per-step dt, projection iterations and
 * residual go to the optional arrays (host or device, length steps).
 * Returns 0 or the first non-zero projection code / error. */
int carpio_gpu_ns_run(carpio_gpu_ns* ns, int steps, double* step_dt,
		int* step_iters, double* step_resid);
/* The time stepper of the handle: NS_explicit_ (s_ns_explicit.hpp, default)
 * or NS_kim_ (s_ns_kim.hpp: Adams-Bashforth advection, per-component
 * Helmholtz predictor solved by the reference's default Jacobi, projection,
 * p = phi / dt - NablaMuNabla(mu, phi) / (2 rho); no time-step restriction). */
#define CARPIO_GPU_STEPPER_EXPLICIT 0
#define CARPIO_GPU_STEPPER_KIM 1
int carpio_gpu_ns_set_stepper(carpio_gpu_ns* ns, int stepper);
/* A mu field (a cell field of the grid's layout, host or device) in place of
 * the uniform mu: NablaMuNabla(mu field) in the predictor
 * (__diffusion_term, s_ns_explicit.hpp:235-241), as unset_uniform_mu +
 * initial_CS("mu", f) give it in the reference (s_ns.hpp:111-118,
 * 277-280; its set_mu cannot be instantiated). NULL: back to the uniform
 * mu. Explicit stepper only. A rho field has no counterpart: the
 * reference's run_one_step asserts a uniform rho (s_ns_explicit.hpp:134). */
int carpio_gpu_ns_set_mu_field(carpio_gpu_ns* ns, const double* mu);

/* Timing of the last carpio_gpu_ns_run, per step (host arrays of length
 * `cap`, any may be NULL): device time of the projection solve launch and of
 * the whole step (CUDA events on the launching stream), inner (FP32) and
 * outer iterations of the solve (with the learned preconditioner: all
 * iterations, and those of the flexible CG before any fallback). *n gets the
 * number of steps recorded. */
int carpio_gpu_ns_profile(carpio_gpu_ns* ns, int cap, int* n,
		double* solve_ms, double* step_ms, int* inner_iters, int* outer_iters);

/* Single operators of Operation_ (s_operation.hpp) on full fields, for
 * callers that drive their own loop and for per-kernel checks.
 *   which: 0 Grad (:46-72)       in a        -> out1 (x faces), out2 (y faces)
 *          1 Div(VecF) (:100-120) in a, b (faces) -> out1
 *          2 InterpolateF2C (:141-164) in a, b -> out1, out2
 *          3 InterpolateC2F (:166-187) in a, b -> out1, out2 (normal + low wall
 *            faces written, the rest left as passed in)
 *          4 VdotNabla (scheme, :313-628) faces a, b, field c -> out1
 *          5 NablaMuNabla(mu) (:664-688) in c -> out1
 *          6 apply_bc (s_equation.hpp:340-378) bc, in/out out1 (in place)
 *          7 max_magnitude (s_vector.hpp:89-103) a, b -> *scalar
 *          8 NablaMuNabla(mu field) (:630-662) mu a, in c -> out1
 *          9 the projection step's predictor (_veo_star_center, s_ns_explicit.hpp:173-213,
 *            the kernel NS_explicit_ stepping runs) on one field with
 *            dt = 1, mu = coef and rho = *scalar (in; 1 when scalar is
 *            NULL or *scalar is 0): faces a, b, field c ->
 *            out1 = (-VdotNabla + NablaMuNabla(mu) / rho) * 1 + c
 * Outputs of 0, 1, 2, 4, 5, 8, 9 are zero outside the cells the reference writes. */
int carpio_gpu_operator(carpio_gpu_grid* g, int which, int scheme,
		double coef, const carpio_gpu_bc* bc, const double* a,
		const double* b, const double* c, double* out1, double* out2,
		double* scalar);

/* Stand-alone Advection_<2> (s_advection.hpp:22-216): a scalar phi carried
 * by a fixed velocity field. Fields are full arrays of the grid's layout
 * (ghosts included), host or device.
 *   create       the handle; scheme upwind1, every boundary Neumann 0 (the
 *                reference's defaults, s_advection.hpp:86-99)
 *   set_scheme   set_advection_scheme (:140-183): CARPIO_GPU_UPWIND1 .. CUI
 *                (minmod is not one of its names: CARPIO_GPU_EINVAL); the
 *                radius-2 schemes need gl >= 2
 *   set_bc       field 0 u, 1 v, 2 phi. ghost_values: NULL (bc->value per
 *                segment) or a field holding, for every ghost cell, the value
 *                a function BC gives there (BC::get_val at the face point
 *                Equation_::apply_bc evaluates, s_equation.hpp:352-357)
 *   initial      initial() (:101-135): the cell fields u, v, phi as set_CS
 *                leaves them (NULL = 0), then the velocities' ghosts and the
 *                face velocities (InterpolateC2F into zeroed face fields)
 *   step         `steps` calls of run_one_step (:185-212) with time step dt:
 *                phi's ghosts refilled, then every normal cell in x-fastest
 *                order updated in place, phi - dt * VdotNabla, so each cell
 *                reads the new values of the cells before it. It also
 *                refills the velocities' ghosts, which changes their corner
 *                ghosts once (read by no later computation).
 *                Equation_::run runs max_step + 1 steps (Time_::is_end,
 *                s_time.hpp:74-80).
 *   get          any of u, v, uf, vf, phi (NULL skips) */
typedef struct carpio_gpu_advection carpio_gpu_advection;
int carpio_gpu_advection_create(carpio_gpu_grid* g, carpio_gpu_advection** out);
int carpio_gpu_advection_destroy(carpio_gpu_advection* a);
int carpio_gpu_advection_set_scheme(carpio_gpu_advection* a, int scheme);
int carpio_gpu_advection_set_bc(carpio_gpu_advection* a, int field,
		const carpio_gpu_bc* bc, const double* ghost_values);
int carpio_gpu_advection_initial(carpio_gpu_advection* a, const double* u,
		const double* v, const double* phi);
int carpio_gpu_advection_step(carpio_gpu_advection* a, double dt, int steps);
int carpio_gpu_advection_get(carpio_gpu_advection* a, double* u, double* v,
		double* uf, double* vf, double* phi);

/* ----- 3. batched Poisson solves -------------------------------------------
 * No counterpart in the reference, which solves one Poisson_ at a time. Many
 * independent Poisson_::run() solves on uniform grids of uneven sizes go into
 * one persistent launch, replayed from a CUDA graph. Each problem is solved as
 * carpio_gpu_poisson_solve solves one grid with the MIXED CG: FP32 inner
 * iterations, FP64 residual, solution and mean removal, the same stopping
 * test. Two kernels: by default one CTA per problem, problems taken largest
 * first from a queue, with the geometric-multigrid V-cycle as the FP32 CG's
 * preconditioner (block barriers only); when the tiles name a cluster size,
 * thread-block clusters in which a problem is owned by a team of 1..16 CTAs
 * (bands of x-rows, plain FP32 CG), whose reductions and halo rows travel
 * through distributed shared memory.
 *
 * The batch keeps its fields on the device in the layout of a grid with one
 * ghost layer ((nx+2) x (ny+2) doubles, y contiguous, ghosts zero).
 * carpio_gpu_batch_upload/download move plain interior arrays (nx*ny doubles,
 * y contiguous; host or device memory) in and out of it. */
typedef struct carpio_gpu_batch carpio_gpu_batch;

typedef struct {
	int nx, ny;                     /* cells */
	double xmin, xmax, ymin, ymax;  /* the box (uniform Grid_) */
	carpio_gpu_bc bc;               /* per segment, as for poisson_solve */
	int mean_removal;               /* remove the means of b and x (all-Neumann) */
	double beta;                    /* uniform beta (Poisson_::set_uniform_beta) */
} carpio_gpu_batch_problem;

/* Launch configuration ("tiles"); 0 in a field lets the library choose. */
typedef struct {
	int threads;        /* threads per CTA: 256 or 512 (cluster teams), 256,
	                       512 or 1024 (multigrid) */
	int cluster;        /* CTAs per cluster: 1, 2, 4, 8 or 16 selects the
	                       cluster-team kernel; 0 the multigrid kernel
	                       (reported as 1) */
	int cells_per_cta;  /* target cells per CTA when sizing a problem's team */
	int use_graph;      /* >= 0: replay a captured CUDA graph; < 0: plain launch */
} carpio_gpu_batch_tiles;

typedef struct {
	carpio_gpu_batch_tiles tiles;  /* the configuration in use */
	int clusters;       /* clusters launched (all resident) */
	int ctas;           /* CTAs launched */
	int smem_bytes;     /* dynamic shared memory per CTA */
	int teams[5];       /* problems with team size 1, 2, 4, 8, 16 */
	double est_ms;      /* the planner's makespan estimate */
	int candidates;     /* configurations the autotuner timed (0: none) */
	double tuned_ms;    /* the autotuner's time for the configuration in use */
} carpio_gpu_batch_info;

/* Plans the batch (teams, cluster slots, shared memory), uploads the
 * coefficients and allocates the device fields (zero). cfg: kind CG,
 * precision MIXED; tol, max_iter, inner_tol and flags apply to every problem.
 * tiles may be NULL. Problems that fit no team are rejected (EINVAL). */
int carpio_gpu_batch_create(int count, const carpio_gpu_batch_problem* probs,
		const carpio_gpu_solver_cfg* cfg, const carpio_gpu_batch_tiles* tiles,
		carpio_gpu_batch** out);
int carpio_gpu_batch_destroy(carpio_gpu_batch* b);
/* which: 0 source, 1 phi (initial guess in, solution out). fields[count]. */
int carpio_gpu_batch_upload(carpio_gpu_batch* b, int which,
		const double* const* fields);
int carpio_gpu_batch_download(carpio_gpu_batch* b, int which,
		double* const* fields);
/* device address of problem i's field in the layout above */
int carpio_gpu_batch_field(carpio_gpu_batch* b, int which, int i, double** dev);
/* sets every problem's field `which` to zero (e.g. phi before a cold solve) */
int carpio_gpu_batch_zero(carpio_gpu_batch* b, int which);
/* Solves every problem on the device-resident fields. stats[count] may be
 * NULL (per problem: code, inner iterations, residual, refinements, device
 * ms); *ms (may be NULL) gets the device time of the whole launch. Returns 0
 * when all converged, 1 if any reached max_iter, or a negative error. */
int carpio_gpu_batch_run(carpio_gpu_batch* b, carpio_gpu_solver_stats* stats,
		double* ms);
/* Times up to max_candidates launch configurations on the fields now held
 * (phi is restored after every trial) and keeps the fastest. */
int carpio_gpu_batch_autotune(carpio_gpu_batch* b, int max_candidates);
int carpio_gpu_batch_get_info(const carpio_gpu_batch* b,
		carpio_gpu_batch_info* info);
/* Host-only planning (no device call): the team size and cluster slot
 * (cluster * 16 + slot) of every problem for the given tiles and number of
 * clusters, and the estimated makespan. */
int carpio_gpu_batch_plan(int count, const carpio_gpu_batch_problem* probs,
		const carpio_gpu_batch_tiles* tiles, int clusters, int* team, int* slot,
		double* est_ms);
/* Host-only: split the problems across `world` processes by estimated work
 * (largest first onto the least-loaded rank); rank_of[count]. */
int carpio_gpu_batch_shard(int count, const carpio_gpu_batch_problem* probs,
		int world, int* rank_of);

/* ----- 4. learned preconditioner: tensor-core operators ---------------------
 * No counterpart in the reference. One 3x3 convolution (stride 1, zero
 * padding 1) of BF16 activations in NHWC layout ([n][h][w][c], c contiguous)
 * with BF16 weights [9][cout][cin0 + cin1] (tap = 3 dy + dx), FP32
 * accumulation on the tensor cores, BF16 output. in1 (may be NULL) is read
 * as channels cin0.. of one concatenated input. Output channels [0, split)
 * go to out0 (split channels per pixel), the rest to out1 (split = 0 means
 * all to out0). relu: max(., 0); mask0/mask1 (may be NULL, layout of
 * out0/out1): zero where the mask is not > 0. Device pointers only; channel
 * counts multiples of 32, cout a multiple of 32 up to 256 or of 192/256
 * above; n*h*w a multiple of 128 with 128-pixel tiles of whole rows or whole
 * images. stream is a cudaStream_t (NULL = default); the call returns when
 * the convolution has finished. */
int carpio_gpu_nn_conv3x3(const void* in0, int cin0, const void* in1, int cin1,
		int n, int h, int w, const void* wt, int cout, void* out0, int split,
		void* out1, const void* mask0, const void* mask1, int relu, void* stream);

/* The learned preconditioner: a 4-level BF16 U-Net (32/64/128/256 channels,
 * 3x3 convolutions, ReLU, average pooling, nearest upsampling, concatenating
 * skips, no biases; carpio_gpu_unet_num_params() FP32 parameters) mapping a
 * field x [n][h][w] (FP32) to z [n][h][w] (FP32); h, w multiples of 8 and at
 * least 16. The convolutions run on the tensor cores; training is Adam on
 * FP32 master weights. loss_mode 0: relative squared error
 * sum (z - t)^2 / sum t^2; 1: relative energy norm (e, A e) / (t, A t),
 * e = z - t, A the all-Neumann 5-point operator with unit face coefficients
 * (the norm conjugate gradients minimise). Field pointers are device memory. */
typedef struct carpio_gpu_unet carpio_gpu_unet;
long carpio_gpu_unet_num_params(void);
/* deterministic He-normal initial weights from `seed` */
int carpio_gpu_unet_create(uint64_t seed, carpio_gpu_unet** out);
int carpio_gpu_unet_destroy(carpio_gpu_unet* u);
/* all parameters as one FP32 vector (host or device memory): the input
 * layer [9][32], the 13 3x3 layers [9][cout][cin] in network order, the
 * output layer [32]; set also resets the optimiser state */
int carpio_gpu_unet_get_params(carpio_gpu_unet* u, float* out);
int carpio_gpu_unet_set_params(carpio_gpu_unet* u, const float* in);
int carpio_gpu_unet_forward(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		float* z, void* stream);
/* loss and gradient (FP32, layout of the parameters; host or device) */
int carpio_gpu_unet_grad(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		const float* t, int loss_mode, float* grad, double* loss);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the batch */
int carpio_gpu_unet_train_step(carpio_gpu_unet* u, int n, int h, int w, const float* x,
		const float* t, int loss_mode, float lr, double* loss);

/* Poisson solve with the learned preconditioner: flexible CG (FCG(m),
 * Notay) in FP64 whose preconditioner is the U-Net on the residual (scaled
 * to unit RMS) followed by `smooth` damped Jacobi sweeps; the network's
 * answer to the initial residual is also the warm start. The true FP64
 * residual judges convergence (the reference's nrm2 test against cfg->tol);
 * after `stall` iterations without a 10 % drop the solve finishes with the
 * plain MIXED CG if `fallback` is set. use_net = 0 runs the same iteration
 * without the network. The grid needs nx, ny multiples of 8 (>= 16) with the
 * network's tiling. Arguments otherwise as carpio_gpu_poisson_solve
 * (resid_hist: the FCG residuals, initial one first); stats: iters = FCG +
 * fallback iterations, outer_iters = FCG iterations. */
typedef struct {
	int use_net;       /* 1: network + smoothing; 0: smoothing only */
	int smooth;        /* Jacobi sweeps after the network */
	double omega;      /* their damping (0 = 0.8) */
	int memory;        /* FCG directions kept, 1..4 */
	int stall;         /* iterations of the stall test (0 = 20) */
	int fallback;      /* finish with the plain CG after a stall */
} carpio_gpu_learned_cfg;

int carpio_gpu_poisson_solve_learned(carpio_gpu_grid* g, const carpio_gpu_bc* bc,
		double beta, const double* source, double* phi,
		const carpio_gpu_solver_cfg* cfg, carpio_gpu_unet* net,
		const carpio_gpu_learned_cfg* lc, double* resid_hist, int hist_cap,
		carpio_gpu_solver_stats* stats);
/* The NS projection with the learned solve (net = NULL: back to the
 * configured projection solver); lc is copied. */
int carpio_gpu_ns_set_learned(carpio_gpu_ns* ns, carpio_gpu_unet* net,
		const carpio_gpu_learned_cfg* lc);

#ifdef __cplusplus
}
#endif
#endif
