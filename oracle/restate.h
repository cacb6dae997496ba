/* Oracle: plain-C restatement of the reference (hyperpower/carpios) algorithms
 * on the projection hot path. TEST INFRASTRUCTURE ONLY: the tests, the smoke
 * check and the benchmark's CPU-baseline leg call it as the checker; the
 * product library never links it.
 *
 * Every routine follows the reference's arithmetic order operation by
 * operation (built with -ffp-contract=off), so on the same inputs it
 * reproduces the reference's doubles bit for bit; tests/test_oracle_golden.py
 * pins that against fixtures produced by the reference's own code.
 *
 * Layout conventions (the reference's):
 *   - a cell field is the SpaceT array of Scalar_ (lib/algebra/space.hpp:184-209):
 *     (nx+2gl) x (ny+2gl) doubles, [I][J] with J (y) contiguous, ghosts included;
 *   - a face field uses the same array: f(i) is the face between cell i and
 *     i+1 along its axis, f(-1) the low wall face (lib/structure/s_operation.hpp:57-70);
 *   - solver vectors number the normal cells x fastest: k = i + j*nx.
 */
#ifndef CARPIO_ORACLE_RESTATE_H
#define CARPIO_ORACLE_RESTATE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Krylov kinds, in the order of the carpio:: free functions */
enum { RS_CG = 0, RS_JACOBI = 1, RS_DIA_BICGSTAB = 2, RS_BICGSTAB = 3,
	RS_IC_CGS = 4, RS_IC_CG = 5 };
#define RS_EZERODIAG (-4)

/* lib/algebra/solver_matrix.hpp:192-260 (Jacobi), 264-316 (CG),
 * 599-672 (Dia_BiCGSTAB), 674-745 (BiCGSTAB). Returns the reference's code
 * (0 converged, 1 max_iter, 2 rho breakdown, 3 omega breakdown) or
 * RS_EZERODIAG where DiaPre (preconditioner.hpp:223-227) would exit().
 * max_iter and tol are in/out exactly as in the reference; hist receives the
 * residual list (lresid), up to hist_cap entries, *hist_len its full length.
 * threads > 1 runs the vector and SpMV loops with OpenMP (not bit-exact). */
int rs_krylov_csr(int kind, int n, const unsigned* rowptr, const unsigned* col,
		const double* val, const double* b, double* x, int* max_iter,
		double* tol, double* hist, int hist_cap, int* hist_len, int threads);

/* lib/algebra/BLAS_Level1.hpp:499-544 and 556-577 */
double rs_dot(int n, const double* x, const double* y);
double rs_nrm2(int n, const double* x);
double rs_residual(int n, const unsigned* rp, const unsigned* ci,
		const double* va, const double* x, const double* b, int full);

/* Grid_::_set_uniform_grid (lib/structure/s_grid.hpp:372-395): cell sizes
 * s[0..n+2gl) and centres c[0..n+2gl), ghosts included. */
void rs_grid_uniform(int n, int gl, double lo, double hi, double* c, double* s);
void rs_grid_sizes(int n, int gl, double lo, const double* cs, double* c, double* s);

/* Boundary description of one field: type per segment (1 Dirichlet,
 * 2 Neumann; segments 0 x-, 1 x+, 2 y-, 3 y+) and a constant value. */
typedef struct {
	int type[4];
	double value[4];
} rs_bc;

/* The assembled system of structure::Solver_::_build_exp/_build_matrix
 * (lib/structure/s_solver.hpp:94-171) for StencilPoisson_ (s_poisson.hpp:60-114)
 * with GhostRegular_ substitution (s_ghost.hpp:140-179, 334-357): same
 * coefficients, same entry order, zero entries trimmed, b = -constant.
 * src is a cell field (NULL = uniform source src_value). Arrays sized
 * rowptr[n+1], col/val[5n], b[n]. Returns nnz. */
int rs_assemble_poisson(int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		double beta, const double* src, double src_value, unsigned* rowptr,
		unsigned* col, double* val, double* b, const double* bfield);

/* Equation_::apply_bc (s_equation.hpp:340-378) on a cell field. */
void rs_apply_bc(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc, double* f);

/* the same with a boundary value per ghost cell (gv, a cell field; NULL =
 * bc->value), for boundary conditions given as functions */
void rs_apply_bc_gv(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc, const double* gv,
		double* f);

/* Operation_ (s_operation.hpp): Grad :46-72, Div(VecF) :100-120,
 * InterpolateF2C :141-164, InterpolateC2F :166-187, NablaMuNabla :664-688. */
void rs_grad(int nx, int ny, int gl, const double* cx, const double* cy,
		const double* phi, double* gx, double* gy);
void rs_div(int nx, int ny, int gl, const double* sx, const double* sy,
		const double* fx, const double* fy, double* div);
void rs_f2c(int nx, int ny, int gl, const double* fx, const double* fy,
		double* cxo, double* cyo);
void rs_c2f(int nx, int ny, int gl, const double* sx, const double* sy,
		const double* u, const double* v, double* fx, double* fy);
void rs_diffusion(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, double mu, const double* f,
		double* out);
void rs_diffusion_var(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const double* mu, const double* f,
		double* out);

/* Advection schemes of NS_::set_advection_scheme (s_ns.hpp:171-211) plus the
 * minmod limiter of src/calculation/advection.hpp:1079-1081. */
enum {
	RS_UPWIND1 = 0, RS_CENTER = 1, RS_CENTER4 = 2, RS_UPWIND2 = 3,
	RS_VANLEER = 4, RS_SUPERBEE = 5, RS_WAHYD = 6, RS_QUICK = 7, RS_CUI = 8,
	RS_MINMOD = 9
};
void rs_advection(int scheme, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const double* uf,
		const double* vf, const double* f, double* out);

/* Advection_::run_one_step (s_advection.hpp:185-212) `steps` times on phi
 * (in place, x-fastest order) with fixed face velocities uf, vf; scheme as
 * rs_advection (RS_MINMOD is not one of Advection_'s). */
void rs_advect_run(int scheme, int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		const double* gv, const double* uf, const double* vf, double dt,
		int steps, double* phi);

/* VectorCenter_::max_magnitude (s_vector.hpp:89-103) */
double rs_max_magnitude(int nx, int ny, int gl, const double* u,
		const double* v);

/* Lid-driven-cavity style explicit projection (NS_explicit_, s_ns_explicit.hpp:
 * 118-229, NS_::restrict_time s_ns.hpp:146-169), projection solved by CG with
 * mean removal of b and x. All fields are full arrays with ghosts and are
 * updated in place. Per-step dt, CG iterations and final residual go to the
 * optional arrays. Returns 0, or the first non-zero CG code. */
typedef struct {
	double rho, mu;            /* uniform rho (set_uniform_rho) and mu */
	double cfl;                /* CFL_number */
	double diff_number;        /* Diffusion_number; >= 100 disables */
	double diff_coef;          /* Diffusion_coefficient */
	int scheme;                /* RS_* advection scheme */
	int cg_max_iter;
	double cg_tol;
	int threads;               /* OpenMP threads for the CG (1 = bit-exact) */
	int proj_kind;             /* RS_* Krylov kind of the projection (0 = CG) */
	int proj_nomean;           /* 1: no mean removal (the shipped solvers) */
	const double* mu_field;    /* set_mu field (NULL: the uniform mu) */
} rs_ns_cfg;

int rs_ns_run(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc_u,
		const rs_bc* bc_v, const rs_ns_cfg* cfg, int steps, double* dt,
		double* u, double* v, double* uf, double* vf, double* phi, double* p,
		double* step_dt, int* step_iters, double* step_resid);

/* StencilHelmholtz_ rows (s_poisson.hpp:185-260) assembled like
 * rs_assemble_poisson (uniform alpha and beta, source field src). */
int rs_assemble_helmholtz(int nx, int ny, int gl, const double* cx,
		const double* sx, const double* cy, const double* sy, const rs_bc* bc,
		double alpha, double beta, const double* src, unsigned* rowptr,
		unsigned* col, double* val, double* b);

/* NS_kim_ stepping (s_ns_kim.hpp:130-280), `steps` steps at time step dt;
 * first: the first of them is the stepper's step 0 (advection without the
 * Adams-Bashforth term). us, vs, usf, vsf persist between calls as the
 * reference's star fields do. The projection uses cfg's solver. */
int rs_kim_run(int nx, int ny, int gl, const double* cx, const double* sx,
		const double* cy, const double* sy, const rs_bc* bc_u,
		const rs_bc* bc_v, const rs_ns_cfg* cfg, int steps, int first, double dt,
		double* u, double* v, double* uf, double* vf, double* phi, double* p,
		double* us, double* vs, double* usf, double* vsf, int* step_iters,
		double* step_resid);

#ifdef __cplusplus
}
#endif
#endif
