// Oracle harness compiled directly against the reference's own headers
// (lib/algebra, lib/structure) with the project shims in oracle/ref/shims.
// It runs the reference code on the workloads the GPU path is checked on and
// writes the inputs and outputs as raw binary arrays plus a text manifest;
// tests/golden/make_golden.py turns those into the committed fixtures.
//
// This is test infrastructure: nothing in the product links or calls it.
//
// Subcommands (all write into <outdir>):
//   csr     <mtx> <rhs|ones> <x0: ones|zeros> <kind> <max_iter> <tol>
//           kind: cg | jacobi | dia_bicgstab | bicgstab | jacobi_class
//           carpio::CG / Jacobi / Dia_BiCGSTAB / BiCGSTAB on a MatrixMarket
//           matrix read with lib/io/mmio.h:220 (as test/algebra/_test_solver.hpp
//           does), CSR built by MatrixSCR_(MatrixSCO_).
//   poisson <case> <n> <solver> <max_iter> <tol> <seed> [stretch]
//           case: c1 | neumann | mixed ; solver: cg | jacobi | dia_bicgstab |
//           bicgstab. Poisson_ (s_poisson.hpp) with the solver replaced by a
//           drop-in structure::Solver_ that assembles the CSR with the
//           reference's _build_exp/_build_matrix and calls the carpio:: free
//           function (mean removal of b and x for the all-Neumann case).
//   cavity  <n> <steps> <scheme> <tol> <max_iter> <dt0> <Re> <dump_every> [stretch]
//           [proj=<kind>[_nomean]] [mu=field]
//           NS_explicit_ (s_ns_explicit.hpp) lid-driven cavity on [0,1]^2,
//           gl = 2, projection by the CG + mean-removal drop-in (proj=: another
//           carpio:: solver, with or without the mean removal; mu=field:
//           mu(x, y) = 1 + x y / 2 in place of the uniform mu).
//   kim     <n> <steps> <scheme> <tol> <max_iter> <dt0> <Re>
//           NS_kim_ (s_ns_kim.hpp) lid-driven cavity, gl = 2, projection by
//           the CG + mean-removal drop-in.
//   ops     <n> <seed> <gl> [stretch]
//           single operators of Operation_ (s_operation.hpp) and
//           Equation_::apply_bc (s_equation.hpp:340-378) on seeded fields;
//           `stretch` (here and for poisson / cavity) builds the grid from
//           cell sizes (make_grid). Also writes the
//           field in_a with Output_Scalar (s_io_file.hpp:43-71) to dump.txt.
//   advect  <n> <steps> <scheme> <dt> <case> [stretch]
//           stand-alone Advection_ (s_advection.hpp) run by Equation_::run
//           with set_time(steps - 1, dt), so `steps` steps. case band: the
//           shipped 2-D TVD example's set-up (u = v = 1, phi = 0, a function
//           BC phi = 1 on 0 <= y <= 0.3 of the x- side, 0 elsewhere); case
//           rotate: solid rotation about (0.5, 0.5) of a cone, default
//           (Neumann 0) BCs. Writes the initial fields the functions give
//           (in_u, in_v, in_phi, every cell incl. ghosts) and phi, u, v at
//           the end.

#include "structure/s_grid.hpp"
#include "structure/s_poisson.hpp"
#include "structure/s_ns_explicit.hpp"
#include "structure/s_ns_kim.hpp"
#include "structure/s_operation.hpp"
#include "structure/s_advection.hpp"
#include "io/mmio.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <random>
#include <string>
#include <vector>

using namespace structure;

typedef Grid_<2> Grid;
typedef std::shared_ptr<Grid> spGrid;
typedef Index_<2> Index;
typedef Poi_<2> Poi;
typedef Scalar_<2> Scalar;
typedef std::shared_ptr<Scalar> spScalar;
typedef Operation_<2> Op;

// structure::Output_Scalar, instantiated in dump_scalar.cpp
void harness_output_scalar(const std::string& filename, const Scalar& s);

// ---------------------------------------------------------------- output ---
static std::string g_out;
static std::ofstream g_meta;

static void out_open(const std::string& dir) {
	g_out = dir;
	std::string cmd = "mkdir -p '" + dir + "'";
	if (std::system(cmd.c_str()) != 0) {
		std::fprintf(stderr, "cannot create %s\n", dir.c_str());
		std::exit(2);
	}
	g_meta.open(dir + "/meta.txt");
}
static void put_scalar(const char* k, double v) {
	char buf[64];
	std::snprintf(buf, sizeof buf, "%.17g", v);
	g_meta << "scalar " << k << " " << buf << "\n";
}
template<class T>
static void put_array(const std::string& name, const char* dtype, const T* p,
		std::size_t n, std::size_t d0, std::size_t d1 = 0) {
	std::string fn = g_out + "/" + name + ".bin";
	FILE* f = std::fopen(fn.c_str(), "wb");
	if (n) std::fwrite(p, sizeof(T), n, f);
	std::fclose(f);
	g_meta << "array " << name << " " << dtype << " " << d0;
	if (d1) g_meta << " " << d1;
	g_meta << "\n";
}
static void put_vec(const std::string& name, const std::vector<double>& v) {
	put_array(name, "f64", v.data(), v.size(), v.size());
}
static void put_arr(const std::string& name, const Arr& a) {
	put_array(name, "f64", a.getPointer(), a.size(), a.size());
}
static void put_list(const std::string& name, const std::list<Vt>& l) {
	std::vector<double> v(l.begin(), l.end());
	put_vec(name, v);
}
// full field with ghosts, SpaceT layout [I][J] with J (y) fastest
static void put_field(const std::string& name, const Scalar& s) {
	const Grid& g = *s.get_grid();
	int NI = g.N(0), NJ = g.N(1);
	std::vector<double> v(std::size_t(NI) * NJ);
	for (int I = 0; I < NI; ++I)
		for (int J = 0; J < NJ; ++J)
			v[std::size_t(I) * NJ + J] = s.VAL(I, J);
	put_array(name, "f64", v.data(), v.size(), NI, NJ);
}
static void get_field(Scalar& s, const std::vector<double>& v) {
	const Grid& g = *s.get_grid();
	int NI = g.N(0), NJ = g.N(1);
	for (int I = 0; I < NI; ++I)
		for (int J = 0; J < NJ; ++J)
			s.VAL(I, J) = v[std::size_t(I) * NJ + J];
}
static void put_csr(const Mat& m) {
	St n = m.iLen(), nz = m.NumNonzeros();
	std::vector<unsigned> rp(n + 1), ci(nz);
	std::vector<double> va(nz);
	for (St i = 0; i <= n; ++i) rp[i] = m.row_ptr(i);
	for (St k = 0; k < nz; ++k) { ci[k] = m.col_ind(k); va[k] = m.val(k); }
	put_array("rowptr", "u32", rp.data(), rp.size(), rp.size());
	put_array("colind", "u32", ci.data(), ci.size(), ci.size());
	put_array("val", "f64", va.data(), va.size(), va.size());
}
// [0,1]^2 with nx x ny cells: uniform (Grid_(min, max, n, gl)), or from
// cell sizes (Grid_(min, gl, csx, csy), s_grid.hpp:35-48, 397-434):
// geometric growth along x, a wave along y, both scaled to length 1
static spGrid make_grid(int nx, int ny, int gl, bool stretch) {
	Poi pmin(0.0, 0.0), pmax(1.0, 1.0);
	if (!stretch) return spGrid(new Grid(pmin, pmax, Index(nx, ny), gl));
	Arr csx(nx), csy(ny);
	double lx = 0, ly = 0;
	for (int i = 0; i < nx; ++i) { csx[i] = std::pow(1.07, double(i)); lx += csx[i]; }
	for (int j = 0; j < ny; ++j) { csy[j] = 1.0 + 0.6 * std::sin(0.9 * j); ly += csy[j]; }
	for (int i = 0; i < nx; ++i) csx[i] /= lx;
	for (int j = 0; j < ny; ++j) csy[j] /= ly;
	return spGrid(new Grid(pmin, gl, csx, csy));
}
static bool stretch_arg(int argc, char** argv, int k) {
	return argc > k + 1 && std::string(argv[k]) == "stretch";
}

static void put_grid(const Grid& g) {
	for (St d = 0; d < 2; ++d) {
		int N = g.N(d);
		std::vector<double> c(N), s(N);
		for (int I = 0; I < N; ++I) { c[I] = g.C_(d, I); s[I] = g.S_(d, I); }
		put_vec(d == 0 ? "grid_cx" : "grid_cy", c);
		put_vec(d == 0 ? "grid_sx" : "grid_sy", s);
	}
}

// ----------------------------------------------------- carpio:: dispatch ---
static int run_carpio(const std::string& kind, const Mat& A, Arr& x,
		const Arr& b, int& max_iter, double& tol, std::list<Vt>& lr) {
	if (kind == "cg") return carpio::CG(A, x, b, max_iter, tol, lr);
	if (kind == "jacobi") return carpio::Jacobi(A, x, b, max_iter, tol, lr);
	if (kind == "dia_bicgstab")
		return carpio::Dia_BiCGSTAB(A, x, b, max_iter, tol, lr);
	if (kind == "bicgstab") return carpio::BiCGSTAB(A, x, b, max_iter, tol, lr);
	if (kind == "ic_cgs") return carpio::IC_CGS(A, x, b, max_iter, tol, lr);
	if (kind == "ic_cg") return carpio::IC_CG(A, x, b, max_iter, tol, lr);
	std::fprintf(stderr, "unknown solver kind %s\n", kind.c_str());
	std::exit(2);
}

static double mean_of(const Arr& a) {
	double s = 0;
	for (St i = 0; i < a.size(); ++i) s += a[i];
	return s / double(a.size());
}
static void remove_mean(Arr& a) {
	double m = mean_of(a);
	for (St i = 0; i < a.size(); ++i) a[i] = a[i] - m;
}

// ------------------------------------------- drop-in structure solver ---
// The seam the GPU library replaces: structure::Solver_<2>::solve() as in
// s_solver.hpp:261-291/329-352, but calling a carpio:: free-function Krylov
// solver chosen by name, with optional null-space (mean) removal.
struct SolveRecord {
	int ret, iters;
	double tol_out;
	std::list<Vt> lr;
	double ms;
};

class Solver_Alg_: public structure::Solver_<2> {
public:
	typedef structure::Solver_<2> Base;
	Solver_Alg_(spGrid g, spGhost gh, spStencil st, const std::string& vn,
			spCenterScalar cs, const std::string& kind, bool mean_removal,
			std::vector<SolveRecord>* rec, bool dump)
		: Base(g, gh, st, vn, cs), _kind(kind), _mean(mean_removal),
		  _rec(rec), _dump(dump) {}
	void solve() {
		auto t0 = std::chrono::steady_clock::now();
		this->_build_exp();
		Mat mat;
		Arr b;
		this->_build_matrix(mat, b);
		Arr x = this->_copy_to_x();
		if (_mean) remove_mean(b);
		if (_dump) {
			put_csr(mat);
			put_arr("b", b);
			put_arr("x0", x);
		}
		SolveRecord r;
		r.iters = this->_max_iter;
		r.tol_out = this->_tol;
		r.ret = run_carpio(_kind, mat, x, b, r.iters, r.tol_out, r.lr);
		if (_mean) remove_mean(x);
		this->_copy_to_cs(x);
		r.ms = std::chrono::duration<double, std::milli>(
				std::chrono::steady_clock::now() - t0).count();
		if (_dump) put_arr("x", x);
		if (_rec) _rec->push_back(r);
	}
protected:
	std::string _kind;
	bool _mean;
	std::vector<SolveRecord>* _rec;
	bool _dump;
};

class PoissonAlg_: public Poisson_<2> {
public:
	PoissonAlg_(spGrid g, const std::string& kind, bool mean, int max_iter,
			double tol, std::vector<SolveRecord>* rec, bool dump)
		: Poisson_<2>(g), _kind(kind), _mean(mean), _mi(max_iter), _tol(tol),
		  _rec(rec), _dump(dump) {}
	int initial() {
		Poisson_<2>::initial();
		std::shared_ptr<Solver_Alg_> s(new Solver_Alg_(this->_grid,
				this->_ghost, this->_stencils["poisson"], "phi",
				this->_css["phi"], _kind, _mean, _rec, _dump));
		s->set_max_iter(_mi);
		s->set_tolerance(_tol);
		this->_solvers["main"] = s;
		return -1;
	}
	void set_dump(bool d) { _dump = d; }
protected:
	std::string _kind;
	bool _mean;
	int _mi;
	double _tol;
	std::vector<SolveRecord>* _rec;
	bool _dump;
};

// ------------------------------------------------------------ csr cmd ---
static int cmd_csr(int argc, char** argv) {
	// csr <mtx> <rhs|ones> <x0> <kind> <max_iter> <tol> <outdir>
	if (argc < 9) return 2;
	std::string mtx = argv[2], rhs = argv[3], x0 = argv[4], kind = argv[5];
	int max_iter = std::atoi(argv[6]);
	double tol = std::atof(argv[7]);
	out_open(argv[8]);
	carpio::MatrixSCO_<double> mco;
	carpio::mm_read_mtx_sparse(mtx, mco);
	Mat A(mco);
	Arr b(A.iLen()), x(A.iLen());
	if (rhs == "ones") b.assign(1.0);
	else carpio::mm_read_array(rhs, b);
	x.assign(x0 == "ones" ? 1.0 : 0.0);
	put_csr(A);
	put_arr("b", b);
	put_arr("x0", x);
	// carpio::Residual (solver_matrix.hpp:583-597) of the start and, below,
	// of the solution
	put_scalar("residual_x0", carpio::Residual(A, x, b));
	std::list<Vt> lr;
	int ret, mi = max_iter;
	double t = tol;
	auto t0 = std::chrono::steady_clock::now();
	if (kind == "jacobi_class") {
		// class form (solver_matrix.hpp:820-910), as test/algebra/_test_solver.hpp uses
		carpio::Solver_Jacobi_<double> s(max_iter, tol);
		ret = s.solve(A, x, b);
		mi = s.num_iter();
		t = s.residual();
		Arr h = s.get_residual_array();
		for (St i = 0; i < h.size(); ++i) lr.push_back(h[i]);
	} else {
		ret = run_carpio(kind, A, x, b, mi, t, lr);
	}
	double ms = std::chrono::duration<double, std::milli>(
			std::chrono::steady_clock::now() - t0).count();
	put_arr("x", x);
	put_scalar("residual_x", carpio::Residual(A, x, b));
	put_list("lresid", lr);
	put_scalar("ret", ret);
	put_scalar("max_iter_in", max_iter);
	put_scalar("tol_in", tol);
	put_scalar("max_iter_out", mi);
	put_scalar("tol_out", t);
	put_scalar("ms", ms);
	return 0;
}

// -------------------------------------------------------- poisson cmd ---
// Case definitions (the GPU tests rebuild the same inputs):
//  c1      [0,1]^2, Dirichlet 0 on segments 0..3, f = -2 pi^2 sin(pi x) sin(pi y)
//  neumann [0,1]^2, all-Neumann (default BC), seeded zero-mean uniform source,
//          mean removed from b and x
//  mixed   [0,1]^2, seg0 Dirichlet 1, seg1 Dirichlet -0.5, seg2 Neumann 0.75,
//          seg3 Neumann -1.25, f = 20 cos(3 pi x) sin(2 pi y)
//  vbeta   as mixed with beta = 1.2 + 0.5 sin(2 pi x) cos(pi y) as a field
static int cmd_poisson(int argc, char** argv) {
	if (argc < 9) return 2;
	std::string cs = argv[2];
	int n = std::atoi(argv[3]);
	std::string kind = argv[4];
	int max_iter = std::atoi(argv[5]);
	double tol = std::atof(argv[6]);
	unsigned seed = unsigned(std::atoi(argv[7]));
	out_open(argv[argc - 1]);
	const bool stretch = stretch_arg(argc, argv, 8);
	spGrid g = make_grid(n, n, 2, stretch);
	put_scalar("stretch", stretch ? 1.0 : 0.0);
	put_grid(*g);
	std::vector<SolveRecord> rec;
	bool mean = (cs == "neumann");
	PoissonAlg_ P(g, kind, mean, max_iter, tol, &rec, true);
	spScalar src(new Scalar(g));
	if (cs == "c1") {
		for (int d = 0; d < 4; ++d) {
			Poisson_<2>::spBC bc(new Poisson_<2>::BC());
			bc->set_default_1_bc(0.0);
			P.add_bc(0, d, "phi", bc);
		}
		P.set_source([](Vt t, Vt x, Vt y, Vt z) {
			return -2.0 * carpio::PI * carpio::PI * std::sin(carpio::PI * x)
					* std::sin(carpio::PI * y);
		});
	} else if (cs == "neumann") {
		std::mt19937_64 rng(seed);
		std::uniform_real_distribution<double> U(-1.0, 1.0);
		for (int i = 0; i < n; ++i)
			for (int j = 0; j < n; ++j) (*src)(i, j) = U(rng);
		spScalar phi(new Scalar(g));
		put_field("source_field", *src);
		P.set_depend(phi, nullptr, src);
	} else if (cs == "mixed" || cs == "vbeta") {
		double vals[4] = { 1.0, -0.5, 0.75, -1.25 };
		for (int d = 0; d < 4; ++d) {
			Poisson_<2>::spBC bc(new Poisson_<2>::BC());
			if (d < 2) bc->set_default_1_bc(vals[d]);
			else bc->set_default_2_bc(vals[d]);
			P.add_bc(0, d, "phi", bc);
		}
		P.set_source([](Vt t, Vt x, Vt y, Vt z) {
			return 20.0 * std::cos(3 * carpio::PI * x)
					* std::sin(2 * carpio::PI * y);
		});
		if (cs == "vbeta")
			P.set_beta([](Vt t, Vt x, Vt y, Vt z) {
				return 1.2 + 0.5 * std::sin(2 * carpio::PI * x) * std::cos(carpio::PI * y);
			});
	} else {
		return 2;
	}
	P.run();
	if (cs == "vbeta") put_field("beta_field", *P.get_CS("beta"));
	put_field("phi", *P.get_CS("phi"));
	put_field("source", *P.get_CS("source"));
	const SolveRecord& r = rec.back();
	put_list("lresid", r.lr);
	put_scalar("ret", r.ret);
	put_scalar("max_iter_out", r.iters);
	put_scalar("tol_out", r.tol_out);
	put_scalar("ms", r.ms);
	return 0;
}

// --------------------------------------------------------- cavity cmd ---
static Vt limiter_minmod(Vt r, Vt R) {
	// src/calculation/advection.hpp:1079-1081: max(0, min(1, r)); in the
	// structured TVD framework (s_operation.hpp:549-596) the face value is
	// phi_C + psi/R (phi_D - phi_C), which on a uniform grid (R = 2) is the
	// adaptive stack's 0.5 psi (phi_D - phi_C).
	return std::max(0.0, std::min(1.0, r));
}
static Vt VdotNabla_TVD_minmod(const VectorFace_<2>& vf, const Scalar& c,
		Index idx) {
	return Op::VdotNabla_TVD(vf, c, idx, limiter_minmod);
}

class NSAlg_: public NS_explicit_<2> {
public:
	NSAlg_(spGrid g, int max_iter, double tol, std::vector<SolveRecord>* rec,
			const std::string& kind = "cg", bool mean = true)
		: NS_explicit_<2>(g) {
		this->_projection = spPoisson(
				new PoissonAlg_(g, kind, mean, max_iter, tol, rec, false));
	}
	void set_scheme(const std::string& s) {
		if (s == "minmod") this->fun_v_dot_nabla = &VdotNabla_TVD_minmod;
		else this->set_advection_scheme(s);
	}
	// one pass of the body of Equation_::run (s_equation.hpp:154-171)
	void step_once() {
		this->run_one_step(this->_time->current_step());
		this->_time->advance();
	}
	double dt() const { return this->_time->dt(); }
	spScalar cs(const std::string& n) { return this->_css[n]; }
	spScalar proj_source() { return this->_projection->get_CS("source"); }
};

static int cmd_cavity(int argc, char** argv) {
	if (argc < 11) return 2;
	int n = std::atoi(argv[2]);
	int steps = std::atoi(argv[3]);
	std::string scheme = argv[4];
	double tol = std::atof(argv[5]);
	int max_iter = std::atoi(argv[6]);
	double dt0 = std::atof(argv[7]);
	double Re = std::atof(argv[8]);
	int dump_every = std::atoi(argv[9]);
	out_open(argv[argc - 1]);
	const bool stretch = stretch_arg(argc, argv, 10);
	// proj=<kind> | proj=<kind>_nomean: another carpio:: solver for the
	// projection, with or without the mean removal (the shipped
	// Solver_IC_CGS_, s_solver.hpp:329-352, removes nothing)
	std::string pkind = "cg";
	bool pmean = true;
	bool mufield = false;
	for (int k = 10; k < argc - 1; ++k) {
		std::string a = argv[k];
		if (a == "mu=field") mufield = true;
		if (a.compare(0, 5, "proj=") != 0) continue;
		pkind = a.substr(5);
		const std::string nm = "_nomean";
		if (pkind.size() > nm.size() && pkind.compare(pkind.size() - nm.size(), nm.size(), nm) == 0) {
			pkind = pkind.substr(0, pkind.size() - nm.size());
			pmean = false;
		}
	}
	spGrid g = make_grid(n, n, 2, stretch);
	put_scalar("stretch", stretch ? 1.0 : 0.0);
	put_grid(*g);
	std::vector<SolveRecord> rec;
	NSAlg_ ns(g, max_iter, tol, &rec, pkind, pmean);
	ns.set_scheme(scheme);
	ns.set_time(steps > 0 ? steps - 1 : 0, dt0);
	NS_<2>::spBC bc0(new NS_<2>::BC()), bc1(new NS_<2>::BC());
	bc0->set_default_1_bc(0);
	bc1->set_default_1_bc(1);
	for (int s = 0; s < 3; ++s) ns.add_bc(0, s, "u", bc0);
	ns.add_bc(0, 3, "u", bc1);
	for (int s = 0; s < 4; ++s) ns.add_bc(0, s, "v", bc0);
	ns.set_uniform_rho(Re);
	ns.set_diffusion_number(0.25, 1.0 / Re);
	if (mufield) {
		// a mu field (s_ns.hpp:111-118, 277-280): NS_::set_mu calls
		// unset_uniform_beta, which NS_ lacks, so it cannot be instantiated;
		// unset_uniform_mu + initial_CS("mu", f) is the working route
		ns.unset_uniform_mu();
		ns.initial_CS("mu", [](Vt, Vt x, Vt y, Vt) { return 1.0 + 0.5 * x * y; });
	}
	ns.initial();
	if (mufield) put_field("mu", *ns.cs("mu"));
	std::vector<double> dts, its, ms, res, rets, step_ms;
	for (int s = 0; s < steps; ++s) {
		auto t0 = std::chrono::steady_clock::now();
		ns.step_once();
		step_ms.push_back(std::chrono::duration<double, std::milli>(
				std::chrono::steady_clock::now() - t0).count());
		dts.push_back(ns.dt());
		rets.push_back(rec.back().ret);
		its.push_back(rec.back().iters);
		ms.push_back(rec.back().ms);
		res.push_back(rec.back().tol_out);
		if (s == 0) {
			// intermediates of the first step, for per-kernel checks
			put_field("s1_us", *ns.cs("us"));
			put_field("s1_vs", *ns.cs("vs"));
			put_field("s1_usf", *ns.cs("usf"));
			put_field("s1_vsf", *ns.cs("vsf"));
			put_field("s1_div", *ns.proj_source());
			put_field("s1_phi", *ns.cs("phi"));
			put_field("s1_u", *ns.cs("u"));
			put_field("s1_v", *ns.cs("v"));
			put_field("s1_uf", *ns.cs("uf"));
			put_field("s1_vf", *ns.cs("vf"));
			put_field("s1_p", *ns.cs("p"));
		}
		if (dump_every > 0 && (s + 1) % dump_every == 0 && s + 1 < steps) {
			char nm[32];
			std::snprintf(nm, sizeof nm, "u_step%d", s + 1);
			put_field(nm, *ns.cs("u"));
		}
	}
	const char* names[] = { "u", "v", "p", "phi", "uf", "vf" };
	for (const char* nm : names) put_field(nm, *ns.cs(nm));
	put_vec("dt", dts);
	put_vec("cg_iters", its);
	put_vec("cg_ret", rets);
	put_vec("cg_ms", ms);
	put_vec("step_ms", step_ms);
	put_vec("cg_resid", res);
	put_scalar("Re", Re);
	put_scalar("dt0", dt0);
	put_scalar("tol", tol);
	return 0;
}

// ------------------------------------------------------------ kim cmd ---
// NS_kim_ (s_ns_kim.hpp) lid-driven cavity: the predictor's Helmholtz solves
// keep the reference's default Jacobi solver (Poisson_::_init_solver), the
// projection is the CG + mean-removal drop-in as for NS_explicit_.
class NSKimAlg_: public NS_kim_<2> {
public:
	NSKimAlg_(spGrid g, int max_iter, double tol, std::vector<SolveRecord>* rec)
		: NS_kim_<2>(g) {
		this->_projection = spPoisson(
				new PoissonAlg_(g, "cg", true, max_iter, tol, rec, false));
	}
	void set_scheme(const std::string& s) {
		if (s == "minmod") this->fun_v_dot_nabla = &VdotNabla_TVD_minmod;
		else this->set_advection_scheme(s);
	}
	void step_once() {
		this->run_one_step(this->_time->current_step());
		this->_time->advance();
	}
	spScalar cs(const std::string& n) { return this->_css[n]; }
	spScalar scr(int d) { return this->_sscr->get_spdata(d); }
};

static int cmd_kim(int argc, char** argv) {
	if (argc < 9) return 2;
	int n = std::atoi(argv[2]);
	int steps = std::atoi(argv[3]);
	std::string scheme = argv[4];
	double tol = std::atof(argv[5]);
	int max_iter = std::atoi(argv[6]);
	double dt0 = std::atof(argv[7]);
	double Re = std::atof(argv[8]);
	out_open(argv[argc - 1]);
	spGrid g = make_grid(n, n, 2, false);
	put_grid(*g);
	std::vector<SolveRecord> rec;
	NSKimAlg_ ns(g, max_iter, tol, &rec);
	ns.set_scheme(scheme);
	ns.set_time(steps > 0 ? steps - 1 : 0, dt0);
	NS_<2>::spBC bc0(new NS_<2>::BC()), bc1(new NS_<2>::BC());
	bc0->set_default_1_bc(0);
	bc1->set_default_1_bc(1);
	for (int s = 0; s < 3; ++s) ns.add_bc(0, s, "u", bc0);
	ns.add_bc(0, 3, "u", bc1);
	for (int s = 0; s < 4; ++s) ns.add_bc(0, s, "v", bc0);
	ns.set_uniform_rho(Re);
	ns.initial();
	std::vector<double> its, res;
	for (int s = 0; s < steps; ++s) {
		ns.step_once();
		its.push_back(rec.back().iters);
		res.push_back(rec.back().tol_out);
		if (s == 0) {
			put_field("s1_xscr", *ns.scr(0));
			put_field("s1_yscr", *ns.scr(1));
			put_field("s1_phi", *ns.cs("phi"));
			put_field("s1_p", *ns.cs("p"));
			put_field("s1_u", *ns.cs("u"));
			put_field("s1_v", *ns.cs("v"));
			put_field("s1_uf", *ns.cs("uf"));
			put_field("s1_vf", *ns.cs("vf"));
		}
	}
	const char* names[] = { "u", "v", "p", "phi", "uf", "vf", "us", "vs" };
	for (const char* nm : names) put_field(nm, *ns.cs(nm));
	put_vec("cg_iters", its);
	put_vec("cg_resid", res);
	return 0;
}

// ------------------------------------------------------------ ops cmd ---
class EqProbe_: public Equation_<2> {
public:
	EqProbe_(spGrid g) : Equation_<2>(g) {
		this->_ghost = spGhost(new GhostRegular_<2>(g, this->_bi));
		this->_time = spTime(new Time_<2>(10, 0.1));
	}
	void put(const std::string& n, spScalar s) { this->_css[n] = s; }
};

static int cmd_ops(int argc, char** argv) {
	if (argc < 6) return 2;
	int n = std::atoi(argv[2]);
	unsigned seed = unsigned(std::atoi(argv[3]));
	int gl = std::atoi(argv[4]);
	out_open(argv[argc - 1]);
	int nx = n, ny = n + 3;  // non-square cell counts on a square box
	const bool stretch = stretch_arg(argc, argv, 5);
	spGrid g = make_grid(nx, ny, gl, stretch);
	put_scalar("stretch", stretch ? 1.0 : 0.0);
	put_grid(*g);
	put_scalar("nx", nx);
	put_scalar("ny", ny);
	put_scalar("gl", gl);
	std::mt19937_64 rng(seed);
	std::uniform_real_distribution<double> U(-1.0, 1.0);
	auto rnd = [&](const std::string& nm) {
		spScalar s(new Scalar(g));
		for (int I = 0; I < g->N(0); ++I)
			for (int J = 0; J < g->N(1); ++J) s->VAL(I, J) = U(rng);
		put_field(nm, *s);
		return s;
	};
	spScalar a = rnd("in_a"), b = rnd("in_b"), uf = rnd("in_uf"),
			vf = rnd("in_vf");
	harness_output_scalar(g_out + "/dump.txt", *a);
	VectorFace_<2> VF(uf, vf, nullptr);
	std::shared_ptr<VectorFace_<2> > spVF(new VectorFace_<2>(uf, vf, nullptr));
	// Grad / Div / interpolations
	auto gr = Op::Grad(a);
	put_field("grad_x", (*gr)[0]);
	put_field("grad_y", (*gr)[1]);
	put_field("div", *Op::Div(spVF));
	auto f2c = Op::InterpolateF2C(spVF);
	put_field("f2c_x", (*f2c)[0]);
	put_field("f2c_y", (*f2c)[1]);
	if (gl >= 1) {
		std::shared_ptr<VectorCenter_<2> > vc(new VectorCenter_<2>(a, b, nullptr));
		spScalar fx(new Scalar(g)), fy(new Scalar(g));
		std::shared_ptr<VectorFace_<2> > vfo(new VectorFace_<2>(fx, fy, nullptr));
		Op::InterpolateC2F(vc, vfo);
		put_field("c2f_x", *fx);
		put_field("c2f_y", *fy);
		put_scalar("max_magnitude", vc->max_magnitude());
		put_scalar("restrict_cfl", Op::TimeRestrict_CourantNumber(0.5, *vc));
		put_scalar("restrict_diff",
				Op::TimeRestrict_DiffusionNumber(0.25, *g, 1e-3));
	}
	// advection schemes and diffusion, interior only
	struct Sch { const char* nm; Vt (*f)(const VectorFace_<2>&, const Scalar&, Index); };
	std::vector<Sch> sch;
	sch.push_back({ "adv_upwind1", &Op::VdotNabla_upwind1 });
	sch.push_back({ "adv_center", &Op::VdotNabla_center });
	if (gl >= 2) {
		sch.push_back({ "adv_vanleer", &Op::VdotNabla_TVD_VanLeer });
		sch.push_back({ "adv_superbee", &Op::VdotNabla_TVD_superbee });
		sch.push_back({ "adv_minmod", &VdotNabla_TVD_minmod });
		sch.push_back({ "adv_upwind2", &Op::VdotNabla_upwind2 });
		sch.push_back({ "adv_quick", &Op::VdotNabla_QUICK });
		sch.push_back({ "adv_cui", &Op::VdotNabla_CUI });
		sch.push_back({ "adv_wahyd", &Op::VdotNabla_TVD_WAHYD });
		sch.push_back({ "adv_center4", &Op::VdotNabla_center4 });
	}
	for (auto& s : sch) {
		Scalar out(g);
		for (typename Grid::Ijk ijk = g->begin_ijk(); !ijk.is_end(); ++ijk)
			out(ijk.current()) = s.f(VF, *a, ijk.current());
		put_field(s.nm, out);
	}
	{
		Scalar out(g);
		for (typename Grid::Ijk ijk = g->begin_ijk(); !ijk.is_end(); ++ijk)
			out(ijk.current()) = Op::NablaMuNabla(0.37, *a, ijk.current());
		put_field("diffusion", out);
	}
	{
		// NablaMuNabla with a mu field (s_operation.hpp:630-662), mu > 0
		spScalar mu(new Scalar(g));
		for (int I = 0; I < g->N(0); ++I)
			for (int J = 0; J < g->N(1); ++J) mu->VAL(I, J) = 1.5 + U(rng);
		put_field("in_mu", *mu);
		Scalar out(g);
		for (typename Grid::Ijk ijk = g->begin_ijk(); !ijk.is_end(); ++ijk)
			out(ijk.current()) = Op::NablaMuNabla(*mu, *a, ijk.current());
		put_field("diffusion_var", out);
	}
	// ghost fill (Equation_::apply_bc) for Dirichlet and Neumann segments
	{
		EqProbe_ eq(g);
		double vals[4] = { 0.5, -2.0, 1.5, 0.25 };
		int types[4] = { 1, 2, 2, 1 };
		for (int d = 0; d < 4; ++d) {
			Equation_<2>::spBC bc(new Equation_<2>::BC());
			if (types[d] == 1) bc->set_default_1_bc(vals[d]);
			else bc->set_default_2_bc(vals[d]);
			eq.add_bc(0, d, "f", bc);
		}
		spScalar f(new Scalar(*b));
		eq.put("f", f);
		eq.apply_bc("f");
		put_field("bc_filled", *f);
	}
	return 0;
}

// ---------------------------------------------------------- advect cmd ---
static int cmd_advect(int argc, char** argv) {
	if (argc < 8) return 2;
	int n = std::atoi(argv[2]);
	int steps = std::atoi(argv[3]);
	std::string scheme = argv[4];
	double dt = std::atof(argv[5]);
	std::string cs = argv[6];
	out_open(argv[argc - 1]);
	const bool stretch = stretch_arg(argc, argv, 7);
	spGrid g = make_grid(n, n, 2, stretch);
	put_grid(*g);
	typedef Advection_<2> Eq;
	Eq eq(g);
	eq.set_time(steps - 1, dt);
	Eq::Function fu, fv, fphi;
	if (cs == "band") {
		fu = [](Vt, Vt, Vt, Vt) { return 1.0; };
		fv = [](Vt, Vt, Vt, Vt) { return 1.0; };
		fphi = [](Vt, Vt, Vt, Vt) { return 0.0; };
		Eq::Function fbc = [](Vt, Vt, Vt y, Vt) {
			return (y >= 0.0 && y <= 0.3) ? 1.0 : 0.0;
		};
		Eq::spBC bc0(new Eq::BC()), bc1(new Eq::BC());
		bc0->set_default_1_bc(0);
		bc1->set_default_1_bc(fbc);
		eq.add_bc(0, 0, "phi", bc1);
		for (int k = 1; k < 4; ++k) eq.add_bc(0, k, "phi", bc0);
	} else if (cs == "rotate") {
		fu = [](Vt, Vt, Vt y, Vt) { return -(y - 0.5); };
		fv = [](Vt, Vt x, Vt, Vt) { return x - 0.5; };
		fphi = [](Vt, Vt x, Vt y, Vt) {
			Vt dx = x - 0.5, dy = y - 0.75;
			Vt r2 = dx * dx + dy * dy;
			return r2 < 0.04 ? 1.0 - r2 / 0.04 : 0.0;
		};
	} else {
		return 2;
	}
	eq.initial_CS("u", fu);
	eq.initial_CS("v", fv);
	eq.initial_CS("phi", fphi);
	// the initial fields as set_CS writes them (s_equation.hpp:266-279)
	const char* nm[3] = { "in_u", "in_v", "in_phi" };
	Eq::Function* fn[3] = { &fu, &fv, &fphi };
	for (int k = 0; k < 3; ++k) {
		Scalar f(g);
		for (int I = 0; I < g->N(0); ++I)
			for (int J = 0; J < g->N(1); ++J)
				f.VAL(I, J) = (*fn[k])(0.0, g->C_(0, I), g->C_(1, J), 0.0);
		put_field(nm[k], f);
	}
	eq.set_advection_scheme(scheme);
	eq.run();
	put_field("phi", *eq.get_CS("phi"));
	put_field("u", *eq.get_CS("u"));
	put_field("v", *eq.get_CS("v"));
	put_field("uf", *eq.get_CS("uf"));
	put_field("vf", *eq.get_CS("vf"));
	return 0;
}

int main(int argc, char** argv) {
	if (argc < 2) {
		std::fprintf(stderr, "usage: ref_harness csr|poisson|cavity|ops ...\n");
		return 2;
	}
	std::string c = argv[1];
	int rc = 2;
	if (c == "csr") rc = cmd_csr(argc, argv);
	else if (c == "poisson") rc = cmd_poisson(argc, argv);
	else if (c == "cavity") rc = cmd_cavity(argc, argv);
	else if (c == "ops") rc = cmd_ops(argc, argv);
	else if (c == "kim") rc = cmd_kim(argc, argv);
	else if (c == "advect") rc = cmd_advect(argc, argv);
	if (rc == 2) std::fprintf(stderr, "bad arguments for %s\n", c.c_str());
	g_meta.close();
	return rc;
}
