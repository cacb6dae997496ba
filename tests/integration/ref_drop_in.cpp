// The reference-side binding a maintainer of hyperpower/carpios adds to use
// the GPU solver: a structure::Solver_<2> subclass (the seam of
// lib/structure/s_solver.hpp:205-207) that keeps the reference's own
// assembly (_build_exp/_build_matrix, s_solver.hpp:94-171) and hands the CSR
// to carpio_gpu::CG instead of carpio::CG. Compiled against the reference's
// headers by tests/test_integration.py; on a machine without a GPU it stops
// after the library reports that no device is present.
#include "structure/s_grid.hpp"
#include "structure/s_poisson.hpp"
#include "carpio_gpu.hpp"

#include <cstdio>
#include <memory>

using namespace structure;

class Solver_GPU_CG_: public structure::Solver_<2> {
public:
	Solver_GPU_CG_(spGrid g, spGhost gh, spStencil st, const std::string& vn,
			spCenterScalar cs)
		: structure::Solver_<2>(g, gh, st, vn, cs) {}
	int code = -100, iters = 0;
	double resid = 0;
	void solve() {
		this->_build_exp();
		Mat mat;
		Arr b;
		this->_build_matrix(mat, b);
		Arr x = this->_copy_to_x();
		iters = this->_max_iter;
		resid = this->_tol;
		std::list<Vt> lr;
		code = carpio_gpu::CG(mat, x, b, iters, resid, lr);   // was carpio::CG
		this->_copy_to_cs(x);
	}
};

class PoissonGPU_: public Poisson_<2> {
public:
	explicit PoissonGPU_(spGrid g) : Poisson_<2>(g) {}
	std::shared_ptr<Solver_GPU_CG_> solver;
	int initial() {
		Poisson_<2>::initial();
		solver.reset(new Solver_GPU_CG_(this->_grid, this->_ghost,
				this->_stencils["poisson"], "phi", this->_css["phi"]));
		solver->set_max_iter(1000);
		solver->set_tolerance(1e-10);
		this->_solvers["main"] = solver;
		return -1;
	}
};

int main() {
	if (carpio_gpu_device_count() < 1) {
		std::printf("linked; no CUDA device\n");
		return 0;
	}
	Poi_<2> pmin(0.0, 0.0), pmax(1.0, 1.0);
	Index_<2> mn(32, 32);
	std::shared_ptr<Grid_<2> > g(new Grid_<2>(pmin, pmax, mn, 2));
	PoissonGPU_ P(g);
	for (int s = 0; s < 4; ++s) {
		Poisson_<2>::spBC bc(new Poisson_<2>::BC());
		bc->set_default_1_bc(0.0);
		P.add_bc(0, s, "phi", bc);
	}
	P.set_source([](Vt, Vt x, Vt y, Vt) {
		return -2.0 * carpio::PI * carpio::PI * std::sin(carpio::PI * x)
				* std::sin(carpio::PI * y);
	});
	P.run();
	std::printf("code %d iters %d resid %.3e\n", P.solver->code, P.solver->iters,
			P.solver->resid);
	return P.solver->code == 0 ? 0 : 1;
}
