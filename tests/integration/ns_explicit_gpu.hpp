// NS_explicit_GPU_: the reference-side binding of the whole projection step.
// A maintainer of hyperpower/carpios adds this class next to NS_explicit_
// (lib/structure/s_ns_explicit.hpp:16-229) and keeps Equation_::run's event
// loop (s_equation.hpp:132-178): initial() builds the GPU handles from the
// reference's own grid, time and boundary conditions, run_one_step() is one
// carpio_gpu_ns_run step (restrict_time, predictor, projection, correction
// on the GPU) that hands the new dt back to the reference's Time_, and
// fields() copies the state back into the Scalar_ arrays for the output
// events. Compiled against the reference's headers.
#ifndef CARPIO_NS_EXPLICIT_GPU_HPP
#define CARPIO_NS_EXPLICIT_GPU_HPP

#include "structure/s_ns_explicit.hpp"
#include "carpio_gpu.h"

#include <stdexcept>
#include <string>

template<structure::St DIM>
class NS_explicit_GPU_: public structure::NS_explicit_<DIM> {
public:
	typedef structure::NS_explicit_<DIM> Base;
	typedef typename Base::spGrid spGrid;
	NS_explicit_GPU_(spGrid g, const double box[4], const carpio_gpu_ns_cfg& cfg)
		: Base(g), cfg_(cfg) {
		for (int k = 0; k < 4; ++k) box_[k] = box[k];
	}
	~NS_explicit_GPU_() {
		if (ns_) carpio_gpu_ns_destroy(ns_);
		if (g_) carpio_gpu_grid_destroy(g_);
	}
	int initial() {
		Base::initial();
		const auto& gr = *this->_grid;
		const int nx = (int)gr.n(0), ny = (int)gr.n(1);
		const int gl = (int)(gr.N(0) - gr.n(0)) / 2;
		check(carpio_gpu_grid_create_uniform(nx, ny, gl, box_[0], box_[1], box_[2],
				box_[3], &g_));
		check(carpio_gpu_ns_create(g_, &cfg_, this->_time->dt(), &ns_));
		return 1;
	}
	int run_one_step(structure::St) {
		double dt = 0.0;
		int its = 0;
		const int rc = carpio_gpu_ns_run(ns_, 1, &dt, &its, nullptr);
		if (rc < 0) check(rc);
		code = rc;
		iters = its;
		this->_time->set_dt(dt);   // restrict_time happened on the GPU
		return -1;
	}
	// the state into the Scalar_ arrays ("u", "v", "phi", "p" cell fields and
	// the face fields "uf", "vf"), SpaceT layout on both sides
	void fields(double* u, double* v, double* uf, double* vf, double* phi, double* p) {
		double dt;
		check(carpio_gpu_ns_get_state(ns_, &dt, u, v, uf, vf, phi, p));
	}
	int code = 0, iters = 0;
private:
	static void check(int rc) {
		if (rc < 0) throw std::runtime_error(std::string("carpio_gpu: ") + carpio_gpu_strerror(rc));
	}
	carpio_gpu_grid* g_ = nullptr;
	carpio_gpu_ns* ns_ = nullptr;
	carpio_gpu_ns_cfg cfg_;
	double box_[4];
};

#endif
