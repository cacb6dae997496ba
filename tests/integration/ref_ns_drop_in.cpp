// The reference-side NS binding (ns_explicit_gpu.hpp) on the reference's own
// classes: a 32 x 32 lid-driven cavity (Re 1000, van Leer, CG projection to
// 1e-10 with mean removal) set up exactly as the reference's examples set
// one up, then Equation_::run for 20 steps with the GPU doing each step.
// Compiled against the reference's headers by tests/test_integration.py;
// with a device it writes u, v, p (SpaceT arrays, doubles) to argv[1].
#include "structure/s_grid.hpp"
#include "ns_explicit_gpu.hpp"

#include <cstdio>
#include <memory>
#include <vector>

using namespace structure;

int main(int argc, char** argv) {
	const int n = 32, steps = 20;
	Poi_<2> pmin(0.0, 0.0), pmax(1.0, 1.0);
	Index_<2> mn(n, n);
	std::shared_ptr<Grid_<2> > g(new Grid_<2>(pmin, pmax, mn, 2));
	carpio_gpu_ns_cfg cfg = {};
	cfg.rho = 1000.0;
	cfg.mu = 1.0;
	cfg.cfl = 0.5;
	cfg.diff_number = 0.25;
	cfg.diff_coef = 1.0 / 1000.0;
	cfg.scheme = CARPIO_GPU_VANLEER;
	for (int s = 0; s < 4; ++s) {
		cfg.bc_u.type[s] = 1;
		cfg.bc_u.value[s] = s == 3 ? 1.0 : 0.0;
		cfg.bc_v.type[s] = 1;
		cfg.bc_v.value[s] = 0.0;
	}
	cfg.projection.kind = CARPIO_GPU_CG;
	cfg.projection.precision = CARPIO_GPU_FP64;
	cfg.projection.max_iter = 100000;
	cfg.projection.tol = 1e-10;
	cfg.projection.mean_removal = 1;
	const double box[4] = { 0.0, 1.0, 0.0, 1.0 };
	NS_explicit_GPU_<2> ns(g, box, cfg);
	// the reference's own set-up calls, as its cavity example makes them
	// (its initial() builds the fields and the projection from them)
	ns.set_advection_scheme("VanLeer");
	ns.set_time(steps - 1, 0.5 / n);   // Time_ runs max_step + 1 steps
	NS_<2>::spBC bc0(new NS_<2>::BC()), bc1(new NS_<2>::BC());
	bc0->set_default_1_bc(0);
	bc1->set_default_1_bc(1);
	for (int s = 0; s < 3; ++s) ns.add_bc(0, s, "u", bc0);
	ns.add_bc(0, 3, "u", bc1);
	for (int s = 0; s < 4; ++s) ns.add_bc(0, s, "v", bc0);
	ns.set_uniform_rho(1000.0);
	ns.set_diffusion_number(0.25, 1.0 / 1000.0);
	if (carpio_gpu_device_count() < 1) {
		std::printf("linked; no CUDA device\n");
		return 0;
	}
	ns.run();
	const size_t N = (size_t)(n + 4) * (n + 4);
	std::vector<double> u(N), v(N), uf(N), vf(N), phi(N), p(N);
	ns.fields(u.data(), v.data(), uf.data(), vf.data(), phi.data(), p.data());
	if (argc > 1) {
		FILE* f = std::fopen(argv[1], "wb");
		if (!f) return 2;
		std::fwrite(u.data(), sizeof(double), N, f);
		std::fwrite(v.data(), sizeof(double), N, f);
		std::fwrite(p.data(), sizeof(double), N, f);
		std::fclose(f);
	}
	std::printf("code %d iters %d\n", ns.code, ns.iters);
	return ns.code == 0 ? 0 : 1;
}
