// The C++ binding (include/carpio_gpu.hpp) and the call sequence of the
// NS_explicit_GPU_ binding, run on a GPU without the reference's headers
// (the machine with the GPU does not have them): minimal stand-ins for
// MatrixSCR_ and ArrayListV with the accessors the templates use.
//
//   binding_gpu csr <dir> <cg|bicgstab>
//                           reads rowptr/colind/val/b (raw little-endian
//                           u32/u32/f64/f64 files) and writes x of
//                           carpio_gpu::CG or carpio_gpu::BiCGSTAB
//   binding_gpu ns <file>   runs the 32 x 32 cavity 20 steps through the
//                           calls NS_explicit_GPU_ makes and writes u, v, p
#include "carpio_gpu.hpp"

#include <cstdio>
#include <cstring>
#include <list>
#include <string>
#include <vector>

// MatrixSCR_'s accessors (lib/algebra/matrix_SparCompRow.hpp)
struct Csr {
	std::vector<uint32_t> rp, ci;
	std::vector<double> va;
	size_t iLen() const { return rp.size() - 1; }
	size_t NumNonzeros() const { return va.size(); }
	uint32_t row_ptr(size_t i) const { return rp[i]; }
	uint32_t col_ind(size_t k) const { return ci[k]; }
	double val(size_t k) const { return va[k]; }
};
// ArrayListV's size() and operator[] (lib/algebra/array_list.hpp)
struct Arr {
	std::vector<double> v;
	size_t size() const { return v.size(); }
	double& operator[](size_t i) { return v[i]; }
	const double& operator[](size_t i) const { return v[i]; }
};

template<class T>
static bool read_all(const std::string& f, std::vector<T>& out) {
	FILE* fp = std::fopen(f.c_str(), "rb");
	if (!fp) return false;
	std::fseek(fp, 0, SEEK_END);
	const long bytes = std::ftell(fp);
	std::fseek(fp, 0, SEEK_SET);
	out.resize(bytes / sizeof(T));
	const size_t got = std::fread(out.data(), sizeof(T), out.size(), fp);
	std::fclose(fp);
	return got == out.size();
}

static int cmd_csr(const std::string& dir, const std::string& kind) {
	Csr A;
	Arr b;
	if (!read_all(dir + "/rowptr", A.rp) || !read_all(dir + "/colind", A.ci)
			|| !read_all(dir + "/val", A.va) || !read_all(dir + "/b", b.v))
		return 2;
	Arr x;
	x.v.assign(b.size(), 0.0);
	int max_iter = 20000;
	double tol = 1e-13;
	std::list<double> lr;
	const int code = kind == "cg" ? carpio_gpu::CG(A, x, b, max_iter, tol, lr)
	                              : carpio_gpu::BiCGSTAB(A, x, b, max_iter, tol, lr);
	std::printf("%s code %d iters %d resid %.3e hist %zu\n", kind.c_str(), code, max_iter,
			tol, lr.size());
	FILE* fp = std::fopen((dir + "/x_" + kind).c_str(), "wb");
	if (!fp) return 2;
	std::fwrite(x.v.data(), sizeof(double), x.size(), fp);
	std::fclose(fp);
	return code;
}

static int cmd_ns(const std::string& file) {
	const int n = 32, steps = 20, gl = 2;
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
	// NS_explicit_GPU_::initial()
	carpio_gpu_grid* g = nullptr;
	carpio_gpu_ns* ns = nullptr;
	if (carpio_gpu_grid_create_uniform(n, n, gl, 0.0, 1.0, 0.0, 1.0, &g)) return 2;
	if (carpio_gpu_ns_create(g, &cfg, 0.5 / n, &ns)) return 2;
	// Equation_::run: max_step + 1 calls of run_one_step
	int worst = 0;
	for (int s = 0; s < steps; ++s) {
		double dt = 0.0;
		int its = 0;
		const int rc = carpio_gpu_ns_run(ns, 1, &dt, &its, nullptr);
		if (rc < 0) return 3;
		if (rc > worst) worst = rc;
	}
	const size_t N = (size_t)(n + 2 * gl) * (n + 2 * gl);
	std::vector<double> u(N), v(N), uf(N), vf(N), phi(N), p(N);
	double dt;
	if (carpio_gpu_ns_get_state(ns, &dt, u.data(), v.data(), uf.data(), vf.data(),
			phi.data(), p.data()))
		return 3;
	carpio_gpu_ns_destroy(ns);
	carpio_gpu_grid_destroy(g);
	FILE* fp = std::fopen(file.c_str(), "wb");
	if (!fp) return 2;
	std::fwrite(u.data(), sizeof(double), N, fp);
	std::fwrite(v.data(), sizeof(double), N, fp);
	std::fwrite(p.data(), sizeof(double), N, fp);
	std::fclose(fp);
	std::printf("ns code %d\n", worst);
	return worst;
}

int main(int argc, char** argv) {
	if (argc < 3) return 2;
	if (carpio_gpu_device_count() < 1) {
		std::printf("linked; no CUDA device\n");
		return 0;
	}
	try {
		if (!std::strcmp(argv[1], "csr") && argc > 3) return cmd_csr(argv[2], argv[3]);
		if (!std::strcmp(argv[1], "ns")) return cmd_ns(argv[2]);
	} catch (const carpio_gpu::Error& e) {
		std::printf("%s\n", e.what());
		return 4;
	}
	return 2;
}
