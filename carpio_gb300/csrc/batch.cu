// Host side of the batched structure-level Poisson solves (device side in
// batch_dev.cuh): the planner, the launch configuration and its autotuner,
// the CUDA graph and the C ABI.
#include "batch_dev.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <queue>
#include <string>
#include <vector>

namespace cg_batch {
// k_batch<T> instantiated in its own translation unit per block size
const void* kernel_256();
const void* kernel_512();
// the one-CTA-per-problem multigrid kernel (batch_mg.cu)
const void* kernel_mg(int T);
long long mg_scratch_floats(int nx, int ny);
}  // namespace cg_batch

namespace {

using namespace cg_dev;
using namespace cg_batch;

// ------------------------------------------------------------------ planner --
// Cost model of one problem on a team (microseconds): iterations times the
// latency of the two team reductions plus the band's per-thread work. The
// iteration counts are those the on-chip solver needs to 1e-8 on these grids
// (about 4.9 N all-Neumann, 2.9 N Dirichlet).
constexpr double kLatOne = 0.7, kLatTeam = 2.0, kPerCell = 0.085;

int iters_estimate(const carpio_gpu_batch_problem& p) {
	const int n = std::max(p.nx, p.ny);
	bool neumann = true;
	for (int k = 0; k < 4; ++k) neumann = neumann && p.bc.type[k] == 2;
	return (int)((neumann ? 4.9 : 2.9) * n) + 10;
}

int rows_max(int nx, int t) { return (nx + t - 1) / t; }

// a row of ny cells padded to whole quads of 4
int row4(int ny) { return (ny + 3) / 4 * 4; }

// p with halo rows and a pad quad per row, the FP32 iterate, r's edge rows,
// one scratch quad per thread
size_t smem_bytes(int nx, int ny, int t, int T) {
	const size_t rm = (size_t)rows_max(nx, t), n4 = (size_t)row4(ny);
	return sizeof(float) * ((rm + 2) * (n4 + 4) + rm * n4 + 2 * n4 + 4 * (size_t)T);
}

// dynamic shared memory at most (the kernel's static arrays take the rest of
// the 227 KB a CTA may have)
constexpr size_t kSmemLimit = 220 * 1024;

struct Plan {
	carpio_gpu_batch_tiles tiles{};
	int clusters = 0;
	std::vector<int> team, kc;
	std::vector<int> cl_team, slot_ptr, slot_list, slot_of;
	size_t smem = 0;
	double est_ms = 0;
	int teams[5] = { 0, 0, 0, 0, 0 };
};

double cost_us(const carpio_gpu_batch_problem& p, int t, int T) {
	const double cells = (double)rows_max(p.nx, t) * row4(p.ny);
	const double per_thread = std::ceil(cells / T);
	return iters_estimate(p) * ((t == 1 ? kLatOne : kLatTeam) + kPerCell * per_thread);
}

int log2i(int t) { int l = 0; while ((1 << l) < t) ++l; return l; }

// LPT of `idx` (by cost) over `slots` slots; returns the makespan and, if
// asked, each problem's slot
double lpt(const std::vector<int>& idx, const std::vector<double>& cost, int slots,
		std::vector<int>* slot_of) {
	std::vector<int> order(idx);
	std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
	using E = std::pair<double, int>;
	std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
	for (int s = 0; s < slots; ++s) pq.push({ 0.0, s });
	double span = 0;
	for (int i : order) {
		E e = pq.top();
		pq.pop();
		e.first += cost[i];
		span = std::max(span, e.first);
		if (slot_of) (*slot_of)[i] = e.second;
		pq.push(e);
	}
	return span;
}

int make_plan(const std::vector<carpio_gpu_batch_problem>& P,
		const carpio_gpu_batch_tiles& tiles, int clusters, Plan& out) {
	const int n = (int)P.size(), T = tiles.threads, S = tiles.cluster;
	const int hard = std::min(kCellsPerCta, kMaxQ * 4 * T);   // cells one CTA can hold
	const int cap = std::min(tiles.cells_per_cta, hard);
	if (clusters < 1 || (T != 256 && T != 512) || cap < 1
			|| (S != 1 && S != 2 && S != 4 && S != 8 && S != 16))
		return CARPIO_GPU_EINVAL;
	out = Plan();
	out.tiles = tiles;
	out.clusters = clusters;
	out.team.assign(n, 1);
	out.kc.assign(n, 1);
	// smallest team that meets the target, then the smallest that fits at all
	for (int i = 0; i < n; ++i) {
		const auto& p = P[i];
		auto fits = [&](int t, int c) {
			return t <= p.nx && (long)rows_max(p.nx, t) * row4(p.ny) <= c
				&& smem_bytes(p.nx, p.ny, t, T) <= kSmemLimit;
		};
		int t = 1;
		while (t < S && t * 2 <= p.nx && !fits(t, cap)) t *= 2;
		if (!fits(t, hard)) return CARPIO_GPU_EINVAL;
		out.team[i] = t;
	}
	// groups by team size; too many groups for the clusters: promote the
	// smallest into the next size up
	std::vector<std::vector<int>> grp(5);
	for (int i = 0; i < n; ++i) grp[log2i(out.team[i])].push_back(i);
	auto ngroups = [&]() { int c = 0; for (auto& g : grp) c += !g.empty(); return c; };
	while (ngroups() > clusters) {
		int l = 0;
		while (grp[l].empty()) ++l;
		int u = l + 1;
		while (u < 5 && grp[u].empty()) ++u;
		if (u >= 5 || (1 << u) > S) return CARPIO_GPU_EINVAL;
		for (int i : grp[l]) {
			if (P[i].nx < (1 << u)) return CARPIO_GPU_EINVAL;   // a band per member
			out.team[i] = 1 << u;
		}
		grp[u].insert(grp[u].end(), grp[l].begin(), grp[l].end());
		grp[l].clear();
	}
	std::vector<double> cost(n);
	for (int i = 0; i < n; ++i) cost[i] = cost_us(P[i], out.team[i], T);
	// clusters per group: one each, the rest to the group with the longest
	// makespan
	std::vector<int> ncl(5, 0);
	for (int l = 0; l < 5; ++l) ncl[l] = grp[l].empty() ? 0 : 1;
	auto span_of = [&](int l) {
		return grp[l].empty() ? 0.0 : lpt(grp[l], cost, ncl[l] * (S >> l), nullptr);
	};
	std::vector<double> span(5);
	for (int l = 0; l < 5; ++l) span[l] = span_of(l);
	for (int c = ngroups(); c < clusters; ++c) {
		int best = -1;
		for (int l = 0; l < 5; ++l)
			if (!grp[l].empty() && (best < 0 || span[l] > span[best])) best = l;
		++ncl[best];
		span[best] = span_of(best);
	}
	// slot lists
	out.cl_team.assign(clusters, 1);
	out.slot_of.assign(n, 0);
	std::vector<std::vector<int>> lists((size_t)clusters * kMaxTeam);
	int c0 = 0;
	out.est_ms = 0;
	for (int l = 0; l < 5; ++l) {
		if (grp[l].empty()) continue;
		const int t = 1 << l, per = S / t;
		std::vector<int> so(n, 0);
		out.est_ms = std::max(out.est_ms, 1e-3 * lpt(grp[l], cost, ncl[l] * per, &so));
		for (int c = c0; c < c0 + ncl[l]; ++c) out.cl_team[c] = t;
		for (int i : grp[l]) {
			const int c = c0 + so[i] / per, s = so[i] % per;
			out.slot_of[i] = c * kMaxTeam + s;
		}
		c0 += ncl[l];
	}
	// clusters left without a group (more clusters than the LPT wanted)
	// run team size 1 and stay idle
	std::vector<int> order(n);
	for (int i = 0; i < n; ++i) order[i] = i;
	std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
	for (int i : order) lists[out.slot_of[i]].push_back(i);
	out.slot_ptr.assign((size_t)clusters * kMaxTeam + 1, 0);
	for (size_t s = 0; s < lists.size(); ++s) {
		out.slot_ptr[s + 1] = out.slot_ptr[s] + (int)lists[s].size();
		out.slot_list.insert(out.slot_list.end(), lists[s].begin(), lists[s].end());
	}
	out.smem = 0;
	for (int i = 0; i < n; ++i) {
		const auto& p = P[i];
		const int t = out.team[i];
		out.smem = std::max(out.smem, smem_bytes(p.nx, p.ny, t, T));
		const long quads = (long)rows_max(p.nx, t) * (row4(p.ny) / 4);
		int k = 1;
		while ((long)k * T < quads) k *= 2;
		out.kc[i] = k;
		out.teams[log2i(t)]++;
	}
	return 0;
}

// FP32 diagonal of a uniform problem as an interior value plus what each
// side's ghost fold adds. The folds depend on the cell size and the boundary
// condition only, so they are read off the FP64 coefficients of a grid with
// the same cells and at least three cells per axis.
void diag_consts(const carpio_gpu_batch_problem& p, float out[5]) {
	const int nx3 = std::max(p.nx, 3), ny3 = std::max(p.ny, 3);
	const double hx = (p.xmax - p.xmin) / p.nx, hy = (p.ymax - p.ymin) / p.ny;
	std::vector<double> cx, sx, cy, sy, D, ax, ay, fold;
	cg_host::uniform_axis(nx3, 1, p.xmin, p.xmin + hx * nx3, cx, sx);
	cg_host::uniform_axis(ny3, 1, p.ymin, p.ymin + hy * ny3, cy, sy);
	cg_host::stencil_host(nx3, ny3, 1, ny3 + 2, cx, sx, cy, sy, p.bc, p.beta, D,
			ax, ay, fold);
	auto d = [&](int i, int j) { return D[(size_t)(i + 1) * (ny3 + 2) + j + 1]; };
	const double base = d(1, 1);
	out[0] = (float)base;
	out[1] = (float)(d(0, 1) - base);
	out[2] = (float)(d(nx3 - 1, 1) - base);
	out[3] = (float)(d(1, 0) - base);
	out[4] = (float)(d(1, ny3 - 1) - base);
}

bool valid_problem(const carpio_gpu_batch_problem& p) {
	if (p.nx < 1 || p.ny < 1 || !(p.xmax > p.xmin) || !(p.ymax > p.ymin)
			|| !std::isfinite(p.beta) || p.beta == 0.0)
		return false;
	for (int k = 0; k < 4; ++k)
		if ((p.bc.type[k] != 1 && p.bc.type[k] != 2) || !std::isfinite(p.bc.value[k]))
			return false;
	return true;
}

const void* batch_kernel(int T) {
	if (T == 256) return cg_batch::kernel_256();
	if (T == 512) return cg_batch::kernel_512();
	return nullptr;
}

// autotuned configurations by batch signature
std::mutex& tune_mu() { static std::mutex* m = new std::mutex(); return *m; }
std::map<std::string, carpio_gpu_batch_tiles>& tune_cache() {
	static auto* c = new std::map<std::string, carpio_gpu_batch_tiles>();
	return *c;
}

}  // namespace

struct carpio_gpu_batch {
	int count = 0;
	std::vector<carpio_gpu_batch_problem> probs;
	carpio_gpu_solver_cfg cfg{};
	std::string signature;
	std::vector<long long> off;         // field offset of each problem
	long long cells = 0;                // field arena length (doubles)
	cg_host::DevBuf src, phi, b, r, D, ax, ay, sx, sy, fold, save;
	cg_host::DevBuf dprob, dteam, dsptr, dslist, dres, dctl;
	// multigrid kernel: one CTA per problem from a queue (mg), its block
	// size and grid, FP32 scratch with per-problem offsets, the order
	bool mg = false;
	int mg_T = 512, mg_grid = 0;
	cg_host::DevBuf w32, w32off, order, queue;
	std::vector<BatchProb> hprob;
	Plan plan;
	const void* kern = nullptr;
	cudaStream_t s = nullptr;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	BatchRes* hres = nullptr;
	BatchCtl* hctl = nullptr;
	carpio_gpu_batch_info info{};
	std::mutex mu;
	~carpio_gpu_batch() {
		if (s) cudaStreamSynchronize(s);
		if (exec) cudaGraphExecDestroy(exec);
		if (graph) cudaGraphDestroy(graph);
		if (e0) cudaEventDestroy(e0);
		if (e1) cudaEventDestroy(e1);
		if (hres) cudaFreeHost(hres);
		if (hctl) cudaFreeHost(hctl);
		if (s) cudaStreamDestroy(s);
	}
};

namespace {

using cg_host::note_cuda_error;

int max_clusters(const void* kern, int T, int S, size_t smem, int* out) {
	CG_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	if (S > 8) CG_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
	cudaLaunchConfig_t lc = {};
	lc.gridDim = dim3(S * cg_host::sm_count());
	lc.blockDim = dim3(T);
	lc.dynamicSmemBytes = smem;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = S;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	lc.attrs = at;
	lc.numAttrs = 1;
	int n = 0;
	cudaError_t e = cudaOccupancyMaxActiveClusters(&n, kern, &lc);
	if (e != cudaSuccess) {
		cudaGetLastError();
		n = 0;
	}
	*out = n;
	return 0;
}

int launch_mg(carpio_gpu_batch* b, cudaStream_t s) {
	BatchArgs a;
	std::memset(&a, 0, sizeof a);
	a.prob = b->dprob.as<BatchProb>();
	a.src = b->src.as<double>();
	a.phi = b->phi.as<double>();
	a.b = b->b.as<double>();
	a.r = b->r.as<double>();
	a.D = b->D.as<double>();
	a.ax = b->ax.as<double>();
	a.ay = b->ay.as<double>();
	a.sx = b->sx.as<double>();
	a.sy = b->sy.as<double>();
	a.fold = b->fold.as<double>();
	a.res = b->dres.as<BatchRes>();
	a.ctl = b->dctl.as<BatchCtl>();
	// after a 1e-2 drop of (r, z): with the V-cycle an iteration gains
	// about a digit
	a.inner_tol = b->cfg.inner_tol > 0 ? b->cfg.inner_tol : 1e-2;
	a.queue = b->queue.as<unsigned>();
	a.order = b->order.as<int>();
	a.count = b->count;
	a.w32 = b->w32.as<float>();
	a.w32off = b->w32off.as<long long>();
	CG_CK(cudaMemsetAsync(b->dres.p, 0, sizeof(BatchRes) * b->count, s));
	CG_CK(cudaMemsetAsync(b->queue.p, 0, sizeof(unsigned), s));
	void* args[] = { &a };
	CG_CK(cudaLaunchKernel(b->kern, dim3(b->mg_grid), dim3(b->mg_T), args, 0, s));
	return 0;
}

int launch(carpio_gpu_batch* b, cudaStream_t s) {
	if (b->mg) return launch_mg(b, s);
	const Plan& pl = b->plan;
	const int T = pl.tiles.threads, S = pl.tiles.cluster;
	BatchArgs a;
	a.prob = b->dprob.as<BatchProb>();
	a.cl_team = b->dteam.as<int>();
	a.slot_ptr = b->dsptr.as<int>();
	a.slot_list = b->dslist.as<int>();
	a.src = b->src.as<double>();
	a.phi = b->phi.as<double>();
	a.b = b->b.as<double>();
	a.r = b->r.as<double>();
	a.D = b->D.as<double>();
	a.ax = b->ax.as<double>();
	a.ay = b->ay.as<double>();
	a.sx = b->sx.as<double>();
	a.sy = b->sy.as<double>();
	a.fold = b->fold.as<double>();
	a.res = b->dres.as<BatchRes>();
	a.ctl = b->dctl.as<BatchCtl>();
	a.inner_tol = b->cfg.inner_tol > 0 ? b->cfg.inner_tol : 3e-2;
	CG_CK(cudaMemsetAsync(b->dres.p, 0, sizeof(BatchRes) * b->count, s));
	cudaLaunchConfig_t lc = {};
	lc.gridDim = dim3(pl.clusters * S);
	lc.blockDim = dim3(T);
	lc.dynamicSmemBytes = pl.smem;
	lc.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeClusterDimension;
	at[0].val.clusterDim.x = S;
	at[0].val.clusterDim.y = 1;
	at[0].val.clusterDim.z = 1;
	lc.attrs = at;
	lc.numAttrs = 1;
	void* args[] = { &a };
	CG_CK(cudaLaunchKernelExC(&lc, b->kern, args));
	return 0;
}

// plan for `tiles`, upload it, capture the graph
int configure(carpio_gpu_batch* b, const carpio_gpu_batch_tiles& tiles) {
	using namespace cg_host;
	const void* kern = batch_kernel(tiles.threads);
	if (!kern) return CARPIO_GPU_EINVAL;
	// shared memory is sized by the plan, the plan by the cluster count: plan
	// once with a cluster per team size (no team is enlarged, so the largest
	// shared memory), then with the real count
	Plan probe;
	int rc;
	if ((rc = make_plan(b->probs, tiles, 5, probe))) return rc;
	int clusters = 0;
	if ((rc = max_clusters(kern, tiles.threads, tiles.cluster, probe.smem, &clusters))) return rc;
	if (clusters < 1) return CARPIO_GPU_EINVAL;
	Plan pl;
	if ((rc = make_plan(b->probs, tiles, clusters, pl))) return rc;
	if (pl.smem > probe.smem) return CARPIO_GPU_EINVAL;
	pl.smem = probe.smem;
	cudaStream_t s = b->s;
	CG_CK(cudaStreamSynchronize(s));
	for (int i = 0; i < b->count; ++i) {
		b->hprob[i].team = pl.team[i];
		b->hprob[i].kc = pl.kc[i];
	}
	if ((rc = to_device(b->dprob, b->hprob.data(), sizeof(BatchProb) * b->count, s))) return rc;
	if ((rc = to_device(b->dteam, pl.cl_team.data(), sizeof(int) * pl.cl_team.size(), s))) return rc;
	if ((rc = to_device(b->dsptr, pl.slot_ptr.data(), sizeof(int) * pl.slot_ptr.size(), s))) return rc;
	if ((rc = to_device(b->dslist, pl.slot_list.data(), sizeof(int) * pl.slot_list.size(), s))) return rc;
	CG_CK(cudaStreamSynchronize(s));
	b->plan = pl;
	b->kern = kern;
	if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
	if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
	if (tiles.use_graph >= 0) {
		CG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		rc = launch(b, s);
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamEndCapture(s, &g);
		if (rc) { if (g) cudaGraphDestroy(g); return rc; }
		if (e != cudaSuccess) { note_cuda_error(e); return CARPIO_GPU_ECUDA; }
		b->graph = g;
		CG_CK(cudaGraphInstantiate(&b->exec, g, 0));
	}
	carpio_gpu_batch_info& in = b->info;
	in.tiles = tiles;
	in.clusters = pl.clusters;
	in.ctas = pl.clusters * tiles.cluster;
	in.smem_bytes = (int)pl.smem;
	for (int k = 0; k < 5; ++k) in.teams[k] = pl.teams[k];
	in.est_ms = pl.est_ms;
	return 0;
}

// the multigrid kernel with T threads per CTA: as many CTAs as fit (at
// most four per SM, at most one per problem), the graph captured
int configure_mg(carpio_gpu_batch* b, int T, int use_graph) {
	using namespace cg_host;
	const void* kern = cg_batch::kernel_mg(T);
	if (!kern) return CARPIO_GPU_EINVAL;
	int per_sm = 0;
	CG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, 0));
	if (per_sm < 1) return CARPIO_GPU_EINVAL;
	per_sm = std::min(per_sm, 4);
	b->kern = kern;
	b->mg = true;
	b->mg_T = T;
	b->mg_grid = std::max(1, std::min(per_sm * sm_count(), b->count));
	cudaStream_t s = b->s;
	CG_CK(cudaStreamSynchronize(s));
	if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
	if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
	if (use_graph >= 0) {
		CG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		int rc = launch(b, s);
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamEndCapture(s, &g);
		if (rc) { if (g) cudaGraphDestroy(g); return rc; }
		if (e != cudaSuccess) { note_cuda_error(e); return CARPIO_GPU_ECUDA; }
		b->graph = g;
		CG_CK(cudaGraphInstantiate(&b->exec, g, 0));
	}
	carpio_gpu_batch_info& in = b->info;
	in.tiles.threads = T;
	in.tiles.cluster = 1;
	in.tiles.cells_per_cta = 0;
	in.tiles.use_graph = use_graph;
	in.clusters = b->mg_grid;
	in.ctas = b->mg_grid;
	in.smem_bytes = 0;
	for (int k = 0; k < 5; ++k) in.teams[k] = 0;
	in.teams[0] = b->count;
	in.est_ms = 0.0;
	b->plan.tiles = in.tiles;
	b->plan.tiles.cluster = 0;
	return 0;
}

int run_once(carpio_gpu_batch* b, float* ms) {
	cudaStream_t s = b->s;
	const cg_host::Watchdog& wd = cg_host::watchdog();
	b->hctl->err = 0;
	b->hctl->pad = 0;
	b->hctl->wait_ns = (unsigned long long)wd.wait_ms * 1000000ull;
	b->hctl->solve_ns = (unsigned long long)wd.solve_ms * 1000000ull;
	CG_CK(cudaMemcpyAsync(b->dctl.p, b->hctl, sizeof(BatchCtl), cudaMemcpyHostToDevice, s));
	CG_CK(cudaEventRecord(b->e0, s));
	if (b->exec) {
		CG_CK(cudaGraphLaunch(b->exec, s));
	} else {
		int rc = launch(b, s);
		if (rc) return rc;
	}
	CG_CK(cudaEventRecord(b->e1, s));
	CG_CK(cudaMemcpyAsync(b->hres, b->dres.p, sizeof(BatchRes) * b->count,
			cudaMemcpyDeviceToHost, s));
	CG_CK(cudaMemcpyAsync(b->hctl, b->dctl.p, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
	CG_CK(cudaStreamSynchronize(s));
	if (ms) CG_CK(cudaEventElapsedTime(ms, b->e0, b->e1));
	return 0;
}

std::vector<carpio_gpu_batch_tiles> candidates(int max_cells) {
	std::vector<carpio_gpu_batch_tiles> out;
	const int Ts[2] = { 512, 256 };
	const int Ss[3] = { 16, 8, 4 };
	const int Cs[3] = { 16384, 8192, 4096 };
	for (int c : Cs)
		for (int S : Ss)
			for (int T : Ts) {
				if (c > max_cells) continue;
				carpio_gpu_batch_tiles t;
				t.threads = T;
				t.cluster = S;
				t.cells_per_cta = c;
				t.use_graph = 0;
				out.push_back(t);
			}
	return out;
}

std::string signature_of(const std::vector<carpio_gpu_batch_problem>& P,
		const carpio_gpu_solver_cfg& cfg) {
	std::string s = std::to_string(P.size()) + ":" + std::to_string(cfg.tol);
	for (const auto& p : P) {
		s += "|" + std::to_string(p.nx) + "x" + std::to_string(p.ny);
		for (int k = 0; k < 4; ++k) s += (char)('0' + p.bc.type[k]);
		s += p.mean_removal ? "m" : "";
	}
	return s;
}

}  // namespace

// ------------------------------------------------------------------ C ABI --
extern "C" {

int carpio_gpu_batch_plan(int count, const carpio_gpu_batch_problem* probs,
		const carpio_gpu_batch_tiles* tiles, int clusters, int* team, int* slot,
		double* est_ms) {
	if (count < 1 || !probs || !tiles || clusters < 1) return CARPIO_GPU_EINVAL;
	std::vector<carpio_gpu_batch_problem> P(probs, probs + count);
	for (const auto& p : P)
		if (!valid_problem(p)) return CARPIO_GPU_EINVAL;
	Plan pl;
	int rc = make_plan(P, *tiles, clusters, pl);
	if (rc) return rc;
	for (int i = 0; i < count; ++i) {
		if (team) team[i] = pl.team[i];
		if (slot) slot[i] = pl.slot_of[i];
	}
	if (est_ms) *est_ms = pl.est_ms;
	return 0;
}

int carpio_gpu_batch_shard(int count, const carpio_gpu_batch_problem* probs,
		int world, int* rank_of) {
	if (count < 0 || (count > 0 && (!probs || !rank_of)) || world < 1)
		return CARPIO_GPU_EINVAL;
	std::vector<double> work(count);
	std::vector<int> idx(count);
	for (int i = 0; i < count; ++i) {
		if (!valid_problem(probs[i])) return CARPIO_GPU_EINVAL;
		work[i] = (double)probs[i].nx * probs[i].ny * iters_estimate(probs[i]);
		idx[i] = i;
	}
	std::vector<int> so(count, 0);
	lpt(idx, work, world, &so);
	for (int i = 0; i < count; ++i) rank_of[i] = so[i];
	return 0;
}

int carpio_gpu_batch_create(int count, const carpio_gpu_batch_problem* probs,
		const carpio_gpu_solver_cfg* cfg, const carpio_gpu_batch_tiles* tiles,
		carpio_gpu_batch** out) {
	using namespace cg_host;
	if (!out || count < 1 || !probs || !cfg) return CARPIO_GPU_EINVAL;
	*out = nullptr;
	if (cfg->kind != CARPIO_GPU_CG || cfg->precision != CARPIO_GPU_MIXED
			|| cfg->max_iter < 0 || !(cfg->tol >= 0))
		return CARPIO_GPU_EINVAL;
	for (int i = 0; i < count; ++i)
		if (!valid_problem(probs[i])) return CARPIO_GPU_EINVAL;
	carpio_gpu_batch* b = new carpio_gpu_batch();
	auto fail = [&](int code) { delete b; return code; };
	b->count = count;
	b->probs.assign(probs, probs + count);
	b->cfg = *cfg;
	b->signature = signature_of(b->probs, *cfg);
	if (cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking) != cudaSuccess
			|| cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess
			|| cudaMallocHost((void**)&b->hres, sizeof(BatchRes) * count) != cudaSuccess
			|| cudaMallocHost((void**)&b->hctl, sizeof(BatchCtl)) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	// coefficients of every problem, on the host with the reference's
	// formulas (one ghost layer)
	std::vector<double> hD, hax, hay, hsx, hsy, hfold;
	b->hprob.resize(count);
	b->off.resize(count);
	long long cells = 0;
	for (int i = 0; i < count; ++i) {
		const auto& p = probs[i];
		std::vector<double> cx, sx, cy, sy, D, ax, ay, fold;
		uniform_axis(p.nx, 1, p.xmin, p.xmax, cx, sx);
		uniform_axis(p.ny, 1, p.ymin, p.ymax, cy, sy);
		stencil_host(p.nx, p.ny, 1, p.ny + 2, cx, sx, cy, sy, p.bc, p.beta, D, ax, ay, fold);
		BatchProb& q = b->hprob[i];
		std::memset(&q, 0, sizeof q);
		q.nx = p.nx;
		q.ny = p.ny;
		q.mean = p.mean_removal ? 1 : 0;
		q.full = ((cfg->flags & CARPIO_GPU_FLAG_FULL_NRM2) || (long)p.nx * p.ny == 1) ? 1 : 0;
		q.max_iter = cfg->max_iter;
		q.tol = cfg->tol;
		q.cell = cells;
		q.axo = (long long)hax.size();
		q.ayo = (long long)hay.size();
		q.sxo = (long long)hsx.size();
		q.syo = (long long)hsy.size();
		q.foldo = (long long)hfold.size();
		{
			// interior face coefficients: from a grid of at least 3 cells
			// when the problem's own has no interior face
			float dc[5];
			diag_consts(p, dc);
			q.d0 = dc[0];
			q.dw = dc[1];
			q.de = dc[2];
			q.ds = dc[3];
			q.dn = dc[4];
		}
		q.cx = p.nx > 1 ? (float)ax[1] : 0.f;
		q.cy = p.ny > 1 ? (float)ay[1] : 0.f;
		b->off[i] = cells;
		cells += (long long)(p.nx + 2) * (p.ny + 2);
		hD.insert(hD.end(), D.begin(), D.end());
		hax.insert(hax.end(), ax.begin(), ax.end());
		hay.insert(hay.end(), ay.begin(), ay.end());
		hsx.insert(hsx.end(), sx.begin(), sx.end());
		hsy.insert(hsy.end(), sy.begin(), sy.end());
		hfold.insert(hfold.end(), fold.begin(), fold.end());
	}
	b->cells = cells;
	cudaStream_t s = b->s;
	int rc;
	const size_t fb = sizeof(double) * (size_t)cells;
	cg_host::DevBuf* fields[4] = { &b->src, &b->phi, &b->b, &b->r };
	for (auto* f : fields) {
		if ((rc = f->ensure(fb))) return fail(rc);
		if (cudaMemsetAsync(f->p, 0, fb, s) != cudaSuccess) {
			note_cuda_error(cudaGetLastError());
			return fail(CARPIO_GPU_ECUDA);
		}
	}
	if ((rc = to_device(b->D, hD.data(), sizeof(double) * hD.size(), s))) return fail(rc);
	if ((rc = to_device(b->ax, hax.data(), sizeof(double) * hax.size(), s))) return fail(rc);
	if ((rc = to_device(b->ay, hay.data(), sizeof(double) * hay.size(), s))) return fail(rc);
	if ((rc = to_device(b->sx, hsx.data(), sizeof(double) * hsx.size(), s))) return fail(rc);
	if ((rc = to_device(b->sy, hsy.data(), sizeof(double) * hsy.size(), s))) return fail(rc);
	if ((rc = to_device(b->fold, hfold.data(), sizeof(double) * hfold.size(), s))) return fail(rc);
	if ((rc = b->dres.ensure(sizeof(BatchRes) * count))) return fail(rc);
	if ((rc = b->dctl.ensure(sizeof(BatchCtl)))) return fail(rc);
	if (cudaStreamSynchronize(s) != cudaSuccess) {
		note_cuda_error(cudaGetLastError());
		return fail(CARPIO_GPU_ECUDA);
	}
	// configuration: the caller's, else an autotuned one for the same
	// signature, else the first candidate that fits. No cluster size asked
	// for: the multigrid kernel (one CTA per problem); a cluster size: the
	// cluster-team kernel (plain FP32 CG, teams of CTAs)
	carpio_gpu_batch_tiles want{};
	if (tiles) want = *tiles;
	bool explicit_tiles = tiles && tiles->threads && tiles->cluster && tiles->cells_per_cta;
	if (!explicit_tiles) {
		std::lock_guard<std::mutex> lk(tune_mu());
		auto it = tune_cache().find(b->signature);
		if (it != tune_cache().end()) {
			const int ug = want.use_graph;
			want = it->second;
			want.use_graph = ug;
			explicit_tiles = true;
		}
	}
	if (want.cluster == 0) {
		// FP32 scratch of every problem, the problems largest first
		std::vector<long long> woff(count);
		long long wtot = 0;
		for (int i = 0; i < count; ++i) {
			woff[i] = wtot;
			wtot += cg_batch::mg_scratch_floats(probs[i].nx, probs[i].ny);
		}
		std::vector<int> ord(count);
		for (int i = 0; i < count; ++i) ord[i] = i;
		std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
			return (long long)probs[x].nx * probs[x].ny > (long long)probs[y].nx * probs[y].ny;
		});
		if ((rc = b->w32.ensure(sizeof(float) * (size_t)wtot))) return fail(rc);
		if ((rc = to_device(b->w32off, woff.data(), sizeof(long long) * count, s))) return fail(rc);
		if ((rc = to_device(b->order, ord.data(), sizeof(int) * count, s))) return fail(rc);
		if ((rc = b->queue.ensure(sizeof(unsigned)))) return fail(rc);
		if ((rc = to_device(b->dprob, b->hprob.data(), sizeof(BatchProb) * count, s))) return fail(rc);
		if (cudaStreamSynchronize(s) != cudaSuccess) {
			note_cuda_error(cudaGetLastError());
			return fail(CARPIO_GPU_ECUDA);
		}
		rc = configure_mg(b, want.threads ? want.threads : 512, want.use_graph);
	} else if (explicit_tiles) {
		rc = configure(b, want);
	} else {
		rc = CARPIO_GPU_EINVAL;
		for (auto c : candidates(kCellsPerCta)) {
			if (want.threads && c.threads != want.threads) continue;
			if (want.cluster && c.cluster != want.cluster) continue;
			if (want.cells_per_cta && c.cells_per_cta != want.cells_per_cta) continue;
			c.use_graph = want.use_graph;
			if ((rc = configure(b, c)) == 0) break;
			if (rc != CARPIO_GPU_EINVAL) break;
		}
	}
	if (rc) return fail(rc);
	*out = b;
	return 0;
}

int carpio_gpu_batch_destroy(carpio_gpu_batch* b) {
	if (!b) return CARPIO_GPU_EINVAL;
	delete b;
	return 0;
}

int carpio_gpu_batch_field(carpio_gpu_batch* b, int which, int i, double** dev) {
	if (!b || !dev || i < 0 || i >= b->count || (which != 0 && which != 1))
		return CARPIO_GPU_EINVAL;
	*dev = (which == 0 ? b->src : b->phi).as<double>() + b->off[i];
	return 0;
}

int carpio_gpu_batch_zero(carpio_gpu_batch* b, int which) {
	if (!b || (which != 0 && which != 1)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(b->mu);
	cg_host::DevBuf& f = which == 0 ? b->src : b->phi;
	CG_CK(cudaMemsetAsync(f.p, 0, sizeof(double) * (size_t)b->cells, b->s));
	CG_CK(cudaStreamSynchronize(b->s));
	return 0;
}

static int batch_copy(carpio_gpu_batch* b, int which, double* const* host,
		const double* const* chost, bool up) {
	if (!b || (which != 0 && which != 1) || (up ? !chost : !host)) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(b->mu);
	double* base = (which == 0 ? b->src : b->phi).as<double>();
	for (int i = 0; i < b->count; ++i) {
		const int nx = b->probs[i].nx, ny = b->probs[i].ny;
		double* d = base + b->off[i] + (ny + 2) + 1;
		const size_t dp = sizeof(double) * (ny + 2), hp = sizeof(double) * ny;
		if (up) {
			if (!chost[i]) return CARPIO_GPU_EINVAL;
			CG_CK(cudaMemcpy2DAsync(d, dp, chost[i], hp, hp, nx, cudaMemcpyDefault, b->s));
		} else {
			if (!host[i]) return CARPIO_GPU_EINVAL;
			CG_CK(cudaMemcpy2DAsync(host[i], hp, d, dp, hp, nx, cudaMemcpyDefault, b->s));
		}
	}
	CG_CK(cudaStreamSynchronize(b->s));
	return 0;
}

int carpio_gpu_batch_upload(carpio_gpu_batch* b, int which, const double* const* fields) {
	return batch_copy(b, which, nullptr, fields, true);
}

int carpio_gpu_batch_download(carpio_gpu_batch* b, int which, double* const* fields) {
	return batch_copy(b, which, fields, nullptr, false);
}

int carpio_gpu_batch_run(carpio_gpu_batch* b, carpio_gpu_solver_stats* stats, double* ms) {
	if (!b) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(b->mu);
	float t = 0;
	int rc = run_once(b, &t);
	if (rc) return rc;
	if (ms) *ms = t;
	const int err = b->hctl->err;
	int code = err;
	bool maxit = false;
	for (int i = 0; i < b->count; ++i) {
		const BatchRes& o = b->hres[i];
		if (!o.ran && !code) code = CARPIO_GPU_ECUDA;
		if (o.ran && o.code == 1) maxit = true;
		if (stats) {
			carpio_gpu_solver_stats& st = stats[i];
			st.code = o.ran ? o.code : (err ? err : CARPIO_GPU_ECUDA);
			st.iters = o.iters;
			st.tol_out = o.resid;
			st.outer_iters = o.updates;
			st.hist_len = 0;
			st.ms = o.ms;
		}
	}
	if (code) return code;
	return maxit ? 1 : 0;
}

int carpio_gpu_batch_autotune(carpio_gpu_batch* b, int max_candidates) {
	using namespace cg_host;
	if (!b || max_candidates < 1) return CARPIO_GPU_EINVAL;
	std::lock_guard<std::mutex> lk(b->mu);
	const size_t fb = sizeof(double) * (size_t)b->cells;
	int rc;
	if ((rc = b->save.ensure(fb))) return rc;
	CG_CK(cudaMemcpyAsync(b->save.p, b->phi.p, fb, cudaMemcpyDeviceToDevice, b->s));
	const carpio_gpu_batch_tiles keep = b->plan.tiles;
	carpio_gpu_batch_tiles best = keep;
	float best_ms = 0;
	int tried = 0;
	// the multigrid kernel's block sizes, or the cluster-team configurations
	std::vector<carpio_gpu_batch_tiles> cands;
	if (b->mg) {
		for (int T : { 512, 256, 1024 }) {
			carpio_gpu_batch_tiles t{};
			t.threads = T;
			cands.push_back(t);
		}
	} else {
		cands = candidates(kCellsPerCta);
	}
	for (auto c : cands) {
		if (tried >= max_candidates) break;
		c.use_graph = keep.use_graph;
		rc = b->mg ? configure_mg(b, c.threads, c.use_graph) : configure(b, c);
		if (rc == CARPIO_GPU_EINVAL) continue;
		if (rc) return rc;
		float ms = 0;
		for (int rep = 0; rep < 2; ++rep) {
			CG_CK(cudaMemcpyAsync(b->phi.p, b->save.p, fb, cudaMemcpyDeviceToDevice, b->s));
			if ((rc = run_once(b, &ms))) return rc;
			if (b->hctl->err) return b->hctl->err;
		}
		++tried;
		if (best_ms == 0 || ms < best_ms) {
			best_ms = ms;
			best = c;
		}
	}
	CG_CK(cudaMemcpyAsync(b->phi.p, b->save.p, fb, cudaMemcpyDeviceToDevice, b->s));
	if ((rc = b->mg ? configure_mg(b, best.threads, best.use_graph) : configure(b, best))) return rc;
	b->info.candidates = tried;
	b->info.tuned_ms = best_ms;
	std::lock_guard<std::mutex> lk2(tune_mu());
	tune_cache()[b->signature] = best;
	return 0;
}

int carpio_gpu_batch_get_info(const carpio_gpu_batch* b, carpio_gpu_batch_info* info) {
	if (!b || !info) return CARPIO_GPU_EINVAL;
	*info = b->info;
	return 0;
}

}  // extern "C"
