// Engine object and C ABI (include/rheocell_gb300.h).
//
// One engine advances one monolayer on one GPU.  Per time step it issues, on
// one stream, the kernels that replace FD_CPUBackend::sim_step
// (src/Backends/FD_CPUBackend.cpp:134-160):
//
//   dry evaluation (xi-only velocity; simplefield, activenematic, and the wet
//   models while friction_cell = 0):
//     [rng] -> cell(eval phi^n + predictor) -> gather(phi*) -> cell(eval phi* +
//     corrector + set_positions) -> [repack] -> gather(phi^{n+1})
//   The force evaluation at phi^{n+1} that closes the reference's step is
//   carried into the next step's first kernel ("pending"), where it is fused
//   with the predictor; its parameters are those in force when the reference
//   would have run it (eval_phase), so the first step after
//   apply_changes_after_equilibration uses the passive forces, as the
//   reference does (FD_CPUBackend.cpp:23-24 vs SimManager.cpp:144).
//
//   wet evaluation (friction_cell > 0):
//     [rng] -> cell(predictor) -> gather(phi*) -> cell(forces, rhs) -> CG ->
//     cell(corrector) -> [repack] -> gather(phi^{n+1}) -> cell(forces, rhs) -> CG
#include "rc_kernels.cuh"
#include "rc_unet_train.cuh"
#include "../../include/rheocell_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace rc;

#define RC_PI_F 3.141592653589793238462643f

// From this many cells on, the per-cell epilogue runs as its own kernel with
// one thread per cell (its FP64 code then shares instructions across cells).
// FP32 engines with a viscous solve always run it: their update-only kernel
// (cell_update_f32) writes per-warp partial sums only.
constexpr int SPLIT_FINISH_CELLS = 256;

// Residual margin of the learned solve (see solve_args).
constexpr double LEARNED_RES_MARGIN = 0.2;

struct rc_engine {
	int device = 0;
	cudaStream_t stream = nullptr;
	cudaStream_t own_stream = nullptr;
	rc_params hp;
	DevParams P;
	PhaseParams ph[2];
	int phase = 0;
	int eval_phase = 0;
	bool pending = false;
	int L = 0, N = 0;
	long long S = 0, S_cap = 0;
	int smem_n = 0;
	int max_n_host = 0;
	int rep_on = 0;
	int cg_blocks = 0;
	int nbx = 0, nby = 0;        // bins of layer 0 (single-monolayer solver paths)
	int n_layers = 1, total_bins = 0;
	int *bin_layer = nullptr;  // layer of each bin
	long long total_box = 0;
	std::vector<LayerDev> layers_h;
	LayerDev *layers = nullptr;

	CellDev *cells = nullptr;
	double *phiA = nullptr, *phiB = nullptr, *dphi_old = nullptr, *mu = nullptr, *dxg = nullptr, *dyg = nullptr;
	double *vx = nullptr, *vy = nullptr, *fx = nullptr, *fy = nullptr, *rep = nullptr;
	int *mapg = nullptr;
	double *phi2 = nullptr, *sq00 = nullptr, *sq01 = nullptr;
	double *walls = nullptr;  // getWalls(k) per box site of every layer; null: periodic boxes
	float *muf = nullptr, *dxf = nullptr, *dyf = nullptr;  // FP32 engines: mu and gradients in FP32
	LayerSolve *lsolve = nullptr;  // wet ensembles: each member's solver bookkeeping
	std::vector<int> layer_blocks[2];  // wet ensembles: solve grid per member (plain FP64, flexible CG)
	int *cnt = nullptr, *cover = nullptr, *cov_off = nullptr, *cov_idx = nullptr;
	int *bin_count = nullptr, *bin_cells = nullptr;
	double *tab_cos = nullptr, *tab_sin = nullptr;
	float *tab_cosf = nullptr, *tab_sinf = nullptr;
	CellSum *csum = nullptr;  // split mode (many cells): per-cell sums for the epilogue kernel
	DevStatus *st = nullptr;
	DevStatus *st_host = nullptr;
	double *rx = nullptr, *ry = nullptr, *px = nullptr, *py = nullptr, *Px = nullptr, *Py = nullptr;
	double *partials = nullptr, *scalars = nullptr;
	unsigned *bar = nullptr;
	float *rxf = nullptr, *ryf = nullptr, *pxf = nullptr, *pyf = nullptr, *apxf = nullptr, *apyf = nullptr;
	float *Pxf = nullptr, *Pyf = nullptr;
	float *exf = nullptr, *eyf = nullptr;
	double *scratch_phi = nullptr, *scratch_rep = nullptr;
	std::vector<void *> allocs;
	std::string err;
	std::string launch_error;  // first failed cooperative launch
	long long launches = 0;    // engine kernels enqueued since the last status read
	int f32_block = CELL_THREADS;  // FP32 cell kernel: patch sites per tile (rc_autotune)
	long long async_steps = 0;
	// stage timers
	bool timing = false;
	struct Mark {
		int stage;
		cudaEvent_t a, b;
	};
	std::vector<Mark> marks;
	std::vector<cudaEvent_t> event_pool;
	double timer_ms[RC_NUM_TIMERS] = {0};
	long long timer_n[RC_NUM_TIMERS] = {0};
	// CUDA graphs of one step, keyed by the host-side step state
	struct StepGraph {
		int pending, eval_phase, phase, smem_n;
		cudaStream_t stream;
		cudaGraphExec_t exec;
		int next_pending, next_eval_phase;
		long long launches;
	};
	std::vector<StepGraph> graphs;
	bool use_graphs = true;
	// learned preconditioner
	int solver = RC_SOLVER_PLAIN;
	float *unet_params = nullptr;  // FP32 network parameters (null: none yet)
	UNetActs unet{};               // activations for the two velocity components
	float *zxf = nullptr, *zyf = nullptr, *Zxf = nullptr, *Zyf = nullptr, *Pxf2 = nullptr, *Pyf2 = nullptr;
	bf16 *unet_pack = nullptr;     // BF16 weights of the tensor-core layers
	UNetActsBF unet_bf{};          // BF16 activations of the tensor-core path
	int cg_blocks_learned = 0;
	// harvested training samples
	float *harv_in = nullptr, *harv_tgt = nullptr, *harv_s = nullptr;
	int *harv_count = nullptr;
	int harv_cap = 0, harv_every = 4, harv_per_solve = 4;
	bool harv_collect = false;
	unsigned long long *phase_ns = nullptr;  // diagnostic solve phase timers (null: off)
	bool phase_on = false;
	double *obs_buf = nullptr;               // diagnostic observables scratch
	size_t obs_cap = 0;
	double *split_buf = nullptr;             // force split and free-energy density of an observation: 6 x S_cap
	CellDev *cells_save = nullptr;           // cell records kept aside while it is formed
	// viscous solve limits (rc_set_cg_limits) and the barrier test hook
	long long cg_max_iters = 0;
	int cg_fail_noconv = 0;
	long long spin_limit = 0;
	int barrier_extra = 0;
	DevStatus *st_save = nullptr;            // rc_viscous_resolve: the engine's status kept aside
};

static cudaEvent_t get_event(rc_engine *e) {
	if(!e->event_pool.empty()) {
		cudaEvent_t v = e->event_pool.back();
		e->event_pool.pop_back();
		return v;
	}
	cudaEvent_t v;
	cudaEventCreate(&v);
	return v;
}

// Brackets one stage launch with events when timing is enabled.
struct StageMark {
	rc_engine *e;
	rc_engine::Mark m;
	StageMark(rc_engine *e_, int stage) : e(e_) {
		if(!e->timing || stage < 0) {
			m.a = nullptr;
			return;
		}
		m.stage = stage;
		m.a = get_event(e);
		m.b = get_event(e);
		cudaEventRecord(m.a, e->stream);
	}
	~StageMark() {
		if(!e->timing || !m.a) return;
		cudaEventRecord(m.b, e->stream);
		e->marks.push_back(m);
	}
};

// Add up completed marks (the stream must be idle).
static void collect_marks(rc_engine *e) {
	for(auto &m : e->marks) {
		float ms = 0;
		if(cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) {
			e->timer_ms[m.stage] += ms;
			e->timer_n[m.stage] += 1;
		}
		e->event_pool.push_back(m.a);
		e->event_pool.push_back(m.b);
	}
	e->marks.clear();
}

static std::string g_create_error;

static int set_err(rc_engine *e, int code, const char *fmt, ...) {
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	if(e) e->err = buf;
	else g_create_error = buf;
	return code;
}

#define CUDA_TRY(e, call)                                                                                    \
	do {                                                                                                     \
		cudaError_t _c = (call);                                                                             \
		if(_c != cudaSuccess) return set_err((e), RC_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(_c)); \
	} while(0)

template<typename T>
static int dalloc(rc_engine *e, T **p, size_t count) {
	void *q = nullptr;
	cudaError_t c = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
	if(c != cudaSuccess) return set_err(e, RC_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", sizeof(T) * count, cudaGetErrorString(c));
	e->allocs.push_back(q);
	*p = (T *) q;
	cudaMemset(q, 0, sizeof(T) * (count ? count : 1));
	return RC_OK;
}

static bool wet_phase(const rc_engine *e, int phase) {
	return (e->P.model == M_POLAR || e->P.model == M_WET) && e->ph[phase].friction_cell != 0.0;
}

static CellArgs cell_args(rc_engine *e) {
	CellArgs a;
	memset(&a, 0, sizeof(a));
	a.cells = e->cells;
	a.N = e->N;
	a.smem_n = e->smem_n;
	a.dphi_old = e->dphi_old;
	a.mu = e->mu;
	a.dxg = e->dxg;
	a.dyg = e->dyg;
	a.muf = e->muf;
	a.dxf = e->dxf;
	a.dyf = e->dyf;
	a.dphif = reinterpret_cast<float *>(e->dphi_old);  // FP32 engines keep dphi^n in FP32
	a.vxg = e->vx;
	a.vyg = e->vy;
	a.fxg = e->fx;
	a.fyg = e->fy;
	a.mapg = e->mapg;
	a.rep = e->rep;
	a.phi2 = e->phi2;
	a.walls = e->walls;
	a.sq00 = e->sq00;
	a.sq01 = e->sq01;
	a.tab_cos = e->tab_cos;
	a.tab_sin = e->tab_sin;
	a.tab_cosf = e->tab_cosf;
	a.tab_sinf = e->tab_sinf;
	a.bin_count = e->bin_count;
	a.bin_cells = e->bin_cells;
	a.nbx = e->nbx;
	a.nby = e->nby;
	a.layers = e->layers;
	a.st = e->st;
	a.P = e->P;
	a.rep_on = e->rep_on;
	a.accumulate_rep = 1;
	return a;
}

// Cell kernel launch: the FP32 variant where the engine runs
// RC_PRECISION_FLOAT (polar and wet nematic models), else FP64; in split
// mode (many cells) followed by the per-cell epilogue kernel.  With a stage
// (RC_TIMER_*), the cell kernel alone is timed under it and the epilogue
// under RC_TIMER_EPILOGUE.  Returns the number of kernels launched.
static int cell_launch(rc_engine *e, int eval, int upd, const CellArgs &a0, cudaStream_t s, int stage = -1) {
	CellArgs a = a0;
	a.split = e->csum != nullptr;
	a.csum = e->csum;
	bool f32;
	{
		StageMark sm(e, stage);
		f32 = e->hp.precision == RC_PRECISION_FLOAT && launch_cell_kernel_f32(e->P.model, eval, upd, a, s, e->f32_block);
		if(!f32) launch_cell_kernel(e->P.model, eval, upd, a, s);
	}
	if(!a.split) return 1;
	StageMark sm(e, stage >= 0 ? RC_TIMER_EPILOGUE : -1);
	launch_cell_finish(e->P.model, eval, upd, f32, a, s);
	return 2;
}

static void gather(rc_engine *e, const double *phi, int phase) {
	BoxArgs b;
	memset(&b, 0, sizeof(b));
	b.cells = e->cells;
	b.phi = phi;
	b.phi2 = e->phi2;
	b.sq00 = e->sq00;
	b.sq01 = e->sq01;
	b.cnt = e->cnt;
	b.cover = e->cover;
	b.bin_count = e->bin_count;
	b.bin_cells = e->bin_cells;
	b.nbx = e->nbx;
	b.nby = e->nby;
	b.layers = e->layers;
	b.n_layers = e->n_layers;
	b.total_bins = e->total_bins;
	b.bin_layer = e->bin_layer;
	b.want_q = (e->P.model == M_NEMATIC || e->P.model == M_WET);
	b.want_cover = wet_phase(e, phase);
	b.check_overlap = (e->P.model == M_POLAR || e->P.model == M_WET);
	b.f32 = e->hp.precision == RC_PRECISION_FLOAT && !b.want_q && !b.want_cover;
	b.bookkeeping = (e->P.model == M_POLAR || e->P.model == M_WET);
	b.restart_every = e->hp.cg_restart_every;
	b.solve_follows = wet_phase(e, phase);
	b.st = e->st;
	b.L = e->L;
	b.lsolve = e->n_layers > 1 ? e->lsolve : nullptr;
	StageMark sm(e, RC_TIMER_GATHER);
	launch_box_gather(b, e->stream);
	e->launches += b.bookkeeping ? 2 : 1;
}

// Arguments of the viscous solve of the evaluation at `phase` with `solver`
// into (vx, vy); returns the grid size.  harvest: record training samples
// when the engine collects them (plain FP64 solves only).
static int solve_args(rc_engine *e, int phase, int solver, bool harvest, double *vx, double *vy, CGArgs &g) {
	memset(&g, 0, sizeof(g));
	g.layer = -1;  // the single monolayer (solve() sets each member of an ensemble)
	g.layers = e->layers;
	g.lsolve = e->lsolve;
	g.cells = e->cells;
	g.mapg = e->mapg;
	g.cnt = e->cnt;
	g.cover = e->cover;
	g.cov_off = e->cov_off;
	g.cov_idx = e->cov_idx;
	g.fx = e->fx;
	g.fy = e->fy;
	g.vx = vx;
	g.vy = vy;
	g.rx = e->rx;
	g.ry = e->ry;
	g.px = e->px;
	g.py = e->py;
	g.apxf = e->apxf;
	g.apyf = e->apyf;
	g.Px = e->Px;
	g.Py = e->Py;
	g.partials = e->partials;
	g.scalars = e->scalars;
	g.bar = e->bar;
	g.st = e->st;
	g.L = e->L;
	g.restart_every = e->hp.cg_restart_every;
	g.xi = e->ph[phase].friction;
	g.eta = e->ph[phase].friction_cell;
	g.tol = e->hp.cg_tolerance > 0 ? e->hp.cg_tolerance : 2.220446049250313e-16;
	// FP32 engines solve in mixed precision (FP32 inner iterations, FP64 refinement)
	g.mixed = e->hp.precision == RC_PRECISION_MIXED || e->hp.precision == RC_PRECISION_FLOAT;
	g.inner_tol = 1e-4;
	g.rxf = e->rxf;
	g.ryf = e->ryf;
	g.pxf = e->pxf;
	g.pyf = e->pyf;
	g.Pxf = e->Pxf;
	g.Pyf = e->Pyf;
	g.exf = e->exf;
	g.eyf = e->eyf;
	g.max_iters = e->cg_max_iters;
	g.fail_noconv = e->cg_fail_noconv;
	g.spin_limit = e->spin_limit;
	g.barrier_extra = e->barrier_extra;
	int blocks = e->cg_blocks;
	if(solver == RC_SOLVER_PLAIN_FP64) g.mixed = 0;  // Eigen's Jacobi CG in FP64 whatever the precision
	if(g.mixed && solver == RC_SOLVER_PLAIN) {
		// mixed precision: Jacobi-preconditioned flexible CG in cover order
		g.fcg = 1;
		g.zxf = e->zxf;
		g.zyf = e->zyf;
		g.Zxf = e->Zxf;
		g.Zyf = e->Zyf;
		g.Pxf2 = e->Pxf2;
		g.Pyf2 = e->Pyf2;
		blocks = e->cg_blocks_learned;
	}
	if(solver == RC_SOLVER_LEARNED || solver == RC_SOLVER_LEARNED_FP32) {
		g.mixed = 1;
		g.fcg = 1;
		// The network-preconditioned solve leaves its error in the operator's
		// smallest-eigenvalue modes (box-smooth, wavelengths of 16-64 sites):
		// max|v - v*| / max|v*| reaches ~50 |r|/|b| against ~4 for Jacobi
		// CG at 1024^2.  It therefore converges to LEARNED_RES_MARGIN times
		// the tolerance, which keeps its velocity error at the plain solve's
		// level (below 1e-7 of the FP64 solution at 1024^2, where the plain
		// tolerance itself left up to 2.6e-7).
		g.tol *= LEARNED_RES_MARGIN;
		g.unet_params = e->unet_params;
		g.unet = e->unet;
		g.unet_tc = solver == RC_SOLVER_LEARNED;
		g.phase_ns = e->phase_on ? e->phase_ns : nullptr;
		g.unet_bf = e->unet_bf;
		g.unet_wpack = e->unet_pack;
		g.zxf = e->zxf;
		g.zyf = e->zyf;
		g.Zxf = e->Zxf;
		g.Zyf = e->Zyf;
		g.Pxf2 = e->Pxf2;
		g.Pyf2 = e->Pyf2;
		blocks = e->cg_blocks_learned;
	}
	else if(harvest && e->harv_cap > 0 && e->harv_collect && !g.mixed) {
		g.harv_in = e->harv_in;
		g.harv_tgt = e->harv_tgt;
		g.harv_s = e->harv_s;
		g.harv_count = e->harv_count;
		g.harv_cap = e->harv_cap;
		g.harv_every = e->harv_every;
		g.harv_per_solve = e->harv_per_solve;
	}
	return blocks;
}

static void solve(rc_engine *e, int phase) {
	CGArgs g;
	const int blocks = solve_args(e, phase, e->solver, true, e->vx, e->vy, g);
	StageMark sm(e, RC_TIMER_SOLVE);
	if(e->n_layers == 1) {
		cudaMemsetAsync(e->bar, 0, sizeof(unsigned) * 4, e->stream);  // the barrier counter starts at zero
		const cudaError_t c = launch_cg(g, blocks, e->stream);
		e->launches += 1;
		if(c != cudaSuccess && e->launch_error.empty()) e->launch_error = cudaGetErrorString(c);
		return;
	}
	// an ensemble: each member's system in turn, on its own box, with the grid
	// a monolayer of its size would get (the same launches as the member alone)
	const bool mixed = g.fcg != 0;
	for(int l = 0; l < e->n_layers; l++) {
		const LayerDev &ly = e->layers_h[(size_t) l];
		CGArgs m = g;
		m.layer = l;
		m.L = ly.L;
		m.cnt = e->cnt + ly.box_off;
		m.cover = e->cover + (size_t) STORE_MAX * ly.box_off;
		const int b = e->layer_blocks[mixed ? 1 : 0][(size_t) l];
		cudaMemsetAsync(e->bar, 0, sizeof(unsigned) * 4, e->stream);
		const cudaError_t c = launch_cg(m, b, e->stream);
		e->launches += 1;
		if(c != cudaSuccess && e->launch_error.empty()) e->launch_error = cudaGetErrorString(c);
	}
}

// Forces (and the viscous solve) at phi^n for the current phase, run at its
// logical time; the dry path leaves it pending for the next predictor.
static void evaluate_end(rc_engine *e, const double *phi, int phase) {
	gather(e, phi, phase);
	if(wet_phase(e, phase)) {
		CellArgs a = cell_args(e);
		a.phi_eval = phi;
		a.pe = e->ph[phase];
		a.pu = e->ph[phase];
		e->launches += cell_launch(e, EV_WET_RHS, UP_NONE, a, e->stream, RC_TIMER_FORCES) - 1;
		e->launches += 1;
		solve(e, phase);
		e->pending = false;
	}
	else {
		e->pending = true;
	}
	e->eval_phase = phase;
}

static void one_step(rc_engine *e) {
	const int cur = e->phase;
	cudaStream_t s = e->stream;
	if(e->P.model == M_POLAR) {
		StageMark sm(e, RC_TIMER_RNG);
		launch_rng(e->cells, e->layers, e->n_layers, e->st, s);
		e->launches += 1;
	}
	CellArgs a = cell_args(e);
	a.phi_eval = e->phiA;
	a.phi_out = e->phiB;
	a.pu = e->ph[cur];
	if(e->pending) {
		a.pe = e->ph[e->eval_phase];
		e->launches += cell_launch(e, EV_LOCAL, UP_PRED, a, s, RC_TIMER_UPDATE) - 1;
	}
	else {
		a.pe = e->ph[cur];
		e->launches += cell_launch(e, EV_NONE, UP_PRED, a, s, RC_TIMER_UPDATE) - 1;
	}
	e->launches += 1;
	gather(e, e->phiB, cur);
	cudaMemsetAsync(e->bin_count, 0, sizeof(int) * (size_t) e->total_bins, s);
	CellArgs c = cell_args(e);
	c.phi_old = e->phiA;
	c.phi_out = e->phiA;
	c.pe = e->ph[cur];
	c.pu = e->ph[cur];
	if(!wet_phase(e, cur)) {
		c.phi_eval = e->phiB;
		e->launches += cell_launch(e, EV_LOCAL, UP_CORR, c, s, RC_TIMER_UPDATE) - 1;
		e->launches += 1;
	}
	else {
		CellArgs f = cell_args(e);
		f.phi_eval = e->phiB;
		f.pe = e->ph[cur];
		f.pu = e->ph[cur];
		e->launches += cell_launch(e, EV_WET_RHS, UP_NONE, f, s, RC_TIMER_FORCES) - 1;
		solve(e, cur);
		c.phi_eval = e->phiB;
		e->launches += cell_launch(e, EV_NONE, UP_CORR, c, s, RC_TIMER_UPDATE) - 1;
		e->launches += 2;
	}
	CellArgs r = cell_args(e);
	r.phi_out = e->phiA;
	{
		StageMark sm(e, RC_TIMER_REPACK);
		launch_repack(r, e->scratch_phi, e->scratch_rep, e->S_cap, s);
	}
	e->launches += 5;
	evaluate_end(e, e->phiA, cur);
}

static void drop_graphs(rc_engine *e) {
	for(auto &g : e->graphs) cudaGraphExecDestroy(g.exec);
	e->graphs.clear();
}

// One step, replayed from a captured CUDA graph when possible.  A graph is
// captured per distinct host-side state (pending evaluation, its phase, the
// current phase, shared-memory sizing, stream); the data-dependent solver
// iteration counts are handled inside the cooperative kernel.
static void run_step(rc_engine *e) {
	if(!e->use_graphs || e->timing || e->stream == nullptr || e->stream == cudaStreamLegacy) {
		one_step(e);
		return;
	}
	for(auto &g : e->graphs) {
		if(g.pending == (int) e->pending && g.eval_phase == e->eval_phase && g.phase == e->phase &&
		   g.smem_n == e->smem_n && g.stream == e->stream) {
			if(cudaGraphLaunch(g.exec, e->stream) != cudaSuccess) {
				if(e->launch_error.empty()) e->launch_error = "graph launch failed";
				return;
			}
			e->pending = g.next_pending != 0;
			e->eval_phase = g.next_eval_phase;
			e->launches += g.launches;
			return;
		}
	}
	rc_engine::StepGraph g;
	g.pending = (int) e->pending;
	g.eval_phase = e->eval_phase;
	g.phase = e->phase;
	g.smem_n = e->smem_n;
	g.stream = e->stream;
	const bool was_pending = e->pending;
	const int was_eval_phase = e->eval_phase;
	const long long l0 = e->launches;
	cudaGraph_t graph = nullptr;
	if(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		cudaGetLastError();
		e->use_graphs = false;
		one_step(e);
		return;
	}
	one_step(e);
	cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
	cudaGraphExec_t exec = nullptr;
	if(ce == cudaSuccess && e->launch_error.empty()) ce = cudaGraphInstantiate(&exec, graph, 0);
	if(graph) cudaGraphDestroy(graph);
	if(ce != cudaSuccess || !e->launch_error.empty()) {
		// capture not possible here: run this and later steps directly
		cudaGetLastError();
		e->launch_error.clear();
		e->use_graphs = false;
		e->pending = was_pending;
		e->eval_phase = was_eval_phase;
		e->launches = l0;
		one_step(e);
		return;
	}
	g.exec = exec;
	g.next_pending = (int) e->pending;
	g.next_eval_phase = e->eval_phase;
	g.launches = e->launches - l0;
	e->graphs.push_back(g);
	if(cudaGraphLaunch(exec, e->stream) != cudaSuccess && e->launch_error.empty()) e->launch_error = "graph launch failed";
}

// Materialise a pending dry evaluation into mu, v, gradients and the map.
static void materialise(rc_engine *e, int accumulate) {
	if(!e->pending) return;
	CellArgs a = cell_args(e);
	a.phi_eval = e->phiA;
	a.pe = e->ph[e->eval_phase];
	a.pu = e->ph[e->eval_phase];
	a.accumulate_rep = accumulate;
	e->launches += cell_launch(e, EV_STORE, UP_NONE, a, e->stream) - 1;
	e->launches += 1;
	if(accumulate) e->pending = false;
}

static int choose_smem(rc_engine *e) {
	int want = std::max(256, (e->max_n_host * 3 + 1) / 2);
	want = ((want + 255) / 256) * 256;
	const int per_site = 8 * cell_smem_arrays(e->P.model);
	const int cap = (200 * 1024) / per_site;
	if(e->max_n_host > cap) return set_err(e, RC_ERR_CAPACITY, "patch of %d sites exceeds shared memory", e->max_n_host);
	e->smem_n = std::min(want, cap);
	return RC_OK;
}

static int check_status(rc_engine *e, rc_step_stats *stats) {
	CUDA_TRY(e, cudaMemcpyAsync(e->st_host, e->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	CUDA_TRY(e, cudaGetLastError());
	if(!e->launch_error.empty()) {
		std::string m = e->launch_error;
		e->launch_error.clear();
		return set_err(e, RC_ERR_CUDA, "viscous solve launch failed: %s", m.c_str());
	}
	const DevStatus &h = *e->st_host;
	e->S = h.S;
	e->max_n_host = std::max(e->max_n_host, h.max_n);
	if(stats) {
		stats->cg_solves += h.cg_solves;
		stats->cg_iterations += h.cg_iters;
		stats->cg_max_iterations = std::max(stats->cg_max_iterations, h.cg_max_iters);
		stats->cg_max_rel_residual = std::max(stats->cg_max_rel_residual, h.cg_max_rel);
		stats->refinements += h.refinements;
		stats->fallbacks += h.fallbacks;
		stats->resized_cells += h.resized_total;
		stats->kernel_launches += e->launches;
	}
	e->launches = 0;
	{
		const size_t off = offsetof(DevStatus, cg_solves);
		const size_t len = offsetof(DevStatus, overflow_used) - off;
		CUDA_TRY(e, cudaMemsetAsync(reinterpret_cast<char *>(e->st) + off, 0, len, e->stream));
	}
	if(h.err) {
		if(h.err & ERR_OVERLAP) return set_err(e, RC_ERR_OVERLAP, "Too many field patches overlap (box site %d)", h.err_where);
		if(h.err & ERR_CAPACITY) return set_err(e, RC_ERR_CAPACITY, "capacity exceeded (cell %d): patch or site storage", h.err_where);
		if(h.err & ERR_BIN) return set_err(e, RC_ERR_CAPACITY, "box bin capacity exceeded");
		if(h.err & ERR_NONFINITE) return set_err(e, RC_ERR_NONFINITE, "non-finite state in cell %d", h.err_where);
		if(h.err & ERR_BARRIER) return set_err(e, RC_ERR_CG, "viscous solve: grid barrier timed out");
		if(h.err & ERR_TYPE) return set_err(e, RC_ERR_INVALID, "Too many field types (cell %d)", h.err_where);
		if(h.err & ERR_MMA) return set_err(e, RC_ERR_CG, "viscous solve: tensor-core completion wait timed out");
		if(h.err & ERR_COPY) return set_err(e, RC_ERR_CUDA, "cell update: bulk-copy completion wait timed out (cell %d)", h.err_where);
		if(h.err & ERR_NOCONV)
			return set_err(e, RC_ERR_CG, "viscous solve: tolerance not reached within the iteration cap (%lld)",
			               e->cg_max_iters);
		return set_err(e, RC_ERR_INVALID, "device error 0x%x", h.err);
	}
	return RC_OK;
}

static void host_cell(const rc_cell_host &h, CellDev &c, int start, int layer = 0) {
	memset(&c, 0, sizeof(c));
	c.layer = layer;
	c.lx = h.lsub_x;
	c.ly = h.lsub_y;
	c.offx = h.offset_x;
	c.offy = h.offset_y;
	c.corner = h.corner;
	c.type = h.type;
	c.start = start;
	c.n = h.lsub_x * h.lsub_y;
	c.xl = h.lsub_x;
	c.yb = h.lsub_y;
	c.comx = c.com_oldx = h.com_x;
	c.comy = c.com_oldy = h.com_y;
	c.unrapx = h.unrap_x;
	c.unrapy = h.unrap_y;
	c.q00 = h.q00;
	c.q01 = h.q01;
	c.thq = h.theta_q;
	c.thq_old = h.theta_q_old;
	c.nqx = h.nemq_x;
	c.nqy = h.nemq_y;
	c.nq_oldx = h.nemq_old_x;
	c.nq_oldy = h.nemq_old_y;
}

// Initial per-cell sums, in the reference's sequential order so they are
// bit-identical: area = sum phi^2 and sumF = sum phi of the loaded field
// (SimBackend.cpp:289-296) and the shape tensor of begin_energy_computation()
// (e.g. WetModel.cpp:126-164; only visible in a download before the first step).
// walls (null: periodic boxes): the wet, polar and simple models' initial
// gradients take derivX/derivY's wall branches (SimpleMultiField.cpp:97-98,
// WetModel.cpp:154-155, WetPolarModel.cpp:119-120; ActiveNematic.cpp:127-128
// keeps the plain differences)
__global__ void init_sums_kernel(CellDev *cells, const LayerDev *layers, const double *phi, int N, const double *walls,
                                 double slip) {
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= N) return;
	CellDev &c = cells[i];
	const int lx = c.lx, ly = c.ly, n = c.n, st = c.start;
	const LayerDev &lay = layers[c.layer];
	const int L = lay.L;
	const double *wl = walls ? walls + lay.box_off : nullptr;
	auto open = [&](int k) { return wl[k] < slip; };
	double area = 0, sumf = 0, s00 = 0, s01 = 0;
	for(int q = 0; q < n; q++) {
		const double p = phi[st + q];
		area += p * p;
		sumf += p;
		const int y = q / lx, x = q - y * lx;
		const int r = (x == lx - 1) ? q - (lx - 1) : q + 1, l = (x == 0) ? q + (lx - 1) : q - 1;
		const int u = (y == ly - 1) ? q - (ly - 1) * lx : q + lx, d = (y == 0) ? q + (ly - 1) * lx : q - lx;
		double dx = .5 * (phi[st + r] - phi[st + l]), dy = .5 * (phi[st + u] - phi[st + d]);
		if(wl) {
			const int k = box_site(c, x, y, L), kx = k % L, ky = k / L;
			const int kr = ky * L + (kx == L - 1 ? 0 : kx + 1), kl = ky * L + (kx == 0 ? L - 1 : kx - 1);
			const int ku = (ky == L - 1 ? 0 : ky + 1) * L + kx, kd = (ky == 0 ? L - 1 : ky - 1) * L + kx;
			if(!(open(kr) && open(kl))) dx = 0.;
			if(!(open(ku) && open(kd))) dy = 0.;
		}
		s00 += -0.5 * (dx * dx - dy * dy);
		s01 += -dx * dy;
	}
	c.area = area;
	c.sumf = sumf;
	c.s00 = s00;
	c.s01 = s01;
}

extern "C" {

int rc_abi_version(void) { return RC_ABI_VERSION; }

}  // extern "C"

// Fills each cell's patch with the generated profile (one block per cell):
// RC_PROFILE_TANH: phi = (1 - tanh((d - radius) / width)) / 2, d the distance
// from the box site to the cell's centre (nearest periodic image);
// RC_PROFILE_DISC: the reference's initial disc (MultiPhaseField::init,
// MultiPhaseField.cpp:149-156), phi = 1 where x^2 + y^2 < radius^2 + 0.5 with
// x = LsubX/2 - (q mod LsubX), y = LsubY/2 - q / LsubX (integer division).
__global__ void generate_phi_kernel(const CellDev *cells, double *phi, rc_generate_spec g, int L) {
	const CellDev &c = cells[blockIdx.x];
	double *out = phi + c.start;
	for(int q = threadIdx.x; q < c.n; q += blockDim.x) {
		const int sy = q / c.lx, sx = q - sy * c.lx;
		double v;
		if(g.profile == RC_PROFILE_DISC) {
			const int x = c.lx / 2 - sx, y = c.ly / 2 - sy;
			v = (double) (x * x + y * y) < g.radius * g.radius + 0.5 ? 1.0 : 0.0;
		}
		else {
			const int k = box_site(c, sx, sy, L);
			const int by = k / L, bx = k - by * L;
			double dx = (double) bx - c.comx, dy = (double) by - c.comy;
			dx -= L * rint(dx / L);
			dy -= L * rint(dy / L);
			const double d = sqrt(dx * dx + dy * dy);
			v = 0.5 * (1.0 - tanh((d - g.radius) / g.width));
		}
		out[q] = v;
	}
}

static int create_engine(const rc_params *params, int n_layers, const rc_box *boxes, const int *n_cells_per_layer,
                         const rc_cell_host *cells, const unsigned long long *rng_states, int device, rc_engine **out,
                         const rc_generate_spec *gen);

extern "C" {

int rc_create(const rc_params *params, const rc_box *box, int n_cells, const rc_cell_host *cells, int device,
              rc_engine **out) {
	if(!params) return set_err(nullptr, RC_ERR_INVALID, "invalid arguments");
	const unsigned long long rs = params->rng_state;
	return create_engine(params, 1, box, &n_cells, cells, &rs, device, out, nullptr);
}

int rc_create_generated(const rc_params *params, const rc_box *box, int n_cells, const rc_cell_host *cells,
                        const rc_generate_spec *spec, int device, rc_engine **out) {
	if(out) *out = nullptr;
	if(!params || !spec) return set_err(nullptr, RC_ERR_INVALID, "invalid arguments");
	if(spec->profile != RC_PROFILE_TANH && spec->profile != RC_PROFILE_DISC)
		return set_err(nullptr, RC_ERR_INVALID, "rc_create_generated: unknown profile %d", spec->profile);
	if(!(spec->radius > 0.0) || (spec->profile == RC_PROFILE_TANH && !(spec->width > 0.0)))
		return set_err(nullptr, RC_ERR_INVALID, "rc_create_generated: radius and width must be positive");
	const unsigned long long rs = params->rng_state;
	return create_engine(params, 1, box, &n_cells, cells, &rs, device, out, spec);
}

int rc_batch_create(const rc_params *params, int n_layers, const rc_box *boxes, const int *n_cells_per_layer,
                    const rc_cell_host *cells, const unsigned long long *rng_states, int device, rc_engine **out) {
	return create_engine(params, n_layers, boxes, n_cells_per_layer, cells, rng_states, device, out, nullptr);
}

}  // extern "C"

static int create_engine(const rc_params *params, int n_layers, const rc_box *boxes, const int *n_cells_per_layer,
                         const rc_cell_host *cells, const unsigned long long *rng_states, int device, rc_engine **out,
                         const rc_generate_spec *gen) {
	if(!out) return set_err(nullptr, RC_ERR_INVALID, "out is NULL");
	*out = nullptr;
	if(!params || !boxes || !n_cells_per_layer || n_layers < 1)
		return set_err(nullptr, RC_ERR_INVALID, "invalid arguments");
	if(params->model < RC_SIMPLEFIELD || params->model > RC_WETMODEL)
		return set_err(nullptr, RC_ERR_INVALID, "unknown interaction model %d", params->model);
	if(params->anchoring) return set_err(nullptr, RC_ERR_UNSUPPORTED, "anchoring is not provided");
	if(params->precision != RC_PRECISION_DOUBLE && params->precision != RC_PRECISION_MIXED &&
	   params->precision != RC_PRECISION_FLOAT)
		return set_err(nullptr, RC_ERR_INVALID, "unknown precision %d", params->precision);
	const bool any_wet = (params->model == RC_WETMODEL || params->model == RC_WETPOLARMODEL) &&
	                     (params->friction_cell[0] != 0.0 || params->friction_cell[1] != 0.0);
	if(params->precision == RC_PRECISION_FLOAT && params->model != RC_WETPOLARMODEL && params->model != RC_WETMODEL)
		return set_err(nullptr, RC_ERR_UNSUPPORTED, "FP32 site arithmetic is provided for wetpolarmodel and wetmodel only");
	bool has_walls = false;
	for(int l = 0; l < n_layers; l++) has_walls |= boxes[l].walls != nullptr;
	if(has_walls && any_wet)
		return set_err(nullptr, RC_ERR_UNSUPPORTED,
		               "walls with a viscous solve are not provided (the reference's wall rows make the assembled "
		               "matrix unsymmetric; its upper-triangle CG then depends on the order of the unknowns)");
	if(has_walls && params->precision == RC_PRECISION_FLOAT)
		return set_err(nullptr, RC_ERR_UNSUPPORTED, "walls are provided by the FP64 cell kernels only");
	std::vector<LayerDev> layers((size_t) n_layers);
	int n_cells = 0, total_bins = 0;
	long long total_box = 0;
	for(int l = 0; l < n_layers; l++) {
		const rc_box &bx = boxes[l];
		if(bx.Lx != bx.Ly || bx.Lx < 3 || bx.Lx > 46340)
			return set_err(nullptr, RC_ERR_INVALID, "The box in the configuration file is not a square (%dx%d)", bx.Lx, bx.Ly);
		if(n_cells_per_layer[l] < 0) return set_err(nullptr, RC_ERR_INVALID, "negative cell count");
		LayerDev &ly = layers[(size_t) l];
		memset(&ly, 0, sizeof(ly));
		ly.L = bx.Lx;
		ly.nbx = (bx.Lx + BIN_X - 1) / BIN_X;
		ly.nby = (bx.Lx + BIN_Y - 1) / BIN_Y;
		ly.bin_off = total_bins;
		ly.box_off = total_box;
		ly.cell_lo = n_cells;
		ly.cell_hi = n_cells + n_cells_per_layer[l];
		ly.rng_state = (rng_states ? rng_states[l] : params->rng_state) & ((1ULL << 48) - 1);
		ly.rng_has = (n_layers == 1) ? params->rng_has_cached : 0;
		ly.rng_cached = (n_layers == 1) ? params->rng_cached : 0.0;
		total_bins += ly.nbx * ly.nby;
		total_box += (long long) bx.Lx * bx.Lx;
		n_cells += n_cells_per_layer[l];
	}
	if(n_cells > 0 && !cells) return set_err(nullptr, RC_ERR_INVALID, "cells is NULL");
	long long S = 0;
	int max_n = 0;
	for(int l = 0; l < n_layers; l++) {
		const int L = layers[(size_t) l].L;
		for(int i = layers[(size_t) l].cell_lo; i < layers[(size_t) l].cell_hi; i++) {
			const rc_cell_host &h = cells[i];
			if(h.lsub_x <= 0 || h.lsub_y <= 0 || h.lsub_x > L || h.lsub_y > L || h.lsub_x > MAX_TABLE_SIDE ||
			   h.lsub_y > MAX_TABLE_SIDE)
				return set_err(nullptr, RC_ERR_INVALID, "cell %d: patch %dx%d does not fit the box/tables", i, h.lsub_x, h.lsub_y);
			if(h.offset_x < 0 || h.offset_x >= h.lsub_x || h.offset_y < 0 || h.offset_y >= h.lsub_y)
				return set_err(nullptr, RC_ERR_INVALID, "cell %d: offset out of range", i);
			if(h.corner < 0 || h.corner >= L * L) return set_err(nullptr, RC_ERR_INVALID, "cell %d: corner out of box", i);
			if(!h.phi && !gen) return set_err(nullptr, RC_ERR_INVALID, "cell %d: phi is NULL", i);
			S += (long long) h.lsub_x * h.lsub_y;
			max_n = std::max(max_n, h.lsub_x * h.lsub_y);
		}
	}
	const int L = layers[0].L;
	if(S >= (1LL << 31) - (1LL << 24)) return set_err(nullptr, RC_ERR_CAPACITY, "too many sites (%lld)", S);

	rc_engine *e = new rc_engine();
	e->device = device;
	e->hp = *params;
	e->L = L;
	e->N = n_cells;
	e->S = S;
	e->n_layers = n_layers;
	e->layers_h = layers;
	e->total_bins = total_bins;
	e->total_box = total_box;
	e->S_cap = std::min((1LL << 31) - 1, S + std::max(S / 4, 65536LL));
	e->max_n_host = max_n;
	int rc;
	cudaError_t ce = cudaSetDevice(device);
	if(ce != cudaSuccess) {
		set_err(nullptr, RC_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(ce));
		delete e;
		return RC_ERR_CUDA;
	}
	auto bail = [&](int code) {
		g_create_error = e->err;
		*out = e;  // caller may read rc_last_error(e) then destroy
		return code;
	};
	if(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking) != cudaSuccess)
		return bail(set_err(e, RC_ERR_CUDA, "stream creation failed"));
	{
		const cudaError_t c = configure_kernels();
		if(c != cudaSuccess) return bail(set_err(e, RC_ERR_CUDA, "kernel configuration failed: %s", cudaGetErrorString(c)));
	}
	e->stream = e->own_stream;

	DevParams &P = e->P;
	memset(&P, 0, sizeof(P));
	P.model = params->model;
	P.L = L;
	P.border = params->border > 0 ? params->border : 4;
	P.dt = params->dt;
	P.J0 = params->J0;
	P.conserved = params->conserved != 0;
	P.gamma = params->gamma;
	P.lambda = params->lambda;
	P.omega = params->omega;
	P.mu = params->mu;
	P.kappa = params->kappa;
	P.passive_alpha = params->passive_alpha;
	{
		float a0 = RC_PI_F * (float) params->R * (float) params->R;  // PI is a float literal (defs.h:4)
		P.a0 = (double) a0;
	}
	P.cg_tol = params->cg_tolerance;
	P.wall_slip = params->wall_slip;
	for(int k = 0; k < 2; k++) {
		e->ph[k].friction = params->friction[k];
		e->ph[k].friction_cell = params->friction_cell[k];
		e->ph[k].zs = params->zetaQ_self[k];
		e->ph[k].zi = params->zetaQ_inter[k];
		e->ph[k].JQ = params->J_Q[k];
		e->ph[k].beta = params->beta[k];
	}
	e->rep_on = (P.model == M_POLAR) && (params->J_Q[0] != 0.0 || params->J_Q[1] != 0.0);
	e->nbx = layers[0].nbx;
	e->nby = layers[0].nby;
	const size_t L2 = (size_t) total_box;  // box arrays of all layers (one layer for the wet paths)
	const size_t cap = (size_t) e->S_cap;
	// the update's per-site inputs are read through 16-byte aligned windows
	// (bulk copies) that may reach up to 8 bytes past the last site
	const size_t capw = cap + 8;
	const bool wet = (P.model == M_POLAR || P.model == M_WET);
	if((rc = dalloc(e, &e->cells, (size_t) std::max(n_cells, 1))) ||
	   (rc = dalloc(e, &e->phiA, capw)) || (rc = dalloc(e, &e->phiB, capw)) || (rc = dalloc(e, &e->dphi_old, capw)) ||
	   (rc = dalloc(e, &e->mu, cap)) || (rc = dalloc(e, &e->dxg, cap)) || (rc = dalloc(e, &e->dyg, cap)) ||
	   (rc = dalloc(e, &e->vx, capw)) || (rc = dalloc(e, &e->vy, capw)) || (rc = dalloc(e, &e->mapg, cap)) ||
	   (rc = dalloc(e, &e->phi2, L2)) || (rc = dalloc(e, &e->sq00, L2)) || (rc = dalloc(e, &e->sq01, L2)) ||
	   (rc = dalloc(e, &e->cnt, L2)) ||
	   (rc = dalloc(e, &e->bin_count, (size_t) total_bins)) || (rc = dalloc(e, &e->bin_layer, (size_t) total_bins)) ||
	   (rc = dalloc(e, &e->bin_cells, (size_t) total_bins * BIN_CAP)) ||
	   (rc = dalloc(e, &e->layers, (size_t) n_layers)) ||
	   (rc = dalloc(e, &e->tab_cos, (size_t) table_base(MAX_TABLE_SIDE + 1))) ||
	   (rc = dalloc(e, &e->tab_sin, (size_t) table_base(MAX_TABLE_SIDE + 1))) ||
	   (rc = dalloc(e, &e->tab_cosf, (size_t) table_base(MAX_TABLE_SIDE + 1))) ||
	   ((n_cells >= SPLIT_FINISH_CELLS || (any_wet && params->precision == RC_PRECISION_FLOAT)) &&
	    (rc = dalloc(e, &e->csum, (size_t) std::max(n_cells, 1)))) ||
	   (rc = dalloc(e, &e->tab_sinf, (size_t) table_base(MAX_TABLE_SIDE + 1))) ||
	   (rc = dalloc(e, &e->st, 1)) || (rc = dalloc(e, &e->st_save, 1)) ||
	   (rc = dalloc(e, &e->scratch_phi, cap + (size_t) n_cells / 2 + 8)) ||
	   (rc = dalloc(e, &e->rep, e->rep_on ? cap : 1)) || (rc = dalloc(e, &e->scratch_rep, e->rep_on ? cap : 1)))
		return bail(rc);
	if(params->precision == RC_PRECISION_FLOAT &&
	   ((rc = dalloc(e, &e->muf, capw)) || (rc = dalloc(e, &e->dxf, capw)) || (rc = dalloc(e, &e->dyf, capw))))
		return bail(rc);
	if(has_walls) {
		// the boxes' wall values (layers without walls stay zero)
		if((rc = dalloc(e, &e->walls, (size_t) total_box))) return bail(rc);
		for(int l = 0; l < n_layers; l++) {
			if(!boxes[l].walls) continue;
			const LayerDev &ly = layers[(size_t) l];
			const cudaError_t c = cudaMemcpy(e->walls + ly.box_off, boxes[l].walls, sizeof(double) * (size_t) ly.L * ly.L,
			                                 cudaMemcpyHostToDevice);
			if(c != cudaSuccess) return bail(set_err(e, RC_ERR_CUDA, "walls upload failed: %s", cudaGetErrorString(c)));
		}
	}
	if(wet) {
		if((rc = dalloc(e, &e->fx, cap)) || (rc = dalloc(e, &e->fy, cap)) || (rc = dalloc(e, &e->cover, L2 * STORE_MAX)) ||
		   (rc = dalloc(e, &e->cov_off, L2 + 1)) || (rc = dalloc(e, &e->cov_idx, cap)) ||
		   (rc = dalloc(e, &e->rx, cap)) || (rc = dalloc(e, &e->ry, cap)) || (rc = dalloc(e, &e->px, cap)) ||
		   (rc = dalloc(e, &e->py, cap)) ||
		   (rc = dalloc(e, &e->Px, L2)) || (rc = dalloc(e, &e->Py, L2)) ||
		   (rc = dalloc(e, &e->partials, 8 * 4096)) || (rc = dalloc(e, &e->scalars, 64)) || (rc = dalloc(e, &e->bar, 4)))
			return bail(rc);
		if(params->precision == RC_PRECISION_MIXED || params->precision == RC_PRECISION_FLOAT) {
			// FP32 inner iterations: the flexible CG in cover order, Jacobi-preconditioned
			if((rc = dalloc(e, &e->rxf, cap)) || (rc = dalloc(e, &e->ryf, cap)) || (rc = dalloc(e, &e->pxf, cap)) ||
			   (rc = dalloc(e, &e->pyf, cap)) || (rc = dalloc(e, &e->exf, cap)) || (rc = dalloc(e, &e->eyf, cap)) ||
			   (rc = dalloc(e, &e->apxf, cap)) || (rc = dalloc(e, &e->apyf, cap)) ||
			   (rc = dalloc(e, &e->Pxf, L2)) || (rc = dalloc(e, &e->Pyf, L2)) || (rc = dalloc(e, &e->zxf, cap)) ||
			   (rc = dalloc(e, &e->zyf, cap)) || (rc = dalloc(e, &e->Zxf, L2)) || (rc = dalloc(e, &e->Zyf, L2)) ||
			   (rc = dalloc(e, &e->Pxf2, L2)) || (rc = dalloc(e, &e->Pyf2, L2)))
				return bail(rc);
			e->cg_blocks_learned = cg_grid_blocks(device, true, (long long) L * L);
		}
		e->cg_blocks = cg_grid_blocks(device, false, (long long) L * L);
		// an ensemble's members keep their own solver bookkeeping (size_rows,
		// restart counter, cold-start flag), zeroed like DevStatus's
		if(n_layers > 1) {
			if((rc = dalloc(e, &e->lsolve, (size_t) n_layers))) return bail(rc);
			for(int l = 0; l < n_layers; l++) {
				const long long sites = (long long) layers[(size_t) l].L * layers[(size_t) l].L;
				e->layer_blocks[0].push_back(cg_grid_blocks(device, false, sites));
				e->layer_blocks[1].push_back(cg_grid_blocks(device, true, sites));
			}
		}
	}
	if(cudaMallocHost(&e->st_host, sizeof(DevStatus)) != cudaSuccess) return bail(set_err(e, RC_ERR_OOM, "pinned alloc failed"));

	// trig tables for the centre of mass, computed like the reference's
	// (MultiPhaseField.cpp:54-65: float argument, double cos/sin)
	{
		std::vector<double> tc(table_base(MAX_TABLE_SIDE + 1)), ts(tc.size());
		for(int l = 1; l <= MAX_TABLE_SIDE; l++)
			for(int i = 0; i < l; i++) {
				volatile float a = (2.0f * RC_PI_F * (float) i);
				volatile float b = a / (float) l;
				tc[table_base(l) + i] = cos((double) b);
				ts[table_base(l) + i] = sin((double) b);
			}
		CUDA_TRY(e, cudaMemcpy(e->tab_cos, tc.data(), sizeof(double) * tc.size(), cudaMemcpyHostToDevice));
		CUDA_TRY(e, cudaMemcpy(e->tab_sin, ts.data(), sizeof(double) * ts.size(), cudaMemcpyHostToDevice));
		std::vector<float> tcf(tc.begin(), tc.end()), tsf(ts.begin(), ts.end());
		CUDA_TRY(e, cudaMemcpy(e->tab_cosf, tcf.data(), sizeof(float) * tcf.size(), cudaMemcpyHostToDevice));
		CUDA_TRY(e, cudaMemcpy(e->tab_sinf, tsf.data(), sizeof(float) * tsf.size(), cudaMemcpyHostToDevice));
	}
	// cells and fields
	{
		std::vector<CellDev> hc((size_t) std::max(n_cells, 1));
		std::vector<double> phi(gen ? 0 : (size_t) S);
		long long start = 0;
		for(int i = 0; i < n_cells; i++) {
			int layer = 0;
			while(layer + 1 < n_layers && i >= layers[(size_t) layer].cell_hi) layer++;
			host_cell(cells[i], hc[i], (int) start, layer);
			if(!gen) memcpy(&phi[(size_t) start], cells[i].phi, sizeof(double) * (size_t) hc[i].n);
			start += hc[i].n;
		}
		CUDA_TRY(e, cudaMemcpy(e->cells, hc.data(), sizeof(CellDev) * (size_t) std::max(n_cells, 1), cudaMemcpyHostToDevice));
		CUDA_TRY(e, cudaMemcpy(e->layers, layers.data(), sizeof(LayerDev) * (size_t) n_layers, cudaMemcpyHostToDevice));
		{
			// bin -> layer, so that a bin's CTA finds its layer with one load
			std::vector<int> bl((size_t) total_bins);
			for(int l = 0; l < n_layers; l++)
				for(int b = 0; b < layers[(size_t) l].nbx * layers[(size_t) l].nby; b++) bl[(size_t) (layers[(size_t) l].bin_off + b)] = l;
			CUDA_TRY(e, cudaMemcpy(e->bin_layer, bl.data(), sizeof(int) * (size_t) total_bins, cudaMemcpyHostToDevice));
		}
		if(S && !gen) CUDA_TRY(e, cudaMemcpy(e->phiA, phi.data(), sizeof(double) * (size_t) S, cudaMemcpyHostToDevice));
		if(S && gen) {
			generate_phi_kernel<<<n_cells, 256, 0, e->stream>>>(e->cells, e->phiA, *gen, L);
			CUDA_TRY(e, cudaGetLastError());
		}
		DevStatus h;
		memset(&h, 0, sizeof(h));
		h.S = S;
		h.S_rows = 0;
		h.restart = 0;
		h.max_n = max_n;
		CUDA_TRY(e, cudaMemcpy(e->st, &h, sizeof(h), cudaMemcpyHostToDevice));
	}
	if((rc = choose_smem(e))) return bail(rc);
	if(n_cells > 0) {
		init_sums_kernel<<<(n_cells + 63) / 64, 64, 0, e->stream>>>(
		    e->cells, e->layers, e->phiA, n_cells, P.model == M_NEMATIC ? nullptr : e->walls, P.wall_slip);
		launch_bins(e->cells, e->layers, n_cells, e->bin_count, e->bin_cells, total_bins, e->st, e->stream);
		// FD_CPUBackend::init: first force evaluation with the phase-0 parameters
		evaluate_end(e, e->phiA, 0);
	}
	if((rc = check_status(e, nullptr))) return bail(rc);
	*out = e;
	return RC_OK;
}

extern "C" {

int rc_step(rc_engine *e, int n_steps, rc_step_stats *stats) {
	if(!e) return RC_ERR_INVALID;
	if(n_steps < 0) return set_err(e, RC_ERR_INVALID, "n_steps < 0");
	if(stats) memset(stats, 0, sizeof(*stats));
	CUDA_TRY(e, cudaSetDevice(e->device));
	int rc = check_status(e, nullptr);  // errors of earlier async work; resets the counters
	if(rc) return rc;
	const int chunk = 16;
	int done = 0;
	while(done < n_steps) {
		if((rc = choose_smem(e))) return rc;
		const int m = std::min(chunk, n_steps - done);
		for(int i = 0; i < m; i++) run_step(e);
		rc = check_status(e, stats);
		if(rc) break;
		done += m;
	}
	if(stats) stats->steps_done = done;
	return rc;
}

int rc_step_async(rc_engine *e, int n_steps) {
	if(!e) return RC_ERR_INVALID;
	if(n_steps < 0) return set_err(e, RC_ERR_INVALID, "n_steps < 0");
	CUDA_TRY(e, cudaSetDevice(e->device));
	int rc = choose_smem(e);
	if(rc) return rc;
	for(int i = 0; i < n_steps; i++) run_step(e);
	e->async_steps += n_steps;
	return RC_OK;
}

int rc_wait(rc_engine *e, rc_step_stats *stats) {
	if(!e) return RC_ERR_INVALID;
	if(stats) memset(stats, 0, sizeof(*stats));
	CUDA_TRY(e, cudaSetDevice(e->device));
	const int rc = check_status(e, stats);
	if(stats) stats->steps_done = e->async_steps;
	e->async_steps = 0;
	return rc;
}

int rc_set_cell_threads(rc_engine *e, int threads) {
	if(!e) return RC_ERR_INVALID;
	bool ok = false;
	for(int b : CELL_F32_BLOCKS) ok = ok || b == threads;
	if(!ok) return set_err(e, RC_ERR_INVALID, "rc_set_cell_threads: %d is not one of 128, 256, 512", threads);
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	if(threads != e->f32_block) {
		e->f32_block = threads;
		drop_graphs(e);
	}
	return RC_OK;
}

int rc_autotune(rc_engine *e, int steps_per_candidate, rc_autotune_report *report) {
	if(!e || steps_per_candidate < 1) return RC_ERR_INVALID;
	rc_autotune_report r;
	memset(&r, 0, sizeof(r));
	r.chosen = e->hp.precision == RC_PRECISION_FLOAT ? e->f32_block : CELL_THREADS;
	if(e->hp.precision != RC_PRECISION_FLOAT) {
		if(report) *report = r;
		return RC_OK;
	}
	CUDA_TRY(e, cudaSetDevice(e->device));
	// each candidate is timed by the stage timers of the launches the tile
	// changes (the cell kernels: updates and force evaluations), so that the
	// viscous solve's run-to-run spread does not decide the tile
	const bool was_timing = e->timing;
	int rc = RC_OK, best = -1;
	for(int b : CELL_F32_BLOCKS) {
		if((rc = rc_set_cell_threads(e, b))) break;
		if((rc = rc_step(e, 1, nullptr))) break;  // one untimed step with this tile
		e->timing = true;
		if((rc = rc_timers(e, nullptr, nullptr, 1))) break;
		if((rc = rc_step(e, steps_per_candidate, nullptr))) break;
		double ms[RC_NUM_TIMERS];
		if((rc = rc_timers(e, ms, nullptr, 1))) break;
		e->timing = was_timing;
		r.threads[r.candidates] = b;
		r.ms_per_step[r.candidates] = (ms[RC_TIMER_UPDATE] + ms[RC_TIMER_FORCES]) / steps_per_candidate;
		if(best < 0 || r.ms_per_step[r.candidates] < r.ms_per_step[best]) best = r.candidates;
		r.candidates++;
	}
	e->timing = was_timing;
	if(rc) return rc;
	if((rc = rc_set_cell_threads(e, r.threads[best]))) return rc;
	r.chosen = e->f32_block;
	if(report) *report = r;
	return RC_OK;
}

int rc_download_phi(rc_engine *e, double *phi, long long n) {
	if(!e || (!phi && n > 0)) return RC_ERR_INVALID;
	if(n != e->S) return set_err(e, RC_ERR_INVALID, "rc_download_phi: n = %lld but the state has %lld sites", n, e->S);
	CUDA_TRY(e, cudaSetDevice(e->device));
	if(n) CUDA_TRY(e, cudaMemcpyAsync(phi, e->phiA, sizeof(double) * (size_t) n, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_upload_phi(rc_engine *e, const double *phi, long long n) {
	if(!e || (!phi && n > 0)) return RC_ERR_INVALID;
	if(n != e->S) return set_err(e, RC_ERR_INVALID, "rc_upload_phi: n = %lld but the state has %lld sites", n, e->S);
	CUDA_TRY(e, cudaSetDevice(e->device));
	materialise(e, 1);
	if(n) CUDA_TRY(e, cudaMemcpyAsync(e->phiA, phi, sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_set_phase(rc_engine *e, int active) {
	if(!e) return RC_ERR_INVALID;
	e->phase = active ? 1 : 0;
	return RC_OK;
}

int rc_get_sizes(const rc_engine *e, int *n_cells, int *lsub_x, int *lsub_y) {
	if(!e) return RC_ERR_INVALID;
	if(n_cells) *n_cells = e->N;
	if(lsub_x || lsub_y) {
		std::vector<CellDev> hc((size_t) std::max(e->N, 1));
		if(cudaMemcpy(hc.data(), e->cells, sizeof(CellDev) * (size_t) std::max(e->N, 1), cudaMemcpyDeviceToHost) != cudaSuccess)
			return RC_ERR_CUDA;
		for(int i = 0; i < e->N; i++) {
			if(lsub_x) lsub_x[i] = hc[i].lx;
			if(lsub_y) lsub_y[i] = hc[i].ly;
		}
	}
	return RC_OK;
}

// FP32 engines keep mu and the gradients in FP32: widen them into the FP64
// arrays that downloads and observables read.
static void widen_fields(rc_engine *e) {
	if(e->muf) launch_widen3(e->muf, e->dxf, e->dyf, e->mu, e->dxg, e->dyg, e->S_cap, e->stream);
}

int rc_download(rc_engine *e, rc_cell_host *cells, unsigned mask) {
	if(!e || (!cells && e->N > 0)) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	materialise(e, 0);
	if(mask & (RC_FIELD_MU | RC_FIELD_GRAD)) widen_fields(e);
	std::vector<CellDev> hc((size_t) std::max(e->N, 1));
	CUDA_TRY(e, cudaMemcpyAsync(hc.data(), e->cells, sizeof(CellDev) * (size_t) std::max(e->N, 1), cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	const bool dry_vel = !wet_phase(e, e->eval_phase);
	(void) dry_vel;
	for(int i = 0; i < e->N; i++) {
		const CellDev &c = hc[i];
		rc_cell_host &h = cells[i];
		if(mask & RC_FIELD_SCALARS) {
			h.lsub_x = c.lx;
			h.lsub_y = c.ly;
			h.offset_x = c.offx;
			h.offset_y = c.offy;
			h.corner = c.corner;
			h.type = c.type;
			h.com_x = c.comx;
			h.com_y = c.comy;
			h.unrap_x = c.unrapx;
			h.unrap_y = c.unrapy;
			h.q00 = c.q00;
			h.q01 = c.q01;
			h.theta_q = c.thq;
			h.theta_q_old = c.thq_old;
			h.nemq_x = c.nqx;
			h.nemq_y = c.nqy;
			h.nemq_old_x = c.nq_oldx;
			h.nemq_old_y = c.nq_oldy;
			h.area = c.area;
			h.sum_f = c.sumf;
			h.perimeter = c.perim;
			h.s00 = c.s00;
			h.s01 = c.s01;
			h.force_rep_x = c.trx;
			h.force_rep_y = c.try_;
		}
		if(mask & ~RC_FIELD_SCALARS) {
			if(h.capacity < c.n) return set_err(e, RC_ERR_INVALID, "cell %d: capacity %d < %d sites", i, h.capacity, c.n);
			const size_t nb = sizeof(double) * (size_t) c.n;
			if((mask & RC_FIELD_PHI) && h.phi) CUDA_TRY(e, cudaMemcpyAsync(h.phi, e->phiA + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
			if(mask & RC_FIELD_VEL) {
				if(h.vx) CUDA_TRY(e, cudaMemcpyAsync(h.vx, e->vx + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
				if(h.vy) CUDA_TRY(e, cudaMemcpyAsync(h.vy, e->vy + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
			}
			if((mask & RC_FIELD_MU) && h.mu) CUDA_TRY(e, cudaMemcpyAsync(h.mu, e->mu + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
			if(mask & RC_FIELD_GRAD) {
				if(h.dx) CUDA_TRY(e, cudaMemcpyAsync(h.dx, e->dxg + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
				if(h.dy) CUDA_TRY(e, cudaMemcpyAsync(h.dy, e->dyg + c.start, nb, cudaMemcpyDeviceToHost, e->stream));
			}
			if((mask & RC_FIELD_MAP) && h.box_index)
				CUDA_TRY(e, cudaMemcpyAsync(h.box_index, e->mapg + c.start, sizeof(int) * (size_t) c.n, cudaMemcpyDeviceToHost, e->stream));
		}
	}
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_upload(rc_engine *e, const rc_cell_host *cells, unsigned mask) {
	if(!e || (!cells && e->N > 0)) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	// the forces of the last evaluation belong to the state before the edit,
	// as on the CPU backend: make them concrete first
	materialise(e, 1);
	std::vector<CellDev> hc((size_t) std::max(e->N, 1));
	CUDA_TRY(e, cudaMemcpyAsync(hc.data(), e->cells, sizeof(CellDev) * (size_t) std::max(e->N, 1), cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	for(int i = 0; i < e->N; i++) {
		CellDev &c = hc[i];
		const rc_cell_host &h = cells[i];
		if(mask & RC_FIELD_SCALARS) {
			if(h.lsub_x != c.lx || h.lsub_y != c.ly) return set_err(e, RC_ERR_INVALID, "cell %d: patch size cannot change on upload", i);
			CellDev n;
			host_cell(h, n, c.start, c.layer);
			n.area = h.area;
			n.sumf = h.sum_f;
			n.perim = h.perimeter;
			n.s00 = h.s00;
			n.s01 = h.s01;
			n.trx = h.force_rep_x;
			n.try_ = h.force_rep_y;
			n.area_old = c.area_old;
			n.sumf_old = c.sumf_old;
			n.com_oldx = c.com_oldx;
			n.com_oldy = c.com_oldy;
			c = n;
		}
		if((mask & RC_FIELD_PHI) && h.phi)
			CUDA_TRY(e, cudaMemcpyAsync(e->phiA + c.start, h.phi, sizeof(double) * (size_t) c.n, cudaMemcpyHostToDevice, e->stream));
	}
	if(mask & RC_FIELD_SCALARS) {
		CUDA_TRY(e, cudaMemcpyAsync(e->cells, hc.data(), sizeof(CellDev) * (size_t) std::max(e->N, 1), cudaMemcpyHostToDevice, e->stream));
		launch_bins(e->cells, e->layers, e->N, e->bin_count, e->bin_cells, e->total_bins, e->st, e->stream);
	}
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_set_timing(rc_engine *e, int enable) {
	if(!e) return RC_ERR_INVALID;
	e->timing = enable != 0;
	return RC_OK;
}

int rc_timers(rc_engine *e, double *ms, long long *launches, int reset) {
	if(!e) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	collect_marks(e);
	for(int i = 0; i < RC_NUM_TIMERS; i++) {
		if(ms) ms[i] = e->timer_ms[i];
		if(launches) launches[i] = e->timer_n[i];
		if(reset) {
			e->timer_ms[i] = 0;
			e->timer_n[i] = 0;
		}
	}
	return RC_OK;
}

int rc_set_stream(rc_engine *e, void *cuda_stream) {
	if(!e) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	e->stream = cuda_stream ? (cudaStream_t) cuda_stream : e->own_stream;
	return RC_OK;
}

// --- learned preconditioner -----------------------------------------------------

static void dfree(rc_engine *e, void *p) {
	if(!p) return;
	cudaFree(p);
	e->allocs.erase(std::remove(e->allocs.begin(), e->allocs.end(), p), e->allocs.end());
}


static bool is_wet_engine(const rc_engine *e) { return e->fx != nullptr; }

int rc_learned_harvest(rc_engine *e, int capacity, int every, int per_solve) {
	if(!e) return RC_ERR_INVALID;
	if(!is_wet_engine(e)) return set_err(e, RC_ERR_UNSUPPORTED, "rc_learned_harvest: the engine has no viscous solve");
	if(e->n_layers > 1) return set_err(e, RC_ERR_UNSUPPORTED, "rc_learned_harvest: not provided for ensembles");
	if(per_solve == 0 && capacity > 0) {
		// stop collecting, keep the stored samples
		CUDA_TRY(e, cudaSetDevice(e->device));
		CUDA_TRY(e, cudaStreamSynchronize(e->stream));
		if(e->harv_collect) drop_graphs(e);
		e->harv_collect = false;
		return RC_OK;
	}
	if(capacity < 0 || (capacity > 0 && (every < 1 || per_solve < 1)))
		return set_err(e, RC_ERR_INVALID, "rc_learned_harvest: capacity %d, every %d, per_solve %d", capacity, every, per_solve);
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	dfree(e, e->harv_in);
	dfree(e, e->harv_tgt);
	dfree(e, e->harv_s);
	dfree(e, e->harv_count);
	e->harv_in = e->harv_tgt = e->harv_s = nullptr;
	e->harv_count = nullptr;
	e->harv_cap = 0;
	e->harv_collect = false;
	drop_graphs(e);
	if(capacity == 0) return RC_OK;
	const size_t L2 = (size_t) e->L * e->L;
	int rc;
	if((rc = dalloc(e, &e->harv_in, (size_t) capacity * L2 * 2)) || (rc = dalloc(e, &e->harv_tgt, (size_t) capacity * L2)) ||
	   (rc = dalloc(e, &e->harv_s, (size_t) capacity)) || (rc = dalloc(e, &e->harv_count, 1)))
		return rc;
	e->harv_cap = capacity;
	e->harv_every = every;
	e->harv_per_solve = per_solve;
	e->harv_collect = true;
	return RC_OK;
}

int rc_learned_harvested(rc_engine *e) {
	if(!e || !e->harv_count) return 0;
	int n = 0;
	cudaSetDevice(e->device);
	cudaStreamSynchronize(e->stream);
	if(cudaMemcpy(&n, e->harv_count, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
	return n;
}

static unsigned long long splitmix(unsigned long long &x) {
	unsigned long long z = (x += 0x9E3779B97F4A7C15ULL);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
	return z ^ (z >> 31);
}

static void shuffle(std::vector<int> &v, unsigned long long &st) {
	for(size_t i = v.size(); i > 1; i--) {
		const size_t j = (size_t) (splitmix(st) % i);
		std::swap(v[i - 1], v[j]);
	}
}

// He initialisation: normal(0, sqrt(2 / (9 c_in))) weights (Box-Muller on
// splitmix64 uniforms), zero biases.
static void init_params(std::vector<float> &p, unsigned long long seed) {
	unsigned long long st = seed ^ 0x5DEECE66DULL;
	p.assign(UNET_PARAMS, 0.f);
	for(int l = 0; l < UNET_LAYERS; l++) {
		const UNetLayerDesc d = unet_layer(l);
		const double sd = sqrt(2.0 / (9.0 * d.ci));
		const int n = 9 * d.ci * d.co;
		for(int k = 0; k < n; k++) {
			const double u1 = ((splitmix(st) >> 11) + 0.5) / 9007199254740992.0;
			const double u2 = ((splitmix(st) >> 11) + 0.5) / 9007199254740992.0;
			p[(size_t) unet_weight_offset(l) + k] = (float) (sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
		}
	}
}

// mean loss of the network in T over samples idx (device copy in didx)
static double eval_loss(UNetTrainer &T, rc_engine *e, const std::vector<int> &idx, int *didx, double *dacc, int cap) {
	if(idx.empty()) return 0.0;
	cudaMemsetAsync(dacc, 0, sizeof(double), e->stream);
	cudaMemcpyAsync(didx, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, e->stream);
	for(size_t b0 = 0; b0 < idx.size(); b0 += (size_t) cap) {
		const int n = (int) std::min((size_t) cap, idx.size() - b0);
		T.batch = n;
		unet_gather(T, e->harv_in, e->harv_tgt, didx + b0, n, e->stream);
		unet_forward(T, T.params, e->stream);
		unet_loss(T, e->stream);
		unet_accumulate_loss(T, dacc, e->stream);
	}
	T.batch = cap;
	double h = 0.0;
	cudaMemcpyAsync(&h, dacc, sizeof(double), cudaMemcpyDeviceToHost, e->stream);
	cudaStreamSynchronize(e->stream);
	return h / (double) idx.size();
}

int rc_learned_train(rc_engine *e, const rc_train_options *o, rc_train_report *rep) {
	if(!e || !o) return RC_ERR_INVALID;
	if(!e->harv_count) return set_err(e, RC_ERR_INVALID, "rc_learned_train: no harvested samples (call rc_learned_harvest first)");
	if(e->L % 4 != 0 || e->L < 8) return set_err(e, RC_ERR_UNSUPPORTED, "rc_learned_train: box side %d is not a multiple of 4", e->L);
	const int epochs = o->epochs > 0 ? o->epochs : 8;
	const int batch = o->batch > 0 ? o->batch : 8;
	const float lr = (float) (o->learning_rate > 0 ? o->learning_rate : 1e-3);
	const double vfrac = o->validation >= 0 ? o->validation : 0.1;
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	const auto t0 = std::chrono::steady_clock::now();
	int count = 0;
	CUDA_TRY(e, cudaMemcpy(&count, e->harv_count, sizeof(int), cudaMemcpyDeviceToHost));
	std::vector<float> sc((size_t) std::max(count, 1));
	if(count) CUDA_TRY(e, cudaMemcpy(sc.data(), e->harv_s, sizeof(float) * (size_t) count, cudaMemcpyDeviceToHost));
	std::vector<int> valid;
	for(int q = 0; q < count; q++)
		if(sc[(size_t) q] > 0.f) valid.push_back(q);
	unsigned long long st = o->seed;
	shuffle(valid, st);
	if(o->max_samples > 0 && (int) valid.size() > o->max_samples) valid.resize((size_t) o->max_samples);
	if(valid.size() < 2) return set_err(e, RC_ERR_INVALID, "rc_learned_train: %zu usable samples", valid.size());
	int nval = (int) llround(vfrac * (double) valid.size());
	if(vfrac > 0 && nval < 1) nval = 1;
	if(nval >= (int) valid.size()) nval = (int) valid.size() - 1;
	std::vector<int> val(valid.begin(), valid.begin() + nval), train(valid.begin() + nval, valid.end());
	UNetTrainer T;
	const int rc0 = unet_trainer_init(T, e->L, batch);
	if(rc0) {
		unet_trainer_free(T);
		return set_err(e, rc0 == -2 ? RC_ERR_INVALID : RC_ERR_OOM, "rc_learned_train: trainer allocation failed");
	}
	int *didx = nullptr;
	double *dacc = nullptr;
	if(cudaMalloc(&didx, sizeof(int) * valid.size()) != cudaSuccess || cudaMalloc(&dacc, sizeof(double)) != cudaSuccess) {
		cudaFree(didx);
		unet_trainer_free(T);
		return set_err(e, RC_ERR_OOM, "rc_learned_train: allocation failed");
	}
	if(o->init || !e->unet_params) {
		std::vector<float> p;
		init_params(p, o->seed);
		cudaMemcpy(T.params, p.data(), sizeof(float) * UNET_PARAMS, cudaMemcpyHostToDevice);
	}
	else
		cudaMemcpy(T.params, e->unet_params, sizeof(float) * UNET_PARAMS, cudaMemcpyDeviceToDevice);
	rc_train_report r;
	memset(&r, 0, sizeof(r));
	r.samples = (int) valid.size();
	r.train_samples = (int) train.size();
	r.validation_samples = (int) val.size();
	r.validation_loss_init = eval_loss(T, e, val, didx, dacc, batch);
	const long long total_steps = (long long) epochs * (long long) ((train.size() + batch - 1) / batch);
	const double lr_final = o->learning_rate_final > 0 ? o->learning_rate_final : (double) lr;
	for(int ep = 0; ep < epochs; ep++) {
		shuffle(train, st);
		cudaMemsetAsync(dacc, 0, sizeof(double), e->stream);
		cudaMemcpyAsync(didx, train.data(), sizeof(int) * train.size(), cudaMemcpyHostToDevice, e->stream);
		for(size_t b0 = 0; b0 < train.size(); b0 += (size_t) batch) {
			const int n = (int) std::min((size_t) batch, train.size() - b0);
			T.batch = n;
			unet_gather(T, e->harv_in, e->harv_tgt, didx + b0, n, e->stream);
			unet_forward(T, T.params, e->stream);
			unet_loss(T, e->stream);
			unet_accumulate_loss(T, dacc, e->stream);
			unet_backward(T, T.params, e->stream);
			// cosine decay from lr to lr_final over the run
			const double frac = total_steps > 1 ? (double) r.steps / (double) (total_steps - 1) : 0.0;
			const double lr_k = lr_final + 0.5 * ((double) lr - lr_final) * (1.0 + cos(3.141592653589793 * frac));
			unet_adam(T, (float) lr_k, e->stream);
			r.steps++;
		}
		T.batch = batch;
		double h = 0.0;
		cudaMemcpyAsync(&h, dacc, sizeof(double), cudaMemcpyDeviceToHost, e->stream);
		cudaStreamSynchronize(e->stream);
		const double mean = h / (double) train.size();
		if(ep == 0) r.loss_first_epoch = mean;
		r.loss_last_epoch = mean;
		r.epochs = ep + 1;
	}
	r.validation_loss = eval_loss(T, e, val, didx, dacc, batch);
	int rc = RC_OK;
	if(!e->unet_params) rc = dalloc(e, &e->unet_params, UNET_PARAMS);
	if(rc == RC_OK) cudaMemcpyAsync(e->unet_params, T.params, sizeof(float) * UNET_PARAMS, cudaMemcpyDeviceToDevice, e->stream);
	if(rc == RC_OK && e->unet_pack) unet_pack_bf16(e->unet_params, e->unet_pack, e->stream);
	const cudaError_t ce = cudaStreamSynchronize(e->stream);
	cudaFree(didx);
	cudaFree(dacc);
	unet_trainer_free(T);
	if(rc) return rc;
	if(ce != cudaSuccess) return set_err(e, RC_ERR_CUDA, "rc_learned_train: %s", cudaGetErrorString(ce));
	r.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
	if(rep) *rep = r;
	return RC_OK;
}

int rc_learned_get_params(rc_engine *e, double *params) {
	if(!e || !params) return RC_ERR_INVALID;
	if(!e->unet_params) return set_err(e, RC_ERR_INVALID, "rc_learned_get_params: the engine has no network parameters");
	CUDA_TRY(e, cudaSetDevice(e->device));
	std::vector<float> h(UNET_PARAMS);
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	CUDA_TRY(e, cudaMemcpy(h.data(), e->unet_params, sizeof(float) * UNET_PARAMS, cudaMemcpyDeviceToHost));
	for(int k = 0; k < UNET_PARAMS; k++) params[k] = h[(size_t) k];
	return RC_OK;
}

int rc_learned_set_params(rc_engine *e, const double *params) {
	if(!e || !params) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	int rc;
	if(!e->unet_params && (rc = dalloc(e, &e->unet_params, UNET_PARAMS))) return rc;
	std::vector<float> h(UNET_PARAMS);
	for(int k = 0; k < UNET_PARAMS; k++) h[(size_t) k] = (float) params[k];
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	CUDA_TRY(e, cudaMemcpy(e->unet_params, h.data(), sizeof(float) * UNET_PARAMS, cudaMemcpyHostToDevice));
	if(e->unet_pack) {
		unet_pack_bf16(e->unet_params, e->unet_pack, e->stream);
		CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	}
	return RC_OK;
}

}  // extern "C"

// Work arrays of `solver` (allocated on first use; the stream must be idle).
static int prepare_solver(rc_engine *e, int solver, const char *who) {
	if(solver != RC_SOLVER_PLAIN && solver != RC_SOLVER_LEARNED && solver != RC_SOLVER_LEARNED_FP32 &&
	   solver != RC_SOLVER_PLAIN_FP64)
		return set_err(e, RC_ERR_INVALID, "%s: unknown solver %d", who, solver);
	if(solver == RC_SOLVER_PLAIN_FP64 && !is_wet_engine(e))
		return set_err(e, RC_ERR_UNSUPPORTED, "%s: the engine has no viscous solve", who);
	if(solver != RC_SOLVER_PLAIN && e->n_layers > 1)
		return set_err(e, RC_ERR_UNSUPPORTED, "%s: ensembles solve each member with the engine's plain solver only", who);
	if(solver == RC_SOLVER_LEARNED || solver == RC_SOLVER_LEARNED_FP32) {
		if(!is_wet_engine(e)) return set_err(e, RC_ERR_UNSUPPORTED, "%s: the engine has no viscous solve", who);
		if(e->L % 4 != 0 || e->L < 8)
			return set_err(e, RC_ERR_UNSUPPORTED, "%s: box side %d is not a multiple of 4", who, e->L);
		if(!e->unet_params) return set_err(e, RC_ERR_INVALID, "%s: no network parameters (train or set them first)", who);
		const size_t cap = (size_t) e->S_cap, L2 = (size_t) e->L * e->L;
		int rc;
		if(!e->rxf) {
			if((rc = dalloc(e, &e->rxf, cap)) || (rc = dalloc(e, &e->ryf, cap)) || (rc = dalloc(e, &e->pxf, cap)) ||
			   (rc = dalloc(e, &e->pyf, cap)) || (rc = dalloc(e, &e->exf, cap)) || (rc = dalloc(e, &e->eyf, cap)) ||
			   (rc = dalloc(e, &e->apxf, cap)) || (rc = dalloc(e, &e->apyf, cap)) || (rc = dalloc(e, &e->Pxf, L2)) ||
			   (rc = dalloc(e, &e->Pyf, L2)))
				return rc;
		}
		if(!e->zxf) {
			if((rc = dalloc(e, &e->zxf, cap)) || (rc = dalloc(e, &e->zyf, cap)) || (rc = dalloc(e, &e->Zxf, L2)) ||
			   (rc = dalloc(e, &e->Zyf, L2)) || (rc = dalloc(e, &e->Pxf2, L2)) || (rc = dalloc(e, &e->Pyf2, L2)))
				return rc;
		}
		if(!e->unet.x0) {
			const size_t p0 = 2 * L2, p1 = p0 / 4, p2 = p0 / 16;
			UNetActs &A = e->unet;
			if((rc = dalloc(e, &A.x0, p0 * 2)) ||
			   (rc = dalloc(e, &A.e0a, p0 * 16)) || (rc = dalloc(e, &A.s0, p0 * 16)) || (rc = dalloc(e, &A.d0a, p0 * 16)) ||
			   (rc = dalloc(e, &A.t0, p0 * 16)) || (rc = dalloc(e, &A.out, p0)) || (rc = dalloc(e, &A.e1a, p1 * 16)) ||
			   (rc = dalloc(e, &A.s1, p1 * 16)) || (rc = dalloc(e, &A.d1a, p1 * 16)) || (rc = dalloc(e, &A.t1, p1 * 16)) ||
			   (rc = dalloc(e, &A.b0, p2 * 16)) || (rc = dalloc(e, &A.t2, p2 * 16)))
				return rc;
		}
		if(solver == RC_SOLVER_LEARNED && !e->unet_pack) {
			const size_t p0 = 2 * L2, p1 = p0 / 4, p2 = p0 / 16;
			UNetActsBF &B = e->unet_bf;
			if((rc = dalloc(e, &e->unet_pack, UNET_PACKED)) || (rc = dalloc(e, &B.e0a, p0 * 16)) ||
			   (rc = dalloc(e, &B.s0, p0 * 16)) || (rc = dalloc(e, &B.d0a, p0 * 16)) || (rc = dalloc(e, &B.t0, p0 * 16)) ||
			   (rc = dalloc(e, &B.e1a, p1 * 16)) || (rc = dalloc(e, &B.s1, p1 * 16)) || (rc = dalloc(e, &B.d1a, p1 * 16)) ||
			   (rc = dalloc(e, &B.t1, p1 * 16)) || (rc = dalloc(e, &B.b0, p2 * 16)) || (rc = dalloc(e, &B.t2, p2 * 16)))
				return rc;
			unet_pack_bf16(e->unet_params, e->unet_pack, e->stream);
			CUDA_TRY(e, cudaStreamSynchronize(e->stream));
		}
		if(!e->cg_blocks_learned) e->cg_blocks_learned = cg_grid_blocks(e->device, true, (long long) e->L * e->L);
	}
	return RC_OK;
}

extern "C" {

int rc_set_solver(rc_engine *e, int solver) {
	if(!e) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	const int rc = prepare_solver(e, solver, "rc_set_solver");
	if(rc) return rc;
	if(solver != e->solver) drop_graphs(e);
	e->solver = solver;
	return RC_OK;
}

int rc_set_cg_limits(rc_engine *e, long long max_iterations, int fail_on_no_convergence) {
	if(!e) return RC_ERR_INVALID;
	if(max_iterations < 0) return set_err(e, RC_ERR_INVALID, "rc_set_cg_limits: max_iterations %lld < 0", max_iterations);
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	drop_graphs(e);
	e->cg_max_iters = max_iterations;
	e->cg_fail_noconv = fail_on_no_convergence != 0;
	return RC_OK;
}

int rc_set_cg_tolerance(rc_engine *e, double tolerance) {
	if(!e) return RC_ERR_INVALID;
	if(!(tolerance >= 0.0) || !std::isfinite(tolerance))
		return set_err(e, RC_ERR_INVALID, "rc_set_cg_tolerance: tolerance %g is not a finite value >= 0", tolerance);
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	drop_graphs(e);
	e->hp.cg_tolerance = tolerance;
	return RC_OK;
}

int rc_test_barrier_timeout(rc_engine *e, long long spin_limit, int unreachable) {
	if(!e) return RC_ERR_INVALID;
	if(spin_limit < 0) return set_err(e, RC_ERR_INVALID, "rc_test_barrier_timeout: spin_limit %lld < 0", spin_limit);
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	drop_graphs(e);
	e->spin_limit = spin_limit;
	e->barrier_extra = unreachable ? 1 : 0;
	return RC_OK;
}

}  // extern "C"

// A re-solve starts cold with zeroed counters and no error; S and the rest of
// the record are the engine's (kept aside and put back after the solve).
__global__ void resolve_status_kernel(DevStatus *st) {
	if(threadIdx.x == 0 && blockIdx.x == 0) {
		st->err = 0;
		st->cg_cold = 1;
		st->cg_solves = st->cg_iters = st->cg_max_iters = st->refinements = st->fallbacks = 0;
		st->cg_max_rel = 0.0;
	}
}

extern "C" {

/*
 * rc_viscous_resolve: the viscous solve of the last force evaluation run
 * again from a cold start with `solver` into caller-owned device arrays; the
 * engine's own velocities, warm-start schedule and counters are left as they
 * were.  It compares solvers on one right-hand side (the learned flexible CG
 * against the plain FP64 CG) without advancing the simulation.  No
 * counterpart in the reference.
 */
int rc_viscous_resolve(rc_engine *e, int solver, double *vx, double *vy, long long n, rc_step_stats *stats) {
	if(!e) return RC_ERR_INVALID;
	if(!vx || !vy) return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve: NULL output array");
	if(n != e->S) return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve: n = %lld but the state has %lld unknowns", n, e->S);
	if(e->n_layers > 1) return set_err(e, RC_ERR_UNSUPPORTED, "rc_viscous_resolve: not provided for ensembles");
	if(e->pending || !wet_phase(e, e->eval_phase))
		return set_err(e, RC_ERR_UNSUPPORTED, "rc_viscous_resolve: the last evaluation had no viscous solve");
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	int rc = prepare_solver(e, solver, "rc_viscous_resolve");
	if(rc) return rc;
	CUDA_TRY(e, cudaMemcpyAsync(e->st_save, e->st, sizeof(DevStatus), cudaMemcpyDeviceToDevice, e->stream));
	resolve_status_kernel<<<1, 32, 0, e->stream>>>(e->st);
	CUDA_TRY(e, cudaGetLastError());
	CUDA_TRY(e, cudaMemsetAsync(e->bar, 0, sizeof(unsigned) * 4, e->stream));
	CGArgs g;
	const int blocks = solve_args(e, e->eval_phase, solver, false, vx, vy, g);
	g.phase_ns = nullptr;
	CUDA_TRY(e, launch_cg(g, blocks, e->stream));
	DevStatus h;
	CUDA_TRY(e, cudaMemcpyAsync(&h, e->st, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaMemcpyAsync(e->st, e->st_save, sizeof(DevStatus), cudaMemcpyDeviceToDevice, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	if(stats) {
		memset(stats, 0, sizeof(*stats));
		stats->cg_solves = h.cg_solves;
		stats->cg_iterations = h.cg_iters;
		stats->cg_max_iterations = h.cg_max_iters;
		stats->cg_max_rel_residual = h.cg_max_rel;
		stats->refinements = h.refinements;
		stats->fallbacks = h.fallbacks;
		stats->kernel_launches = 2;
	}
	if(h.err & ERR_BARRIER) return set_err(e, RC_ERR_CG, "rc_viscous_resolve: grid barrier timed out");
	if(h.err & ERR_MMA) return set_err(e, RC_ERR_CG, "rc_viscous_resolve: tensor-core completion wait timed out");
	if(h.err & ERR_NOCONV) return set_err(e, RC_ERR_CG, "rc_viscous_resolve: tolerance not reached within the iteration cap");
	if(h.err) return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve: device error 0x%x", h.err);
	return RC_OK;
}

int rc_solver_profile(rc_engine *e, int enable, double *ms, int n) {
	if(!e) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	int rc;
	if(!e->phase_ns && (rc = dalloc(e, &e->phase_ns, 32))) return rc;
	if(ms && n > 0) {
		unsigned long long h[32];
		CUDA_TRY(e, cudaMemcpy(h, e->phase_ns, sizeof(h), cudaMemcpyDeviceToHost));
		for(int k = 0; k < n && k < 32; k++) ms[k] = (double) h[k] * 1e-6;
	}
	if((enable != 0) != e->phase_on) drop_graphs(e);
	if(enable) CUDA_TRY(e, cudaMemset(e->phase_ns, 0, sizeof(unsigned long long) * 32));
	e->phase_on = enable != 0;
	return RC_OK;
}

// --- diagnostic observables ---------------------------------------------------

static int obs_scratch(rc_engine *e, size_t n) {
	if(e->obs_cap >= n) return RC_OK;
	dfree(e, e->obs_buf);
	e->obs_buf = nullptr;
	e->obs_cap = 0;
	int rc;
	if((rc = dalloc(e, &e->obs_buf, n))) return rc;
	e->obs_cap = n;
	return RC_OK;
}

// The last force evaluation formed again with its force split recorded in
// split_buf (Fpassive x/y, Factive x/y, Pressure per site, stride S_cap), the
// way the reference's interactions leave them in BaseField for its
// ForceField and StressField observables.  The re-evaluation reads the
// current phi and box sums and rewrites mu, gradients, the map and the
// forces (or dry velocities) with the values they already hold; the polar
// Repulsion accumulator is not advanced, and the cell records are put back,
// so the engine's trajectory is unchanged.
static int observe_split(rc_engine *e) {
	if(e->hp.precision == RC_PRECISION_FLOAT)
		return set_err(e, RC_ERR_UNSUPPORTED, "force observables are formed by the FP64 cell kernels only");
	int rc;
	if(!e->split_buf && (rc = dalloc(e, &e->split_buf, 6 * (size_t) e->S_cap))) return rc;
	if(!e->cells_save && (rc = dalloc(e, &e->cells_save, (size_t) std::max(e->N, 1)))) return rc;
	if(e->N == 0) return RC_OK;
	CUDA_TRY(e, cudaMemcpyAsync(e->cells_save, e->cells, sizeof(CellDev) * (size_t) e->N, cudaMemcpyDeviceToDevice, e->stream));
	CellArgs a = cell_args(e);
	a.phi_eval = e->phiA;
	a.pe = e->ph[e->eval_phase];
	a.pu = e->ph[e->eval_phase];
	a.accumulate_rep = 0;
	a.fsplit = e->split_buf;
	a.fsplit_stride = e->S_cap;
	cell_launch(e, wet_phase(e, e->eval_phase) ? EV_WET_RHS : EV_STORE, UP_NONE, a, e->stream);
	CUDA_TRY(e, cudaGetLastError());
	CUDA_TRY(e, cudaMemcpyAsync(e->cells, e->cells_save, sizeof(CellDev) * (size_t) e->N, cudaMemcpyDeviceToDevice, e->stream));
	return RC_OK;
}

// Box fields (f0, f1) of an observable kind into the scratch area.
static int observe_box_fields(rc_engine *e, int kind, int layer, int only_type, double *f0, double *f1) {
	const LayerDev &lay = e->layers_h[(size_t) layer];
	if(kind <= RC_OBS_NEMATIC) {
		materialise(e, 0);  // current velocities (dry models)
		launch_obs_field(e->cells, e->layers, lay, e->bin_count, e->bin_cells, e->phiA, e->vx, e->vy, kind, layer,
		                 only_type, f0, f1, e->stream);
		return RC_OK;
	}
	int rc;
	if((rc = observe_split(e))) return rc;
	const double *sp = e->split_buf;
	const size_t st = (size_t) e->S_cap;
	if(kind == RC_OBS_FORCE) {
		// get_total_force_x/y: the velocity times the interaction's friction
		launch_obs_sites(e->cells, e->layers, lay, e->bin_count, e->bin_cells, e->phiA, e->vx, e->vy,
		                 e->ph[e->phase].friction, layer, only_type, f0, f1, e->stream);
	}
	else if(kind == RC_OBS_FORCE_PASSIVE || kind == RC_OBS_FORCE_ACTIVE) {
		const double *g = sp + (kind == RC_OBS_FORCE_PASSIVE ? 0 : 2) * st;
		launch_obs_sites(e->cells, e->layers, lay, e->bin_count, e->bin_cells, e->phiA, g, g + st, 1.0, layer,
		                 only_type, f0, f1, e->stream);
	}
	else if(kind == RC_OBS_PRESSURE) {
		launch_obs_sites(e->cells, e->layers, lay, e->bin_count, e->bin_cells, e->phiA, sp + 4 * st, nullptr, 1.0, layer,
		                 only_type, f0, f1, e->stream);
	}
	else {
		// the free-energy density gradient 2 gamma lambda grad(phi) of the
		// models that set it (WetModel.cpp:608-609, SimpleMultiField.cpp:179-180)
		const double g2 = (e->P.model == M_WET || e->P.model == M_SIMPLE) ? 2 * e->P.gamma * e->P.lambda : 0.0;
		launch_obs_thermo(e->cells, e->layers, lay, e->bin_count, e->bin_cells, e->phiA, sp + 5 * st, e->mu, e->dxg,
		                  e->dyg, g2, kind - RC_OBS_THERMO, layer, only_type, f0, f1, e->stream);
	}
	return RC_OK;
}

int rc_observe_field(rc_engine *e, int kind, int layer, int only_type, int size_grid, double *fx, double *fy,
                     double *coarse_x, double *coarse_y) {
	if(!e || !fx || !fy) return RC_ERR_INVALID;
	if(kind < RC_OBS_VELOCITY || kind > RC_OBS_CHEMPOT2) return set_err(e, RC_ERR_INVALID, "rc_observe_field: kind %d", kind);
	if(layer < 0 || layer >= e->n_layers) return set_err(e, RC_ERR_INVALID, "rc_observe_field: layer %d", layer);
	CUDA_TRY(e, cudaSetDevice(e->device));
	const LayerDev &lay = e->layers_h[(size_t) layer];
	const size_t L2 = (size_t) lay.L * lay.L;
	int rc;
	if((rc = obs_scratch(e, 4 * L2))) return rc;
	double *f0 = e->obs_buf, *f1 = f0 + L2, *c0 = f1 + L2, *c1 = c0 + L2;
	if((rc = observe_box_fields(e, kind, layer, only_type, f0, f1))) return rc;
	if(size_grid > 0) {
		launch_obs_coarse(f0, c0, lay.L, size_grid, e->stream);
		launch_obs_coarse(f1, c1, lay.L, size_grid, e->stream);
	}
	CUDA_TRY(e, cudaGetLastError());
	CUDA_TRY(e, cudaMemcpyAsync(fx, f0, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaMemcpyAsync(fy, f1, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	if(size_grid > 0 && coarse_x) CUDA_TRY(e, cudaMemcpyAsync(coarse_x, c0, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	if(size_grid > 0 && coarse_y) CUDA_TRY(e, cudaMemcpyAsync(coarse_y, c1, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_observe_stress(rc_engine *e, int kind, int layer, int only_type, int size_grid, double *xx, double *yy,
                      double *xy) {
	if(!e || !xx || !yy) return RC_ERR_INVALID;
	if(kind < RC_OBS_FORCE || kind > RC_OBS_PRESSURE) return set_err(e, RC_ERR_INVALID, "rc_observe_stress: kind %d", kind);
	if(layer < 0 || layer >= e->n_layers) return set_err(e, RC_ERR_INVALID, "rc_observe_stress: layer %d", layer);
	if(size_grid < 1) return set_err(e, RC_ERR_INVALID, "rc_observe_stress: size_grid %d", size_grid);
	CUDA_TRY(e, cudaSetDevice(e->device));
	const LayerDev &lay = e->layers_h[(size_t) layer];
	const size_t L2 = (size_t) lay.L * lay.L;
	int rc;
	if((rc = obs_scratch(e, 5 * L2))) return rc;
	double *f0 = e->obs_buf, *f1 = f0 + L2, *o0 = f1 + L2, *o1 = o0 + L2, *o2 = o1 + L2;
	if((rc = observe_box_fields(e, kind, layer, only_type, f0, f1))) return rc;
	const bool pressure = kind == RC_OBS_PRESSURE;
	// pressure: both components come from the pressure field (StressField.cpp:192-193)
	launch_obs_stress(f0, pressure ? f0 : f1, o0, o1, pressure ? nullptr : o2, lay.L, size_grid, e->stream);
	CUDA_TRY(e, cudaGetLastError());
	CUDA_TRY(e, cudaMemcpyAsync(xx, o0, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaMemcpyAsync(yy, o1, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	if(xy && !pressure) CUDA_TRY(e, cudaMemcpyAsync(xy, o2, sizeof(double) * L2, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

int rc_observe_cells(rc_engine *e, double *cell_obs, double *layer_obs) {
	if(!e) return RC_ERR_INVALID;
	CUDA_TRY(e, cudaSetDevice(e->device));
	const size_t nc = (size_t) std::max(e->N, 1), nl = (size_t) e->n_layers;
	int rc;
	if((rc = obs_scratch(e, 6 * nc + 4 * nl))) return rc;
	materialise(e, 0);  // current gradients (dry models)
	widen_fields(e);
	double *co = e->obs_buf, *lo = co + 6 * nc;
	launch_obs_cells(e->cells, e->layers, e->N, e->n_layers, e->dxg, e->dyg, co, lo, e->stream);
	CUDA_TRY(e, cudaGetLastError());
	if(cell_obs && e->N) CUDA_TRY(e, cudaMemcpyAsync(cell_obs, co, sizeof(double) * 6 * (size_t) e->N, cudaMemcpyDeviceToHost, e->stream));
	if(layer_obs) CUDA_TRY(e, cudaMemcpyAsync(layer_obs, lo, sizeof(double) * 4 * nl, cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	return RC_OK;
}

long long rc_site_count(const rc_engine *e) { return e ? e->S : 0; }

int rc_layer_count(const rc_engine *e) { return e ? e->n_layers : 0; }

const char *rc_last_error(const rc_engine *e) { return e ? e->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

namespace {

constexpr long long NA_MAX_UNKNOWNS = RC_NOALLOC_MAX_UNKNOWNS;
constexpr long long NA_MAX_BOX_SITES = RC_NOALLOC_MAX_BOX_SITES;
constexpr long long NA_MAX_BLOCKS = 4096;

constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t NA_OFF_ST = 0;
constexpr size_t NA_OFF_BAR = NA_OFF_ST + na_round(sizeof(rc::DevStatus));
constexpr size_t NA_OFF_SCALARS = NA_OFF_BAR + na_round(2 * sizeof(unsigned));
constexpr size_t NA_OFF_PARTIALS = NA_OFF_SCALARS + na_round(64 * sizeof(double));
constexpr size_t NA_OFF_VEC = NA_OFF_PARTIALS + na_round(8 * NA_MAX_BLOCKS * sizeof(double));
constexpr size_t NA_VEC = na_round(NA_MAX_UNKNOWNS * sizeof(double));
constexpr size_t NA_OFF_BOX = NA_OFF_VEC + 4 * NA_VEC;
constexpr size_t NA_BOX = na_round(NA_MAX_BOX_SITES * sizeof(double));
constexpr size_t NA_OFF_COV_OFF = NA_OFF_BOX + 2 * NA_BOX;
constexpr size_t NA_OFF_COV_IDX = NA_OFF_COV_OFF + na_round((NA_MAX_BOX_SITES + 1) * sizeof(int));
constexpr size_t NA_BYTES = NA_OFF_COV_IDX + na_round(NA_MAX_UNKNOWNS * sizeof(int));

// The fixed solver area (about 1.8 MB): status, barrier words, reduction
// slots, four work vectors (residual and scaled direction of both
// components), two box-grid sums and the CSR cover lists, laid out at the
// offsets above.  One area per device, shared by every caller.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// Device address of the area, looked up once per device.
std::mutex g_noalloc_mu;
std::vector<unsigned char *> g_noalloc_ptr;

// Resets what the solve needs zero at its start: the status record (then S
// and the cold-start flag) and the grid barrier's arrival counter.  The work
// arrays are initialised by the solve itself.
__global__ void noalloc_header_kernel(rc::DevStatus *st, unsigned *bar, long long S) {
	if(threadIdx.x == 0 && blockIdx.x == 0) {
		memset(st, 0, sizeof(*st));
		st->S = S;
		st->cg_cold = 1;
		bar[0] = 0u;
		bar[1] = 0u;
	}
}

}  // namespace

extern "C" {

/*
 * rc_viscous_resolve_noalloc: the viscous solve of the last force evaluation,
 * run again from a cold start into caller-owned device arrays, with every
 * solver work array taken from a fixed, statically sized device area instead
 * of engine or runtime allocations.  It exists for hosts that must not
 * allocate device memory while they run: a driver that has already handed
 * the HBM to its own pool for an ensemble of engines, or one that cannot take
 * the device-wide synchronisation cudaMalloc/cudaFree imply in the middle of
 * its time loop.  The reference has no counterpart (Eigen allocates its CG
 * work vectors on every solve, WetModel.cpp:279-376).
 */
int rc_viscous_resolve_noalloc(rc_engine *e, double *vx, double *vy, long long n, int *iterations) {
	if(!e) return RC_ERR_INVALID;
	if(e->n_layers > 1) return set_err(e, RC_ERR_UNSUPPORTED, "rc_viscous_resolve_noalloc: not provided for ensembles");
	if(!vx || !vy) return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve_noalloc: NULL output array");
	if(n != e->S)
		return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve_noalloc: n = %lld but the state has %lld unknowns", n, e->S);
	if(e->pending || !wet_phase(e, e->eval_phase))
		return set_err(e, RC_ERR_UNSUPPORTED, "rc_viscous_resolve_noalloc: the last evaluation had no viscous solve");
	if(e->S > NA_MAX_UNKNOWNS)
		return set_err(e, RC_ERR_CAPACITY,
		               "rc_viscous_resolve_noalloc: %lld unknowns per component, the fixed area holds at most %lld",
		               e->S, NA_MAX_UNKNOWNS);
	if((long long) e->L * e->L > NA_MAX_BOX_SITES)
		return set_err(e, RC_ERR_CAPACITY,
		               "rc_viscous_resolve_noalloc: box of %d x %d sites, the fixed area holds at most %lld sites", e->L,
		               e->L, NA_MAX_BOX_SITES);
	if(e->cg_blocks > NA_MAX_BLOCKS / 2)
		return set_err(e, RC_ERR_CAPACITY, "rc_viscous_resolve_noalloc: %d solver blocks, at most %lld", e->cg_blocks,
		               NA_MAX_BLOCKS / 2);
	CUDA_TRY(e, cudaSetDevice(e->device));
	unsigned char *base = nullptr;
	{
		std::lock_guard<std::mutex> lock(g_noalloc_mu);
		if(g_noalloc_ptr.size() <= (size_t) e->device) g_noalloc_ptr.resize((size_t) e->device + 1, nullptr);
		if(!g_noalloc_ptr[(size_t) e->device]) {
			void *q = nullptr;
			const cudaError_t c = cudaGetSymbolAddress(&q, g_noalloc_scratch);
			if(c != cudaSuccess)
				return set_err(e, RC_ERR_CUDA, "rc_viscous_resolve_noalloc: cudaGetSymbolAddress failed: %s",
				               cudaGetErrorString(c));
			g_noalloc_ptr[(size_t) e->device] = (unsigned char *) q;
		}
		base = g_noalloc_ptr[(size_t) e->device];
	}
	rc::DevStatus *st = (rc::DevStatus *) (base + NA_OFF_ST);
	unsigned *bar = (unsigned *) (base + NA_OFF_BAR);
	double *vec = (double *) (base + NA_OFF_VEC);
	const size_t vs = NA_VEC / sizeof(double), bs = NA_BOX / sizeof(double);
	noalloc_header_kernel<<<1, 32, 0, e->stream>>>(st, bar, e->S);
	CUDA_TRY(e, cudaGetLastError());
	CGArgs g;
	memset(&g, 0, sizeof(g));
	g.layer = -1;  // the single monolayer
	g.cells = e->cells;
	g.mapg = e->mapg;
	g.cnt = e->cnt;
	g.cover = e->cover;
	g.cov_off = (int *) (base + NA_OFF_COV_OFF);
	g.cov_idx = (int *) (base + NA_OFF_COV_IDX);
	g.fx = e->fx;
	g.fy = e->fy;
	g.vx = vx;
	g.vy = vy;
	g.rx = vec;
	g.ry = vec + vs;
	g.px = vec + 2 * vs;
	g.py = vec + 3 * vs;
	g.Px = (double *) (base + NA_OFF_BOX);
	g.Py = g.Px + bs;
	g.partials = (double *) (base + NA_OFF_PARTIALS);
	g.scalars = (double *) (base + NA_OFF_SCALARS);
	g.bar = bar;
	g.st = st;
	g.L = e->L;
	g.restart_every = 0;
	g.xi = e->ph[e->eval_phase].friction;
	g.eta = e->ph[e->eval_phase].friction_cell;
	g.tol = e->hp.cg_tolerance > 0 ? e->hp.cg_tolerance : 2.220446049250313e-16;
	g.mixed = 0;
	CUDA_TRY(e, launch_cg(g, e->cg_blocks, e->stream));
	rc::DevStatus h;
	CUDA_TRY(e, cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
	CUDA_TRY(e, cudaStreamSynchronize(e->stream));
	if(h.err & ERR_BARRIER) return set_err(e, RC_ERR_CG, "rc_viscous_resolve_noalloc: grid barrier timed out");
	if(h.err) return set_err(e, RC_ERR_INVALID, "rc_viscous_resolve_noalloc: device error 0x%x", h.err);
	if(iterations) *iterations = h.cg_iters;
	return RC_OK;
}

}  // extern "C"

namespace rc {
__global__ void conversion_selftest_kernel(const double *in, float *exact, float *fast, float *cuda_rn, double *widened,
                                           long long n) {
	for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
		const double v = in[i];
		exact[i] = d2f_int(v);
		fast[i] = d2f_fast(v);
		const float r = __double2float_rn(v);
		cuda_rn[i] = r;
		widened[i] = f2d_int(r);
	}
}
}  // namespace rc

extern "C" {

int rc_selftest_conversions(const double *in, float *exact, float *fast, float *cuda_rn, double *widened, long long n,
                            int device) {
	if(!in || !exact || !fast || !cuda_rn || !widened || n <= 0)
		return set_err(nullptr, RC_ERR_INVALID, "rc_selftest_conversions: invalid arguments");
	int prev = 0;
	if(cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess)
		return set_err(nullptr, RC_ERR_CUDA, "rc_selftest_conversions: no device %d", device);
	double *din = nullptr, *dw = nullptr;
	float *de = nullptr, *df = nullptr, *dc = nullptr;
	const size_t nd = sizeof(double) * (size_t) n, nf = sizeof(float) * (size_t) n;
	cudaError_t c = cudaMalloc(&din, nd);
	if(c == cudaSuccess) c = cudaMalloc(&dw, nd);
	if(c == cudaSuccess) c = cudaMalloc(&de, nf);
	if(c == cudaSuccess) c = cudaMalloc(&df, nf);
	if(c == cudaSuccess) c = cudaMalloc(&dc, nf);
	if(c == cudaSuccess) c = cudaMemcpy(din, in, nd, cudaMemcpyHostToDevice);
	if(c == cudaSuccess) {
		const long long blocks = std::min<long long>((n + 255) / 256, 4096);
		conversion_selftest_kernel<<<(unsigned) blocks, 256>>>(din, de, df, dc, dw, n);
		c = cudaGetLastError();
	}
	if(c == cudaSuccess) c = cudaMemcpy(exact, de, nf, cudaMemcpyDeviceToHost);
	if(c == cudaSuccess) c = cudaMemcpy(fast, df, nf, cudaMemcpyDeviceToHost);
	if(c == cudaSuccess) c = cudaMemcpy(cuda_rn, dc, nf, cudaMemcpyDeviceToHost);
	if(c == cudaSuccess) c = cudaMemcpy(widened, dw, nd, cudaMemcpyDeviceToHost);
	cudaFree(din);
	cudaFree(dw);
	cudaFree(de);
	cudaFree(df);
	cudaFree(dc);
	cudaSetDevice(prev);  // the caller's current device is left as it was
	if(c != cudaSuccess) return set_err(nullptr, RC_ERR_CUDA, "rc_selftest_conversions: %s", cudaGetErrorString(c));
	return RC_OK;
}

void rc_destroy(rc_engine *e) {
	if(!e) return;
	cudaSetDevice(e->device);
	if(e->stream) cudaStreamSynchronize(e->stream);
	for(void *p : e->allocs) cudaFree(p);
	if(e->st_host) cudaFreeHost(e->st_host);
	collect_marks(e);
	for(auto &g : e->graphs) cudaGraphExecDestroy(g.exec);
	for(cudaEvent_t v : e->event_pool) cudaEventDestroy(v);
	if(e->own_stream) cudaStreamDestroy(e->own_stream);
	delete e;
}

}  // extern "C"
