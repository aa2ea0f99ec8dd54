// Host-visible launch interface of the engine's kernels (implemented in
// rc_cells.cu, rc_box.cu and rc_cg.cu).
#pragma once

#include "rc_common.cuh"
#include "rc_unet.cuh"
#include "rc_unet_tc.cuh"

namespace rc {

enum EvalMode { EV_NONE = 0, EV_STORE = 1, EV_WET_RHS = 2, EV_LOCAL = 3 };
enum UpdMode { UP_NONE = 0, UP_PRED = 1, UP_CORR = 2 };

// Per-cell sums handed from a cell kernel to the per-cell epilogue kernel
// (split mode): the FP64 kernels' block totals, or the FP32 kernel's
// per-warp partials (combined in FP64 by the epilogue kernel).
struct CellSum {
	double acc[12];
	double area[CELL_MAX_THREADS / 32];
	float part[CELL_MAX_THREADS / 32][12];
	int imin[2];
	int nw;  // FP32 kernel: warps that wrote area/part
	int pad;
	double perim;
};

struct CellArgs {
	CellDev *cells;
	const LayerDev *layers;
	int N;
	int smem_n;            // per-site capacity of the dynamic shared memory
	const double *phi_eval;  // phi at which forces are evaluated; PRED update also reads phi^n here
	const double *phi_old;   // CORR: phi^n
	double *phi_out;         // PRED: phi*; CORR: phi^{n+1}
	double *dphi_old;
	double *mu, *dxg, *dyg, *vxg, *vyg, *fxg, *fyg;
	// FP32 engines: the force evaluation's mu and gradients in FP32 (they feed
	// only the FP32 update; downloads and observables widen them into mu, dxg, dyg)
	float *muf, *dxf, *dyf;
	float *dphif;  // FP32 kernels: dphi^n in FP32, in the dphi_old buffer
	int *mapg;
	double *rep;
	const double *phi2, *sq00, *sq01;
	const double *walls;     // wall values per box site (getWalls), null for periodic boxes
	const double *tab_cos, *tab_sin;
	const float *tab_cosf, *tab_sinf;  // the same tables rounded to FP32 (FP32 kernels)
	CellSum *csum;                     // split mode: sums for the epilogue kernel
	int split;                         // 1: the per-cell epilogue runs in cell_finish_kernel
	int *bin_count, *bin_cells;
	int nbx, nby;
	DevStatus *st;
	DevParams P;
	PhaseParams pe;        // parameters of the evaluation
	PhaseParams pu;        // parameters of the update (directed active forces)
	int rep_on;            // track the polar Repulsion accumulator
	int accumulate_rep;    // this evaluation adds to it (not a re-evaluation for download)
	// force split of an observation (null otherwise): per site, at
	// fsplit + f * fsplit_stride + start + q, f = 0..4: Fpassive_x, Fpassive_y,
	// Factive_x, Factive_y, Pressure (BaseField members the reference's
	// interactions fill, e.g. WetModel.cpp:605,636-637,655-656)
	double *fsplit;
	long long fsplit_stride;
};

struct BoxArgs {
	const CellDev *cells;
	const LayerDev *layers;
	int n_layers, total_bins;
	const double *phi;
	double *phi2, *sq00, *sq01;
	int *cnt, *cover;      // cover[slot * L*L + k]
	const int *bin_count, *bin_cells;
	const int *bin_layer;  // layer of each bin
	int nbx, nby;
	int want_q, want_cover, check_overlap;
	int f32;               // FP32 engines: phi^2 summed in FP32 (the cell kernel reads it in FP32)
	int bookkeeping;       // wet models: size_rows / restart bookkeeping of this evaluation
	int restart_every;
	int solve_follows;     // a viscous solve follows this evaluation
	DevStatus *st;
	int L;
	LayerSolve *lsolve;    // wet ensembles: per-member bookkeeping (null: DevStatus)
};

struct CGArgs {
	const CellDev *cells;
	const int *mapg;
	const int *cnt, *cover;
	int *cov_off, *cov_idx;  // CSR cover lists built by the solve
	const double *fx, *fy;   // right-hand sides
	double *vx, *vy;         // solution; warm start
	double *rx, *ry, *px, *py;  // residual; scaled direction T p
	double *Px, *Py;         // box-grid sums of p
	double *partials;        // per-block partial sums
	double *scalars;         // solver scalars (see rc_cg.cu)
	unsigned *bar;           // barrier counter and generation
	DevStatus *st;
	int L;
	int restart_every;
	double xi, eta, tol;
	int mixed;               // FP32 inner iterations inside FP64 refinement
	int fcg;                 // the inner iterations are the flexible CG in cover order (network or Jacobi)
	double inner_tol;        // mixed: relative residual reduction per refinement sweep
	float *rxf, *ryf, *pxf, *pyf, *apxf, *apyf, *Pxf, *Pyf;
	float *exf, *eyf;        // mixed: correction of one refinement sweep
	// learned preconditioner for the inner iterations of the mixed path
	// (flexible CG); null: Jacobi
	const float *unet_params;
	UNetActs unet;           // activations for the two components (batch 2)
	int unet_tc;             // 1: BF16 tensor-core layers (unet_bf, unet_wpack)
	UNetActsBF unet_bf;
	const bf16 *unet_wpack;
	float *zxf, *zyf;        // z = M r
	float *Zxf, *Zyf;        // box sums of z
	float *Pxf2, *Pyf2;      // second buffer of the direction's box sums
	// training samples harvested from the plain FP64 solve; null: none.
	// Sample q: harv_in[q][L2][2] = (R/s, W), harv_tgt[q][L2] = (X* - X)/s,
	// harv_s[q] = s (0 marks an unused slot); *harv_count samples stored.
	unsigned long long *phase_ns;  // diagnostic per-phase times of the learned solve (null: off)
	float *harv_in, *harv_tgt, *harv_s;
	int *harv_count;
	int harv_cap, harv_every, harv_per_solve;
	// iteration cap per component (0: Eigen's default of twice the unknowns);
	// fail_noconv: a solve that stops at the cap above its tolerance sets
	// ERR_NOCONV (Eigen reports that only through info(), which the
	// reference does not read)
	long long max_iters;
	int fail_noconv;
	// grid-barrier polls before a wait gives up (0: the default, about 1-2 s);
	// barrier_extra: arrivals the first barrier waits for beyond the grid's
	// blocks -- a test hook that makes the wait run out (nothing arrives)
	int barrier_extra;
	long long spin_limit;
	// ensembles: the member whose system this launch solves (-1: the single
	// monolayer); its box arrays (cnt, cover) and L are the member's, its
	// unknowns the contiguous run of its cells' sites, its bookkeeping lsolve[layer]
	int layer;
	const LayerDev *layers;
	LayerSolve *lsolve;
};

cudaError_t configure_kernels();
void launch_cell_kernel(int model, int eval, int upd, const CellArgs &a, cudaStream_t s);
// FP32 site arithmetic (rc_cells_f32.cu) for the polar and wet nematic
// models; block: threads per cell (CELL_F32_BLOCKS); false if the model has
// no FP32 kernel
bool launch_cell_kernel_f32(int model, int eval, int upd, const CellArgs &a, cudaStream_t s, int block);
cudaError_t configure_kernels_f32();
// split mode: the per-cell epilogue, one thread per cell (f32: after the FP32 kernel)
void launch_cell_finish(int model, int eval, int upd, bool f32, const CellArgs &a, cudaStream_t s);
size_t cell_smem_bytes(int model, int smem_n);
int cell_smem_arrays(int model);
void launch_rng(CellDev *cells, LayerDev *layers, int n_layers, DevStatus *st, cudaStream_t s);
// out_k[i] = in_k[i] for three float arrays of n elements (FP32 engines' mu and gradients)
void launch_widen3(const float *a, const float *b, const float *c, double *x, double *y, double *z, long long n,
                   cudaStream_t s);
void launch_bins(CellDev *cells, const LayerDev *layers, int N, int *bin_count, int *bin_cells, int total_bins,
                 DevStatus *st, cudaStream_t s);
void launch_repack(CellArgs a, double *scratch_phi, double *scratch_rep, long long cap, cudaStream_t s);
void launch_box_gather(const BoxArgs &a, cudaStream_t s);
int cg_grid_blocks(int device, bool learned, long long box_sites);
// diagnostic observables (rc_obs.cu)
void launch_obs_field(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                      const int *bin_cells, const double *phi, const double *vx, const double *vy, int kind, int layer,
                      int only_type, double *fx, double *fy, cudaStream_t s);
void launch_obs_coarse(const double *f, double *out, int L, int sg, cudaStream_t s);
void launch_obs_sites(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                      const int *bin_cells, const double *phi, const double *g0, const double *g1, double scale, int layer,
                      int only_type, double *fx, double *fy, cudaStream_t s);
void launch_obs_thermo(const CellDev *cells, const LayerDev *layers, const LayerDev &lay_h, const int *bin_count,
                       const int *bin_cells, const double *phi, const double *fd, const double *mu, const double *dxg,
                       const double *dyg, double g2, int sub, int layer, int only_type, double *fx, double *fy,
                       cudaStream_t s);
void launch_obs_stress(const double *fx, const double *fy, double *xx, double *yy, double *xy, int L, int sg, cudaStream_t s);
void launch_obs_cells(const CellDev *cells, const LayerDev *layers, int N, int n_layers, const double *dxg,
                      const double *dyg, double *cell_obs, double *layer_obs, cudaStream_t s);
cudaError_t launch_cg(const CGArgs &a, int blocks, cudaStream_t s);

}  // namespace rc
