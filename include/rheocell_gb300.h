/*
 * rheocell_gb300 -- C ABI of the GB300 multi-phase-field time-step engine.
 *
 * This is the drop-in boundary for RheoCell's time-step hot path.  In the
 * reference, SimManager::run (src/Managers/SimManager.cpp:131-178) drives a
 * backend chosen by BackendFactory::make_backend
 * (src/Backends/BackendFactory.cpp:12-113, which already reserves the
 * `backend = CUDA` / `backend_precision` slot at :37-65).  A CUDA backend
 * class written on top of this header replaces FD_CPUBackend
 * (src/Backends/FD_CPUBackend.cpp) and the force evaluation of the selected
 * interaction (src/Interactions/{SimpleMultiField,ActiveNematic,
 * WetPolarModel,WetModel}.cpp); the C++ caller above it is unchanged.
 *
 * Conventions
 *  - Plain C types only; no exception crosses the ABI.  Every function that
 *    can fail returns 0 on success and a negative rc_status otherwise;
 *    rc_last_error() then holds a message.  The C++ caller turns a non-zero
 *    status into RCexception(rc_last_error(e)), as the reference's main()
 *    catches RCexception (src/rheoCell.cpp:40-43).
 *  - Ownership: the device owns the simulation state between calls.  Host
 *    memory handed to a call is borrowed for the duration of that call.
 *  - Threading: one host thread per engine; the engine issues all its work
 *    on one CUDA stream (its own, or the one given to rc_set_stream).
 *  - All state is FP64, as the reference's `number` (src/Utilities/LR_vector.h:7-11).
 */
#ifndef RHEOCELL_GB300_H
#define RHEOCELL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define RC_ABI_VERSION 1

typedef enum rc_status {
	RC_OK = 0,
	RC_ERR_INVALID = -1,      /* bad argument or inconsistent input        */
	RC_ERR_CUDA = -2,         /* a CUDA call failed                        */
	RC_ERR_OOM = -3,          /* device allocation failed                  */
	RC_ERR_OVERLAP = -4,      /* more than 20 patches cover one box site   */
	RC_ERR_NONFINITE = -5,    /* NaN/Inf in the state                      */
	RC_ERR_CG = -6,           /* the viscous solve failed (max iterations) */
	RC_ERR_CAPACITY = -7,     /* a patch outgrew the engine's capacity     */
	RC_ERR_UNSUPPORTED = -8   /* feature not provided by this build        */
} rc_status;

/* interaction_type values (src/Interactions/InteractionFactory.cpp:13-58). */
typedef enum rc_model {
	RC_SIMPLEFIELD = 0,   /* "simplefield"    */
	RC_ACTIVENEMATIC = 1, /* "activenematic"  */
	RC_WETPOLARMODEL = 2, /* "wetpolarmodel"  */
	RC_WETMODEL = 3       /* "wetmodel"       */
} rc_model;

/* backend_precision values (src/Backends/BackendFactory.cpp:14-16,38-63). */
typedef enum rc_precision {
	RC_PRECISION_DOUBLE = 0, /* FP64 everywhere; the parity path                    */
	RC_PRECISION_MIXED = 1,  /* FP64 fields; FP32 viscous-solve inner iterations,
	                            FP64 dots and FP64 true-residual refinement        */
	RC_PRECISION_FLOAT = 2   /* wetpolarmodel and wetmodel: FP32 site arithmetic,
	                            FP64 field storage and FP64 cell-area integrals;
	                            the viscous solve as RC_PRECISION_MIXED            */
} rc_precision;

/*
 * Interaction and integrator parameters.  Arrays of two hold the value in
 * force before interaction->apply_changes_after_equilibration() ([0], the
 * values the interaction's constructor sets) and after it ([1], the input-file
 * values); see e.g. WetModel.cpp:4-21 and :88-96.  The C++ caller fills both
 * from the input file and the constructor defaults.
 */
typedef struct rc_params {
	int model;             /* rc_model                                          */
	int precision;         /* rc_precision                                      */
	int R;                 /* cell radius (int, as BaseInteraction::R)          */
	int border;            /* patch growth border, 4 (src/Fields/BaseField.cpp:5) */
	double dt;             /* FDBackend dt                                      */
	double J0;             /* FD_CPUBackend J0 (default 1)                      */
	double gamma, lambda, omega, mu, kappa;
	double passive_alpha;  /* wet models                                        */
	double cg_tolerance;   /* CGtolerance; <= 0 means Eigen's default (epsilon) */
	int cg_restart_every;  /* warm solves between cold restarts: 100 (wetmodel), 10 (wetpolarmodel) */
	int anchoring;         /* reserved; must be 0 (update_anchoring is not provided) */
	double friction[2];    /* xi                                               */
	double friction_cell[2]; /* eta; 0 selects the dry path v = f / xi         */
	double zetaQ_self[2];
	double zetaQ_inter[2];
	double J_Q[2];
	double beta[2];        /* wetpolarmodel perimeter term                      */
	/* drand48 state (48 bits) and Utils::gaussian's cached deviate, as left by
	 * the host after reading the topology and configuration. */
	unsigned long long rng_state;
	int rng_has_cached;
	double rng_cached;
	/* 1: conserved dynamics of sim_type = FD_CH (src/Backends/FD_CHBackend.cpp:44-118),
	 * d(phi)/dt = J0 lap(mu) - v.grad(phi); 0: FD_CPU, d(phi)/dt = -J0 mu - v.grad(phi) */
	int conserved;
	/* wall_slip (src/Interactions/BaseInteraction.cpp:10,23; 0.5 unless set):
	 * a box site whose wall value is below it is open; used only with walls */
	double wall_slip;
} rc_params;

/*
 * The simulation box: a periodic square of Lx x Ly sites (Lx == Ly;
 * src/Boxes/SquareBox.cpp).  `walls` (NULL: none) holds Lx*Ly values of the
 * box's getWalls(k) for the square wall boxes (box = square with type =
 * square_walls, circle_walls or triangle_walls: SquareWalls.cpp:23-55,
 * CircleWalls.cpp:23-45, TriangleWalls.cpp:24-60), copied at create.  With
 * walls, the stencils, the adhesion term and the forces of the wetmodel,
 * wetpolarmodel and simplemultifield interactions take the reference's wall
 * branches (BaseInteraction.h:196-263, WetModel.cpp:531-536,664-690,
 * WetPolarModel.cpp:267-272,329-337); activenematic ignores walls, as the
 * reference's does.  A viscous solve with walls is not provided
 * (RC_ERR_UNSUPPORTED): the reference's wall rows make its assembled matrix
 * unsymmetric (WetModel.cpp:295-335), and its upper-triangle CG then
 * depends on the order of the unknowns.
 */
typedef struct rc_box {
	int Lx, Ly;
	const double *walls;
} rc_box;

/*
 * One phase-field patch (src/Fields/BaseField.h:121-224).  Scalars are copied
 * in on create/upload and out on download.  Per-site arrays are host pointers
 * of at least `capacity` elements (storage order, LsubX fastest); a NULL
 * pointer skips that array.
 */
typedef struct rc_cell_host {
	int lsub_x, lsub_y;      /* LsubX, LsubY                                  */
	int offset_x, offset_y;  /* offset[0..1]                                  */
	int corner;              /* sub_corner_bottom_left (box site index)       */
	int type;                /* topology type                                  */
	double com_x, com_y;     /* CoM                                            */
	double unrap_x, unrap_y; /* unrap_sub_corner_bottom_left_x/_y              */
	double q00, q01;         /* Q00, Q01                                       */
	double theta_q, theta_q_old;
	double nemq_x, nemq_y, nemq_old_x, nemq_old_y;
	double area, sum_f, perimeter, s00, s01;
	double force_rep_x, force_rep_y;  /* total_force_repulsion_x/_y           */
	int capacity;            /* elements available behind each pointer below  */
	double *phi;             /* fieldScalar                                    */
	double *vx, *vy;         /* velocity (interaction->get_velocity_x/_y)      */
	double *mu;              /* freeEnergy                                     */
	double *dx, *dy;         /* fieldDX, fieldDY                               */
	int *box_index;          /* map_sub_to_box (download only)                 */
} rc_cell_host;

/* rc_download / rc_upload field mask. */
#define RC_FIELD_SCALARS 0x01u  /* per-cell scalars and patch geometry */
#define RC_FIELD_PHI     0x02u
#define RC_FIELD_VEL     0x04u
#define RC_FIELD_MU      0x08u
#define RC_FIELD_GRAD    0x10u
#define RC_FIELD_MAP     0x20u
#define RC_FIELD_ALL     0x3fu

typedef struct rc_step_stats {
	long long steps_done;    /* sim_step calls completed by this rc_step      */
	int cg_solves;           /* viscous solves run (x and y counted apart)    */
	int cg_iterations;       /* CG iterations summed over those solves        */
	int cg_max_iterations;   /* largest iteration count of one solve          */
	double cg_max_rel_residual; /* largest |r|/|b| at exit                    */
	int resized_cells;       /* patches that changed size                     */
	int refinements;         /* mixed precision: outer refinement sweeps      */
	long long kernel_launches; /* engine kernels launched by the call         */
	int fallbacks;           /* mixed/learned solves whose refinement stalled
	                            and that the plain FP64 CG finished           */
	int reserved;
} rc_step_stats;

typedef struct rc_engine rc_engine;

/* Version of this ABI (RC_ABI_VERSION).  No counterpart in the reference. */
int rc_abi_version(void);

/*
 * Create an engine from a loaded configuration.  Replaces
 * FD_CPUBackend::init (src/Backends/FD_CPUBackend.cpp:19-42): uploads the
 * patches and performs the first force evaluation with the phase-0
 * parameters, as the reference does before apply_changes_after_equilibration.
 * `device` is the CUDA ordinal; cells[i].phi must hold lsub_x*lsub_y values.
 */
int rc_create(const rc_params *params, const rc_box *box, int n_cells,
              const rc_cell_host *cells, int device, rc_engine **out);

/*
 * Create an engine that advances n_layers independent monolayers together
 * (an ensemble: every launch covers all of them).  Layer l has box boxes[l]
 * and the next n_cells_per_layer[l] entries of `cells` (layer-major);
 * rng_states[l] is its drand48 state (NULL: params->rng_state for all).  All
 * layers share `params`.  Batches are provided for dry evaluations
 * (friction_cell = 0 in both phases); downloads and uploads address the cells
 * in the same layer-major order.  A monolayer simulation is a batch of one.
 * No counterpart in the reference, which runs one monolayer per process
 * (src/rheoCell.cpp:13-29); each layer here is what one such process reads
 * (SimBackend::read_next_configuration, src/Backends/SimBackend.cpp:220-314).
 */
/*
 * rc_create with every patch's phi generated on the device instead of copied
 * from host arrays (cells[i].phi is ignored and may be NULL; the other fields
 * of cells[i] -- patch geometry, centre, Q, the drand48-drawn director --
 * are taken as in rc_create).  It replaces, for a start from generated
 * discs, the reference's confGenerator writing the configuration file and
 * SimBackend::read_next_configuration parsing it back
 * (src/Managers/GeneratorManager.cpp:130-158, src/Backends/SimBackend.cpp:220-314):
 * at 1024^2 that file is about 0.4 GB of text.
 *   RC_PROFILE_TANH: phi = (1 - tanh((d - radius) / width)) / 2, d the
 *     distance of the box site from the cell's centre (com_x, com_y), nearest
 *     periodic image;
 *   RC_PROFILE_DISC: the reference's initial disc (MultiPhaseField::init,
 *     src/Fields/MultiPhaseField.cpp:149-156): phi = 1 where
 *     x^2 + y^2 < radius^2 + 0.5, x = LsubX/2 - (q mod LsubX),
 *     y = LsubY/2 - q / LsubX, else 0 (confGenerator's files hold the same
 *     values for radius = its init_radius).
 */
#define RC_PROFILE_TANH 0
#define RC_PROFILE_DISC 1
typedef struct rc_generate_spec {
	int profile;     /* RC_PROFILE_TANH or RC_PROFILE_DISC */
	double radius;   /* tanh: R; disc: the disc radius      */
	double width;    /* tanh: interface width lambda        */
} rc_generate_spec;
int rc_create_generated(const rc_params *params, const rc_box *box, int n_cells, const rc_cell_host *cells,
                        const rc_generate_spec *spec, int device, rc_engine **out);

int rc_batch_create(const rc_params *params, int n_layers, const rc_box *boxes, const int *n_cells_per_layer,
                    const rc_cell_host *cells, const unsigned long long *rng_states, int device, rc_engine **out);

/* Number of monolayers the engine advances.  No counterpart in the reference
 * (one monolayer per process there). */
int rc_layer_count(const rc_engine *e);

/*
 * Advance n_steps time steps (FD_CPUBackend::sim_step,
 * src/Backends/FD_CPUBackend.cpp:134-160, called n_steps times).  stats may
 * be NULL.  Returns after the work is complete on the device.
 */
int rc_step(rc_engine *e, int n_steps, rc_step_stats *stats);

/*
 * Enqueue n_steps time steps on the engine's stream and return at once.
 * Errors raised on the device are reported by the next rc_wait.  Patch sizes
 * are not re-examined between the steps of one call, so a patch that grows
 * past the engine's current shared-memory sizing is reported as
 * RC_ERR_CAPACITY; rc_step does that check every 16 steps.  The same steps
 * as rc_step (FD_CPUBackend::sim_step, src/Backends/FD_CPUBackend.cpp:134-160);
 * the reference has no asynchronous form.
 */
int rc_step_async(rc_engine *e, int n_steps);

/* Wait for enqueued work; report device errors and the statistics
 * accumulated since the last rc_wait / rc_step (stats may be NULL).  No
 * counterpart in the reference, whose sim_step returns when the step is done
 * (src/Managers/SimManager.cpp:148-159). */
int rc_wait(rc_engine *e, rc_step_stats *stats);

/*
 * Select the parameter set: 0 before, 1 after
 * apply_simulation_changes_after_equilibration (src/Backends/SimBackend.cpp:316-325).
 */
int rc_set_phase(rc_engine *e, int active);

/* Number of cells and, if the pointers are non-NULL, each patch's size:
 * BaseField::LsubX / LsubY (src/Fields/BaseField.h:198-199). */
int rc_get_sizes(const rc_engine *e, int *n_cells, int *lsub_x, int *lsub_y);

/*
 * Copy device state into host mirrors (SimBackend::apply_simulation_data_changes,
 * src/Backends/SimBackend.cpp:327-329, which the reference calls before every
 * print).  Velocities, mu and gradients are those of the last force
 * evaluation.  Fails with RC_ERR_INVALID if a capacity is too small.
 */
int rc_download(rc_engine *e, rc_cell_host *cells, unsigned fields_mask);

/*
 * Copy host edits into device state (SimBackend::apply_changes_to_simulation_data,
 * src/Backends/SimBackend.cpp:331-333).  Patch sizes cannot change here.  After
 * upload the next step uses the forces of the last evaluation (computed
 * before the edit), as the reference's CPU backend does.
 */
int rc_upload(rc_engine *e, const rc_cell_host *cells, unsigned fields_mask);

/*
 * Flat transfers of phi: the patches of all cells concatenated in cell order,
 * each in storage order (the layout of the reference's stacked solver
 * unknowns, field_start_index, WetModel.cpp:203-209).  n must equal
 * rc_site_count(e).  One copy each way; host memory may be pinned.  The
 * upload follows rc_upload's semantics for RC_FIELD_PHI.
 */
int rc_download_phi(rc_engine *e, double *phi, long long n);
int rc_upload_phi(rc_engine *e, const double *phi, long long n);

/*
 * Stage timers (CUDA events on the engine's stream), the device-side
 * counterpart of the reference's TimingManager stages "First Step" and
 * "Forces" (src/Backends/FDBackend.cpp:41-43).  While enabled, every stage
 * launch is bracketed by two events; rc_timers() adds up the elapsed times of
 * the completed ones (it synchronises) and reports, per stage, the total
 * milliseconds and the number of launches.  reset != 0 zeroes the totals.
 */
#define RC_TIMER_UPDATE 0   /* per-cell kernels: update (and fused dry forces) */
#define RC_TIMER_GATHER 1   /* box gather (and solver bookkeeping)            */
#define RC_TIMER_FORCES 2   /* wet force / right-hand-side evaluation         */
#define RC_TIMER_SOLVE  3   /* viscous solve                                  */
#define RC_TIMER_REPACK 4   /* patch resize repack                            */
#define RC_TIMER_RNG    5   /* polar noise stream                             */
#define RC_TIMER_EPILOGUE 6 /* per-cell epilogue kernel of a split update:
                               cell sums, positions, directed forces        */
#define RC_NUM_TIMERS   7
int rc_set_timing(rc_engine *e, int enable);
int rc_timers(rc_engine *e, double *ms, long long *launches, int reset);

/* Issue the engine's work on this cudaStream_t (NULL: the engine's own).
 * No counterpart in the reference (CPU only). */
int rc_set_stream(rc_engine *e, void *cuda_stream);

/*
 * No counterpart in the reference.  Re-run the viscous solve of the last
 * force evaluation (both components, from a cold start, plain FP64 CG at the
 * engine's tolerance) into vx and vy, device arrays of n = rc_site_count(e)
 * doubles in the order of rc_download_phi, without allocating any memory:
 * the solver's work arrays live in one fixed device area of about 1.8 MB per
 * device, so the state must have at most RC_NOALLOC_MAX_UNKNOWNS unknowns
 * and a box of at most RC_NOALLOC_MAX_BOX_SITES sites (RC_ERR_CAPACITY
 * otherwise, nothing launched).  For hosts that may not allocate device
 * memory inside their time loop.  The first call on a device looks the area
 * up (cudaGetSymbolAddress); with CUDA's lazy module loading (the default)
 * that lookup may load the library's device code and with it the area, i.e.
 * the first call per device can allocate: make it during set-up, before the
 * time loop and before any stream capture.  Later calls allocate nothing.
 * The area is shared: calls on one device must not overlap in time (from any
 * engine or stream), or they race.  Runs on the engine's stream and returns
 * when the solve is done; it does not wait for work the caller has pending
 * on vx and vy in other streams (finish or order that first).  `iterations`
 * (may be NULL) receives the CG iterations of both components.
 * RC_ERR_UNSUPPORTED if the last evaluation had no viscous solve.
 */
#define RC_NOALLOC_MAX_UNKNOWNS 32768
#define RC_NOALLOC_MAX_BOX_SITES 16384
int rc_viscous_resolve_noalloc(rc_engine *e, double *vx, double *vy, long long n, int *iterations);

/*
 * The learned preconditioner's network (no counterpart in the reference).
 * RC_UNET_PARAMS parameters: 11 layers of 3x3 convolutions on the periodic
 * box grid, each 9*ci*co weights w[tap][ci][co] then co biases; the layer
 * list is in rheocell_gb300/csrc/rc_unet.cuh.
 *
 * rc_unet_loss_grad: one FP32 forward, loss and backward pass on the device
 * for host data: input [batch][L][L][2], target [batch][L][L]; loss = mean
 * over samples of |f - target|^2 / |target|^2; grad (RC_UNET_PARAMS values)
 * and output ([batch][L][L]) may be NULL.  L must be a multiple of 4.
 */
#define RC_UNET_PARAMS 25937
/*
 * Tile-shape autotuning of the FP32 cell kernel (precision RC_PRECISION_FLOAT;
 * no counterpart in the reference, whose update is one serial loop,
 * FD_CPUBackend.cpp:44-120).  Each cell patch is swept by one CTA in tiles of
 * `threads` patch sites; rc_autotune times every candidate tile (128, 256,
 * 512 sites) over `steps_per_candidate` steps of this engine's own workload
 * (one untimed step first) by the stage timers of the cell kernels (updates
 * and force evaluations; ms_per_step reports their time per step) and keeps
 * the fastest.  The simulation advances by
 * 3 x (steps_per_candidate + 1) steps.  The FP32 results of different tiles
 * differ by rounding only (their per-warp partial sums are grouped
 * differently).  FP64 engines keep one tile (their summation order is part of
 * their parity with the reference): candidates = 0.
 * rc_set_cell_threads sets the tile directly (128, 256 or 512).
 */
typedef struct rc_autotune_report {
    int candidates;          /* tiles tried */
    int threads[4];          /* patch sites per tile of each candidate */
    double ms_per_step[4];   /* measured step time of each (CUDA events) */
    int chosen;              /* tile in use afterwards */
} rc_autotune_report;
int rc_autotune(rc_engine *e, int steps_per_candidate, rc_autotune_report *report);
int rc_set_cell_threads(rc_engine *e, int threads);

/* rc_unet_forward_tc: the network's forward pass as the solve runs it
 * (BF16 activations, tensor-core layers, FP32 first and last layers);
 * input [batch][L][L][2], output [batch][L][L].  No counterpart in the
 * reference (the learned preconditioner is this engine's own). */
int rc_unet_forward_tc(int L, int batch, const double *params, const double *input, double *output, int device);
/* rc_unet_loss_grad: one training pass of the network (FP32 forward,
 * relative-L2 loss against target [batch][L][L], backward): the loss, the
 * gradient of all RC_UNET_PARAMS parameters and the output.  No counterpart
 * in the reference. */
int rc_unet_loss_grad(int L, int batch, const double *params, const double *input, const double *target,
                      double *loss, double *grad, double *output, int device);

/*
 * Learned preconditioner for the wet models' viscous solve (no counterpart
 * in the reference, whose solve is Eigen's Jacobi-preconditioned CG,
 * WetModel.cpp:361-376).
 *
 * The patch-stacked system reduces exactly to a box-grid one: with
 * T(k) = xi + eta D(k), R[k] = sum_{j at k} r_j / T(k), W[k] = n(k) / T(k),
 * the box sums V = S v solve V - eta W (N4 V) = R, and v_j = (r_j + eta
 * (N4 V)[k_j]) / T(k_j).  The network maps (R/s, W) to V/s (s = |r| /
 * sqrt(S)); inside flexible CG (FCG(1)) it serves as the preconditioner of
 * the FP32 inner iterations of the mixed-precision solve, whose FP64
 * iterative refinement keeps the RC_PRECISION_MIXED guarantees (true FP64
 * residual below cg_tolerance; a sweep that fails to halve the residual
 * hands over to plain FP64 CG).
 *
 * rc_learned_harvest: collect training samples from the following plain
 * FP64 solves (RC_SOLVER_PLAIN with RC_PRECISION_DOUBLE, or
 * RC_SOLVER_PLAIN_FP64): at sweeps 0,
 * every, 2*every, ... (at most per_solve points per solve) each velocity
 * component gives the pair (box residual, box error), until `capacity`
 * samples are stored.  capacity = 0 stops harvesting and frees the store;
 * per_solve = 0 (capacity > 0) stops collecting and keeps the samples.
 * rc_learned_harvested: samples stored so far (synchronises).
 * rc_learned_train: Adam on the stored samples (device forward and backward
 * kernels); the trained parameters become the engine's.
 * rc_set_solver: RC_SOLVER_PLAIN (default), RC_SOLVER_PLAIN_FP64 or
 * RC_SOLVER_LEARNED (needs parameters, from training or
 * rc_learned_set_params, and a box side that is a multiple of 4).
 */
#define RC_SOLVER_PLAIN 0
#define RC_SOLVER_LEARNED 1        /* network on the tensor cores (BF16 activations) */
#define RC_SOLVER_LEARNED_FP32 2   /* the same network in FP32 on the CUDA cores     */
#define RC_SOLVER_PLAIN_FP64 3     /* Eigen's Jacobi CG in FP64 whatever the engine's
                                      precision (RC_SOLVER_PLAIN follows it: the
                                      FP32 inner iterations for mixed and float) */

typedef struct rc_train_options {
	int epochs;                 /* passes over the training samples (<= 0: 8)         */
	int batch;                  /* samples per Adam step (<= 0: 8)                     */
	double learning_rate;       /* Adam step size (<= 0: 1e-3)                         */
	double validation;          /* fraction held out for validation (< 0: 0.1)         */
	unsigned long long seed;    /* initialisation and shuffling                        */
	int init;                   /* 1: fresh initialisation; 0: continue from the current parameters */
	int max_samples;            /* use at most this many samples (<= 0: all)           */
	double learning_rate_final; /* cosine decay of the step size to this value over the run (<= 0: constant) */
} rc_train_options;

typedef struct rc_train_report {
	int samples;                /* valid harvested samples used                        */
	int train_samples, validation_samples;
	int epochs, steps;
	double loss_first_epoch;    /* mean training loss over the first epoch             */
	double loss_last_epoch;     /* ... over the last epoch                             */
	double validation_loss_init;/* validation loss before training                     */
	double validation_loss;     /* ... after                                           */
	double ms;                  /* wall time of the training                           */
} rc_train_report;

int rc_learned_harvest(rc_engine *e, int capacity, int every, int per_solve);
int rc_learned_harvested(rc_engine *e);
int rc_learned_train(rc_engine *e, const rc_train_options *options, rc_train_report *report);
int rc_learned_get_params(rc_engine *e, double *params);
int rc_learned_set_params(rc_engine *e, const double *params);
int rc_set_solver(rc_engine *e, int solver);

/*
 * rc_viscous_resolve: run the viscous solve of the last force evaluation
 * again, from a cold start, with `solver` (RC_SOLVER_PLAIN: the engine's
 * precision -- FP64 CG for RC_PRECISION_DOUBLE; RC_SOLVER_PLAIN_FP64: FP64 CG
 * for any precision; or a learned solver, which needs parameters) into vx
 * and vy, device arrays of n = rc_site_count(e)
 * doubles in the order of rc_download_phi.  The engine's velocities,
 * warm-start schedule and counters are unchanged, so solvers can be compared
 * on one right-hand side without advancing the simulation.  `stats` (may be
 * NULL) receives the solve's counters.  RC_ERR_UNSUPPORTED if the last
 * evaluation had no viscous solve.  Synchronises.  No counterpart in the
 * reference (the closest is calling Eigen's solve() twice,
 * WetModel.cpp:364-375).
 */
int rc_viscous_resolve(rc_engine *e, int solver, double *vx, double *vy, long long n, rc_step_stats *stats);

/*
 * rc_set_cg_limits: cap every viscous solve at max_iterations iterations
 * per component (0: Eigen's default, twice the number of unknowns,
 * WetModel.cpp:361-376 with Eigen's ConjugateGradient defaults).  With
 * fail_on_no_convergence != 0, a solve that stops at the cap with its
 * residual above the tolerance makes rc_step fail with RC_ERR_CG (the
 * reference, like Eigen, carries on silently; it never reads
 * solverCG.info()).
 */
int rc_set_cg_limits(rc_engine *e, long long max_iterations, int fail_on_no_convergence);

/*
 * rc_set_cg_tolerance: the relative residual at which every following
 * viscous solve stops (the CGtolerance key, WetModel.cpp:59-60; 0: Eigen's
 * default, machine epsilon).  Lets a host solve one right-hand side to a
 * much tighter tolerance (with rc_viscous_resolve) as the reference
 * solution other solves are measured against.
 */
int rc_set_cg_tolerance(rc_engine *e, double tolerance);

/*
 * Test hook of the solve's failure detection (no counterpart in the
 * reference).  spin_limit: polls of a grid-barrier wait before it gives up
 * (0: the default, about 1-2 s).  unreachable != 0 makes the first grid
 * barrier of every later solve wait for one arrival more than the grid has
 * blocks, which never comes: every block gives up after spin_limit polls,
 * the kernel returns, and rc_step fails with RC_ERR_CG ("grid barrier timed
 * out") with the CUDA context intact.  The engine's state is then undefined;
 * destroy it.
 */
int rc_test_barrier_timeout(rc_engine *e, long long spin_limit, int unreachable);

/*
 * Diagnostic timers of the learned solve, read on the device clock by one
 * block at the end of each phase (each phase's time includes the grid
 * barrier that ends it).  enable = 1 zeroes and starts them, 0 stops them;
 * ms (may be NULL) receives the totals so far, up to n of: network input
 * gather, first layer, tensor-core layers at levels 0, 1, 2, last layer,
 * preconditioned residual, flexible-CG phases A, B, C, everything else,
 * then (within the tensor-core layers) weight staging, operand staging,
 * MMA issue and completion, epilogue as one write-out thread sees them, the
 * MMA thread's waits (row staged, accumulator slot free) and issue, and one
 * staging thread's waits (buffer free) and loads.  No counterpart in the
 * reference.
 */
int rc_solver_profile(rc_engine *e, int enable, double *ms, int n);

/*
 * Self-test of the engine's double <-> float conversions on the integer
 * pipes (the FP32 cell kernels use them in place of the conversion
 * instructions, which issue on the narrow FP64 pipe of GB300).  On device
 * `device`, converts the n doubles of `in` (host array) by the exact form
 * (round to nearest even; below the FP32 normal range to signed zero) into
 * `exact`, by the short streaming form (round to nearest, ties away; below
 * the normal range to signed zero; beyond the FP32 range, infinities and NaN
 * to NaN) into `fast`, and by CUDA's __double2float_rn into `cuda_rn`, and
 * widens cuda_rn back to double by the integer form into `widened` (host
 * arrays of n).  No counterpart in the reference.
 */
int rc_selftest_conversions(const double *in, float *exact, float *fast, float *cuda_rn, double *widened, long long n,
                            int device);

/*
 * Diagnostic observables computed on the device from the current state.
 *
 * rc_observe_field: the box fields of the reference's field observables --
 * RC_OBS_VELOCITY (VelocityField::calc_field, src/Observables/
 * VelocityField.cpp:69-78: sum of v * phi), RC_OBS_SHAPE (ShapeField.cpp:
 * 69-78: S00 * phi, S01 * phi) and RC_OBS_NEMATIC (NematicField.cpp:69-78:
 * Q00 * phi, Q01 * phi) -- summed over the cells of monolayer `layer` (of
 * type only_type; -1: all) in index order, into fx, fy (L*L each, row-major
 * box sites).  With size_grid > 0 also the coarse-grained fields
 * (VelocityField.cpp:105-121) into coarse_x, coarse_y (may be NULL).
 * The force kinds are the box fields of ForceField / StressField::calc_field
 * (src/Observables/ForceField.cpp:79-96, StressField.cpp:84-100) from the
 * last force evaluation: RC_OBS_FORCE the total force, velocity times the
 * friction (get_total_force_x/y); RC_OBS_FORCE_PASSIVE and
 * RC_OBS_FORCE_ACTIVE the interaction's Fpassive / Factive split
 * (e.g. WetModel.cpp:636-637,655-656); RC_OBS_PRESSURE the pressure
 * Rep - CH - A (WetModel.cpp:605) in fx and the phi field in fy.  Their
 * coarse fields are ForceField's window means (ForceField.cpp:141-160).
 * RC_OBS_THERMO, RC_OBS_THERMO_XY and RC_OBS_CHEMPOT2 are the unweighted box
 * sums of ThermodynamicStressField::calc_field (ThermodynamicStressField.cpp:
 * 75-99): xx and yy of f_d - mu phi + d phi g (g = 2 gamma lambda grad(phi)
 * where the interaction sets it, WetModel.cpp:607-609, SimpleMultiField.cpp:
 * 178-180), then xy = d_x phi g_y with the sum of mu, then the sums of mu^2
 * and phi; their coarse fields are its window means (:131-150).
 * The split is formed by evaluating the forces again at the current state,
 * which leaves the simulation unchanged (FP64 engines only).
 *
 * rc_observe_stress: StressField's coarse stress of one of the force kinds
 * (StressField.cpp:171-199): per box site, over the size_grid^2 periodic
 * window, with e the unit vector from the window site to the centre,
 * xx = sum fx ex / sg^2, yy = sum fy ey / sg^2,
 * xy = sum (fx ey + fy ex) / (2 sg^2); for RC_OBS_PRESSURE xx and yy of the
 * pressure field (xy is not formed and may be NULL).
 *
 * rc_observe_cells: per cell (6 doubles each, cell order): unwrapped centre
 * of mass x, y; area; elongation |S|; aspect ratio sqrt(s1/s2) - 1;
 * orientation atan2(S01, S00)/2 -- from the current gradients, as
 * scripts/calcAvgShape.py:274-336 forms them; and per monolayer (4 doubles
 * each): mean area, area variance, mean elongation, mean aspect ratio.
 * Either pointer may be NULL.
 */
#define RC_OBS_VELOCITY 0
#define RC_OBS_SHAPE 1
#define RC_OBS_NEMATIC 2
#define RC_OBS_FORCE 3
#define RC_OBS_FORCE_PASSIVE 4
#define RC_OBS_FORCE_ACTIVE 5
#define RC_OBS_PRESSURE 6
#define RC_OBS_THERMO 7      /* ThermodynamicStressField xx, yy */
#define RC_OBS_THERMO_XY 8   /* ThermodynamicStressField xy, sum of mu */
#define RC_OBS_CHEMPOT2 9    /* ThermodynamicStressField sum of mu^2, sum of phi */
int rc_observe_field(rc_engine *e, int kind, int layer, int only_type, int size_grid, double *fx, double *fy,
                     double *coarse_x, double *coarse_y);
int rc_observe_stress(rc_engine *e, int kind, int layer, int only_type, int size_grid, double *xx, double *yy,
                      double *xy);
int rc_observe_cells(rc_engine *e, double *cell_obs, double *layer_obs);

/* Sites (sum of LsubX*LsubY) in the current configuration: the reference's
 * stacked unknown count size_rows (src/Interactions/WetModel.cpp:203-209). */
long long rc_site_count(const rc_engine *e);

/* Message of the last failure on this engine (or of the last failed create):
 * the text the reference's RCexception carries to main
 * (src/rheoCell.cpp:40-43). */
const char *rc_last_error(const rc_engine *e);

/* Release the engine's device memory, stream and graphs: the backend's
 * destruction (SimBackend::~SimBackend, src/Backends/SimBackend.cpp:37-39;
 * FD_CPUBackend::~FD_CPUBackend, src/Backends/FD_CPUBackend.cpp:9).  NULL is
 * a no-op. */
void rc_destroy(rc_engine *e);

#ifdef __cplusplus
}
#endif

#endif /* RHEOCELL_GB300_H */
