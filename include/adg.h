/*
 * adg.h -- C ABI of the GB300 (sm_103a) ADER-DG element path.
 *
 * Drop-in boundary for the hot path of AmrDG<P>::ADER
 * (reference: Source/NumericalMethod/AmrDG/AmrDG.h:1071-1165) and the
 * L2ProjInterp AMR transfer operators (AmrDG_Interpolater.tpp:7-448).
 * Plain C types only: sizes, host pointers and device pointers.  Every entry
 * point returns an int status (ADG_OK = 0); adg_last_error() gives the text.
 *
 * Data layout (HBM): one packed array per AMR level, element-major
 * U_w[cell][q][n] (q = conserved variable, n = spatial Legendre mode, the
 * reference's MultiIndex order AmrDG.h:62-122), cells ordered x-fastest over
 * the level's valid cells.  The context owns all device memory of the
 * hierarchy; adg_get_state/adg_set_state copy a level in or out (host or
 * device pointers, see ADG_MEM_*).
 */
#ifndef ADG_H
#define ADG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADG_OK 0
#define ADG_ERR_ARG 1          /* invalid argument / unsupported (D, P) */
#define ADG_ERR_CUDA 2         /* CUDA runtime error */
#define ADG_ERR_LAYOUT 3       /* invalid box layout (nesting, overlap) */
#define ADG_ERR_NUMERIC 4      /* device status: NaN or non-positive density */
#define ADG_ERR_STATE 5        /* call out of order (e.g. step before init) */
#define ADG_ERR_NOALLOC_CAPACITY 6 /* problem larger than the fixed scratch of adg_ader_step_noalloc */
#define ADG_ERR_IO 7           /* plotfile missing, malformed or not matching the configuration */

#define ADG_MEM_HOST 0
#define ADG_MEM_DEVICE 1
#define ADG_MEM_HOST_ASYNC 2 /* page-locked host buffer; the copy is queued on the context's stream and the
                                call returns at once: adg_synchronize before the buffer is read or reused */

/* Initial conditions (Source/Model/CompressibleEuler/Compressible_Euler.h:120-368). */
#define ADG_IC_VORTEX 0     /* isentropic vortex, free stream (u_inf, v_inf) */
#define ADG_IC_KH_NOISE 1   /* KH: sin(4 pi x) + seeded noise of amplitude noise_amp */
#define ADG_IC_KH_REF 2     /* reference KH (Gaussian-localised v) */
#define ADG_IC_BLAST3D 3    /* spherical blast in [0,1]^3 */
#define ADG_IC_CONST 4      /* uniform free stream */

typedef struct adg_config {
  int D, P;                 /* spatial dimension 2|3; polynomial degree 1..6 at D = 2, 1..3 at D = 3
                               (the learned seed: P <= 3 at D = 2, P <= 2 at D = 3) */
  double gamma;             /* adiabatic index (Compressible_Euler.cpp:42-47) */
  double c_dt;              /* CFL safety factor (Solver::c_dt) */
  int n_cell[3];            /* level-0 cells per dimension */
  double prob_lo[3], prob_hi[3];
  int periodic[3];          /* 1 periodic, 0 outflow (zero-gradient mode copy) */
  int ic;                   /* ADG_IC_* */
  double u_inf, v_inf, beta, xc, yc;
  uint64_t seed;            /* noise seed of ADG_IC_KH_NOISE */
  double noise_amp;
  int max_grid;             /* max cells per box edge */
  /* AMR (max_level = 0: single level) */
  int max_level;
  int blocking_factor;
  int dtn_regrid;           /* regrid every n steps (Mesh::dtn_regrid) */
  int tag_kind;             /* ADG_TAG_* */
  double tag_threshold;     /* threshold of ADG_TAG_DENSITY_GRADIENT / ADG_TAG_PRESSURE_JUMP */
  double grid_eff;
  int n_error_buf;
  int reflux_box_quirk;     /* 1: reference's per-box reflux mask (AmrDG_Interpolater.tpp:41-56) */
  int picard_sweeps;        /* predictor sweeps; <= 0 means P (AmrDG.h:1103-1119) */
  int elems_per_block;      /* 0: autotuned default */
  /* TVB limiter of the finest level after every limiter_t-th ADER step
   * (AmrDG.h:990-997, Limiter_w AmrDG.h:1657-1855; 0: off): a linear mode is
   * kept where |slope| <= tvb_c[l] * tvb_M * h^2 (h the level's smallest cell
   * size), else the characteristic minmod of the slope and the neighbours'
   * mean differences (limiter_type "TVB", TVB_M, AMR_TVB_C, t_limit of
   * setNumericalSettings, Source/main.cpp:147). */
  int limiter_t;
  double tvb_M;
  double tvb_c[8];
  /* Regrid once dt_regrid of simulated time has passed since the last regrid
   * (Mesh::dt_regrid, AmrDG.h:936-941; <= 0: off).  The decision reads the
   * time from the device, one synchronisation per step while it is on. */
  double dt_regrid;
  /* Per-level coefficient of the reference's tagging criteria (amr_c of
   * setGeometrySettings, Source/main.cpp:125-138; <= 0 means 1.0). */
  double amr_c[8];
  /* ADG_TAG_VORTEX: 1 moves the tagged disc's centre with the free stream
   * (xc + u_inf t, yc + v_inf t); 0 keeps it at (xc, yc) as the reference's
   * current code does (Compressible_Euler.h:629-630). */
  int tag_advect;
  /* Initial condition of the finer levels (Solver::setValidationMode,
   * Solver.h:711-734): 0 the projection of the coarser level; 1 the analytic
   * IC on every level, then average down and the ghost fill of every level
   * (AMR_sync_initial_condition, AmrDG_Level.tpp:94-118); 2 as 1, but the
   * finer levels' coarse-fine ghost cells keep their own analytic projection
   * until the first step's ghost fill (how the reference's recorded
   * static-refinement convergence runs were initialised). */
  int validation_mode;
  /* 1: no coarse-fine flux correction (the reference's "NO REFLUX" runs). */
  int no_reflux;
} adg_config;

/* Refinement criteria (tag_kind). */
#define ADG_TAG_DENSITY_GRADIENT 0 /* max_d |rho_{i+1} - rho_{i-1}| / (2 rho_i) > tag_threshold (cell means) */
#define ADG_TAG_PRESSURE_JUMP 1    /* the same on the cell-mean pressure */
#define ADG_TAG_VORTEX 2           /* Compressible_Euler.h:615-644: cell centre within amr_c[l]^2 of the vortex
                                      centre (distances wrapped once by half the domain) */
#define ADG_TAG_KH_TVB 3           /* Compressible_Euler.h:645-682: a characteristic slope of the cell fails
                                      minmodB's test |slope| <= tvb_c[l] * amr_c[l] * h^2 */

typedef struct adg_ctx adg_ctx;

/* Context: builds the element operators for (D, P) and owns device state.
 * Replaces AmrDG<P>::init (Source/NumericalMethod/AmrDG/AmrDG.tpp:82-246). */
int adg_ctx_create(const adg_config* cfg, adg_ctx** out);
int adg_ctx_destroy(adg_ctx* ctx);
const char* adg_last_error(const adg_ctx* ctx);

/* Stream all work is issued on (default: the context's own stream). */
int adg_set_stream(adg_ctx* ctx, void* cuda_stream);

/* Build the level-0 layout and project the initial condition on the device.
 * Replaces Solver::init + AmrDG::set_initial_condition
 * (Source/Core/Solver.h:502-597, Source/NumericalMethod/AmrDG/AmrDG.h:782-836),
 * then computes the first Dt (AmrDG.h:1253-1357). */
int adg_init(adg_ctx* ctx);

/* Level state in/out: n_cells * Q * Np_s doubles, element-major, cells in
 * x-fastest order over the level's valid cells.  Setting a level that has a
 * finer level makes that level's coarse-fine ghosts stale; they are projected
 * again once, before the next kernel that reads them (a step, adg_ader,
 * adg_predictor, adg_tags) or by adg_fill_ghosts.  lev = ADG_ALL_LEVELS:
 * every level in one copy, packed in level order (level 0's cells, then
 * level 1's, ...; counts from adg_level_cells). */
#define ADG_ALL_LEVELS (-1)
int adg_num_levels(const adg_ctx* ctx, int* nlev);
int adg_level_cells(const adg_ctx* ctx, int lev, int64_t* ncells);
int adg_get_state(adg_ctx* ctx, int lev, double* dst, int mem);
int adg_set_state(adg_ctx* ctx, int lev, const double* src, int mem);
/* Step readback: register a page-locked host buffer with room for
 * capacity_cells * Q * Np_s doubles (at least the level's valid cells) that
 * receives level lev's state, as adg_get_state returns it (the level's
 * current valid cells, adg_level_cells), at the end of every step of
 * adg_step and adg_advance (also the timed forms).  The copy waits only for
 * the step's last writer of that level
 * (the corrector or limiter for the finest level, the average down onto it
 * for the others) and runs on its own stream beside the rest of the step;
 * the next step and anything queued after adg_advance are ordered after it,
 * and it is complete after adg_synchronize.  host = NULL clears; a cleared
 * or replaced buffer may be released after adg_synchronize.  Regrids keep
 * the registration while the level's cells fit; one that removes the level
 * or grows it past the capacity drops it, and no copy of the new layout goes
 * into the buffer (adg_readback_active then reports 0 and the buffer does
 * not hold that step's state: read it with adg_get_state).  lev =
 * ADG_ALL_LEVELS registers one buffer for every level packed in level order
 * (as adg_get_state with ADG_ALL_LEVELS; capacity = all levels' cells), each
 * level copied into its place as soon as it is final.  Steps of
 * adg_time_kernels do not read back.  For a caller that keeps the state on
 * the host: the per-step output of U_w(l, q) at the end of a step of
 * AmrDG::evolve (after the limiter and the average down,
 * Source/NumericalMethod/AmrDG/AmrDG.h:988-1025). */
int adg_set_readback(adg_ctx* ctx, int lev, double* host, int64_t capacity_cells);
int adg_readback_active(adg_ctx* ctx, int lev, int* active);
/* Waits for everything queued on the context's stream (copies of
 * ADG_MEM_HOST_ASYNC, steps of adg_advance and their readback). */
int adg_synchronize(adg_ctx* ctx);

/* Time step size: current Dt (device-computed), set an explicit Dt, or
 * recompute it from the state (set_Dt, AmrDG.h:1253-1357). */
int adg_get_dt(adg_ctx* ctx, double* dt);
int adg_set_dt(adg_ctx* ctx, double dt);
int adg_compute_dt(adg_ctx* ctx, double* dt);
int adg_get_time(adg_ctx* ctx, double* t);

/* One ADER predictor-corrector step of every level with the current Dt
 * (AmrDG<P>::ADER, AmrDG.h:1071-1165), without the Dt update. */
int adg_ader(adg_ctx* ctx);

/* One full step of the evolve loop body (AmrDG.h:935-1029): regrid when due,
 * ADER, average down, ghost fill, t += Dt, new Dt. */
int adg_step(adg_ctx* ctx);

/* n steps; use_graph != 0 replays a captured CUDA graph of the step
 * (re-captured when the layout changes). */
int adg_advance(adg_ctx* ctx, int nsteps, int use_graph);

/* AMR layout: number of regrids so far; boxes of a level
 * (out[6*b + {lo0,lo1,lo2,hi0,hi1,hi2}], up to cap boxes); refinement tags
 * of the valid cells of a level from the current state (1 byte per cell, the
 * level's cell order).  (AmrDG_TagCellRef.tpp:4-52, Mesh::regrid) */
int adg_regrid_count(const adg_ctx* ctx, int* n);
/* DOF updates done so far (sum over steps of valid elements of every level
 * times Q * Np_s) and the host wall time spent in regrids. */
int adg_dof_updates(const adg_ctx* ctx, int64_t* total, double* regrid_ms);
/* The same count over leaf elements only (valid elements not covered by a
 * finer level).  No reference counterpart. */
int adg_leaf_dof_updates(const adg_ctx* ctx, int64_t* total);
/* Lp norm (p = 1 or 2) of component q of the solution minus the analytic
 * initial condition, over the leaf cells, with the reference's quadrature
 * (N = P + 1 GL points per dimension for p = 1, 2N for p = 2):
 * LpNorm_DG_AMR, AmrDG.h:1399-1578 (the vortex after one period returns to
 * its initial state, so this is the error the reference's convergence runs
 * report). */
int adg_lp_norm(adg_ctx* ctx, int p, int q, double* out);
/* Elements the TVB limiter has modified so far (the reference's
 * n_limited_total, AmrDG.h:996). */
int adg_limited_count(adg_ctx* ctx, int64_t* n);
/* Host wall time of the regrids so far by phase, ms[0..n) with n <= 6:
 * [0] tag kernels and the wait for the state, [1] clustering,
 * [2] hierarchy and remap tables, [3] table upload, [4] remap launches,
 * [5] CUDA graph capture/update after a layout change.  No reference
 * counterpart (an instrumentation entry point of this library). */
int adg_regrid_profile(const adg_ctx* ctx, double* ms, int n);
int adg_get_boxes(const adg_ctx* ctx, int lev, int* out, int cap, int* nbox);
/* Layout from the caller (e.g. the BoxArrays of an AMReX hierarchy after its
 * regrid, Mesh.h:156-196): nbox[l] boxes of level l < nlev in
 * boxes[6 * (sum of earlier counts + b) + {lo0,lo1,lo2,hi0,hi1,hi2}], level
 * cell indices.  Levels must be properly nested; level 0 must cover the
 * domain.  The state is remapped as AMR_remake_level / AMR_make_new_fine_level
 * do (AmrDG_Level.tpp:52-132): old data where a cell stays valid, the L2
 * projection of the coarser level elsewhere.  The context stops regridding
 * on its own first step (it still regrids every dtn_regrid steps when
 * dtn_regrid > 0: give 0 to leave the layout to the caller). */
int adg_set_layout(adg_ctx* ctx, int nlev, const int* nbox, const int* boxes);
/* Cell indices (i, j, k) of the valid cells of a level in the order of the
 * level's state arrays (3 ints per cell). */
int adg_level_cell_coords(const adg_ctx* ctx, int lev, int* ijk);
int adg_tags(adg_ctx* ctx, int lev, uint8_t* out);

/* L2ProjInterp transfer operators (AmrDG_Interpolater.tpp:283-398) for a caller
 * that keeps its own FillPatch / average-down machinery and wants the
 * projections on the GPU.  mem: ADG_MEM_HOST or ADG_MEM_DEVICE for every array.
 * adg_interp_scatter (amr_scatter): fine[i] = Minv P_cf[child[i]] coarse[i] for
 * i < n; coarse and fine [n][Q][Np_s]; child[i] in [0, 2^D), bit (D-1-d) set
 * for the upper half in direction d (host children out of range: ADG_ERR_ARG;
 * device ones give NaN).
 * adg_interp_gather (amr_gather): coarse[i] = 2^-D Minv sum_l P_fc[l] fine[i][l];
 * fine [n][2^D][Q][Np_s] with children numbered as above, coarse [n][Q][Np_s].
 * adg_average_down (Solver::AMR_average_fine_coarse): every covered cell of
 * the context's layout from its children, finest level first.
 * adg_fill_ghosts (the coarse-interpolated part of FillPatchTwoLevels): the
 * context's coarse-fine ghost elements from their coarse parents.
 * The coarse-fine flux correction (FluxRegister + L2ProjInterp::reflux) has no
 * entry point of its own: it is part of adg_ader's corrector. */
int adg_interp_scatter(adg_ctx* ctx, const double* coarse, const int8_t* child, int64_t n, double* fine, int mem);
int adg_interp_gather(adg_ctx* ctx, const double* fine, int64_t n, double* coarse, int mem);
int adg_average_down(adg_ctx* ctx);
int adg_fill_ghosts(adg_ctx* ctx);
/* The TVB limiter of the finest level on the current state (Limiter_w,
 * AmrDG.h:1657-1855), the stage the evolve loop runs between ADER and the
 * average down (AmrDG.h:990-997): call it after adg_ader, whose predictor
 * records the cell means an outflow boundary's neighbour takes.  Needs
 * limiter_t > 0 at creation; *n_limited (may be NULL) receives the elements
 * this call modified. */
int adg_limit(adg_ctx* ctx, int64_t* n_limited);

/* Zero-copy boundary to the caller's per-box device arrays.
 *
 * The reference keeps the state as one MultiFab per (level, q) whose
 * FArrayBoxes hold the Np_s modes of U_w as components, with nghost ghost
 * cells (Source/NumericalMethod/AmrDG/AmrDG.tpp:300-333, Solver.h:408-457).
 * An adg_patch describes one box of that hierarchy: its level and valid box,
 * the ghost width of its arrays, the Q device pointers (FArrayBox data of
 * U_w(level, q), x fastest over the grown box, then y, z and the component)
 * and the strides of j, k and the component in doubles.
 * adg_set_patches registers patches that tile the context's current layout
 * exactly (every valid cell in one patch; a layout from adg_set_layout with
 * the same BoxArrays, or the context's own); after a layout change they must
 * be registered again (ADG_ERR_LAYOUT until then).  adg_read_patches copies
 * every valid cell of the patches into the context's state, adg_write_patches
 * the state into the patches' valid cells (ghost cells are the caller's
 * FillPatch); both are device-to-device kernels queued on the context's
 * stream (adg_synchronize before the host reads the arrays), so an AMReX
 * build with device MultiFabs needs no host copy per step.  No reference
 * counterpart beyond the data layout. */
typedef struct adg_patch {
  int level;
  int lo[3], hi[3];      /* valid box in the level's cell index space */
  int nghost;            /* ghost cells on every side of the arrays */
  double* U_w[5];        /* device pointer per conserved variable q < Q */
  int64_t jstride, kstride, nstride;  /* doubles between j, k and component neighbours */
} adg_patch;
int adg_set_patches(adg_ctx* ctx, const adg_patch* patches, int n);
int adg_read_patches(adg_ctx* ctx);
int adg_write_patches(adg_ctx* ctx);

/* Completed steps of the evolve loop (the reference's n, AmrDG.h:868-877,
 * 1012); a restart from a plotfile continues its count. */
int adg_get_step(const adg_ctx* ctx, int64_t* n);

/* Plotfiles (checkpoint / restart).
 *
 * adg_write_plotfile replaces Solver::PlotFile (Source/Core/Solver.h:922-968):
 * one AMReX plotfile per conserved variable q, <data_dir>/tstep_<tstep>_q_<q>_plt,
 * holding the Np_s modal coefficients of U_w as components named
 * "<var_names[q]>_<m>", the level hierarchy (boxes, domains, cell sizes,
 * refinement ratio 2), the current time and tstep as every level's step.
 * level < 0 writes every level, level >= 0 only that one.  var_names NULL:
 * the reference's Compressible_Euler names (mass_density, momentum_x,
 * momentum_y, energy_density in 2D; momentum_z before energy_density in 3D).
 * Directories are created as needed; existing files are overwritten.
 *
 * adg_read_plotfile replaces Solver::ReadPlotFile (Source/Core/Solver.h:599-652)
 * and the FillPatch that follows it in Solver::init (:572-593): it reads the
 * Q plotfiles of tstep, restores the boxes of levels 0..min(finest, max_level),
 * the state, the time and the step count, fills the coarse-fine ghosts and
 * recomputes Dt; the next step regrids first, as the reference's evolve loop
 * does after a restart (AmrDG.h:868-877, 938-940).  Everything is checked
 * (dimension, component count, level-0 domain, ratio 2, consistent boxes over
 * q) before the context changes: on ADG_ERR_IO it is as before the call.
 * time may be NULL. */
int adg_write_plotfile(adg_ctx* ctx, const char* data_dir, int tstep, int level, const char* const* var_names);
int adg_read_plotfile(adg_ctx* ctx, const char* data_dir, int tstep, double* time);
/* Header of one plotfile directory without a context or a GPU (all levels'
 * multifab and FAB headers are checked, no data is read): dimension,
 * component count, finest level, time and level-0 step.  Any output may be
 * NULL.  Returns ADG_ERR_IO for a missing or malformed plotfile, with the
 * reason in err (err_cap bytes, may be NULL). */
int adg_plotfile_info(const char* plotfile_dir, int* dim, int* ncomp, int* finest_level, double* time, int* step,
                      char* err, int err_cap);

/* Per-stage entry points (parity testing). */
/* Predictor only for level lev: writes H_w (Q * Np_st per cell, element-major)
 * for the valid cells to dst (device pointer). (AmrDG.tpp:495-537, 744-827) */
int adg_predictor(adg_ctx* ctx, int lev, double* dst_dev);

/* Device status word: bit 0 NaN, bit 1 non-positive density, bit 2 pressure
 * floored (Compressible_Euler.h:586); cleared on read. */
int adg_status(adg_ctx* ctx, uint32_t* status);

/* Kernel launches issued by this context since creation (all kernels). */
int adg_launch_count(const adg_ctx* ctx, int64_t* n);

/* Select the CUDA device for contexts created afterwards by this thread. */
int adg_set_device(int device);

/* n steps like adg_advance, bracketed by CUDA events recorded on the
 * context's stream; *ms receives the device time of the n steps. */
int adg_advance_timed(adg_ctx* ctx, int nsteps, int use_graph, double* ms);
/* The same with the L2 evicted before every step (a device memset of
 * flush_bytes, outside the timed region): ms = the sum over the steps of
 * the device time from the step's start (regrid included) to its end.
 * No reference counterpart (benchmark timing). */
int adg_advance_timed_flushed(adg_ctx* ctx, int nsteps, int use_graph, int64_t flush_bytes, double* ms);

/* n steps with CUDA events around every kernel on the context's stream;
 * ms[k] receives the average duration of kernel kind k per step:
 * 0 predictor (+ corrector volume term and face traces; with a seed
 * attached: the seed inference, the seeded predictor and the fallback),
 * 1 numerical flux, 2 corrector update, 3 time-step reduction, 4 AMR
 * synchronisation, 5 the seed inference alone, 6 the seeded predictor alone,
 * 7 the fallback pass (5-7: 0 without a seed). */
int adg_time_kernels(adg_ctx* ctx, int nsteps, double* ms, int nkinds);

/* Autotuner of the predictor's elements per block (the launch shape of its
 * largest kernel; results do not depend on it, bit for bit): times every
 * choice the configuration is built with for nsteps steps of the context's
 * current layout, from a snapshot of the state that is restored afterwards
 * (the context's state, time, step count and counters are unchanged), keeps
 * the fastest in the context and records it per GPU model, (D, P), level-0
 * grid, finest level and stage (plain FP64, or the attached seed's mode) in
 * a text file: ADG_TUNE_CACHE, else $HOME/.cache/adg_gb300/tune.txt.
 * Contexts created with elems_per_block = 0 take the recorded choice at
 * adg_init and adg_seed_attach.  With a seed attached the seeded predictor is
 * tuned, else the plain one.  *E_out (may be NULL) receives the choice,
 * ms[i] (cap entries, may be NULL) the per-step predictor time of choice i in
 * the order of the configuration's choices.  No reference counterpart. */
int adg_autotune(adg_ctx* ctx, int nsteps, int* E_out, double* ms, int cap);
/* The elements-per-block choices the configuration is built with (up to cap)
 * and the ones in use by the plain and the seeded predictor. */
int adg_block_choices(const adg_ctx* ctx, int* choices, int cap, int* n, int* E_plain, int* E_seeded);

/* Page-locked host buffers for host<->device state copies. */
int adg_host_alloc(size_t bytes, void** ptr);
int adg_host_free(void* ptr);

/* ---------------------------------------------------------------------------
 * Learned predictor seed.  A multilayer perceptron (Q*Np_s + 1 inputs: the
 * element's modal state and Dt/dx; three hidden layers with GELU; Q*Np_st
 * outputs: the space-time predictor H_w) trained on the GPU with FP32
 * kernels on pairs the Picard predictor itself generates.  Attached to a
 * context it supplies the predictor's initial guess: `sweeps` Picard sweeps
 * from the seed replace the P sweeps of AmrDG<P>::ADER (AmrDG.h:1099-1119);
 * the first sweep's change judges every element and elements whose residual
 * exceeds `tol` (relative to the element's largest cell mean) rerun the full
 * FP64 Picard predictor.  The corrector is always FP64.
 * ------------------------------------------------------------------------- */
typedef struct adg_seed adg_seed;
int adg_seed_create(int D, int P, int hidden, uint64_t rng_seed, adg_seed** out);
int adg_seed_destroy(adg_seed* s);
/* Append (features, targets) of the current state of ctx's valid elements,
 * targets from a Picard predictor of target_sweeps sweeps. */
int adg_seed_collect(adg_ctx* ctx, adg_seed* s, int target_sweeps);
int adg_seed_num_samples(const adg_seed* s, int64_t* n);
/* Standardise the data set (first call) and train epochs of Adam. */
int adg_seed_train(adg_seed* s, int epochs, int batch, double lr, double* last_epoch_loss);
/* Network on standardised inputs X (n x n_in, host) -> Y (n x n_out, host). */
int adg_seed_forward(adg_seed* s, const float* X, int n, float* Y);
/* Loss and parameter gradients of the MSE on (X, T) (host, standardised). */
int adg_seed_gradients(adg_seed* s, const float* X, const float* T, int n, float* grads, double* loss);
/* Parameters: W1 b1 W2 b2 W3 b3 W4 b4 (row-major, in x out), then
 * x_mean, x_istd, y_mean, y_std. */
int adg_seed_num_params(const adg_seed* s, int64_t* n_weights, int64_t* n_total);
int adg_seed_get_params(adg_seed* s, float* out);
int adg_seed_set_params(adg_seed* s, const float* in);
/* mode 0 detaches; 1: sweeps in FP64; 2: sweeps in FP32. */
int adg_seed_attach(adg_ctx* ctx, adg_seed* s, int mode, int sweeps, double tol);
/* Which kernels compute the seed during steps: 1 (default) the fused
 * tensor-core kernel (features, the four layers as TF32 tcgen05 MMAs with
 * TMEM accumulators, H_w assembly) when the hidden width is 128; 0 the SIMT
 * kernels (features, four FP32 SGEMMs, assembly).  No reference counterpart. */
int adg_seed_set_path(adg_ctx* ctx, int path);
/* The seeds H_w of every element of the current layout (valid elements of
 * all levels, then the coarse-fine ghosts; Q * Np_st per element) into
 * dst_dev (device pointer) through the given path.  No reference counterpart. */
int adg_seed_infer(adg_ctx* ctx, double* dst_dev, int path);
/* Elements whose seed was rejected (fallback to the full Picard), and
 * elements predicted, since attach. */
int adg_seed_stats(adg_ctx* ctx, int64_t* fallbacks, int64_t* predicted);

/* Measured FP64 multiply-add throughput of this GPU (DFMA chains), GFLOP/s. */
int adg_fp64_peak_probe(double* gflops);

/* One ADER predictor-corrector step (AmrDG::ADER physics, all sweeps) of a
 * single-level grid, periodic in every direction, that allocates nothing.
 * No counterpart in the reference: it exists for callers that cannot
 * allocate GPU memory when they need a step (code running inside another
 * framework's memory arena or pool, or a loop that must not call the
 * allocator after start-up).  The caller passes the state U_w (device
 * pointer, element-major [cell][q][n], cells x-fastest; updated in place)
 * and the step size; all intermediates live in one fixed device array of
 * ADG_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  Problems whose intermediates do not fit return
 * ADG_ERR_NOALLOC_CAPACITY (about 12,800 elements at D=2, P=3).  The first
 * call on a device looks up the array's device address (make it before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race.  Work is issued on `stream` (NULL: default stream), asynchronously.
 * A CUDA error already pending when the call starts returns ADG_ERR_CUDA
 * before any launch and is left pending for its owner. */
#define ADG_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int adg_ader_step_noalloc(int D, int P, const int n_cell[3], const double prob_lo[3], const double prob_hi[3],
                          double gamma, double dt, double* U_w, void* stream);

/* Algorithmic FP64 flops per element-step (the method's dense matvec count)
 * and the FP64 operations the generated kernels actually issue per element. */
int adg_flops_per_element(int D, int P, double* algorithmic, double* issued);

#ifdef __cplusplus
}
#endif

#endif /* ADG_H */
