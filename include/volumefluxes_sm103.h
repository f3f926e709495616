/*
 * volumefluxes_sm103.h -- C ABI of the GB300 (sm_103a) shallow-water step library.
 *
 * One handle owns one 2D simulation on one CUDA device: its state buffers,
 * bottom topography, time-derivative scratch and a device-resident step
 * record (time, dt, CFL maxima). The entry points below are what a
 * VolumeFluxes.jl backend binds with `ccall` to replace the reference's
 * per-loop KernelAbstractions launches; each cites the reference interface it
 * stands in for (paths are within the VolumeFluxes.jl project).
 *
 * Conventions
 *  - All functions return 0 on success and a negative VF_E* code on failure;
 *    vf_last_error() gives a message. Nothing aborts, nothing traps on the
 *    device.
 *  - Host arrays use the reference's Volume layout: one plane per variable
 *    (w, hu, hv), each column-major with x fastest
 *    (src/volume/volume.jl:24-51, src/backends/buffer.jl:29-42). Element type
 *    is double for real_bytes == 8 and float for real_bytes == 4.
 *  - Host pointers need only be valid for the duration of the call. Calls on
 *    one handle are synchronous and not reentrant; distinct handles may be
 *    used from distinct threads.
 */
#ifndef VOLUMEFLUXES_SM103_H
#define VOLUMEFLUXES_SM103_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VF_ABI_VERSION 2
#define VF_MAX_SOURCES 8

/* Error codes. */
#define VF_OK 0
#define VF_EINVAL (-1)   /* invalid argument or unsupported configuration */
#define VF_ENOMEM (-2)   /* device or host allocation failed */
#define VF_ECUDA (-3)    /* CUDA runtime error */
#define VF_ESTATE (-4)   /* call out of order (e.g. stepping before a state upload) */

/* Source terms, applied in the order listed
 * (src/system.jl:62-75: directional terms inside the x/y loop, the rest after). */
#define VF_SRC_BOTTOM 1       /* SourceTermBottom, src/sourceterms/source_term_bottom.jl:24-41 */
#define VF_SRC_CONST_RAIN 2   /* ConstantRain(rate [m/h]), src/sourceterms/source_term_rain.jl:24-30,71-76 */
#define VF_SRC_CONST_INFIL 3  /* ConstantInfiltration(rate [m/s]), src/sourceterms/source_term_infiltration.jl:73-88 */
#define VF_SRC_TIME_RAIN 4    /* TimeDependentRain(rates [m/h], times), src/sourceterms/source_term_rain.jl:32-54;
                                 table from vf_set_source_table */
#define VF_SRC_HORTON 5       /* HortonInfiltration: rate = fc, aux = (f0, k), per-cell factor from
                                 vf_set_source_field, src/sourceterms/source_term_infiltration.jl:21-70 */
#define VF_SRC_RAIN_FIELD 6   /* per-cell rain [m/s] from vf_set_source_field: FunctionalRain evaluated at
                                 cell centres by the caller, src/sourceterms/source_term_rain.jl:57-76 */

/* ImplicitFriction laws, src/friction.jl:30-43. */
#define VF_FRICTION_NONE 0
#define VF_FRICTION_BSA2012 1
#define VF_FRICTION_FCG2016 2
#define VF_FRICTION_BH2021 3

#define VF_STEPPER_FE 1       /* ForwardEulerStepper, src/timestepper/forwardeuler.jl:23-47 */
#define VF_STEPPER_RK2 2      /* RungeKutta2, src/timestepper/rungekutta.jl:21-52 */
#define VF_BC_WALL 1          /* WallBC, src/bc.jl:81-110 */
#define VF_BC_PERIODIC 2      /* PeriodicBC, src/bc.jl:29-40 */
#define VF_BC_NEUMANN 3       /* NeumannBC as src/bc.jl:49-60 computes it: left columns mirror the interior,
                                 bottom rows copy the top interior rows, right and top ghosts evolve by the
                                 all-cell passes alone (ghost copied onto ghost) */
#define VF_REC_LINEAR 1       /* LinearReconstruction(theta), src/reconstruction/linearreconstruction.jl:22-102 */
#define VF_REC_NONE 2         /* NoReconstruction, src/reconstruction/noreconstruction.jl:30-46 */

/* Everything the reference's ConservedSystem + Simulator constructors carry
 * for this path (src/system.jl:37-53, src/simulator.jl:72-91,
 * src/equations/swe_2D.jl:28, src/grid.jl:82-90). */
typedef struct vf_config {
  int32_t abi_version;       /* VF_ABI_VERSION */
  int32_t nx, ny, gc;        /* interior cells and ghost layers (gc must be 2) */
  double extent[4];          /* x0, x1, y0, y1 */
  int32_t real_bytes;        /* 8: Float64 state, 4: Float32 state */
  double g, rho, depth_cutoff, desingularizing_kappa;
  int32_t reconstruction;    /* VF_REC_* */
  double theta;
  int32_t n_sources;
  int32_t source_kind[VF_MAX_SOURCES];
  double source_rate[VF_MAX_SOURCES];
  double source_aux[VF_MAX_SOURCES][2];
  int32_t friction;          /* VF_FRICTION_* */
  double friction_Cz;
  int32_t stepper;           /* VF_STEPPER_* */
  int32_t bc;                /* VF_BC_* */
  double cfl;
  int32_t bottom_is_constant;/* 1: ConstantBottomTopography(bottom_constant) */
  double bottom_constant;
  int32_t device;            /* CUDA device ordinal */
} vf_config;

typedef struct vf_handle vf_handle;

/* Stands in for ConservedSystem(...) + Simulator(backend, system, stepper, grid; cfl)
 * (src/system.jl:37-53, src/simulator.jl:72-91) with create_buffer on the
 * device (src/backends/buffer.jl:40-42). Validates the configuration the way
 * the reference's constructors do (gc > 1 for LinearReconstruction,
 * src/reconstruction/linearreconstruction.jl:59; is_compatible,
 * src/equations/equation.jl:74-84). */
int vf_create(const vf_config* cfg, vf_handle** out);
void vf_destroy(vf_handle* h);

/* Stands in for BottomTopography2D(B, backend, grid): convert_to_backend of the
 * corner array (src/bottom_topography.jl:51-57), (nx+2gc+1) x (ny+2gc+1),
 * x fastest. */
int vf_upload_bottom(vf_handle* h, const void* B_corners);

/* Data of the time- or cell-dependent source term at position `index` of the
 * source list. vf_set_source_table: TimeDependentRain's n breakpoints `times`
 * and rates `rates` [m/h] (the reference's constructor, src/sourceterms/
 * source_term_rain.jl:35-41). vf_set_source_field: HortonInfiltration's factor
 * (src/sourceterms/source_term_infiltration.jl:37-44) or a rain field [m/s]
 * over the total grid (nx+2gc) x (ny+2gc), x fastest, in the real type. A
 * field may be re-uploaded between steps (a FunctionalRain re-evaluated at the
 * new time). */
int vf_set_source_table(vf_handle* h, int32_t index, const double* times, const double* rates, int32_t n);
int vf_set_source_field(vf_handle* h, int32_t index, const void* field);

/* Stands in for set_current_state!(sim, state) (src/simulator.jl:119-135):
 * writes the interior planes (nx*ny each, x fastest), then the device
 * boundary update (src/bc.jl:81-110). */
int vf_set_interior_state(vf_handle* h, const void* w, const void* hu, const void* hv);
/* Full-volume upload (ghost cells included), 3 planes of (nx+2gc)*(ny+2gc). */
int vf_upload_state(vf_handle* h, const void* state);
/* Stands in for collect(current_state(sim)) (src/simulator.jl:98). */
int vf_download_state(vf_handle* h, void* state);
/* Stands in for collect(current_interior_state(sim).h/.hu/.hv)
 * (src/simulator.jl:114-115, src/volume/interior_volume_variable.jl:168-176).
 * Any of the three pointers may be NULL. */
int vf_get_interior_state(vf_handle* h, void* w, void* hu, void* hv);

/* Stands in for perform_step!(sim, max_dt) (src/simulator.jl:145-177): one
 * full FE/RK2 step including friction, dry clamp and boundary update, with
 * time-dependent sources evaluated at t (the simulator's current time).
 * Writes the dt used (current_timestep) to *dt_out. Does not advance t; the
 * caller does t += dt as simulate_to_time does (src/simulator.jl:205). */
int vf_step(vf_handle* h, double max_dt, double t, double* dt_out);

/* Float64 arithmetic of the per-step kernels (vf_step, vf_simulate and the
 * wide members of a batch). VF_ARITH_REFERENCE (the default): every operation
 * rounds as the reference's Julia code does, so results equal the reference
 * CPU path bit for bit. VF_ARITH_FAITHFUL: quotients correct to about one ulp
 * (a refined hardware reciprocal shared by quotients with one divisor),
 * library cube roots and fused multiply-adds; the same passes and branches,
 * held to the 1e-12 relative max-norm tolerance against the reference path
 * instead of to its bits, and fewer FP64 instructions per cell. Stands in for
 * nothing in the reference (whose CPU and KernelAbstractions backends both
 * round every operation); VF_EINVAL for Float32 handles or another mode. */
#define VF_ARITH_REFERENCE 0
#define VF_ARITH_FAITHFUL 1
int vf_set_arithmetic(vf_handle* h, int32_t mode);

/* Stands in for the loop of simulate_to_time (src/simulator.jl:179-212) with
 * the time kept on the device: from t0, step while t < endtime with
 * max_dt = endtime - t when match_endtime (else +Inf), capped by
 * maximum_timestep when it is >= 0. Stops early, after the step where
 * t + dt >= stop_time (the IntervalWriter trigger, src/callbacks.jl:49-55),
 * or after max_steps steps when max_steps > 0. No host synchronisation
 * happens between steps. Outputs (any may be NULL): final time, steps taken,
 * dt of the last step. */
int vf_simulate(vf_handle* h, double t0, double endtime, int32_t match_endtime, double maximum_timestep,
                double stop_time, int64_t max_steps, double* t_out, int64_t* steps_out, double* last_dt_out);

/* Total water volume sum((w - B_cell) * dx * dy) over the interior, summed in
 * Float64 on the device in a fixed order (the water-volume bookkeeping of
 * examples/example_tools.jl:49-106). */
int vf_water_volume(vf_handle* h, double* out);

/* (w, hu, hv) of n interior cells (0-based i, j) of the current state, in the
 * real type, without downloading the state: the gauge reads a callback such
 * as an IntervalWriter (src/callbacks.jl:40-55) makes every interval, where
 * the reference collects the whole interior (examples/example_tools.jl:99).
 * Any output may be NULL. */
int vf_sample_cells(vf_handle* h, const int32_t* i, const int32_t* j, int32_t n, void* w_out, void* hu_out,
                    void* hv_out);

/* Device-resident access for callers that keep data on the GPU: the current
 * state's device base pointer, its row pitch and plane stride in elements,
 * and the element offset of total cell (0, 0). Valid until the next step. */
int vf_device_state(vf_handle* h, void** base, int64_t* pitch, int64_t* plane_stride, int64_t* offset00);
/* The CUDA stream all of the handle's work is issued on (cudaStream_t). */
int vf_stream(vf_handle* h, void** stream);

/* Times n_steps steps already resident on the device with CUDA events on the
 * handle's stream (no host copies); writes the elapsed milliseconds. Uses
 * match_endtime = false and max_dt = +Inf, as perform_step!(sim, Inf). */
int vf_time_steps(vf_handle* h, int64_t n_steps, float* ms_out);

/* Like vf_time_steps, with CUDA events around each kernel of each step:
 * *ms_flux and *ms_stage receive the summed durations of the flux passes and
 * of the stage (RK2) or apply (forward Euler) passes. */
int vf_time_kernels(vf_handle* h, int64_t n_steps, float* ms_flux, float* ms_stage);

/* Self-test of the bounded wait the TMA tile kernels use for their tile
 * copies (an mbarrier in shared memory): one warp waits on a barrier that is
 * completed (arrive = 1) or never completed (arrive = 0) and gives up after
 * `iterations` polls; *gave_up receives 1 when the wait ran out. The kernel
 * returns either way. No reference counterpart (failure-detection test hook). */
int vf_selftest_tile_wait(int32_t device, int32_t arrive, int32_t iterations, int32_t* gave_up);

/* Self-test of the Float64 quotient every Float64 kernel uses (correctly
 * rounded reciprocals shared by a divisor's quotients, with the IEEE division
 * for the operands the method excludes): q[i] = a[i] / b[i] for n host
 * pairs, computed on the device. It must equal IEEE division bit for bit. No
 * reference counterpart (test hook). */
int vf_selftest_quotients(int32_t device, const double* a, const double* b, int32_t n, double* q);

/* Self-test of the near-dry velocity quotient of the Float32 kernels (face
 * sides and cells with |h| below the near-dry threshold divide (hu, hv) by
 * the desingularised depth this way): q[i] as the kernels compute a[i] / b[i],
 * and q64[i] = the IEEE Float64 quotient rounded to Float32, both on the
 * device for n host pairs. The two must be equal bit for bit wherever the
 * operands and the quotient are normal Float32 numbers (the Float32 kernels
 * flush subnormals to zero). No reference counterpart (test hook). */
int vf_selftest_near_dry_quotients(int32_t device, const float* a, const float* b, int32_t n, float* q, float* q64);

/* ---- Batched ensemble ------------------------------------------------------
 * Advances many independent simulations, each a handle set up as above, each
 * to its own end time with its own CFL dt: the loop of simulate_to_time
 * (src/simulator.jl:179-212, with callback = nothing) run for every handle at
 * once. The reference steps one Simulator at a time; these calls have no
 * counterpart there and replace a host loop over simulate_to_time calls.
 *
 * One thread-block cluster per simulation runs its whole time loop on the
 * device; launches are grouped by cluster size (one launch per group,
 * concurrent streams), and the GPU's block scheduler starts a pending
 * simulation whenever a cluster finishes. Simulations of at least wide_cells
 * cells instead run the plain whole-grid kernels on their own stream, fed in
 * CUDA-graph chunks by the host whenever the batch is polled or waited on.
 * Per-handle results are bitwise those of vf_simulate on the same handle in
 * Float64, and independent of which other simulations share the batch in both
 * precisions. */
#define VF_BATCH_OK 0          /* reached its end time */
#define VF_BATCH_TIMEOUT 1     /* the launch's watchdog (time_limit_s) stopped it */
#define VF_BATCH_STALLED 2     /* t + dt rounded to t: no progress possible */
#define VF_BATCH_MAX_STEPS 3   /* stopped after max_steps steps */

typedef struct vf_batch_options {
  int32_t tiles_per_cta;   /* target 32x16 tiles per CTA when sizing a cluster; 0: default (16) */
  int32_t max_cluster;     /* largest cluster (1..16); 0: default (16) */
  double time_limit_s;     /* watchdog from the batch's start, in seconds; <= 0: default (600 s) */
  int32_t seg_rows;        /* rows per strip segment of Float32 column-marching members
                              (8..256); 0: 64, halved down to 8 until every warp has two */
  int64_t wide_cells;      /* members with at least this many interior cells run the plain
                              whole-grid kernels on their own stream instead of a cluster;
                              0: default (262144), < 0: never */
} vf_batch_options;

typedef struct vf_batch vf_batch;

/* Starts the batch and returns without waiting. The handles must have state
 * (and bottom, tables, fields) uploaded, must be distinct, must live on one
 * device, and must not be used by other calls until collected. t0[i] and
 * endtime[i] are per handle; match_endtime and maximum_timestep (< 0: none)
 * act as in vf_simulate; max_steps <= 0 means no limit. opt may be NULL. */
int vf_batch_launch(vf_handle* const* hs, int32_t n, const double* t0, const double* endtime,
                    int32_t match_endtime, double maximum_timestep, int64_t max_steps,
                    const vf_batch_options* opt, vf_batch** out);
/* Number of simulations of the batch that have finished (non-blocking). */
int vf_batch_poll(vf_batch* b, int32_t* n_done);
/* 1 if simulation i has finished, else 0 (non-blocking); negative on error. */
int vf_batch_is_done(vf_batch* b, int32_t i);
/* Hands a finished simulation back to its handle (its current state becomes
 * the final state) and reports its final time, steps, last dt and
 * VF_BATCH_* status (any pointer may be NULL). VF_ESTATE if not finished. */
int vf_batch_collect(vf_batch* b, int32_t i, double* t_out, int64_t* steps_out, double* last_dt_out,
                     int32_t* status_out);
/* Blocks until every simulation of the batch has finished. */
int vf_batch_wait(vf_batch* b);
/* Waits, collects what is not collected yet, and frees the batch. */
int vf_batch_free(vf_batch* b);
/* launch + wait + collect every simulation + free. Outputs are arrays of n
 * (any may be NULL). */
int vf_batch_simulate(vf_handle* const* hs, int32_t n, const double* t0, const double* endtime,
                      int32_t match_endtime, double maximum_timestep, int64_t max_steps,
                      const vf_batch_options* opt, double* t_out, int64_t* steps_out, double* last_dt_out,
                      int32_t* status_out);
/* Cluster size the batch would give handle h under opt (NULL: defaults). */
int vf_batch_cluster_size(vf_handle* h, const vf_batch_options* opt, int32_t* csize_out);
/* Message for the last batch failure (b may be NULL for vf_batch_launch). */
const char* vf_batch_last_error(vf_batch* b);

/* ---- Serving ---------------------------------------------------------------
 * A request loop over whole simulations (no counterpart in the reference).
 * A request is a configuration, its bottom corners, an initial interior state,
 * t0 and an end time; the engine keeps its state on the device from admission
 * to completion and writes the final interior state to the caller's output
 * buffers. An engine thread per server admits requests oldest-first within an
 * HBM budget (the device bytes vf_create allocates per request), launches
 * each round's admissions as one batch beside the batches still running
 * (continuous batching) and completes requests as their done flags appear.
 * Requests take SourceTermBottom, ConstantRain and ConstantInfiltration
 * sources. Input buffers must stay valid until the request is admitted,
 * output buffers until it is reported done. */
typedef struct vf_server vf_server;

/* opt: batch options of every launch (NULL: defaults); max_steps <= 0: none. */
int vf_server_create(int32_t device, int64_t hbm_budget_bytes, const vf_batch_options* opt, int64_t max_steps,
                     vf_server** out);
/* Queues a request; *ticket_out identifies it. VF_ENOMEM if it alone exceeds the budget. */
int vf_server_submit(vf_server* s, const vf_config* cfg, const void* B_corners, const void* w, const void* hu,
                     const void* hv, double t0, double endtime, void* out_w, void* out_hu, void* out_hv,
                     int64_t* ticket_out);
/* Non-blocking: writes up to `capacity` tickets that finished (done or failed)
 * since the last poll to done_tickets and their count to *n_done. Returns
 * VF_ECUDA once if the engine met a launch error since the last poll. */
int vf_server_poll(vf_server* s, int64_t* done_tickets, int32_t capacity, int32_t* n_done);
/* When the request was submitted, admitted and finished, in seconds since the
 * server was created. */
int vf_server_timing(vf_server* s, int64_t ticket, double* submit_s, double* admit_s, double* done_s);
/* Outcome of a finished request: final time, steps, last dt, VF_BATCH_*
 * status; returns the request's error code if it failed. */
int vf_server_result(vf_server* s, int64_t ticket, double* t_out, int64_t* steps_out, double* last_dt_out,
                     int32_t* status_out);
/* Forgets a finished request. */
int vf_server_release(vf_server* s, int64_t ticket);
/* Device bytes charged to running requests, queue and running counts, batches launched. */
int vf_server_stats(vf_server* s, int64_t* used_bytes, int32_t* queued, int32_t* running, int64_t* launches);
/* Waits for running batches and frees everything. */
int vf_server_destroy(vf_server* s);
const char* vf_server_last_error(vf_server* s);

/* ---- Differentiation -------------------------------------------------------
 * Reverse-mode gradients of a gauge loss with a frozen dt sequence. The
 * reference differentiates through its CPU path with ForwardDiff dual numbers
 * (test/test_swe_ad.jl, examples/optimization.jl); these calls replace that
 * for large parameter counts: one reverse sweep gives dLoss/dB for every
 * bottom corner and dLoss/dCz at once. Covered: RungeKutta2 and
 * ForwardEulerStepper, LinearReconstruction and NoReconstruction, WallBC and
 * PeriodicBC, a BottomTopography2D, SourceTermBottom, ConstantRain,
 * ConstantInfiltration, TimeDependentRain, HortonInfiltration and any
 * ImplicitFriction law (not NeumannBC, or FunctionalRain, whose field the host
 * re-evaluates between steps). The run's time starts at 0. At kinks
 * (minmod switches, dry faces, the dry clamp) the gradient is the
 * derivative of the branch the forward pass took. */

/* One step with exactly this dt (no CFL limit): the forward pass with a frozen
 * dt sequence. t is the simulator's time (time-dependent sources). */
int vf_step_fixed(vf_handle* h, double dt, double t);

typedef struct vf_adjoint vf_adjoint;

/* Takes the handle's current state as U^0 of an n_steps run; checkpoints every
 * checkpoint_every steps (<= 0: round(sqrt(n_steps))). */
int vf_adjoint_create(vf_handle* h, int32_t n_steps, int32_t checkpoint_every, vf_adjoint** out);
/* Runs the n_steps from U^0 on the handle, keeping checkpoints: with
 * frozen_dts (n_steps values) as given, else with the CFL dt of every step,
 * written to dts_out (may be NULL). Leaves the handle at U^n_steps. */
int vf_adjoint_forward(vf_adjoint* a, const double* frozen_dts, double* dts_out);
/* loss = sum_g (w[gauge_i[g], gauge_j[g]] - target[g])^2 over interior cells
 * (0-based) of the final state, and its gradient: grad_B receives
 * dLoss/dB for every corner, (nx+2gc+1) x (ny+2gc+1) doubles, x fastest;
 * *grad_Cz receives dLoss/dCz. Any output may be NULL. */
int vf_adjoint_backward(vf_adjoint* a, const int32_t* gauge_i, const int32_t* gauge_j, const double* target,
                        int32_t n_gauges, double* loss_out, double* grad_B, double* grad_Cz);
void vf_adjoint_destroy(vf_adjoint* a);
const char* vf_adjoint_last_error(vf_adjoint* a);

/* Largest interior row count vf_water_volume_static accepts. */
#define VF_STATIC_MAX_ROWS 16384

/* Water volume sum((w - B_cell) * dx * dy) of a state the caller owns on the
 * device, for callers that cannot let a library allocate device memory (code
 * whose device memory belongs to another allocator that must account for
 * every byte, such as CUDA.jl's pool, or loops that cannot afford the
 * synchronisation cudaMalloc may imply). It calls no cudaMalloc/cudaFree:
 * inputs and the output are the caller's, and its scratch (one Float64
 * partial sum per interior row) is a fixed file-scope device array of
 * VF_STATIC_MAX_ROWS doubles (128 KiB) that every GPU using the library holds
 * until the process exits. No counterpart in the reference: an addition for
 * allocation-free callers.
 *
 *  state_dev  dense reference-layout volume on the device, (nx+2gc) x (ny+2gc)
 *             x 3, x fastest; only the w plane is read
 *  B_dev      dense corner array (nx+2gc+1) x (ny+2gc+1), or NULL when
 *             bottom_is_constant
 *  out_dev    device double receiving the volume; written asynchronously on
 *             `stream` (a cudaStream_t, NULL for the default stream)
 *
 * Returns VF_EINVAL for ny > VF_STATIC_MAX_ROWS or bad arguments (message
 * from vf_last_error(NULL)). All calls share the scratch array, which keeps the
 * last call's contents: calls whose kernels overlap on the GPU race. A call
 * outside stream capture looks the array up with cudaGetSymbolAddress (its
 * address changes when the device or its primary context is reset); a call
 * during capture reuses the last address found on that device. Make one call
 * on a device before any capture, and again after a reset of the device. */
int vf_water_volume_static(const void* state_dev, const void* B_dev, int32_t nx, int32_t ny, int32_t gc,
                           int32_t real_bytes, double dx, double dy, int32_t bottom_is_constant,
                           double bottom_constant, double* out_dev, void* stream);

/* Message for the last failure on this handle (or of vf_create when h is NULL). */
const char* vf_last_error(vf_handle* h);
/* Kernel launches issued by this handle since creation. */
int64_t vf_launch_count(vf_handle* h);

#ifdef __cplusplus
}
#endif
#endif
