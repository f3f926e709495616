/*
 * vf_oracle.h -- C interface of the CPU oracle for the 2D shallow-water time step.
 *
 * TEST INFRASTRUCTURE ONLY. The oracle is a line-by-line CPU restatement of
 * VolumeFluxes.jl's practical 2D shallow-water path (src/ files cited in
 * vf_oracle.cpp). Only the tests, the smoke check and the CPU-baseline leg of
 * bench.py may load it; the product library never links or calls it.
 *
 * Layout follows the reference's Volume (src/volume/volume.jl:24-51): one
 * plane per conserved variable (w, hu, hv), each plane column-major with x
 * fastest, total size (nx+2gc) x (ny+2gc). Bottom topography lives on cell
 * corners, (nx+2gc+1) x (ny+2gc+1), x fastest
 * (src/bottom_topography.jl:51-82).
 */
#ifndef VF_ORACLE_H
#define VF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Source-term codes, kept in the order the caller lists them
 * (src/system.jl:67-73 walks the vector in order). */
enum {
  VFO_SRC_BOTTOM = 1,        /* SourceTermBottom, src/sourceterms/source_term_bottom.jl:24-41 */
  VFO_SRC_CONST_RAIN = 2,    /* ConstantRain(rate in m/h), source_term_rain.jl:24-30,71-76 */
  VFO_SRC_CONST_INFIL = 3,   /* ConstantInfiltration(rate in m/s), source_term_infiltration.jl:73-88 */
  VFO_SRC_TIME_RAIN = 4,     /* TimeDependentRain(rates [m/h], times), source_term_rain.jl:32-54 (table set later) */
  VFO_SRC_HORTON = 5,        /* HortonInfiltration: rate=fc, aux0=f0, aux1=k, per-cell factor set later,
                                source_term_infiltration.jl:21-70 */
  VFO_SRC_RAIN_FIELD = 6     /* per-cell rain rate [m/s] over the total grid (FunctionalRain evaluated
                                by the caller at cell centres), source_term_rain.jl:57-68 */
};

enum { VFO_FRICTION_NONE = 0, VFO_FRICTION_BSA2012 = 1, VFO_FRICTION_FCG2016 = 2, VFO_FRICTION_BH2021 = 3 };
enum { VFO_STEPPER_FE = 1, VFO_STEPPER_RK2 = 2 };
enum { VFO_BC_WALL = 1, VFO_BC_PERIODIC = 2, VFO_BC_NEUMANN = 3 };
enum { VFO_REC_LINEAR = 1, VFO_REC_NONE = 2 };
enum { VFO_MAX_SOURCES = 8 };

typedef struct {
  int nx, ny, gc;
  double extent[4];          /* x0, x1, y0, y1 */
  int real_bytes;            /* 8: Float64 state, 4: Float32 state */
  double g, rho, depth_cutoff, desingularizing_kappa;
  int reconstruction;        /* VFO_REC_LINEAR */
  double theta;
  int n_sources;
  int source_kind[VFO_MAX_SOURCES];
  double source_rate[VFO_MAX_SOURCES];
  double source_aux[VFO_MAX_SOURCES][2];
  int friction;              /* VFO_FRICTION_* */
  double friction_Cz;
  int stepper;               /* VFO_STEPPER_* */
  int bc;                    /* VFO_BC_WALL */
  double cfl;
  int bottom_is_constant;    /* 1: ConstantBottomTopography(bottom_constant) */
  double bottom_constant;
} vfo_params;

typedef struct vfo_sim vfo_sim;

/* B_corners: (nx+2gc+1)*(ny+2gc+1) doubles, ignored when bottom_is_constant. */
int vfo_create(const vfo_params* p, const double* B_corners, vfo_sim** out);
void vfo_destroy(vfo_sim* s);
/* Tables and per-cell arrays of source term `index` (its position in the
 * source list): TimeDependentRain times/rates (n entries); HortonInfiltration
 * factor or rain field over the total grid (nx+2gc)*(ny+2gc), x fastest. */
int vfo_set_source_table(vfo_sim* s, int index, const double* times, const double* rates, int n);
int vfo_set_source_field(vfo_sim* s, int index, const double* field);
/* The deterministic exp used for Horton infiltration (identical on the device). */
double vfo_exp(double x);
/* Interior planes, nx*ny each, x fastest; then the boundary update
 * (src/simulator.jl:119-135). */
int vfo_set_interior(vfo_sim* s, const double* w, const double* hu, const double* hv);
/* Full current state, 3 planes of (nx+2gc)*(ny+2gc). */
int vfo_get_state(const vfo_sim* s, double* out);
int vfo_get_interior(const vfo_sim* s, double* w, double* hu, double* hv);
/* One perform_step! (src/simulator.jl:145-177); returns the dt used. */
int vfo_perform_step(vfo_sim* s, double max_dt, double* dt_out);
/* simulate_to_time (src/simulator.jl:179-212) without callbacks.
 * maximum_timestep < 0 means none. Stops early after max_steps steps when
 * max_steps > 0. */
int vfo_simulate_to_time(vfo_sim* s, double endtime, int match_endtime, double maximum_timestep,
                         long long max_steps, long long* steps_out);
double vfo_time(const vfo_sim* s);
void vfo_set_time(vfo_sim* s, double t);
double vfo_current_timestep(const vfo_sim* s);
int vfo_set_threads(int n);
int vfo_get_threads(void);

/* Known-answer hooks used by the unit tests. */
double vfo_minmod(double a, double b, double c);
double vfo_minmod_slope(double l, double c, double r, double theta);
/* which: 0 B_cell, 1 face_left X, 2 face_right X, 3 face_left Y, 4 face_right Y.
 * i, j are the reference's 1-based total-grid indices. */
double vfo_bottom_lookup(const double* B, int n1p1, int n2p1, int i, int j, int which);
/* Wall boundary update in place on a full 3-plane state. */
int vfo_update_bc_wall(double* state, int nx, int ny, int gc);
/* Periodic boundary update in place on a full 3-plane state. */
int vfo_update_bc_periodic(double* state, int nx, int ny, int gc);
int vfo_update_bc_neumann(double* state, int nx, int ny, int gc);
double vfo_cbrt(double x);
double vfo_desingularize(double h, double kappa);

/* Float64 dual-number run (the stand-in for ForwardDiff through this path):
 * from the given interior state at t = 0, n_steps steps with the frozen dt
 * sequence dts (t += dt after each), bottom corners B + eps*Bdot (Bdot may be
 * NULL) and friction Cz + eps*Cz_dot; returns loss = sum over gauges of
 * (w[i,j] - target)^2 (interior 0-based indices) and d loss / d eps. `like`
 * (may be NULL) lends its source tables and per-cell source fields. */
int vfo_dual_gauge_loss(const vfo_params* p, const double* B, const double* Bdot, double Cz_dot, const double* w,
                        const double* hu, const double* hv, const double* dts, int n_steps, const int* gauge_i,
                        const int* gauge_j, const double* target, int n_gauges, double* loss, double* dloss,
                        const vfo_sim* like);

/* The same run in plain Float64 (the loss of vfo_dual_gauge_loss without a
 * derivative). */
int vfo_frozen_gauge_loss(const vfo_params* p, const double* B, const double* w, const double* hu, const double* hv,
                          const double* dts, int n_steps, const int* gauge_i, const int* gauge_j,
                          const double* target, int n_gauges, double* loss, const vfo_sim* like);

/* The same run in extended precision (long double: 64-bit significand on
 * x86, 113-bit on Arm), the reference of the gradient's finite-difference
 * checks: bottom B + eps*Bdir and friction Cz + eps*Cz_dir1 + eps^2*Cz_dir2
 * formed in that precision; the loss comes back as hi + lo. */
int vfo_ext_gauge_loss(const vfo_params* p, const double* B, const double* Bdir, double Cz_dir1, double Cz_dir2,
                       double eps, const double* w, const double* hu, const double* hv, const double* dts,
                       int n_steps, const int* gauge_i, const int* gauge_j, const double* target, int n_gauges,
                       double* loss_hi, double* loss_lo, const vfo_sim* like);

/* Branch-outcome counters (instrumentation of the gradient checks): on != 0
 * zeroes them and starts counting every branch outcome of the path (minmod
 * case, reconstruction clause, wet face sides, the kappa early-out, the
 * operand winning each wave-speed max/min, the desingularised depth, the dry
 * clamp); on == 0 zeroes them and stops. vfo_branch_counts writes up to n
 * counters and returns how many exist. */
void vfo_branch_counting(int on);
int vfo_branch_counts(unsigned long long* out, int n);

#ifdef __cplusplus
}
#endif
#endif
