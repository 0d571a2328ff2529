/*
 * excalibur_gb300.h -- C ABI of the GB300 photon-geodesic tracer.
 *
 * Plain C: POD structs, raw pointers and sizes, no torch types. Every entry
 * point takes a `void* stream` (a cudaStream_t; NULL = legacy default
 * stream), enqueues its work on it and returns an ExcError code. Array
 * pointers inside the structs are DEVICE pointers owned by the caller; the
 * library never frees them. Per-photon outcomes are written to `status[]`,
 * never raised: a photon the reference would abort with an exception gets a
 * failure status and keeps its last accepted state.
 *
 * Reference interfaces replaced (lmagristella/excalibur-tool):
 *   exc_trace            Integrator.integrate / integrate_single
 *                        (excalibur/integration/integrator.py:218-409, :434-476)
 *                        with RK4.step / Leapfrog4.step / RK45Adaptive.step (:9-152)
 *   exc_geodesic_rhs     Metric.geodesic_equations
 *                        (metrics/perturbed_flrw_metric_fast.py:227-273,
 *                         metrics/schwarzschild_metric_fast.py:253-303)
 *   exc_interp           InterpolatorFast.value_gradient_and_time_derivative
 *                        (grid/interpolator_4d_fast.py:443-502; legacy strict
 *                         grid/interpolator_fast.py:294-306)
 *   exc_eval_cosmology   LCDM_Cosmology.a_of_eta / adot_of_eta
 *                        (core/cosmology.py:199-206, :84-93)
 *   exc_metric_tensor    Metric.metric_tensor (diagonal part)
 *                        (perturbed_flrw_metric_fast.py:126-141,
 *                         schwarzschild_metric_fast.py:190-201)
 *   exc_null_init        Photons._solve_u0_from_null_condition
 *                        (photon/photons.py:540-568; same formula as the
 *                         cone generators :393-405)
 *   exc_null_error       Photon.null_condition_relative_error
 *                        (photon/photon.py:46-68)
 */
#ifndef EXCALIBUR_GB300_H
#define EXCALIBUR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EXC_ABI_VERSION 2
#define EXC_MAX_FIELDS 32

/* ---- return codes of every entry point ---------------------------------- */
typedef enum {
  EXC_SUCCESS = 0,
  EXC_ERR_INVALID = -1,      /* bad argument (message via exc_last_error) */
  EXC_ERR_CUDA = -2,         /* a CUDA runtime call failed */
  EXC_ERR_UNSUPPORTED = -3,  /* valid but not built (e.g. precision/metric combo) */
  EXC_ERR_NO_DEVICE = -4
} ExcError;

/* ---- per-photon status written by exc_trace ----------------------------- */
enum {
  EXC_PH_STEPS = 0,          /* reached max_steps accepted steps ("steps" stop mode) */
  EXC_PH_LEFT_BOX = 1,       /* position left [box_lo, box_hi) after an accepted step */
  EXC_PH_A_STOP = 2,         /* a(eta) <= a_stop after an accepted step */
  EXC_PH_MAX_ITER = 3,       /* iteration cap (the reference's max_iter, integrator.py:261) */
  EXC_PH_OUTSIDE_GRID = 4,   /* interpolator error mode: point outside the strict interior */
  EXC_PH_HORIZON = 5,        /* r <= r_s (schwarzschild_metric_fast.py:269-270) */
  EXC_PH_NONFINITE = 6,      /* NaN/Inf state or acceleration, or overflow of r**3 */
  EXC_PH_TIMED_OUT = 7,      /* device deadline reached */
  EXC_PH_ABORTED = 8,        /* host abort flag seen */
  EXC_PH_NOT_RUN = 9,        /* never dequeued (launch ended early) */
  EXC_PH_BAD_FIELD = 10,     /* field_index outside [0, n_fields) */
  EXC_PH_RETRACE = 11        /* EXC_PREC_MIXED_RAW only: a stage point or a stop decision came
                                within the mixed tracer's error window of a discontinuity of the
                                reference's RHS (a cell face of the base-node gradient, a stop
                                threshold); the photon's state, dt and outputs are left untouched
                                for the FP64 tracer (EXC_PREC_MIXED does that re-trace itself) */
};

/* ---- enums -------------------------------------------------------------- */
enum { EXC_METRIC_FLRW = 1, EXC_METRIC_SCHWARZSCHILD = 2 };
enum { EXC_COSMO_STATIC = 0, EXC_COSMO_TABLE = 1, EXC_COSMO_TABLE_FD = 2 };
enum { EXC_BOUNDARY_PERIODIC = 0, EXC_BOUNDARY_CLAMP = 1, EXC_BOUNDARY_ERROR = 2 };
/* EXC_GRAD_BASE_NODE: the fast interpolators (grid/interpolator_4d_fast.py,
 *   grid/interpolator_fast.py): trilinear value, central difference at the
 *   cell's base node, boundary per ExcField.boundary.
 * EXC_GRAD_TRILINEAR: the slow Interpolator (grid/interpolator.py:4-206):
 *   trilinear value with the bounds rule rel in [0, n-1) per spatial axis
 *   (EXC_PH_OUTSIDE_GRID outside); gradient = trilinear blend of the central
 *   differences at the cell's eight corners (base index clipped to [1, n-2]);
 *   4-D: quadrilinear value (time index clipped to [0, nt-2], weights not,
 *   no time bounds check), gradient on the snapshot nearest in time (round
 *   half to even, clipped), dPhi/deta from the snapshots either side of
 *   clip(floor(rel_t), 1, nt-2). Needs boundary EXC_BOUNDARY_ERROR and n >= 3
 *   per spatial axis. The mixed-precision tracer takes it on 3-D grids; its value
 *   and gradient are continuous across interior cell faces, so only stage points
 *   near the outer cells are handed back to the FP64 re-trace. */
enum { EXC_GRAD_BASE_NODE = 0, EXC_GRAD_TRILINEAR = 1 };
/* EXC_DTYPE_F32X2: a float64 grid stored as interleaved float32 pairs, node i
 * at data[2i] = hi = (float)x_i and data[2i + 1] = lo = (float)(x_i - hi);
 * read by the mixed-precision tracer, whose FP32 arithmetic then takes grid
 * differences without cancellation (hi differences are exact), and by its
 * FP64 re-trace pass as hi + lo (x_i to 2^-48 relative). */
enum { EXC_DTYPE_F64 = 0, EXC_DTYPE_F32 = 1, EXC_DTYPE_F32X2 = 2 };
enum { EXC_STEPPER_RK4 = 0, EXC_STEPPER_RK45 = 1, EXC_STEPPER_LEAPFROG4 = 2 };
enum { EXC_TABLEAU_REFERENCE = 0, EXC_TABLEAU_FEHLBERG = 1 };
/* EXACT:     reference operation order, no FMA contraction (parity path).
 * FAST:      same formulas, FMA contraction, reciprocal constants.
 * MIXED:     FP32 RHS + interpolation, double-float (hi + lo FP32) state; rays
 *            that come within the error window of a discontinuity of the
 *            reference's RHS are re-traced by the FAST FP64 tracer in a second
 *            launch on the same stream (FLRW, RK4 or RK45, no records). RK45:
 *            the error norm and step-size control in FP64, the null-condition
 *            renormalisation in FP64.
 * MIXED_RAW: the mixed launch alone; such rays end with EXC_PH_RETRACE.
 * RETRACE:   the second launch alone: the FAST FP64 tracer over the photons
 *            whose status is EXC_PH_RETRACE (the others are not touched), so a
 *            caller can overlap one batch's re-trace with the next batch's
 *            MIXED_RAW launch on another stream. */
enum { EXC_PREC_FP64_EXACT = 0, EXC_PREC_FP64_FAST = 1, EXC_PREC_MIXED = 2, EXC_PREC_MIXED_RAW = 3,
       EXC_PREC_RETRACE = 4 };

/* stop_flags bits (the "steps" stop and max_iter always apply) */
#define EXC_STOP_BOX   1
#define EXC_STOP_A     2
/* With EXC_STOP_BOX, FLRW: the box stop lands on the face. Before each trial step the
 * distance to the box along the current velocity is taken; when the step would reach
 * within EXC_FACE_MARGIN of a face (lambda_face < margin * |dt|, dt after the reference's
 * [dt_min, dt_max] clip), the step is shortened to end on it and the photon ends
 * (EXC_PH_LEFT_BOX) once that step is accepted; no other box test is made. The end point is
 * then a smooth function of the initial direction, whatever the step sequence (the first
 * step past the face, the default, moves in whole steps as the direction changes). Not in
 * the reference, which has no box stop. */
#define EXC_STOP_FACE  4

/* Grid staging of the FP64 tracers (ExcTraceArgs.staging; an autotuner knob): the a(eta) table
 * read through the read-only data cache (EXC_STAGING_CACHE, the default) or copied once per
 * block into shared memory at kernel start (EXC_STAGING_SHARED; tables of at most
 * EXC_STAGING_MAX_TABLE entries). Same values either way. The mixed-precision tracer always
 * keeps its FP32 copy of the table in shared memory when it fits. */
enum { EXC_STAGING_CACHE = 0, EXC_STAGING_SHARED = 1 };
#define EXC_STAGING_MAX_TABLE 12288
#define EXC_FACE_MARGIN 1.05



/* obs_flags bits */
#define EXC_OBS_ENDPOINTS 1   /* a, Phi at both ends; deflection; min_r */
#define EXC_OBS_PATH      2   /* path length, chord, stable excess (time delay) */
#define EXC_OBS_ISW       4   /* trapezoid integral of dPhi/deta along the path */

/* columns of ExcTraceArgs.obs ([n_photons][EXC_OBSCOL_N], float64) */
enum {
  EXC_OBSCOL_A_OBS = 0, EXC_OBSCOL_A_EM = 1, EXC_OBSCOL_PHI_OBS = 2, EXC_OBSCOL_PHI_EM = 3,
  EXC_OBSCOL_ISW_INT = 4,       /* int dPhi/deta deta (SI), trapezoid over accepted states */
  EXC_OBSCOL_PATH = 5,          /* sum |dx| over accepted states (naive, reference definition) */
  EXC_OBSCOL_CHORD = 6,         /* |x_N - x_0| */
  EXC_OBSCOL_EXCESS = 7,        /* path - chord, cancellation-free form */
  EXC_OBSCOL_V0X = 8, EXC_OBSCOL_V0Y = 9, EXC_OBSCOL_V0Z = 10,   /* first cartesian spatial velocity */
  EXC_OBSCOL_V1X = 11, EXC_OBSCOL_V1Y = 12, EXC_OBSCOL_V1Z = 13, /* last cartesian spatial velocity */
  EXC_OBSCOL_MIN_R = 14,        /* min |x - lens_center| over accepted states */
  EXC_OBSCOL_ETA_OBS = 15, EXC_OBSCOL_ETA_EM = 16,
  EXC_OBSCOL_N = 20
};

/* A potential grid. C-order [n0][n1][n2] (3-D) or [n0][n1][n2][n3] with time
 * innermost (4-D), like the reference's field arrays (grid/grid.py:57-81,
 * interpolator_4d_fast.py:286-298). */
typedef struct ExcField {
  const void* data;
  int32_t dtype;           /* EXC_DTYPE_* */
  int32_t ndim;            /* 3 or 4 */
  int32_t boundary;        /* EXC_BOUNDARY_* */
  int32_t grad_mode;       /* EXC_GRAD_* */
  int64_t n[4];
  double origin[4];
  double spacing[4];
  /* Query offset added to a position before every lookup in this grid: the
   * comparison runners integrate in observer-local coordinates and wrap their
   * interpolator so that it queries x + shift (_ShiftedInterpolator,
   * _excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw.py:39-56).
   * All zero = no shift (x + 0.0 leaves every position unchanged). */
  double shift[3];
} ExcField;

/* Spacetime: metric parameters, cosmology table and potential grids. */
typedef struct ExcMetric {
  int32_t kind;            /* EXC_METRIC_* */
  int32_t analytical;      /* analytical_geodesics flag */
  int32_t free_time;       /* Schwarzschild free_time_geodesic flag */
  int32_t cosmology;       /* EXC_COSMO_* (FLRW) */
  double c, c2, c4;        /* float64(c), float64(c**2), float64(c**4) */
  double two_over_c2;      /* float64 of the exact rational 2/c**2 */
  /* Schwarzschild */
  double mass, radius, r_s;
  double center[3];
  /* cosmology table (EXC_COSMO_TABLE*) */
  const double* a_table;
  int64_t a_table_n;
  double eta_min, eta_step;
  double H0, omega_m, omega_r, omega_k, omega_lambda;
  /* potential grids (FLRW) */
  int32_t n_fields;
  int32_t reserved;
  ExcField fields[EXC_MAX_FIELDS];
} ExcMetric;

typedef struct ExcTraceArgs {
  int64_t n_photons;
  double* state;                 /* [n][8] in/out: (x^0..x^3, u^0..u^3) */
  int32_t* status;               /* [n] out: EXC_PH_* */
  int32_t* n_steps;              /* [n] out: accepted steps (optional) */
  int32_t* n_iter;               /* [n] out: iterations incl. rejected (optional) */
  double* dt_state;              /* [n] in/out: per-photon dt (optional; NULL = use dt) */
  const int32_t* field_index;    /* [n] grid used by each photon (optional; NULL = 0) */
  double* obs;                   /* [n][EXC_OBSCOL_N] out (optional) */
  double* records;               /* [n][max_records][record_cols] out (optional) */
  int32_t* n_records;            /* [n] out (required with records) */
  int32_t record_every;          /* reference semantics (integrator.py:271-274,387-394) */
  int32_t max_records;
  int32_t record_cols;           /* 14 (FLRW) or 12 (Schwarzschild) */
  int32_t stepper;               /* EXC_STEPPER_* */
  int32_t tableau;               /* EXC_TABLEAU_* (RK45) */
  int32_t precision;             /* EXC_PREC_* */
  int32_t renormalize_every;     /* 0 = off (integrator.py:376-377) */
  int32_t stop_flags;            /* EXC_STOP_* */
  int32_t obs_flags;             /* EXC_OBS_* bits */
  int32_t block_size;            /* 0 = library default (FP64 builds with blocks_per_sm 0 too:
                                    32-thread blocks, as many an SM as fill the batch's last
                                    wave; otherwise 128) */
  int32_t blocks_per_sm;         /* 0 = library default (EXC_PREC_MIXED with a queue: the
                                    mixed pass's; its FP64 re-trace pass sizes itself on the
                                    device from the share of rays handed back) */
  int32_t staging;               /* EXC_STAGING_*: where the FP64 tracers read the a(eta) table */
  double dt, dt_min, dt_max, rtol, atol;
  int64_t max_iter;              /* reference: 10000 */
  int64_t max_steps;             /* "steps" stop value */
  double box_lo[3], box_hi[3];   /* EXC_STOP_BOX: keep while lo <= x < hi (EXC_STOP_FACE: end on a face) */
  double a_stop;                 /* EXC_STOP_A: stop once a <= a_stop */
  double lens_center[3];         /* cartesian centre for min_r (FLRW) */
  uint32_t* queue;               /* device scratch >= 2 uint32, zeroed by the call;
                                    NULL = static per-photon assignment */
  const int32_t* abort_flag;     /* device flag polled by the kernel (optional) */
  int64_t deadline_cycles;       /* 0 = none; else SM clock cycles after kernel start */
} ExcTraceArgs;

/* ---- entry points ------------------------------------------------------- */
int exc_abi_version(void);
const char* exc_strerror(int code);
const char* exc_last_error(void);         /* message of the last failing call (thread-local) */

int exc_trace(const ExcMetric* metric, const ExcTraceArgs* args, void* stream);

int exc_geodesic_rhs(const ExcMetric* metric, int32_t precision,
                     const double* state, double* out, int32_t* status,
                     const int32_t* field_index, int64_t n, void* stream);

int exc_interp(const ExcField* field, const double* points /* [n][4]: x,y,z,t */,
               double* out /* [n][5]: val, gx, gy, gz, dval/dt */, int32_t* status,
               int64_t n, void* stream);

int exc_eval_cosmology(const ExcMetric* metric, const double* eta, double* a,
                       double* adot, int64_t n, void* stream);

int exc_metric_tensor(const ExcMetric* metric, const double* x /* [n][4] */,
                      double* g_diag /* [n][4] */, int32_t* status,
                      const int32_t* field_index, int64_t n, void* stream);

int exc_null_init(const ExcMetric* metric, double* state /* [n][8], u^0 written */,
                  double sign, int32_t* status, const int32_t* field_index,
                  int64_t n, void* stream);

int exc_null_error(const ExcMetric* metric, const double* state, double* rel_err,
                   int32_t* status, const int32_t* field_index, int64_t n, void* stream);

/* ---- no-allocation variant ----------------------------------------------
 * No counterpart in the reference. exc_trace_noalloc runs exc_trace with its
 * work-queue scratch taken from a fixed array inside the library instead of
 * ExcTraceArgs.queue (which must be NULL), for callers that cannot allocate
 * device memory themselves -- e.g. an application that owns every device buffer
 * and forbids allocation in its processing loop, or a latency-bound loop that
 * cannot afford the implicit device synchronisation of cudaMalloc/cudaFree.
 * Inputs and outputs are still the caller's. Limits: the array is
 * EXC_NOALLOC_SCRATCH_BYTES per GPU, held until the process exits; a launch
 * uses 8 bytes of it (the queue head), on devices 0..EXC_NOALLOC_MAX_DEVICES-1.
 * The first call on a device looks up the array's address (with that device
 * current); make that first call before any stream capture. The address is
 * cached per device and per CUDA context: a call from another context on the
 * same device looks it up again. cudaDeviceReset unloads the library's device
 * code; a later call may then reuse a stale address if the new primary context
 * gets the old handle, so a process that resets a device must not call this
 * entry point again afterwards. All calls share the one array, so calls that
 * overlap on the GPU (e.g. concurrent streams) race on the queue: serialise
 * them. Nothing here calls cudaMalloc/cudaFree. */
#define EXC_NOALLOC_SCRATCH_BYTES 256
#define EXC_NOALLOC_MAX_DEVICES 64
int exc_trace_noalloc(const ExcMetric* metric, const ExcTraceArgs* args, void* stream);

/* ---- device-side photon generation (photon/photons.py:295-459, 540-568): initial
 * states written on the device, then u^0 from the null condition (exc_null_init).
 *   PATCH_GRID   n_side^2 pixel centres of a square tangent-plane patch:
 *                d = axis + (A half) e1 + (B half) e2, A, B = (i + 1/2) / n_side * 2 - 1
 *                (first index A), normalised.
 *   PATCH_POINTS the same at given (A, B) = uv[i] ([n][2] float64, device).
 *   CONE_GRID    theta_i = (i + 1/2) half / n_theta, phi_j = 2 pi j / n_phi (no on-axis ray),
 *                (sin t cos p, sin t sin p, cos t) turned from +z onto the axis by the
 *                Rodrigues rotation v cos + (k x v) sin + k (v . k)(1 - cos) with
 *                rot_axis = k, rot_cos, rot_sin (the host's rotate_to_direction values).
 *   FULL_SKY     n directions uniform on the sphere from a counter-based generator
 *                (splitmix64 of seed and photon index; not numpy's stream).
 * u_spatial = speed * d; origin (eta, x, y, z) for every photon; u^0 = sign * |u^0|.
 * status ([n], optional) gets the null initialisation's status. */
/* EXC_GEN_CONE_RANDOM (Photons.generate_cone_random, photon/photons.py:33-157): n
 *   directions with theta uniform in [0, half) from the cone axis and azimuth uniform in
 *   [0, 2 pi), rotated like CONE_GRID; counter-based random numbers (seed, photon index),
 *   so the stream is not numpy's.
 * EXC_GEN_IMPACT_BINS (Photons.generate_impact_parameter_bins, photons.py:570-701): parallel
 *   rays along `axis` from screen points origin + b (cos p e1 + sin p e2), photon i in the bin
 *   ib with bin_offsets[ib] <= i < bin_offsets[ib + 1]; b uniform in area in
 *   [b_edges[ib], b_edges[ib + 1]], p uniform in [0, 2 pi) (random_phi) or j 2 pi / n_ib for
 *   the bin's j-th photon; `spherical` converts positions and velocities to (r, theta, phi)
 *   with the reference's formulas (core/coordinates.py:31-84), origin[1..3] then being the
 *   cartesian observer. n = bin_offsets[n_bins]. */
enum { EXC_GEN_PATCH_GRID = 0, EXC_GEN_PATCH_POINTS = 1, EXC_GEN_CONE_GRID = 2, EXC_GEN_FULL_SKY = 3,
       EXC_GEN_CONE_RANDOM = 4, EXC_GEN_IMPACT_BINS = 5 };
typedef struct ExcPhotonGen {
  int32_t mode;
  int32_t n_side;            /* PATCH_GRID */
  int32_t n_theta, n_phi;    /* CONE_GRID */
  int64_t n;                 /* PATCH_POINTS, FULL_SKY, CONE_RANDOM, IMPACT_BINS */
  double origin[4];
  double axis[3];
  double e1[3], e2[3];       /* PATCH_*: tangent basis */
  double half;               /* PATCH_*: tan(patch / 2); CONE_*: cone half-angle (rad) */
  double rot_axis[3];        /* CONE_* rotation */
  double rot_cos, rot_sin;
  const double* uv;          /* PATCH_POINTS */
  uint64_t seed;             /* FULL_SKY, CONE_RANDOM, IMPACT_BINS */
  double speed;
  double sign;
  int32_t n_bins;            /* IMPACT_BINS */
  int32_t random_phi;
  int32_t spherical;
  int32_t reserved;
  const double* b_edges;     /* [n_bins + 1], device */
  const int64_t* bin_offsets;  /* [n_bins + 1], device, cumulative photon counts from 0 */
} ExcPhotonGen;

/* Number of photons a generator produces. */
int64_t exc_gen_count(const ExcPhotonGen* gen);
/* states: [exc_gen_count(gen)][8] float64, device. */
int exc_generate_photons(const ExcMetric* metric, const ExcPhotonGen* gen, double* states, int32_t* status,
                         void* stream);

/* ---- lens potential on a grid: replaces the host-side field construction of
 * spherical_mass(M, R, center).potential(X, Y, Z) (objects/spherical_mass.py:29-49)
 * on the meshgrid of numpy.linspace(origin, origin + n * spacing, n, endpoint=False)
 * that the comparison runners build before every run
 * (_excalibur_runs/excalibur_run_compare_schwarzschild_vs_flrw.py:474-479).
 * out: [n0][n1][n2] float64, device. neg_gm, three_r2, two_r3 are the reference's
 * scalar subexpressions -G*M, 3*R**2 and 2*R**3, evaluated by the caller with the
 * reference's own (Python) arithmetic; the grid is then bit-identical to numpy's. */
int exc_spherical_mass_grid(const int64_t n[3], const double origin[3], const double spacing[3],
                            const double center[3], double radius, double neg_gm, double three_r2,
                            double two_r3, double* out, void* stream);

/* ---- launch-schedule autotuner (no reference counterpart: the reference has no
 * GPU schedule). Runs exc_trace on a sample batch for each candidate (block size
 * 32, 64, 96, 128) x (blocks per SM 2 .. 8, and 0 = the occupancy limit) -- the lane
 * count sets how evenly a batch of similar trajectories fills its last wave, and the
 * warps an SM how they share its FP64 throughput --, then the three fastest of those again with the a(eta) table
 * staged in shared memory (EXC_STAGING_SHARED; FP64 launches of an FLRW metric with a
 * table of at most EXC_STAGING_MAX_TABLE entries), and returns the one with the highest
 * rate (args->staging is ignored; plan->staging is the chosen staging). The sample's
 * buffers are scratch: before every trial the library copies pristine_state
 * ([n][8] float64, device) into args->state; args->dt_state must be NULL (trials
 * start from args->dt); args->block_size / blocks_per_sm are ignored. With
 * args->n_iter given, the rate is the sum of n_iter (steps tried) per second, so a
 * trial may be cut short by args->deadline_cycles (a time box over a large,
 * shuffled sample measures the steady state rather than the longest trajectory);
 * without it the rate is 1 / elapsed time. One untimed warm-up trial precedes the
 * timed ones. Synchronous on `stream`; allocates no device memory. */
#define EXC_TUNE_MAX_TRIALS 48
typedef struct ExcLaunchPlan {
  int32_t block_size;
  int32_t blocks_per_sm;
  float best_ms;
  float best_rate;          /* steps tried per second (or 1/s) of the chosen candidate */
  int32_t n_trials;
  int32_t trial_block[EXC_TUNE_MAX_TRIALS];
  int32_t trial_blocks_per_sm[EXC_TUNE_MAX_TRIALS];
  float trial_ms[EXC_TUNE_MAX_TRIALS];
  float trial_rate[EXC_TUNE_MAX_TRIALS];
  int32_t staging;          /* EXC_STAGING_* of the chosen candidate */
  int32_t trial_staging[EXC_TUNE_MAX_TRIALS];
} ExcLaunchPlan;

int exc_autotune(const ExcMetric* metric, const ExcTraceArgs* args, const double* pristine_state,
                 ExcLaunchPlan* plan, void* stream);

/* The FP64 builds' default launch size (block_size and blocks_per_sm both 0): 32-thread blocks,
 * this many an SM for n_photons similar trajectories on sm_count SMs with at most occupancy
 * 32-thread blocks resident an SM -- the batch over the waves it needs at that limit, rounded up
 * to whole warps an SM, so that its last wave is as full as the others. Host only. */
int32_t exc_balanced_blocks_per_sm(int64_t n_photons, int32_t sm_count, int32_t occupancy);

/* ---- FP64 pipe probe (measurement only; no reference counterpart) --------
 * Throughput of the FP64 operations the parity build issues, measured on the
 * current device with IEEE semantics and no FMA contraction (the parity
 * build's flags): rates_out[EXC_PROBE_*] in operations per second over the
 * whole GPU. A bench turns the algorithmic operation mix of a photon-step into
 * FP64-pipe time with them (a division costs several multiply/add slots).
 * `scratch` is a caller-owned device buffer of at least exc_probe_scratch_len()
 * doubles. Synchronous on `stream`. */
enum { EXC_PROBE_ADDMUL = 0, EXC_PROBE_DIV = 1, EXC_PROBE_SQRT = 2, EXC_PROBE_FMOD = 3, EXC_PROBE_N = 4 };
int64_t exc_probe_scratch_len(void);
int exc_probe_fp64_rates(double* scratch, int64_t n_scratch, double* rates_out, void* stream);

/* Check of the parity build's division by launch constants (no reference counterpart): the
 * quotient x * RN(1/c) with Markstein's FMA correction against the IEEE quotient x / c, bit for
 * bit, over n_samples x (random signs and significands over 2^-200 .. 2^200, and every second
 * one placed next to a rounding midpoint of x / c) for the divisors[k] (device, n_div of them,
 * taken in turn). *mismatches (device) is zeroed, then counts the quotients that differ. */
int exc_probe_div_rn(const double* divisors, int32_t n_div, int64_t n_samples, uint64_t seed,
                     unsigned long long* mismatches, void* stream);

/* ---- redshift maps from recorded trajectories ---------------------------
 * Replace the host loop of _postprocessing/compute_redshift_map.py:98-171
 * (compute_redshift_map: per photon, the rows holding a NaN dropped as
 * load_trajectories does at :47-48, then RedshiftCalculator(...)
 * .compute_all_components(), excalibur/observables/redshift.py:340-399) and
 * extract_sky_positions (:54-95); the maps are pixel means (exc_sky_bin) in place
 * of create_2d_map's scipy griddata (_postprocessing/compute_time_delay_map.py:313-357).
 * records: [n_photons][n_rows][n_cols] float64, device, NaN-padded (the runners'
 * trajectory-file layout; FLRW rows [eta, x, y, z, u0..u3, a, Phi, dPhi/dx,
 * dPhi/dy, dPhi/dz, dPhi/deta], n_cols >= 14). */
enum {
  EXC_RS_Z_H = 0,
  EXC_RS_Z_SW = 1,
  EXC_RS_Z_ISW = 2,          /* -simpson(Phi_dot c^2, eta) / c^2, scipy's irregular-spacing rule */
  EXC_RS_Z_D = 3,            /* Doppler; 0 without endpoint velocities */
  EXC_RS_Z_TOTAL = 4,
  EXC_RS_Z_TOTAL_EXACT = 5,
  EXC_RS_PHI_OBS = 6,        /* columns 6..17: NaN for a photon without clean rows */
  EXC_RS_PHI_EM = 7,
  EXC_RS_A_OBS = 8,
  EXC_RS_A_EM = 9,
  EXC_RS_ETA_OBS = 10,
  EXC_RS_ETA_EM = 11,
  EXC_RS_X_OBS = 12,         /* 3 columns */
  EXC_RS_X_EM = 15,          /* 3 columns */
  EXC_RS_N_ROWS = 18,        /* clean rows; components stay 0 below 2, as in compute_redshift_map */
  /* time delay over the recorded rows (_postprocessing/compute_time_delay_map.py:97-126,
   * 244-310): 0 below two clean rows, as compute_time_delays leaves them */
  EXC_RS_PATH = 19,          /* sum of |x_{k+1} - x_k| over consecutive clean rows, m */
  EXC_RS_CHORD = 20,         /* |x_last - x_first|, m */
  EXC_RS_TIME_DELAY = 21,    /* path / c - chord / c, s */
  EXC_RS_TD_KEPT = 22,       /* 1 when load_trajectories (:76-92) keeps the photon: a clean row,
                                every clean |x| < 1e26 m and |eta| < 3e18 s; else 0 */
  EXC_RS_NCOLS = 23
};
/* out: [n_photons][EXC_RS_NCOLS] float64, device. scratch: n_photons * n_rows int32,
 * device, used only when n_rows > 257 (NULL allowed otherwise: up to 257 rows, the ISW
 * Simpson sum is one numpy summation block and the kernel reads each row once). v_obs, v_em:
 * [n_photons][3] float64 peculiar velocities at the first and last clean row (the
 * reference's velocity_func evaluated there), or both NULL. */
int exc_record_redshift(const double* records, int64_t n_photons, int32_t n_rows, int32_t n_cols, double c,
                        const double* v_obs, const double* v_em, int32_t* scratch, double* out, void* stream);
/* dirs: [n_photons][3], the unit spatial velocity (columns 5..7) of each photon's first clean
 * row; NaN for a photon without one. */
int exc_sky_directions(const double* records, int64_t n_photons, int32_t n_rows, int32_t n_cols, double* dirs,
                       void* stream);
/* x_proj, y_proj: [n] tangent-plane coordinates of dirs about mean_dir with the in-plane basis
 * (basis_x, basis_y): the angle from mean_dir along the in-plane unit vector, 0 within 1e-10
 * rad of it, NaN for a NaN direction. The three host vectors are passed by value. */
int exc_sky_project(const double* dirs, int64_t n, const double mean_dir[3], const double basis_x[3],
                    const double basis_y[3], double* x_proj, double* y_proj, void* stream);
/* Pixel means of scattered samples over extent = {x0, x1, y0, y1} (host): pixel
 * (iy, ix) with ix = min(floor((x - x0) / (x1 - x0) * nx), nx - 1), iy likewise; samples
 * outside the extent or with a non-finite x, y or value are skipped. sum [ny][nx] float64 and
 * count [ny][nx] uint64 are zeroed first; mean [ny][nx] = sum / count, NaN where count = 0. */
int exc_sky_bin(const double* x, const double* y, const double* values, int64_t n, int32_t nx, int32_t ny,
                const double extent[4], double* sum, unsigned long long* count, double* mean, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* EXCALIBUR_GB300_H */
