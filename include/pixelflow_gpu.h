/*
 * pixelflow_gpu.h -- C ABI of the GB300 immersed-boundary step.
 *
 * Drop-in for the step loop of PixelFlow's ibm2 / ibm3 programs
 * (nobu-n2002/PixelFlow, src/omp_parallel/ibm_2d_uniform_omp_cpu.f90 and
 * ibm_3d_uniform_omp_cpu.f90).  The reference has no plugin or FFI layer;
 * its seam is the set of Fortran subroutines called from `program main`.
 * Each entry point below names the reference routine it replaces.
 *
 * Conventions
 *  - Plain C types only; every call returns PF_OK (0) or a negative PF_E_*
 *    code, and pf_last_error() gives a message for the calling thread.
 *  - Field arrays cross the boundary in the reference's own layout: Fortran
 *    column-major a(0:ld1-1, 0:ld2-1[, 0:l+1]) of double, i fastest, with
 *    the ghost layer at 0 and m+1.  ld1 >= m+2 and ld2 >= n+2 are the
 *    caller's leading dimensions (md+1 and nd+1 of lib/global.f90:6,12).
 *  - A case owns its device memory and one CUDA stream; calls on one case
 *    are not thread safe, calls on different cases are.  Compute calls are
 *    asynchronous; pf_get_state / pf_norms / pf_synchronize wait.
 */
#ifndef PIXELFLOW_GPU_H
#define PIXELFLOW_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF_ABI_VERSION 3

enum {
  PF_OK = 0,
  PF_E_INVALID = -1,   /* bad argument or unsupported size */
  PF_E_CUDA = -2,      /* CUDA runtime failure */
  PF_E_NOMEM = -3,     /* device allocation failed or over the memory budget */
  PF_E_NONFINITE = -4, /* NaN or Inf found in the fields */
  PF_E_TIMEOUT = -5,   /* a bounded device wait gave up */
  PF_E_STATE = -6,     /* call made in the wrong order / handle closed */
  PF_E_BUSY = -7       /* no free slot (batch and serving forms) */
};

enum { PF_PREC_FP64 = 0, PF_PREC_MIXED = 1 };

/* Namelist values of config/controlDict.txt (lib/global.f90:18-26, 47-54)
 * plus the grid size from the porosity file header (lib/grid.f90:38,283).
 * dx = width/(m-1), dy = height/(n-1), dz = depth/(l-1), dt = time/istep_max
 * are derived as grid.f90:50-52 and :297-300 do. */
typedef struct pf_params {
  int32_t dim, m, n, l; /* dim 2 (ibm2) or 3 (ibm3); l ignored for dim 2 */
  double xnue, xlambda, density, width, height, depth, time;
  double inlet_velocity, outlet_pressure, aoa;
  int32_t istep_max, iter_max;
  double thickness, threshold, relux_factor;
  int32_t nonslip;
  int32_t inflow_porosity; /* 1: inflow and initial velocities scaled by the
                              porosity, as ibm_2d_backstep_omp_cpu.f90 does
                              (:533-534, :615-618); 0: the uniform programs */
  int32_t wall_mode;       /* 1 (3D, plain FP64 only): the air-condition
                              program, ibm_3d_air_condition_omp_cpu.f90 --
                              walls on all six faces by the table below,
                              non-periodic ghosts; 0: the uniform programs */
  int32_t walls[6];        /* wall table, faces top, bottom, east, west,
                              north, south (:10-15): 0 wall, 1 inlet (where
                              porosity >= 0.9), 2 outlet (where >= 0.9) */
  int32_t slip_y;          /* 1 (2D, plain FP64 only): symmetry rows at j = 1
                              and j = n (dp/dy = 0, v = 0, u mirrored) in
                              place of the periodic wrap -- the option the
                              reference keeps commented out in
                              boundrary_matrix (ibm_2d_uniform_omp_cpu.f90:
                              438-450) and boundary (:503-518); 0: periodic */
} pf_params;

/* Options that only this library reads (the &gpu_control group). */
typedef struct pf_options {
  int32_t precision;       /* PF_PREC_FP64: plain step.  PF_PREC_MIXED: FP32
                              stencils and SOR sweeps inside an FP64
                              defect-correction loop */
  int32_t outer_max;       /* mixed: defect-correction passes per step */
  int32_t inner_sweeps;    /* mixed: FP32 SOR iterations per pass */
  int32_t track_sor_error; /* 1: compute the reference's SOR max-change */
  double dc_tol;           /* mixed: stop passes once max|r| <= dc_tol */
  int32_t use_graph;       /* 1: replay each step from a CUDA graph */
  int32_t sweep_form;      /* mixed, FP32 sweeps: PF_SWEEP_SPLIT one launch
                              per colour; PF_SWEEP_FUSED both colours in one
                              launch where the case allows it (3D, even n and
                              l; split otherwise); PF_SWEEP_AUTO times both
                              on the case at creation and keeps the faster.
                              Same results bit for bit */
  int32_t fused_rows;      /* mixed, fused sweep: y rows per tile (0: auto) */
  int32_t fused_planes;    /* mixed, fused sweep: cap on the (tile, plane)
                              pairs of one CTA (0: one wave of CTAs) */
  int32_t sor_path;        /* plain FP64, 3D: PF_SOR_AUTO walks per-colour
                              cell lists with the pure-fluid cells (porosity
                              1 around them) first, whose six neighbours are
                              summed exactly and whose coefficients are the
                              one fluid constant; PF_SOR_CELLS updates every
                              cell with its own six stored coefficients.  The
                              same red-black iterates up to the rounding of
                              the fluid cells' neighbour sum */
  int32_t reserved[1];
} pf_options;

enum { PF_SWEEP_AUTO = 0, PF_SWEEP_SPLIT = 1, PF_SWEEP_FUSED = 2 };
enum { PF_SOR_AUTO = 0, PF_SOR_CELLS = 1 };

typedef struct pf_case pf_case;

/* Message for the last failed call on this thread ("" if none). */
const char *pf_last_error(void);
const char *pf_strerror(int code);
int pf_abi_version(void);
/* Select the CUDA device that later pf_create calls on this thread use. */
int pf_set_device(int device);
int pf_device_count(int *count);
/* Fill *opt with defaults (plain FP64, error tracking on, graphs on). */
void pf_default_options(pf_options *opt);

/* Create a case.  porosity_values: m*n[*l] raw values in the order of the
 * porosity CSV records (i fastest), as read by grid_conditions
 * (lib/grid.f90:36-47 2D, :281-294 3D); the threshold clamp of grid.f90:43
 * and the ghost fill of :92-106 / :349-378 are applied here.
 * Replaces: read_settings + grid_conditions[_yz_periodic] set-up. */
int pf_create(const pf_params *prm, const pf_options *opt, const double *porosity_values,
              pf_case **out);
int pf_destroy(pf_case *c);

/* Create a case whose porosity is generated on the GPU from analytic shapes,
 * with the profile of the reference's preprocessing tools
 * (tools/cylinder/make_porosity_2d_cylinder.py:119-122):
 *   porosity = max(threshold, 0.5*tanh(sdf/(edge*dx)) + 0.5),
 * sdf = min over the shapes of the signed distance (positive in the fluid),
 * node (i,j,k) at ((i-1)dx, (j-1)dy, (k-1)dz).  Circles and ellipses (2D,
 * ellipse distance to first order) and spheres (3D); at most PF_MAX_SHAPES.
 * Same set-up as pf_create otherwise. */
enum { PF_SHAPE_CIRCLE = 0, PF_SHAPE_ELLIPSE = 1, PF_SHAPE_SPHERE = 2 };
#define PF_MAX_SHAPES 32
typedef struct pf_shape {
  int32_t kind, reserved;
  double cx, cy, cz; /* centre (cz ignored in 2D) */
  double a, b;       /* radius / semi-axes */
  double angle;      /* ellipse rotation (radians) */
} pf_shape;
int pf_create_shapes(const pf_params *prm, const pf_options *opt, const pf_shape *shapes, int nshapes,
                     double edge, pf_case **out);

/* initial_conditions followed by boundary
 * (ibm_2d_uniform_omp_cpu.f90:67-70 / ibm_3d_uniform_omp_cpu.f90:68-71). */
int pf_initial_conditions(pf_case *c);

/* Host <-> device field exchange in the Fortran layout described above.
 * w is ignored for 2D cases (may be NULL). */
int pf_set_state(pf_case *c, const double *u, const double *v, const double *w, const double *p,
                 int ld1, int ld2);
int pf_get_state(pf_case *c, double *u, double *v, double *w, double *p, int ld1, int ld2);

/* Asynchronous output at istep_out (the reference writes its VTK files from
 * the host arrays, lib/output.f90:421-537, :968-1088): pf_snapshot_begin
 * copies the state as of the last enqueued step on the device and starts the
 * device->host copy on a second stream, so the caller can enqueue further
 * steps at once; pf_snapshot_wait waits for that copy and unpacks it into the
 * caller's arrays (same layout as pf_get_state; a null field is skipped).  One
 * snapshot may be in flight per case (PF_E_BUSY otherwise). */
int pf_snapshot_begin(pf_case *c);
int pf_snapshot_wait(pf_case *c, double *u, double *v, double *w, double *p, int ld1, int ld2);
int pf_get_porosity(pf_case *c, double *poro, int ld1, int ld2);

/* solve_p: divergence, predictor, coefficients/RHS, boundrary_matrix and the
 * red-black SOR (ibm_2d_uniform_omp_cpu.f90:142-286, 293-406, 410-454;
 * ibm_3d_uniform_omp_cpu.f90:151-426, 433-614, 618-663).  Snapshots the
 * velocities first, as the step loop does (2D :84-96, 3D :85-100). */
int pf_solve_p(pf_case *c);
/* Velocity projection loop (2D :103-115, 3D :109-125). */
int pf_projection(pf_case *c);
/* boundary (2D :460-538, 3D :669-752). */
int pf_boundary(pf_case *c);
/* nsteps passes of the main step loop body (2D :80-125, 3D :81-132):
 * snapshot, solve_p, projection, boundary. */
int pf_step(pf_case *c, int nsteps);
int pf_synchronize(pf_case *c);

/* One pass of the step loop body (2D :80-125, 3D :81-132) from host arrays
 * to host arrays, for a caller whose fields live on the host between steps:
 * the result equals pf_set_state(u, v, w, p) + pf_step(c, 1) +
 * pf_get_state(u_out, ...), bit for bit.  For 3D periodic plain-FP64 cases
 * with ld1 = m+2 and ld2 = n+2 the input copies run in slabs of planes beside
 * the divergence and the predictor of the planes already in place (the first
 * use allocates three fields of device staging, counted by
 * pf_memory_bytes); other cases make the three calls.  A null output field is
 * not read back.  Waits for the result. */
int pf_step_host(pf_case *c, const double *u, const double *v, const double *w, const double *p,
                 double *u_out, double *v_out, double *w_out, double *p_out, int ld1, int ld2);

/* max|div u| of the porosity-weighted divergence that output_divergent_2d/3d
 * writes (lib/output.f90:217-224, :929-941) on the current fields, and the
 * SOR `error` of the last solve_p (the value the reference prints at
 * ibm_2d_uniform_omp_cpu.f90:400 / ibm_3d:608; 0 when tracking is off).
 * Returns PF_E_NONFINITE if max_div is NaN or Inf. */
int pf_norms(pf_case *c, double *max_div, double *sor_error);

/* Force sums of the current state, as output_force_log_2d / _3d compute them
 * (lib/output.f90:244-305, :1090-1165; called every step by
 * ibm_2d_drag_omp_cpu.f90:121): force_p = pressure part (x, y, z), force_v =
 * wall-friction part; z = 0 in 2D.  F = force_p + force_v, and the reference's
 * Cd/Cl are F / (density * inlet_velocity^2 * radius).  Deterministic (fixed
 * summation order); waits for the case's stream. */
int pf_forces(pf_case *c, double force_p[3], double force_v[3]);

/* Pin a caller-owned host buffer so pf_set_state / pf_get_state copy it
 * asynchronously at full link speed (cudaHostRegister); optional. */
int pf_host_register(void *ptr, size_t bytes);
int pf_host_unregister(void *ptr);

/* Timing of the stages inside pf_step, with CUDA events on the case's
 * stream.  While profiling is on, steps run without graph replay.
 * pf_profile_end returns the summed device time of the SOR half-sweep
 * kernels, their launch count, and the time of whole steps. */
int pf_profile_begin(pf_case *c);
int pf_profile_end(pf_case *c, double *sor_ms, int64_t *sor_launches, double *step_ms,
                   int64_t *steps);

/* Per-step durations (ms) of the last profiling session, up to max_steps
 * values; *n receives the count written. */
int pf_profile_step_times(pf_case *c, double *ms, int64_t max_steps, int64_t *n);

/* The last profiling session's device time (ms, summed over its steps) of
 * the step's four stages, in the order of the reference's loop body:
 * ms[0] divergence + predictor, ms[1] the Poisson right-hand side (and, in
 * the precision form, nothing else), ms[2] the SOR (every half-sweep with
 * its halo updates; the precision form's passes of FP64 residual, FP32
 * sweeps and FP64 accumulation), ms[3] projection + boundary. */
int pf_profile_stages(pf_case *c, double ms[4]);

/* Number of kernels this case has launched (graph replays count every
 * kernel node), for accounting in benchmarks. */
int pf_kernel_launches(pf_case *c, int64_t *count);

/* Device memory held by the case, in bytes. */
int pf_memory_bytes(pf_case *c, size_t *bytes);

/* ---- Batched form -------------------------------------------------------
 * Many independent cases (2D and 3D, uneven sizes) resident on one GPU,
 * advanced by one persistent kernel per dimension: each thread-block cluster
 * claims a case from a device queue (largest work first) and runs all stages
 * of its steps itself, separated by hardware cluster barriers.  Cases larger
 * than large_cells run full-GPU steps on their own streams at the same time.  Cases run the
 * precision form (PF_PREC_MIXED) with the per-case options given at add time.
 * No counterpart in the reference, which runs one case per process; the
 * per-case step is the same routine sequence as pf_step. */
typedef struct pf_batch pf_batch;
typedef struct pf_batch_options {
  int32_t cluster;           /* CTAs per cluster: 1, 2, 4, 8 or 16 */
  int32_t threads;           /* threads per CTA: 256, 512 or 1024 */
  int32_t max_cases;         /* slots */
  int32_t global_passes;     /* 1: 2D cases never keep their correction in
                                shared memory (default 0: they do when the
                                rows of a CTA fit in 226 KB) */
  uint64_t hbm_budget_bytes; /* admission limit for the cases' device memory */
  int32_t large_cells;       /* cases with more cells run full-GPU steps on their
                                own stream, concurrently with the persistent
                                kernel (default 100000) */
  int32_t use_graph;         /* 1 (default): the descriptor upload and the
                                persistent launches of a call run as a CUDA
                                graph, captured once per composition (cases
                                per dimension, shared memory, launch shape)
                                and replayed by later calls of the same
                                composition (the last 16 compositions are
                                kept); the large cases replay their own
                                step graphs.  0: plain launches */
  int32_t reserved[6];
} pf_batch_options;
void pf_batch_default_options(pf_batch_options *opt); /* cluster 4, 512 threads, 1024 slots, 150 GiB */
int pf_batch_create(const pf_batch_options *opt, pf_batch **out);
int pf_batch_destroy(pf_batch *b);
/* Device bytes a case needs (same accounting as the admission check). */
int pf_case_bytes(const pf_params *prm, const pf_options *opt, size_t *bytes);
/* Add a case (initial conditions applied).  PF_E_NOMEM when it does not fit
 * the budget now, PF_E_BUSY when no slot is free. */
int pf_batch_add(pf_batch *b, const pf_params *prm, const pf_options *opt, const double *porosity_values,
                 int *slot);
int pf_batch_add_shapes(pf_batch *b, const pf_params *prm, const pf_options *opt, const pf_shape *shapes,
                        int nshapes, double edge, int *slot);
int pf_batch_remove(pf_batch *b, int slot);
/* Advance slots[q] by nsteps[q] steps, all in one persistent launch per
 * dimension; returns when the launch has finished. */
int pf_batch_step_slots(pf_batch *b, const int *slots, const int *nsteps, int n);
int pf_batch_step(pf_batch *b, int nsteps); /* every occupied slot */
int pf_batch_synchronize(pf_batch *b);
int pf_batch_get_state(pf_batch *b, int slot, double *u, double *v, double *w, double *p, int ld1, int ld2);
int pf_batch_norms(pf_batch *b, int slot, double *max_div, double *sor_error);
int pf_batch_memory(pf_batch *b, size_t *in_use, size_t *budget);
int pf_batch_kernel_launches(pf_batch *b, int64_t *n);
/* Change the launch shape (CTAs per cluster, threads per CTA) used by later
 * steps; the autotuner calls this between timed trials. */
int pf_batch_configure(pf_batch *b, int cluster, int threads);
/* Device time (CUDA events on the batch stream) of the last step call. */
int pf_batch_last_ms(pf_batch *b, double *ms);
/* Graphs of the persistent launch captured so far, and calls that replayed
 * one without capturing. */
int pf_batch_graph_stats(pf_batch *b, int64_t *captured, int64_t *replays);

/* max|div u| without allocating device memory.  No counterpart in the
 * reference: it exists for callers that must not call cudaMalloc at this
 * point -- cudaMalloc/cudaFree synchronise the whole device, which stalls a
 * loop that keeps other work running on other streams, and some programs run
 * under a memory budget owned by another allocator.  u, v, w (NULL in 2D)
 * and porosity are the caller's DEVICE arrays in the Fortran layout of
 * pf_get_state / pf_get_porosity (leading dimensions ld1 >= m+2,
 * ld2 >= n+2); *max_div is a DEVICE double written on `stream` (a
 * cudaStream_t, NULL for the legacy default stream).  Same value as
 * pf_norms' max_div.  The reduction uses a fixed scratch array compiled into
 * the library (PF_NOALLOC_MAX_ROWS partials, 2 MiB, held by every GPU that
 * loads the library until exit); cases with n*l > PF_NOALLOC_MAX_ROWS are
 * rejected with PF_E_INVALID.  All calls share that array, so calls that
 * overlap on the GPU race and must be serialised by the caller.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress); make
 * it before any stream capture begins.  That address is kept per device
 * ordinal for the rest of the process: it belongs to the device's primary
 * context, so call this only with the primary context current, and not after
 * a cudaDeviceReset of that device. */
#define PF_NOALLOC_MAX_ROWS 262144
int pf_max_div_noalloc(const pf_params *prm, const double *u, const double *v, const double *w,
                       const double *porosity, int ld1, int ld2, double *max_div, void *stream);

/* The precision form's FP32 sweep: *fused = 1 when the case runs both
 * colours in one launch; split_ms / fused_ms (either may be NULL) = the
 * time per sweep of each form measured at creation under PF_SWEEP_AUTO
 * (0 when not measured). */
int pf_sweep_info(pf_case *c, int *fused, float *split_ms, float *fused_ms);

/* Testing of the failure path of the fused correction sweep (no reference
 * counterpart): from the next step on, the sweep's producer skips staging
 * step `stage` of each run, so the consumers' bounded wait for it runs out
 * (about 0.2 s), every CTA drains its own copies and the case's error word
 * is set; pf_synchronize, pf_get_state and pf_norms then return
 * PF_E_TIMEOUT for the rest of the case's life.  stage < 0 restores normal
 * operation of later steps (the error word stays).  PF_E_STATE when the case
 * does not run the fused sweep.  After PF_E_TIMEOUT the case's fields are
 * undefined: the sweeps that gave up stopped part way through a pass, so
 * the correction and the pressure hold a mix of old and new values (no
 * result is computed from a stage that never landed).  Restart the case
 * from a saved state. */
int pf_debug_fused_drop_stage(pf_case *c, int stage);

/* The schedule pf_step_host follows for a 3D case with l planes (no device
 * work): per slab of input planes, six ints -- the planes k0, k1 it brings
 * (ghost planes 0 and l+1 included), then the divergence planes and the
 * predictor planes issued once it is in place (lo, hi; empty when hi < lo).
 * Plane 1 of the predictor runs after the last slab.  Writes up to
 * `capacity` slabs and returns the number of slabs. */
int pf_debug_step_host_plan(int l, int *slabs, int capacity);

/* The plain sweep's cell lists (no reference counterpart): *listed = 1 when
 * the case's SOR walks cell lists (PF_SOR_AUTO, 3D plain FP64 without
 * walls); fluid[c] / total[c] = the pure-fluid cells and all cells of
 * colour c (either array may be NULL). */
int pf_sor_info(pf_case *c, int *listed, int fluid[2], int total[2]);

/* The precision form's split FP32 sweep (no reference counterpart): *listed
 * = 1 when it walks chunk lists (PF_SOR_AUTO, 3D without walls, grids of
 * more than one wave of CTAs); fluid[c] / total[c] = the chunks of four
 * cells whose porosity operands are all 1.0f and all chunks of colour c
 * (either array may be NULL). */
int pf_dc_list_info(pf_case *c, int *listed, int fluid[2], int total[2]);

/* Testing of the exact six-term sum of the list sweep's fluid cells (no
 * reference counterpart): out[i] = x[6i] + ... + x[6i+5] rounded once to
 * FP64, ok[i] = 0 where an input is Inf/NaN or the sum is not a normal
 * number (the sweep then adds in FP64).  Host arrays; allocates. */
int pf_debug_sum6(const double *x, int n, double *out, int *ok);

#ifdef __cplusplus
}
#endif
#endif /* PIXELFLOW_GPU_H */
