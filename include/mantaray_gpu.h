/*
 * mantaray_gpu.h -- C ABI of the GB300 ray-integration library
 * (libmantaray_gpu.so).
 *
 * Drop-in boundary for the hot path of mines-oceanography/mantaray: the Rust
 * extension module `_mantaray` (src/ffi.rs:18-85) and the drivers beneath it
 * (ManyRays::trace_many, src/ray.rs:98-127; SingleRay::trace_individual,
 * src/ray.rs:198-213) over the field types of src/bathymetry/ and
 * src/current/.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every function returns MR_OK (0) or a negative MR_ERR_* code; the
 *    message of the last failure on the calling thread is mr_last_error().
 *  - Field handles own device (HBM) copies of their grids, made once at
 *    creation on the device current at that time, and are immutable: one
 *    handle may serve any number of concurrent trace calls.
 *  - Trajectories are stored traj[5][rows_cap][n] (f64; variables t, x, y,
 *    kx, ky; time-major, ray fastest): the (time_step, ray) layout of the
 *    reference's xarray result (python/mantaray/core.py:114-125).  Rows past
 *    a ray's last row are NaN (core.py:116-119 pads with NaN).
 *  - n_rows[i] counts the rows the reference records for ray i: the initial
 *    state plus one row per step taken, the last one included when the stop
 *    rule ends the ray (src/wave_ray_path.rs:600-626).
 *  - Per-ray failures do not fail the call: the reference turns every RHS
 *    error into NaN (src/wave_ray_path.rs:220-234) and stops the ray;
 *    status[i] says which way each ray ended.
 */
#ifndef MANTARAY_GPU_H
#define MANTARAY_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ------------------------------------------------------ */
#define MR_OK 0
/* An argument is invalid (null pointer, size mismatch, axis with fewer than
 * two points, unknown option).  Error::InvalidArgument, src/error.rs:12-14. */
#define MR_ERR_INVALID_ARGUMENT (-1)
/* A CUDA runtime call failed (message names the call). */
#define MR_ERR_CUDA (-2)
/* A file could not be opened or read.  Error::IOError, src/error.rs:26-28;
 * the reference panics here (src/ffi.rs:36-38). */
#define MR_ERR_IO (-3)
/* Not a NetCDF-3 classic/64-bit-offset file, or a variable is missing.
 * Error::ReadError, src/error.rs:34-36. */
#define MR_ERR_READ (-4)
/* rows_cap < mr_num_steps(t0, t_end, dt) + 1. */
#define MR_ERR_CAPACITY (-5)
/* Device or host allocation failed. */
#define MR_ERR_OUT_OF_MEMORY (-6)

/* ---- per-ray status ------------------------------------------------------ */
#define MR_RAY_COMPLETE 0 /* all ceil((t_end - t0)/dt) steps taken */
#define MR_RAY_STOPPED 1  /* ended by the solout rule (src/wave_ray_path.rs:236-246) */

/* ---- trace options (bit flags, OR-ed into `options`) ---------------------
 * Stop rule: which derivative the solout test sees after each step.  The
 * stepper crate (ode_solvers 0.4.0) is not in the reference tree, so both
 * readings are offered; they differ only by whether a ray whose new state is
 * finite but out of the domain records one more, all-NaN, row.
 *   MR_STOP_STAGE1: the first-stage derivative of the step just taken.
 *   MR_STOP_FRESH:  the derivative evaluated at the new state.
 * Right-hand-side arithmetic of the plain FP64 kernel:
 *   MR_MATH_IDENTITY: (default, 0) the reference's quantities from one
 *                     expm1, one reciprocal, two rsqrt and kx/k, ky/k (exact
 *                     identities, FMAs; a few ulps from the reference's
 *                     calls), about 3x as fast on the FP64 pipe.
 *   MR_MATH_LIBM:     the reference's own calls (atan2, cos, sin, cosh, tanh,
 *                     sinh, three sqrt) in its own order; reproduces the
 *                     reference's single-step known answers to f64::EPSILON.
 * Both hold every step within 1e-9 (relative) of the reference.  Field
 * lookups and interpolation are bit-identical to the reference in both. */
#define MR_STOP_STAGE1 0x0
#define MR_STOP_FRESH 0x1
#define MR_MATH_IDENTITY 0x0
#define MR_MATH_LIBM 0x10

typedef struct mr_bathymetry mr_bathymetry;
typedef struct mr_current mr_current;

/* ---- bathymetry ---------------------------------------------------------- */

/* Gridded bathymetry (replaces CartesianNetcdf3, src/bathymetry/
 * cartesian_netcdf3.rs:35-43 and :167-256): f32 axes x[nx], y[ny], f64 depth
 * of depth_len values read with flat index nx*j + i (:465-471).  depth_len
 * may differ from nx*ny exactly as in the reference (lookups past the end
 * become IndexOutOfBounds, i.e. NaN).  nx, ny >= 2 (the reference panics on
 * a one-point axis at its first lookup). */
int mr_bathymetry_grid(size_t nx, size_t ny, const float *x, const float *y,
                       const double *depth, size_t depth_len,
                       mr_bathymetry **out);

/* CartesianNetcdf3::open(path, x_name, y_name, depth_name)
 * (cartesian_netcdf3.rs:167-256): reads a NetCDF-3 file; i8/u8/i16/i32/f32/
 * f64 variables are converted as the reference converts them. */
int mr_bathymetry_open(const char *path, const char *x_name, const char *y_name,
                       const char *depth_name, mr_bathymetry **out);

/* ConstantDepth (src/bathymetry/constant_depth.rs:98-129). */
int mr_bathymetry_constant(float h, mr_bathymetry **out);

/* ConstantSlope (src/bathymetry/constant_slope.rs:28-77). */
int mr_bathymetry_slope(float h0, float x0, float y0, float dhdx, float dhdy,
                        mr_bathymetry **out);

/* ArrayDepth test field (src/bathymetry/array_depth.rs:9-35): n x n values,
 * arr[i*n + j] = array[i][j]. */
int mr_bathymetry_array(size_t n, const float *arr, mr_bathymetry **out);

void mr_bathymetry_destroy(mr_bathymetry *b);

/* ---- current ------------------------------------------------------------- */

/* Gridded current (replaces CartesianCurrent, src/current/
 * cartesian_current.rs:18-27 and :58-213): f64 axes and u, v with flat index
 * nx*j + i (:421-427).  nx, ny >= 2. */
int mr_current_grid(size_t nx, size_t ny, const double *x, const double *y,
                    const double *u, size_t u_len, const double *v,
                    size_t v_len, mr_current **out);

/* CartesianCurrent::open(path, x_name, y_name, u_name, v_name)
 * (cartesian_current.rs:58-213). */
int mr_current_open(const char *path, const char *x_name, const char *y_name,
                    const char *u_name, const char *v_name, mr_current **out);

/* ConstantCurrent (src/current/constant_current.rs:50-108); (0, 0) is the
 * reference's DEFAULT_CURRENT (:41). */
int mr_current_constant(double u, double v, mr_current **out);

void mr_current_destroy(mr_current *c);

/* ---- tracing ------------------------------------------------------------- */

/* Number of RK4 steps: ceil((t_end - t0) / dt) cast as Rust casts to usize
 * (saturating, NaN -> 0).  A trace call needs rows_cap >= this + 1. */
uint64_t mr_num_steps(double t0, double t_end, double dt);

/* ManyRays::new(bathymetry, current, rays).trace_many(t0, t_end, dt)
 * (src/ray.rs:98-127) on the GPU, plain FP64 form.  Host buffers: x0, y0,
 * kx0, ky0 [n]; traj [5][rows_cap][n]; n_rows [n]; status [n].  Synchronous.
 * Page-locked output buffers are written by the kernel directly. */
int mr_trace(const mr_bathymetry *b, const mr_current *c, size_t n,
             const double *x0, const double *y0, const double *kx0,
             const double *ky0, double t0, double t_end, double dt,
             int options, size_t rows_cap, double *traj, int32_t *n_rows,
             uint8_t *status);

/* Same, all buffers in device memory; asynchronous on `stream` (a
 * cudaStream_t; NULL = the calling thread's default stream).  One kernel
 * launch, no allocation. */
int mr_trace_device(const mr_bathymetry *b, const mr_current *c, size_t n,
                    const double *x0, const double *y0, const double *kx0,
                    const double *ky0, double t0, double t_end, double dt,
                    int options, size_t rows_cap, double *traj,
                    int32_t *n_rows, uint8_t *status, void *stream);

/* SingleRay::trace_individual(0, duration, step_size) as returned by the
 * extension's single_ray (src/ffi.rs:25-49): rows[rows_cap][5] of
 * (t, x, y, kx, ky) tuples, *n_rows of them valid. */
int mr_single_ray(const mr_bathymetry *b, const mr_current *c, double x0,
                  double y0, double kx0, double ky0, double duration,
                  double step_size, size_t rows_cap, double *rows,
                  int32_t *n_rows);

/* _mantaray.single_ray(x0, y0, kx0, ky0, duration, step_size, bathymetry,
 * current) (src/ffi.rs:25-49): opens the two NetCDF-3 files with the
 * reference's fixed variable names (x, y, depth; x, y, u, v). */
int mr_single_ray_files(const char *bathymetry_path, const char *current_path,
                        double x0, double y0, double kx0, double ky0,
                        double duration, double step_size, size_t rows_cap,
                        double *rows, int32_t *n_rows);

/* _mantaray.ray_tracing(x0, y0, kx0, ky0, duration, step_size, bathymetry,
 * current) (src/ffi.rs:51-85), traj layout as mr_trace. */
int mr_ray_tracing_files(const char *bathymetry_path, const char *current_path,
                         size_t n, const double *x0, const double *y0,
                         const double *kx0, const double *ky0,
                         double duration, double step_size, size_t rows_cap,
                         double *traj, int32_t *n_rows, uint8_t *status);

/* ---- batched FP32 form ------------------------------------------------------
 * ManyRays::trace_many (src/ray.rs:98-127) for millions of rays from many
 * sources over several (bathymetry, current) scenarios, in single precision:
 * the same ray equations, step and cell-gradient rule as the plain form, with
 * FP32 right-hand side and interpolation, positions held as FP32 offsets from
 * per-ray FP64 origins, and Kahan-compensated accumulation.  One persistent
 * kernel; rays that end (grid exit, dry cell) are replaced from a device work
 * queue.  Results: the state every `decimation` steps (f32) and the last
 * valid state of each ray (f64).  All array arguments are device pointers.
 * Calls on one mr_batch must not overlap on the GPU (they share its work
 * queue). */
typedef struct mr_batch mr_batch;
typedef struct mr_batch_graph mr_batch_graph;

/* Launch shape of the persistent kernel. */
typedef struct mr_batch_config {
  int block;           /* threads per block: a multiple of 32 in [32, 256] */
  int blocks_per_sm;   /* blocks per SM of the persistent grid; with one ray per
                          lane, more than the kernel's register-hungry build
                          holds selects its 72-register build (same results) */
  int rays_per_lane;   /* 1 or 2 rays interleaved per thread */
  int rebase_interval; /* steps between FP64 origin rebases */
  int order;           /* 1: sort the rays by starting cell and direction before
                          tracing, so a warp's rays share cell records (results
                          per ray are unchanged); 0: trace in index order */
  int staging;         /* where a ray entering a new cell gets the cell's records
                          (results per ray are the same for every choice):
                          MR_STAGING_NONE from global memory;
                          MR_STAGING_TILE from the warp's 8 x 8-cell tile in
                          shared memory, loaded by the tensor memory
                          accelerator and moved to where most of its rays are
                          (one scenario with its current gridded on the
                          bathymetry's grid only);
                          MR_STAGING_AHEAD from the lane's slot of shared
                          memory, into which the records of the cell the ray
                          is heading into are copied (cp.async) a step ahead
                          (every scenario's current gridded on its
                          bathymetry's grid).
                          Other combinations: MR_ERR_INVALID_ARGUMENT.  One ray
                          per lane. */
  int sweep_steps;     /* 0: each ray is traced to its end in one launch.  > 0:
                          the call runs in sweeps of at most sweep_steps steps
                          per ray (ceil(max_steps / sweep_steps) launches);
                          between two sweeps the rays still running are sorted
                          again by where they are (2 x 2-cell blocks), so that
                          the rays a GPU runs at once stay in one part of the
                          field and share its cell records in L2 (results per
                          ray are the same).  Needs order = 1, one ray per
                          lane and MR_STAGING_NONE; the running rays' states,
                          list and sort keys take 76 bytes per ray of scratch,
                          grown on demand by direct calls and owned by each
                          graph. */
} mr_batch_config;

#define MR_STAGING_NONE 0
#define MR_STAGING_TILE 1
#define MR_STAGING_AHEAD 2

/* Per-ray status of the batched form. */
#define MR_BATCH_COMPLETE 0       /* max_steps steps taken */
#define MR_BATCH_OUT_OF_DOMAIN 1  /* a stage left the grid (reference: NaN stop) */
#define MR_BATCH_DRY 2            /* depth <= 0 (reference: NaN group velocity) */
#define MR_BATCH_BAD_WAVENUMBER 3 /* k <= 0 or non-finite */

int mr_batch_default_config(mr_batch_config *cfg);

/* Packs n_scenarios (bathymetry, current) pairs into FP32 cell records on
 * the fields' device.  Bathymetry must be gridded with ascending, evenly
 * spaced axes; the current gridded or constant. */
int mr_batch_create(size_t n_scenarios, const mr_bathymetry *const *bathy,
                    const mr_current *const *current, mr_batch **out);
void mr_batch_destroy(mr_batch *b);

/* Traces n rays from t0 with step dt for at most max_steps steps.
 * ray_scenario [n] (null: all scenario 0); x0, y0, kx0, ky0 [n];
 * saved [5][save_cap][n] f32 (t, x, y, kx, ky) every `decimation` steps, step
 * 0 included (decimation 0: no rows; rows a ray does not reach are NaN);
 * end_state [5][n] f64; n_steps, n_saved [n]; status [n].  Inputs are device
 * memory; outputs device memory or page-locked host memory, which the kernel
 * writes in place (the decimated rows then reach the host while it runs). */
int mr_batch_trace_device(mr_batch *b, size_t n, const uint8_t *ray_scenario,
                          const double *x0, const double *y0, const double *kx0,
                          const double *ky0, double t0, double dt,
                          int64_t max_steps, int64_t decimation, size_t save_cap,
                          float *saved, double *end_state, int32_t *n_steps,
                          int32_t *n_saved, uint8_t *status,
                          const mr_batch_config *cfg, void *stream);

/* The same call captured once in a CUDA graph over buffers sized for n_max
 * rays (saved is [5][save_cap][n_max], end_state [5][n_max]); each launch
 * replays it for the first n <= n_max rays of those buffers. */
int mr_batch_graph_create(mr_batch *b, size_t n_max, const uint8_t *ray_scenario,
                          const double *x0, const double *y0, const double *kx0,
                          const double *ky0, double t0, double dt,
                          int64_t max_steps, int64_t decimation, size_t save_cap,
                          float *saved, double *end_state, int32_t *n_steps,
                          int32_t *n_saved, uint8_t *status,
                          const mr_batch_config *cfg, mr_batch_graph **out);
int mr_batch_graph_launch(mr_batch_graph *g, size_t n, void *stream);
void mr_batch_graph_destroy(mr_batch_graph *g);

/* mr_batch_trace_device without any device allocation.  No counterpart in
 * the reference.  For callers that cannot call cudaMalloc when they trace
 * (device memory owned by another runtime's pool, or a loop that must not
 * allocate): the kernel's scratch -- its work-queue head and this call's copy
 * of the scenario table -- lives in a static 16 KiB device array that every
 * GPU loading the library keeps until exit, instead of in memory the library
 * allocates.  Limit: at most MR_BATCH_STATIC_MAX_SCENARIOS scenarios
 * (MR_ERR_CAPACITY beyond).  The first call on a device looks up the array's
 * device address; make that first call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race, so serialise them.
 * Arguments and results as mr_batch_trace_device. */
#define MR_BATCH_STATIC_MAX_SCENARIOS 64
int mr_batch_trace_device_static(mr_batch *b, size_t n, const uint8_t *ray_scenario,
                                 const double *x0, const double *y0, const double *kx0,
                                 const double *ky0, double t0, double dt,
                                 int64_t max_steps, int64_t decimation, size_t save_cap,
                                 float *saved, double *end_state, int32_t *n_steps,
                                 int32_t *n_saved, uint8_t *status,
                                 const mr_batch_config *cfg, void *stream);

/* ---- differentiation form --------------------------------------------------
 * Gradients of any function of the rays' end states with respect to the
 * initial states (x, y, kx, ky) and every node of the depth, u and v grids:
 * a hand-written discrete adjoint of the RK4 stepper (ode_solvers 0.4.0 as
 * called at src/ray.rs:207-208) over the reference's equations
 * (src/wave_ray_path.rs:118-216), with the grid lookups in the working
 * precision and no f32 casts (the reference's casts make the map a staircase
 * below any finite-difference step).  The forward pass stores every
 * `checkpoint_every`-th state; the adjoint pass recomputes each segment from
 * its checkpoint.  mr_diff_tangent is the forward-mode (tangent-linear)
 * derivative of the same map, for checking.  precision: 64 (double arrays)
 * or 32 (float arrays; node gradients are still accumulated in double).
 * Fields are row-major [ny][nx] on regular grids; all arrays are device
 * memory; calls are asynchronous on `stream`. */
typedef struct mr_diff_grid {
  size_t nx, ny;   /* points per axis, >= 2 */
  double x0, y0;   /* first axis values */
  double dx, dy;   /* spacing, > 0 */
} mr_diff_grid;

/* End states [4][n] (x, y, kx, ky) after `steps` steps of dt; status[i] = 1
 * (and NaN) for rays that left the grids or met depth <= 0.  checkpoints:
 * [ceil(steps / checkpoint_every)][4][n]. */
int mr_diff_forward(int precision, const mr_diff_grid *bgrid, const void *depth,
                    const mr_diff_grid *cgrid, const void *u, const void *v,
                    size_t n, const void *x0, const void *y0, const void *kx0,
                    const void *ky0, double dt, int64_t steps,
                    int64_t checkpoint_every, void *checkpoints, void *end_state,
                    uint8_t *status, void *stream);

/* Given grad_end [4][n] = dL/d(end state), writes grad_state0 [4][n] =
 * dL/d(initial state) and sets grad_depth [bny*bnx], grad_u, grad_v
 * [cny*cnx] (f64) to dL/d(node).  Rays with status != 0 contribute nothing.
 * segment: scratch [checkpoint_every][16][n] (every step's four RK4 stage
 * states). */
int mr_diff_backward(int precision, const mr_diff_grid *bgrid, const void *depth,
                     const mr_diff_grid *cgrid, const void *u, const void *v,
                     size_t n, const void *x0, const void *y0, const void *kx0,
                     const void *ky0, double dt, int64_t steps,
                     int64_t checkpoint_every, const void *checkpoints,
                     const uint8_t *status, const void *grad_end, void *segment,
                     void *grad_state0, double *grad_depth, double *grad_u,
                     double *grad_v, void *stream);

/* Directional derivative of the end states along dstate0 [4][n] and the
 * node perturbations d_depth, d_u, d_v (each may be null): d_end [4][n]. */
int mr_diff_tangent(int precision, const mr_diff_grid *bgrid, const void *depth,
                    const mr_diff_grid *cgrid, const void *u, const void *v,
                    size_t n, const void *x0, const void *y0, const void *kx0,
                    const void *ky0, const void *dstate0, const void *d_depth,
                    const void *d_u, const void *d_v, double dt, int64_t steps,
                    void *end_state, void *d_end, uint8_t *status, void *stream);

/* ---- initial states on the device -------------------------------------------
 * The reference's notebooks build initial states on the host: a launch point
 * or a start line, directions, and |k| from the period by the dispersion
 * relation (notebooks/canonical_examples/utils.py:11-26,
 * notebooks/agulhas/notebook/src.py:60-82).  These write them straight into
 * device arrays for the batched form.  Ray r gets direction
 * theta0 + (theta1 - theta0) * u and period period0 + (period1 - period0) * v
 * with u, v in [0, 1) from SplitMix64 of (seed, r) (u evenly spaced,
 * (j + 0.5) / count, with MR_SEED_EVEN_DIRECTIONS); |k| solves
 * (2 pi / T)^2 = g k tanh(k h), g = 9.8, by Newton iteration in FP64 at the
 * depth h the bathymetry handle's lookup gives at the launch point (NaN
 * states where there is none).  Device arrays; asynchronous on `stream`. */
#define MR_SEED_EVEN_DIRECTIONS 0x1

/* n_sources points (sx, sy: device arrays), rays_per_source rays each, ray
 * r = s * rays_per_source + j; outputs [n_sources * rays_per_source]. */
int mr_seed_point_sources(const mr_bathymetry *b, size_t n_sources, const double *sx,
                          const double *sy, size_t rays_per_source, double theta0,
                          double theta1, double period0, double period1, uint64_t seed,
                          int flags, double *x0, double *y0, double *kx0, double *ky0,
                          void *stream);

/* n rays evenly spaced from (xa, ya) to (xb, yb) (numpy.linspace points). */
int mr_seed_line(const mr_bathymetry *b, double xa, double ya, double xb, double yb, size_t n,
                 double theta0, double theta1, double period0, double period1, uint64_t seed,
                 int flags, double *x0, double *y0, double *kx0, double *ky0, void *stream);

/* ---- NetCDF-3 access (host only, no GPU) ---------------------------------- */

/* Reads variable `name` of a NetCDF-3 file converted to f64 (the reference's
 * `as f64` conversions).  Writes min(len, cap) values; *len = its length;
 * *nc_type = its NetCDF type code (1 byte, 2 char/u8, 3 short, 4 int,
 * 5 float, 6 double). */
int mr_netcdf3_read_f64(const char *path, const char *name, double *out,
                        size_t cap, size_t *len, int *nc_type);

/* ---- diagnostics ----------------------------------------------------------- */

/* Message of the last failing call on this thread ("" if none). */
const char *mr_last_error(void);

/* Measured FMA throughput of the current device in TFLOP/s (fp64 != 0: the
 * FP64 pipe, else FP32), from a chain-of-FMA kernel on every SM.  The
 * roofline denominator for the compute-bound integrators.  No counterpart in
 * the reference (measurement only). */
int mr_measure_fma_peak(int fp64, double *tflops);

/* Library version, major*10000 + minor*100 + patch. */
int mr_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MANTARAY_GPU_H */
