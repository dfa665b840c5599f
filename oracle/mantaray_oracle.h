/*
 * mantaray_oracle.h -- CPU restatement of the reference ray-integration path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * (tests, the smoke check and the CPU baseline leg of the benchmark).  It is
 * never linked into, loaded by, or called from the product library.
 *
 * Every function restates one reference function op for op (same operand
 * order, same f32/f64 casts, no FMA contraction: compiled with
 * -ffp-contract=off against glibc libm, the libm the reference's Rust f64
 * methods call on Linux).  Citations are path:line inside the reference
 * project (mines-oceanography/mantaray).
 *
 * Parity pins: the known-answer values of the reference's own unit tests
 * (src/wave_ray_path.rs:296-626, src/interpolator.rs:86-161,
 * src/bathymetry/cartesian_netcdf3.rs:562-834,
 * src/current/cartesian_current.rs:645-992, python/tests/test_core.py) are
 * ported in tests/test_oracle_golden.py.  The RK4 stepper lives in the
 * un-vendored crate ode_solvers 0.4.0; its textbook scheme is restated here and
 * pinned by the single-step EPSILON tests of src/wave_ray_path.rs:403-548.
 */
#ifndef MANTARAY_ORACLE_H
#define MANTARAY_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error values of src/error.rs:7-37 that the hot path can produce. */
enum {
  OR_OK = 0,
  OR_ARGUMENT_OUT_OF_BOUNDS = 1, /* Error::ArgumentOutOfBounds (k <= 0) */
  OR_INVALID_ARGUMENT = 2,       /* Error::InvalidArgument (bilinear) */
  OR_INDEX_OUT_OF_BOUNDS = 3     /* Error::IndexOutOfBounds */
};

/* Stop rule of the RK4 loop: which derivative `solout` is handed
 * (src/wave_ray_path.rs:236-246).  ode_solvers 0.4.0 is not in the tree, so
 * this is a switch: STAGE1 = the first-stage derivative of the step just
 * taken; FRESH = the derivative re-evaluated at the new state. */
enum { OR_STOP_STAGE1 = 0, OR_STOP_FRESH = 1 };

/* Per-ray status written by or_trace. */
enum { OR_RAY_COMPLETE = 0, OR_RAY_STOPPED = 1 };

typedef struct or_bathy or_bathy;
typedef struct or_current or_current;

/* CartesianNetcdf3 in memory (src/bathymetry/cartesian_netcdf3.rs:35-43):
 * f32 axes, f64 depth, flat index nx*j + i.  depth_len may differ from
 * nx*ny, as in the reference (index checked at :465-471). */
or_bathy *or_bathy_grid(size_t nx, size_t ny, const float *x, const float *y,
                        const double *depth, size_t depth_len);
/* ConstantDepth (src/bathymetry/constant_depth.rs:98-129). */
or_bathy *or_bathy_constant(float h);
/* ConstantSlope (src/bathymetry/constant_slope.rs:28-77). */
or_bathy *or_bathy_slope(float h0, float x0, float y0, float dhdx, float dhdy);
/* ArrayDepth (src/bathymetry/array_depth.rs:9-35): square n x n,
 * arr[i*n + j] = array[i][j] with i the x index. */
or_bathy *or_bathy_array(size_t n, const float *arr);
void or_bathy_free(or_bathy *b);

/* CartesianCurrent in memory (src/current/cartesian_current.rs:18-27). */
or_current *or_current_grid(size_t nx, size_t ny, const double *x,
                            const double *y, const double *u, size_t u_len,
                            const double *v, size_t v_len);
/* ConstantCurrent (src/current/constant_current.rs:50-108). */
or_current *or_current_constant(double u, double v);
void or_current_free(or_current *c);

/* interpolator::bilinear (src/interpolator.rs:39-84).
 * pts = 4 x (x, y, value), target = (tx, ty). */
int or_bilinear(const float pts[12], float tx, float ty, float *out);

/* nearest (cartesian_netcdf3.rs:274-296), f32. */
int or_nearest_f32(float target, const float *arr, size_t n, float *out);
/* nearest (cartesian_current.rs:231-253), f64. */
int or_nearest_f64(double target, const double *arr, size_t n, double *out);

/* four_corners: out = [x1,y1, x1,y2, x2,y2, x2,y1] (as the reference's
 * vec![(x1, y1), (x1, y2), (x2, y2), (x2, y1)]). */
int or_bathy_four_corners(const or_bathy *b, float x, float y, uint64_t out[8]);
int or_current_four_corners(const or_current *c, double x, double y,
                            uint64_t out[8]);

/* depth_and_gradient: out = (h, dh/dx, dh/dy). */
int or_depth_and_gradient(const or_bathy *b, float x, float y, float out[3]);
/* current_and_gradient: out = (u, v, du/dx, du/dy, dv/dx, dv/dy). */
int or_current_and_gradient(const or_current *c, double x, double y,
                            double out[6]);

/* WaveRayPath::group_velocity / dkdt_bathy / odes / system. */
int or_group_velocity(double k, double h, double *out);
void or_dkdt_bathy(double k, double h, double dhdx, double dhdy,
                   double out[2]);
int or_odes(const or_bathy *b, const or_current *c, double x, double y,
            double kx, double ky, double out[4]);

/* Number of RK4 steps ode_solvers takes: ceil((t_end - t0) / dt) cast to
 * usize with Rust's saturating semantics. */
uint64_t or_num_steps(double t0, double t_end, double dt);

/* ManyRays::trace_many (src/ray.rs:98-127) + SingleRay::trace_individual
 * (src/ray.rs:198-213) over n rays, `threads` OpenMP threads (<=0: all).
 * traj is [5][rows_cap][n] f64 (t, x, y, kx, ky), time-major per variable;
 * rows after a ray's last row are NaN.  n_rows[i] = rows recorded (initial
 * state included).  Returns 0, or -1 when rows_cap < num_steps + 1. */
int or_trace(const or_bathy *b, const or_current *c, size_t n,
             const double *x0, const double *y0, const double *kx0,
             const double *ky0, double t0, double t_end, double dt,
             int stop_rule, size_t rows_cap, double *traj, int32_t *n_rows,
             uint8_t *status, int threads);

/* Same integration without storing trajectories: only the final row of each
 * ray (5 x n, t,x,y,kx,ky) and its row count.  Used for timed CPU samples of
 * workloads whose full trajectories would not fit in host memory. */
int or_trace_final(const or_bathy *b, const or_current *c, size_t n,
                   const double *x0, const double *y0, const double *kx0,
                   const double *ky0, double t0, double t_end, double dt,
                   int stop_rule, double *final_state, int32_t *n_rows,
                   uint8_t *status, int threads);

/* The differentiation model (f64 lookups, see the .cpp): end states [4][n]
 * (x, y, kx, ky) after `steps` RK4 steps, NaN with status 1 for rays that
 * met a NaN derivative.  Fields are raw row-major arrays [ny][nx] on grids
 * with origin (x0, y0) and spacing (dx, dy).  Returns 0 or -1. */
int or_diff_end_states(const double *depth, size_t bnx, size_t bny, double bx0,
                       double by0, double bdx, double bdy, const double *u,
                       const double *v, size_t cnx, size_t cny, double cx0,
                       double cy0, double cdx, double cdy, size_t n,
                       const double *x0, const double *y0, const double *kx0,
                       const double *ky0, double dt, uint64_t steps,
                       double *end_state, uint8_t *status, int threads);

#ifdef __cplusplus
}
#endif
#endif
