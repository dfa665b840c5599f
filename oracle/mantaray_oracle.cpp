// mantaray_oracle.cpp -- CPU restatement of the reference ray-integration
// path.  TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never part of
// the product library.  Build: oracle/Makefile (g++ -O3 -ffp-contract=off
// -fopenmp).  Citations are path:line inside mines-oceanography/mantaray.
//
// Floating-point contract: every expression keeps the reference's operand
// order and precision.  f32 arithmetic stays in f32 (no promotion: the file
// is compiled without -ffast-math, FLT_EVAL_METHOD is 0 on x86_64 and
// aarch64), no contraction into FMA, glibc libm for the transcendental
// functions.

#include "mantaray_oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double G = 9.8;  // src/wave_ray_path.rs:23

// Rust `v as usize` for floats: saturating, NaN -> 0 (Rust >= 1.45).
inline uint64_t as_usize(double v) {
  if (!(v > 0.0)) return 0;
  if (v >= 18446744073709551616.0) return UINT64_MAX;
  return static_cast<uint64_t>(v);
}
inline uint64_t as_usize(float v) { return as_usize(static_cast<double>(v)); }

// Rust f32::fract / f64::fract: self - self.trunc().
inline float fract(float v) { return v - std::trunc(v); }
inline double fract(double v) { return v - std::trunc(v); }

enum BathyKind { B_GRID = 0, B_CONST = 1, B_SLOPE = 2, B_ARRAY = 3 };
enum CurrentKind { C_GRID = 0, C_CONST = 1 };

}  // namespace

struct or_bathy {
  int kind;
  std::vector<float> x, y;     // grid axes (f32, cartesian_netcdf3.rs:37-39)
  std::vector<double> depth;   // grid depth (f64, cartesian_netcdf3.rs:42)
  float h;                     // constant depth
  float h0, x0, y0, dhdx, dhdy;  // constant slope
  size_t an;                   // array depth: n x n
  std::vector<float> arr;
};

struct or_current {
  int kind;
  std::vector<double> x, y, u, v;  // cartesian_current.rs:18-27
  double cu, cv;                   // constant current
};

namespace {

// interpolator::bilinear, src/interpolator.rs:39-84 (f32 throughout).
int bilinear(const float p[4][3], float tx, float ty, float *out) {
  // src/interpolator.rs:46-50: a target coincident with a corner returns it.
  for (int i = 0; i < 4; ++i) {
    if (tx == p[i][0] && ty == p[i][1]) {
      *out = p[i][2];
      return OR_OK;
    }
  }
  const float *a = p[0], *b = p[1], *c = p[2], *d = p[3];
  // :59-61 translate b, d and the target with respect to a.
  const float bt0 = b[0] - a[0], bt1 = b[1] - a[1];
  const float dt0 = d[0] - a[0], dt1 = d[1] - a[1];
  const float tt0 = tx - a[0], tt1 = ty - a[1];
  // :64-67 determinant of the change of basis.
  const float p1 = bt0 * dt1;
  const float p2 = dt0 * bt1;
  const float det = p1 - p2;
  if (det == 0.0f) return OR_INVALID_ARGUMENT;
  // :69-72 inverse change-of-basis matrix.
  const float m00 = dt1 / det;
  const float m01 = -(dt0 / det);
  const float m10 = -(bt1 / det);
  const float m11 = bt0 / det;
  // :74-75 target in the unit square.
  const float q00 = m00 * tt0, q01 = m01 * tt1;
  const float x = q00 + q01;
  const float q10 = m10 * tt0, q11 = m11 * tt1;
  const float y = q10 + q11;
  // :78-83 bilinear form, evaluated left to right.
  const float a00 = a[2];
  const float a10 = b[2] - a[2];
  const float a01 = d[2] - a[2];
  const float a11 = ((c[2] - a[2]) - a10) - a01;
  const float r1 = a10 * x;
  const float r2 = a01 * y;
  const float r3 = (a11 * x) * y;
  *out = ((a00 + r1) + r2) + r3;
  return OR_OK;
}

// nearest, src/bathymetry/cartesian_netcdf3.rs:274-296 and
// src/current/cartesian_current.rs:231-253 (same rule in f32 / f64).
template <typename T>
int nearest(T target, const T *arr, size_t n, T *out) {
  if (n == 0) return OR_INDEX_OUT_OF_BOUNDS;
  if (n == 1) {
    *out = T(0);
    return OR_OK;
  }
  const T spacing = std::fabs(arr[1] - arr[0]);
  const T index = (target - arr[0]) / spacing;
  if (index < T(0) || index > static_cast<T>(n - 1)) return OR_INDEX_OUT_OF_BOUNDS;
  *out = index;
  return OR_OK;
}

// Edge / on-grid / interior corner rule of four_corners,
// cartesian_netcdf3.rs:343-387 and cartesian_current.rs:292-336.
template <typename T>
void corner_pair(T idx, size_t n, uint64_t *lo, uint64_t *hi) {
  const T low = T(0);
  const T high = static_cast<T>(n - 1);
  if (idx == low) {
    *lo = as_usize(idx);
    *hi = as_usize(idx) + 1;
  } else if (idx == high) {
    *lo = as_usize(idx) - 1;
    *hi = as_usize(idx);
  } else if (fract(idx) == T(0)) {
    *lo = as_usize(std::round(idx));
    *hi = *lo + 1;
  } else {
    *lo = as_usize(std::floor(idx));
    *hi = as_usize(std::ceil(idx));
  }
}

template <typename T>
int four_corners(T x, T y, const T *ax, size_t nx, const T *ay, size_t ny,
                 uint64_t out[8]) {
  T xi, yi;
  int e = nearest(x, ax, nx, &xi);
  if (e) return e;
  e = nearest(y, ay, ny, &yi);
  if (e) return e;
  uint64_t x1, x2, y1, y2;
  corner_pair(xi, nx, &x1, &x2);
  corner_pair(yi, ny, &y1, &y2);
  // vec![(x1, y1), (x1, y2), (x2, y2), (x2, y1)]
  out[0] = x1; out[1] = y1;
  out[2] = x1; out[3] = y2;
  out[4] = x2; out[5] = y2;
  out[6] = x2; out[7] = y1;
  return OR_OK;
}

// depth_at_indexes, cartesian_netcdf3.rs:465-471 (and val_from_arr,
// cartesian_current.rs:421-427): flat index nx*j + i checked against the
// array length.
inline int flat_value(const std::vector<double> &arr, size_t nx, uint64_t i,
                      uint64_t j, double *out) {
  const uint64_t idx = static_cast<uint64_t>(nx) * j + i;
  if (idx >= arr.size()) return OR_INDEX_OUT_OF_BOUNDS;
  *out = arr[idx];
  return OR_OK;
}

// CartesianNetcdf3::depth_and_gradient, cartesian_netcdf3.rs:98-135.
int grid_depth_and_gradient(const or_bathy *b, float x, float y, float out[3]) {
  if (std::isnan(x) || std::isnan(y)) {
    out[0] = out[1] = out[2] = std::numeric_limits<float>::quiet_NaN();
    return OR_OK;
  }
  const size_t nx = b->x.size(), ny = b->y.size();
  uint64_t c[8];
  int e = four_corners<float>(x, y, b->x.data(), nx, b->y.data(), ny, c);
  if (e) return e;
  // interpolate, :417-445: corner depths cast to f32.
  float pts[4][3];
  for (int i = 0; i < 4; ++i) {
    double d;
    e = flat_value(b->depth, nx, c[2 * i], c[2 * i + 1], &d);
    if (e) return e;
    pts[i][0] = b->x[c[2 * i]];
    pts[i][1] = b->y[c[2 * i + 1]];
    pts[i][2] = static_cast<float>(d);
  }
  float depth;
  e = bilinear(pts, x, y, &depth);
  if (e) return e;
  // :119-132 cell forward differences in f64: sw = corner 0, nw = corner 1,
  // se = corner 3.
  const double x_space = static_cast<double>(b->x[1]) - static_cast<double>(b->x[0]);
  const double y_space = static_cast<double>(b->y[1]) - static_cast<double>(b->y[0]);
  double d_se, d_sw, d_nw;
  if ((e = flat_value(b->depth, nx, c[6], c[7], &d_se))) return e;
  if ((e = flat_value(b->depth, nx, c[0], c[1], &d_sw))) return e;
  if ((e = flat_value(b->depth, nx, c[2], c[3], &d_nw))) return e;
  const double xg = (d_se - d_sw) / x_space;
  const double yg = (d_nw - d_sw) / y_space;
  out[0] = depth;
  out[1] = static_cast<float>(xg);
  out[2] = static_cast<float>(yg);
  return OR_OK;
}

int depth_and_gradient(const or_bathy *b, float x, float y, float out[3]) {
  const float nan = std::numeric_limits<float>::quiet_NaN();
  switch (b->kind) {
    case B_GRID:
      return grid_depth_and_gradient(b, x, y, out);
    case B_CONST:  // constant_depth.rs:122-128
      if (std::isnan(x) || std::isnan(y)) {
        out[0] = out[1] = out[2] = nan;
      } else {
        out[0] = b->h; out[1] = 0.0f; out[2] = 0.0f;
      }
      return OR_OK;
    case B_SLOPE:  // constant_slope.rs:67-76, f32
      if (std::isnan(x) || std::isnan(y)) {
        out[0] = out[1] = out[2] = nan;
      } else {
        const float t1 = b->dhdx * (x - b->x0);
        const float t2 = b->dhdy * (y - b->y0);
        out[0] = (b->h0 + t1) + t2;
        out[1] = b->dhdx;
        out[2] = b->dhdy;
      }
      return OR_OK;
    case B_ARRAY: {  // array_depth.rs:68-75 (`as usize` saturates, NaN -> 0)
      const uint64_t i = as_usize(x), j = as_usize(y);
      if (i >= b->an || j >= b->an) {
        out[0] = out[1] = out[2] = nan;
      } else {
        out[0] = b->arr[i * b->an + j]; out[1] = 0.0f; out[2] = 0.0f;
      }
      return OR_OK;
    }
  }
  return OR_INVALID_ARGUMENT;
}

// CartesianCurrent::current_and_gradient, cartesian_current.rs:487-542.
int grid_current_and_gradient(const or_current *c, double x, double y,
                              double out[6]) {
  const size_t nx = c->x.size(), ny = c->y.size();
  uint64_t k[8];
  int e = four_corners<double>(x, y, c->x.data(), nx, c->y.data(), ny, k);
  if (e) return e;
  const float tx = static_cast<float>(x), ty = static_cast<float>(y);
  // interpolate, :365-398: coordinates and values cast to f32.
  float res[2];
  const std::vector<double> *fields[2] = {&c->u, &c->v};
  for (int f = 0; f < 2; ++f) {
    float pts[4][3];
    for (int i = 0; i < 4; ++i) {
      double val;
      e = flat_value(*fields[f], nx, k[2 * i], k[2 * i + 1], &val);
      if (e) return e;
      pts[i][0] = static_cast<float>(c->x[k[2 * i]]);
      pts[i][1] = static_cast<float>(c->y[k[2 * i + 1]]);
      pts[i][2] = static_cast<float>(val);
    }
    e = bilinear(pts, tx, ty, &res[f]);
    if (e) return e;
  }
  // :515-536 cell forward differences in f64.
  const double x_space = c->x[1] - c->x[0];
  const double y_space = c->y[1] - c->y[0];
  double u_se, u_sw, u_nw, v_se, v_sw, v_nw;
  if ((e = flat_value(c->u, nx, k[6], k[7], &u_se))) return e;
  if ((e = flat_value(c->u, nx, k[0], k[1], &u_sw))) return e;
  if ((e = flat_value(c->u, nx, k[2], k[3], &u_nw))) return e;
  if ((e = flat_value(c->v, nx, k[6], k[7], &v_se))) return e;
  if ((e = flat_value(c->v, nx, k[0], k[1], &v_sw))) return e;
  if ((e = flat_value(c->v, nx, k[2], k[3], &v_nw))) return e;
  out[0] = static_cast<double>(res[0]);
  out[1] = static_cast<double>(res[1]);
  out[2] = (u_se - u_sw) / x_space;  // du/dx
  out[3] = (u_nw - u_sw) / y_space;  // du/dy
  out[4] = (v_se - v_sw) / x_space;  // dv/dx
  out[5] = (v_nw - v_sw) / y_space;  // dv/dy
  return OR_OK;
}

int current_and_gradient(const or_current *c, double x, double y, double out[6]) {
  if (c->kind == C_GRID) return grid_current_and_gradient(c, x, y, out);
  // constant_current.rs:100-108
  out[0] = c->cu; out[1] = c->cv;
  out[2] = out[3] = out[4] = out[5] = 0.0;
  return OR_OK;
}

// WaveRayPath::group_velocity, src/wave_ray_path.rs:177-188.
int group_velocity(double k, double h, double *out) {
  if (h <= 0.0) {
    *out = std::numeric_limits<double>::quiet_NaN();
    return OR_OK;
  }
  if (k <= 0.0) return OR_ARGUMENT_OUT_OF_BOUNDS;
  const double kh = k * h;
  const double ch = std::cosh(kh);
  const double th = std::tanh(kh);
  const double num = th + kh / (ch * ch);  // .powi(2) is x * x
  const double den = std::sqrt((k * G) * th);
  *out = (G / 2.0) * (num / den);
  return OR_OK;
}

// WaveRayPath::dkdt_bathy, src/wave_ray_path.rs:207-216, left to right.
void dkdt_bathy(double k, double h, double dhdx, double dhdy, double out[2]) {
  const double kh = k * h;
  const double s = std::sinh(kh);
  const double c = std::cosh(kh);
  const double r = std::sqrt((G * k) * std::tanh(kh));
  const double f = (((((-0.5) * k) * 1.0) / s) * 1.0) / c;
  out[0] = (f * r) * dhdx;
  out[1] = (f * r) * dhdy;
}

// WaveRayPath::odes, src/wave_ray_path.rs:118-150.
int odes(const or_bathy *b, const or_current *c, double x, double y, double kx,
         double ky, double out[4]) {
  float hg[3];
  int e = depth_and_gradient(b, static_cast<float>(x), static_cast<float>(y), hg);
  if (e) return e;
  const double h = static_cast<double>(hg[0]);
  const double dhdx = static_cast<double>(hg[1]);
  const double dhdy = static_cast<double>(hg[2]);
  double cur[6];
  e = current_and_gradient(c, x, y, cur);
  if (e) return e;
  const double k = std::sqrt(kx * kx + ky * ky);
  const double theta = std::atan2(ky, kx);
  double cg;
  e = group_velocity(k, h, &cg);
  if (e) return e;
  const double cgx = cg * std::cos(theta) + cur[0];
  const double cgy = cg * std::sin(theta) + cur[1];
  double dkb[2];
  dkdt_bathy(k, h, dhdx, dhdy, dkb);
  // du = (du/dx, du/dy), dv = (dv/dx, dv/dy)
  out[0] = cgx;
  out[1] = cgy;
  out[2] = (dkb[0] - kx * cur[2]) - ky * cur[4];
  out[3] = (dkb[1] - kx * cur[3]) - ky * cur[5];
  return OR_OK;
}

// impl System for WaveRayPath::system, src/wave_ray_path.rs:220-234:
// any error becomes an all-NaN derivative.
inline void system(const or_bathy *b, const or_current *c, const double s[4],
                   double ds[4]) {
  if (odes(b, c, s[0], s[1], s[2], s[3], ds) != OR_OK) {
    ds[0] = ds[1] = ds[2] = ds[3] = std::numeric_limits<double>::quiet_NaN();
  }
}

// solout, src/wave_ray_path.rs:236-246.
inline bool all_nan(const double v[4]) {
  return std::isnan(v[0]) && std::isnan(v[1]) && std::isnan(v[2]) && std::isnan(v[3]);
}

// One classical RK4 step (ode_solvers 0.4.0 Rk4::step, textbook scheme):
// k1 = f(y); k2 = f(y + k1*h/2); k3 = f(y + k2*h/2); k4 = f(y + k3*h);
// y' = y + (k1 + k2*2 + k3*2 + k4) * (h/6), each vector op elementwise.
inline void rk4_step(const or_bathy *b, const or_current *c, const double y[4],
                     const double k1[4], double half, double dt, double yn[4]) {
  double k2[4], k3[4], k4[4], tmp[4];
  for (int i = 0; i < 4; ++i) tmp[i] = y[i] + k1[i] * half;
  system(b, c, tmp, k2);
  for (int i = 0; i < 4; ++i) tmp[i] = y[i] + k2[i] * half;
  system(b, c, tmp, k3);
  for (int i = 0; i < 4; ++i) tmp[i] = y[i] + k3[i] * dt;
  system(b, c, tmp, k4);
  const double sixth = dt / 6.0;
  for (int i = 0; i < 4; ++i) {
    const double acc = ((k1[i] + k2[i] * 2.0) + k3[i] * 2.0) + k4[i];
    yn[i] = y[i] + acc * sixth;
  }
}

// Rk4::integrate (ode_solvers 0.4.0) for one ray, as called from
// SingleRay::trace_individual (src/ray.rs:198-213).  `emit(row, t, y)` stores
// a row.  Returns rows recorded; *stopped tells whether solout ended it.
template <typename Emit>
uint64_t integrate(const or_bathy *b, const or_current *c, const double y0[4],
                   double t0, uint64_t nsteps, double dt, int stop_rule,
                   Emit emit, bool *stopped) {
  double y[4] = {y0[0], y0[1], y0[2], y0[3]};
  double t = t0;
  const double half = dt / 2.0;
  emit(0, t, y);
  uint64_t rows = 1;
  *stopped = false;
  double k1[4];
  system(b, c, y, k1);
  for (uint64_t s = 0; s < nsteps; ++s) {
    double yn[4];
    rk4_step(b, c, y, k1, half, dt, yn);
    t = t + dt;
    emit(rows, t, yn);
    ++rows;
    for (int i = 0; i < 4; ++i) y[i] = yn[i];
    double fresh[4];
    system(b, c, y, fresh);  // next step's first stage (system ignores t)
    const double *dy = (stop_rule == OR_STOP_FRESH) ? fresh : k1;
    if (all_nan(dy) || all_nan(y)) {
      *stopped = true;
      break;
    }
    for (int i = 0; i < 4; ++i) k1[i] = fresh[i];
  }
  return rows;
}

}  // namespace

extern "C" {

or_bathy *or_bathy_grid(size_t nx, size_t ny, const float *x, const float *y,
                        const double *depth, size_t depth_len) {
  or_bathy *b = new (std::nothrow) or_bathy();
  if (!b) return nullptr;
  b->kind = B_GRID;
  b->x.assign(x, x + nx);
  b->y.assign(y, y + ny);
  b->depth.assign(depth, depth + depth_len);
  return b;
}

or_bathy *or_bathy_constant(float h) {
  or_bathy *b = new (std::nothrow) or_bathy();
  if (!b) return nullptr;
  b->kind = B_CONST;
  b->h = h;
  return b;
}

or_bathy *or_bathy_slope(float h0, float x0, float y0, float dhdx, float dhdy) {
  or_bathy *b = new (std::nothrow) or_bathy();
  if (!b) return nullptr;
  b->kind = B_SLOPE;
  b->h0 = h0; b->x0 = x0; b->y0 = y0; b->dhdx = dhdx; b->dhdy = dhdy;
  return b;
}

or_bathy *or_bathy_array(size_t n, const float *arr) {
  or_bathy *b = new (std::nothrow) or_bathy();
  if (!b) return nullptr;
  b->kind = B_ARRAY;
  b->an = n;
  b->arr.assign(arr, arr + n * n);
  return b;
}

void or_bathy_free(or_bathy *b) { delete b; }

or_current *or_current_grid(size_t nx, size_t ny, const double *x,
                            const double *y, const double *u, size_t u_len,
                            const double *v, size_t v_len) {
  or_current *c = new (std::nothrow) or_current();
  if (!c) return nullptr;
  c->kind = C_GRID;
  c->x.assign(x, x + nx);
  c->y.assign(y, y + ny);
  c->u.assign(u, u + u_len);
  c->v.assign(v, v + v_len);
  return c;
}

or_current *or_current_constant(double u, double v) {
  or_current *c = new (std::nothrow) or_current();
  if (!c) return nullptr;
  c->kind = C_CONST;
  c->cu = u; c->cv = v;
  return c;
}

void or_current_free(or_current *c) { delete c; }

int or_bilinear(const float pts[12], float tx, float ty, float *out) {
  float p[4][3];
  std::memcpy(p, pts, sizeof(p));
  return bilinear(p, tx, ty, out);
}

int or_nearest_f32(float target, const float *arr, size_t n, float *out) {
  return nearest<float>(target, arr, n, out);
}

int or_nearest_f64(double target, const double *arr, size_t n, double *out) {
  return nearest<double>(target, arr, n, out);
}

int or_bathy_four_corners(const or_bathy *b, float x, float y, uint64_t out[8]) {
  return four_corners<float>(x, y, b->x.data(), b->x.size(), b->y.data(),
                             b->y.size(), out);
}

int or_current_four_corners(const or_current *c, double x, double y,
                            uint64_t out[8]) {
  return four_corners<double>(x, y, c->x.data(), c->x.size(), c->y.data(),
                              c->y.size(), out);
}

int or_depth_and_gradient(const or_bathy *b, float x, float y, float out[3]) {
  return depth_and_gradient(b, x, y, out);
}

int or_current_and_gradient(const or_current *c, double x, double y,
                            double out[6]) {
  return current_and_gradient(c, x, y, out);
}

int or_group_velocity(double k, double h, double *out) {
  return group_velocity(k, h, out);
}

void or_dkdt_bathy(double k, double h, double dhdx, double dhdy, double out[2]) {
  dkdt_bathy(k, h, dhdx, dhdy, out);
}

int or_odes(const or_bathy *b, const or_current *c, double x, double y,
            double kx, double ky, double out[4]) {
  return odes(b, c, x, y, kx, ky, out);
}

uint64_t or_num_steps(double t0, double t_end, double dt) {
  return as_usize(std::ceil((t_end - t0) / dt));
}

int or_trace(const or_bathy *b, const or_current *c, size_t n,
             const double *x0, const double *y0, const double *kx0,
             const double *ky0, double t0, double t_end, double dt,
             int stop_rule, size_t rows_cap, double *traj, int32_t *n_rows,
             uint8_t *status, int threads) {
  const uint64_t nsteps = or_num_steps(t0, t_end, dt);
  if (nsteps >= rows_cap) return -1;
  const size_t plane = rows_cap * n;
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
  for (long long r = 0; r < static_cast<long long>(n); ++r) {
    const size_t i = static_cast<size_t>(r);
    const double s0[4] = {x0[i], y0[i], kx0[i], ky0[i]};
    auto emit = [&](uint64_t row, double t, const double *y) {
      double *base = traj + row * n + i;
      base[0] = t;
      base[plane] = y[0];
      base[2 * plane] = y[1];
      base[3 * plane] = y[2];
      base[4 * plane] = y[3];
    };
    bool stopped = false;
    const uint64_t rows = integrate(b, c, s0, t0, nsteps, dt, stop_rule, emit, &stopped);
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (uint64_t row = rows; row < rows_cap; ++row) {
      double *base = traj + row * n + i;
      for (int v = 0; v < 5; ++v) base[v * plane] = nan;
    }
    n_rows[i] = static_cast<int32_t>(rows);
    status[i] = stopped ? OR_RAY_STOPPED : OR_RAY_COMPLETE;
  }
  (void)threads;
  return 0;
}

int or_trace_final(const or_bathy *b, const or_current *c, size_t n,
                   const double *x0, const double *y0, const double *kx0,
                   const double *ky0, double t0, double t_end, double dt,
                   int stop_rule, double *final_state, int32_t *n_rows,
                   uint8_t *status, int threads) {
  const uint64_t nsteps = or_num_steps(t0, t_end, dt);
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 8) num_threads(threads)
#endif
  for (long long r = 0; r < static_cast<long long>(n); ++r) {
    const size_t i = static_cast<size_t>(r);
    const double s0[4] = {x0[i], y0[i], kx0[i], ky0[i]};
    double last[5] = {0, 0, 0, 0, 0};
    auto emit = [&](uint64_t, double t, const double *y) {
      last[0] = t; last[1] = y[0]; last[2] = y[1]; last[3] = y[2]; last[4] = y[3];
    };
    bool stopped = false;
    const uint64_t rows = integrate(b, c, s0, t0, nsteps, dt, stop_rule, emit, &stopped);
    for (int v = 0; v < 5; ++v) final_state[v * n + i] = last[v];
    n_rows[i] = static_cast<int32_t>(rows);
    status[i] = stopped ? OR_RAY_STOPPED : OR_RAY_COMPLETE;
  }
  (void)threads;
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// The differentiation model: the reference's equations with the grid lookups
// in f64 (no f32 casts), which makes the step map smooth inside each cell
// (the f32 casts of the reference make it a staircase at the ulp level, below
// any finite-difference step).  Same corner rule as the reference
// (idx in [0, n-1], the last cell for idx == n-1), f64 bilinear, f64 cell
// forward differences, and the reference's RHS expressions.  This is the
// function the GPU adjoint and tangent-linear kernels differentiate; it is
// here so finite differences of it can check them.

namespace {

struct Grid64 {
  const double *v0, *v1;  // one or two fields on the grid
  size_t nx, ny;
  double x0, y0, dx, dy;
};

// Cell (i, j) and in-cell fractions of (x, y); false outside the grid.
bool cell64(const Grid64 &g, double x, double y, size_t *i, size_t *j, double *fx, double *fy) {
  const double ix = (x - g.x0) / g.dx, iy = (y - g.y0) / g.dy;
  if (!(ix >= 0.0 && ix <= static_cast<double>(g.nx - 1) && iy >= 0.0 &&
        iy <= static_cast<double>(g.ny - 1)))
    return false;
  double fi = std::floor(ix), fj = std::floor(iy);
  if (fi > static_cast<double>(g.nx - 2)) fi = static_cast<double>(g.nx - 2);
  if (fj > static_cast<double>(g.ny - 2)) fj = static_cast<double>(g.ny - 2);
  *i = static_cast<size_t>(fi);
  *j = static_cast<size_t>(fj);
  *fx = ix - fi;
  *fy = iy - fj;
  return true;
}

inline double bilin64(const double *a, size_t nx, size_t i, size_t j, double fx, double fy,
                      double *ddx, double *ddy) {
  const double v00 = a[nx * j + i], v10 = a[nx * j + i + 1];
  const double v01 = a[nx * (j + 1) + i], v11 = a[nx * (j + 1) + i + 1];
  *ddx = v10 - v00;  // forward differences (divided by the spacing by the caller)
  *ddy = v01 - v00;
  return ((v00 + (v10 - v00) * fx) + (v01 - v00) * fy) + (((v11 - v10) - v01) + v00) * fx * fy;
}

int odes_f64interp(const Grid64 &bg, const Grid64 &cg, double x, double y, double kx, double ky,
                   double out[4]) {
  size_t i, j;
  double fx, fy, gx, gy;
  if (!cell64(bg, x, y, &i, &j, &fx, &fy)) return OR_INDEX_OUT_OF_BOUNDS;
  const double h = bilin64(bg.v0, bg.nx, i, j, fx, fy, &gx, &gy);
  const double hx = gx / bg.dx, hy = gy / bg.dy;
  if (!cell64(cg, x, y, &i, &j, &fx, &fy)) return OR_INDEX_OUT_OF_BOUNDS;
  double ux, uy, vx, vy;
  const double u = bilin64(cg.v0, cg.nx, i, j, fx, fy, &ux, &uy);
  const double v = bilin64(cg.v1, cg.nx, i, j, fx, fy, &vx, &vy);
  ux /= cg.dx; uy /= cg.dy; vx /= cg.dx; vy /= cg.dy;
  const double k = std::sqrt(kx * kx + ky * ky);
  double cgv;
  int e = group_velocity(k, h, &cgv);
  if (e) return e;
  double dkb[2];
  dkdt_bathy(k, h, hx, hy, dkb);
  out[0] = cgv * (kx / k) + u;
  out[1] = cgv * (ky / k) + v;
  out[2] = (dkb[0] - kx * ux) - ky * vx;
  out[3] = (dkb[1] - kx * uy) - ky * vy;
  return OR_OK;
}

}  // namespace

extern "C" {

int or_diff_end_states(const double *depth, size_t bnx, size_t bny, double bx0, double by0,
                       double bdx, double bdy, const double *u, const double *v, size_t cnx,
                       size_t cny, double cx0, double cy0, double cdx, double cdy, size_t n,
                       const double *x0, const double *y0, const double *kx0, const double *ky0,
                       double dt, uint64_t steps, double *end_state, uint8_t *status,
                       int threads) {
  if (bnx < 2 || bny < 2 || cnx < 2 || cny < 2) return -1;
  const Grid64 bg{depth, nullptr, bnx, bny, bx0, by0, bdx, bdy};
  const Grid64 cg{u, v, cnx, cny, cx0, cy0, cdx, cdy};
#ifdef _OPENMP
  if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
  for (long long r = 0; r < static_cast<long long>(n); ++r) {
    const size_t i = static_cast<size_t>(r);
    double y[4] = {x0[i], y0[i], kx0[i], ky0[i]};
    const double half = dt / 2.0, sixth = dt / 6.0;
    bool ok = true;
    auto f = [&](const double *s, double *d) {
      if (odes_f64interp(bg, cg, s[0], s[1], s[2], s[3], d) != OR_OK) {
        d[0] = d[1] = d[2] = d[3] = std::numeric_limits<double>::quiet_NaN();
      }
    };
    for (uint64_t st = 0; st < steps && ok; ++st) {
      double k1[4], k2[4], k3[4], k4[4], tmp[4];
      f(y, k1);
      for (int q = 0; q < 4; ++q) tmp[q] = y[q] + k1[q] * half;
      f(tmp, k2);
      for (int q = 0; q < 4; ++q) tmp[q] = y[q] + k2[q] * half;
      f(tmp, k3);
      for (int q = 0; q < 4; ++q) tmp[q] = y[q] + k3[q] * dt;
      f(tmp, k4);
      for (int q = 0; q < 4; ++q) y[q] = y[q] + (((k1[q] + k2[q] * 2.0) + k3[q] * 2.0) + k4[q]) * sixth;
      if (std::isnan(y[0]) || std::isnan(y[1]) || std::isnan(y[2]) || std::isnan(y[3])) ok = false;
    }
    for (int q = 0; q < 4; ++q) end_state[q * n + i] = ok ? y[q] : std::numeric_limits<double>::quiet_NaN();
    status[i] = ok ? OR_RAY_COMPLETE : OR_RAY_STOPPED;
  }
  (void)threads;
  return 0;
}

}  // extern "C"
