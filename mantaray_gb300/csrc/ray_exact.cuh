// ray_exact.cuh -- the reference's ray equations on the GPU, operation for
// operation.
//
// Used by the plain FP64 kernel.  The translation unit that includes it is
// compiled with -fmad=false (no a*b+c contraction, as Rust compiles the
// reference) and IEEE division/sqrt (nvcc defaults without fast math).  f32
// work stays f32, f64 work stays f64, casts are round-to-nearest, exactly as
// in the reference.  Transcendentals (tanh, cosh, sinh, atan2, cos, sin) are
// CUDA's; they can differ from glibc's by an ulp, which is the only source of
// difference from the CPU oracle.
#pragma once

#include <math.h>
#include <stdint.h>

#include "fields.h"

namespace mr {

constexpr double kG = 9.8;  // src/wave_ray_path.rs:23

// Rust `v as usize`: saturating, NaN -> 0.
__device__ __forceinline__ uint64_t as_usize(float v) {
  if (!(v > 0.0f)) return 0ull;
  if (v >= 18446744073709551616.0f) return ~0ull;
  return static_cast<uint64_t>(v);
}
__device__ __forceinline__ uint64_t as_usize(double v) {
  if (!(v > 0.0)) return 0ull;
  if (v >= 18446744073709551616.0) return ~0ull;
  return static_cast<uint64_t>(v);
}
__device__ __forceinline__ float rfract(float v) { return v - truncf(v); }
__device__ __forceinline__ double rfract(double v) { return v - trunc(v); }
__device__ __forceinline__ float rround(float v) { return roundf(v); }
__device__ __forceinline__ double rround(double v) { return round(v); }
__device__ __forceinline__ float rfloor(float v) { return floorf(v); }
__device__ __forceinline__ double rfloor(double v) { return floor(v); }
__device__ __forceinline__ float rceil(float v) { return ceilf(v); }
__device__ __forceinline__ double rceil(double v) { return ceil(v); }

// interpolator::bilinear, src/interpolator.rs:39-84.  Corners in the order
// [(x1,y1), (x1,y2), (x2,y2), (x2,y1)] given as px/py/pv.
__device__ __forceinline__ int bilinear_exact(const float px[4], const float py[4],
                                              const float pv[4], float tx, float ty,
                                              float *out) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (tx == px[i] && ty == py[i]) {  // :46-50 coincident corner
      *out = pv[i];
      return RHS_OK;
    }
  }
  const float bt0 = px[1] - px[0], bt1 = py[1] - py[0];
  const float dt0 = px[3] - px[0], dt1 = py[3] - py[0];
  const float tt0 = tx - px[0], tt1 = ty - py[0];
  const float det = bt0 * dt1 - dt0 * bt1;  // :64
  if (det == 0.0f) return RHS_INVALID_ARGUMENT;
  const float m00 = dt1 / det;
  const float m01 = -(dt0 / det);
  const float m10 = -(bt1 / det);
  const float m11 = bt0 / det;
  const float x = m00 * tt0 + m01 * tt1;  // :74
  const float y = m10 * tt0 + m11 * tt1;  // :75
  const float a00 = pv[0];
  const float a10 = pv[1] - pv[0];
  const float a01 = pv[3] - pv[0];
  const float a11 = pv[2] - pv[0] - a10 - a01;
  *out = a00 + a10 * x + a01 * y + a11 * x * y;  // :83, left to right
  return RHS_OK;
}

// nearest + the edge/on-grid/interior corner rule (cartesian_netcdf3.rs:274-390
// in f32, cartesian_current.rs:231-339 in f64).  a0/sp/high are the host
// precomputed a[0], |a[1]-a[0]| and (n-1) as T.
template <typename T>
__device__ __forceinline__ int corner_pair(T target, T a0, T sp, T high, uint64_t n,
                                           uint64_t *lo, uint64_t *hi) {
  T idx;
  if (n == 1) {
    idx = T(0);
  } else {
    idx = (target - a0) / sp;
    if (idx < T(0) || idx > high) return RHS_INDEX_OUT_OF_BOUNDS;
  }
  if (idx == T(0)) {
    *lo = as_usize(idx);
    *hi = *lo + 1;
  } else if (idx == high) {
    *lo = as_usize(idx) - 1;
    *hi = as_usize(idx);
  } else if (rfract(idx) == T(0)) {
    *lo = as_usize(rround(idx));
    *hi = *lo + 1;
  } else {
    *lo = as_usize(rfloor(idx));
    *hi = as_usize(rceil(idx));
  }
  return RHS_OK;
}

__device__ __forceinline__ int flat_value(const double *arr, uint64_t len, uint64_t nx,
                                          uint64_t i, uint64_t j, double *out) {
  const uint64_t idx = nx * j + i;
  if (idx >= len) return RHS_INDEX_OUT_OF_BOUNDS;
  *out = __ldg(arr + idx);
  return RHS_OK;
}

// BathymetryData::depth_and_gradient for every kind.  out = (h, dh/dx, dh/dy).
__device__ __forceinline__ int depth_and_gradient_exact(const BathyDev &b, float x, float y,
                                                        float out[3]) {
  const float nan = __int_as_float(0x7fffffff);
  if (b.kind == BATHY_GRID) {
    // cartesian_netcdf3.rs:98-135
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = nan;
      return RHS_OK;
    }
    uint64_t x1, x2, y1, y2;
    int e = corner_pair<float>(x, b.x0, b.xsp, b.xhigh, b.nx, &x1, &x2);
    if (e) return e;
    e = corner_pair<float>(y, b.y0, b.ysp, b.yhigh, b.ny, &y1, &y2);
    if (e) return e;
    // The axis arrays are indexed like the reference's Vec (x1, x2 < nx
    // whenever nx >= 2, which the handle constructor enforces).
    double d_sw, d_nw, d_ne, d_se;
    if ((e = flat_value(b.depth, b.depth_len, b.nx, x1, y1, &d_sw))) return e;
    if ((e = flat_value(b.depth, b.depth_len, b.nx, x1, y2, &d_nw))) return e;
    if ((e = flat_value(b.depth, b.depth_len, b.nx, x2, y2, &d_ne))) return e;
    if ((e = flat_value(b.depth, b.depth_len, b.nx, x2, y1, &d_se))) return e;
    const float ax1 = __ldg(b.x + x1), ax2 = __ldg(b.x + x2);
    const float ay1 = __ldg(b.y + y1), ay2 = __ldg(b.y + y2);
    const float px[4] = {ax1, ax1, ax2, ax2};
    const float py[4] = {ay1, ay2, ay2, ay1};
    const float pv[4] = {__double2float_rn(d_sw), __double2float_rn(d_nw),
                         __double2float_rn(d_ne), __double2float_rn(d_se)};
    float depth;
    e = bilinear_exact(px, py, pv, x, y, &depth);
    if (e) return e;
    const double xg = (d_se - d_sw) / b.xspace;  // :126-128
    const double yg = (d_nw - d_sw) / b.yspace;  // :130-132
    out[0] = depth;
    out[1] = __double2float_rn(xg);
    out[2] = __double2float_rn(yg);
    return RHS_OK;
  }
  if (b.kind == BATHY_CONSTANT) {
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = nan;
    } else {
      out[0] = b.h; out[1] = 0.0f; out[2] = 0.0f;
    }
    return RHS_OK;
  }
  if (b.kind == BATHY_SLOPE) {
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = nan;
    } else {
      out[0] = b.s_h0 + b.s_dhdx * (x - b.s_x0) + b.s_dhdy * (y - b.s_y0);
      out[1] = b.s_dhdx;
      out[2] = b.s_dhdy;
    }
    return RHS_OK;
  }
  // BATHY_ARRAY
  const uint64_t i = as_usize(x), j = as_usize(y);
  if (i >= b.an || j >= b.an) {
    out[0] = out[1] = out[2] = nan;
  } else {
    out[0] = __ldg(b.arr + i * b.an + j); out[1] = 0.0f; out[2] = 0.0f;
  }
  return RHS_OK;
}

// CurrentData::current_and_gradient.  out = (u, v, du/dx, du/dy, dv/dx, dv/dy).
__device__ __forceinline__ int current_and_gradient_exact(const CurrentDev &c, double x,
                                                          double y, double out[6]) {
  if (c.kind == CURRENT_CONSTANT) {
    out[0] = c.cu; out[1] = c.cv;
    out[2] = out[3] = out[4] = out[5] = 0.0;
    return RHS_OK;
  }
  // cartesian_current.rs:487-542
  uint64_t x1, x2, y1, y2;
  int e = corner_pair<double>(x, c.x0, c.xsp, c.xhigh, c.nx, &x1, &x2);
  if (e) return e;
  e = corner_pair<double>(y, c.y0, c.ysp, c.yhigh, c.ny, &y1, &y2);
  if (e) return e;
  double u_sw, u_nw, u_ne, u_se, v_sw, v_nw, v_ne, v_se;
  if ((e = flat_value(c.u, c.u_len, c.nx, x1, y1, &u_sw))) return e;
  if ((e = flat_value(c.u, c.u_len, c.nx, x1, y2, &u_nw))) return e;
  if ((e = flat_value(c.u, c.u_len, c.nx, x2, y2, &u_ne))) return e;
  if ((e = flat_value(c.u, c.u_len, c.nx, x2, y1, &u_se))) return e;
  if ((e = flat_value(c.v, c.v_len, c.nx, x1, y1, &v_sw))) return e;
  if ((e = flat_value(c.v, c.v_len, c.nx, x1, y2, &v_nw))) return e;
  if ((e = flat_value(c.v, c.v_len, c.nx, x2, y2, &v_ne))) return e;
  if ((e = flat_value(c.v, c.v_len, c.nx, x2, y1, &v_se))) return e;
  const float ax1 = __double2float_rn(__ldg(c.x + x1)), ax2 = __double2float_rn(__ldg(c.x + x2));
  const float ay1 = __double2float_rn(__ldg(c.y + y1)), ay2 = __double2float_rn(__ldg(c.y + y2));
  const float px[4] = {ax1, ax1, ax2, ax2};
  const float py[4] = {ay1, ay2, ay2, ay1};
  const float tx = __double2float_rn(x), ty = __double2float_rn(y);
  const float pu[4] = {__double2float_rn(u_sw), __double2float_rn(u_nw),
                       __double2float_rn(u_ne), __double2float_rn(u_se)};
  const float pv[4] = {__double2float_rn(v_sw), __double2float_rn(v_nw),
                       __double2float_rn(v_ne), __double2float_rn(v_se)};
  float u, v;
  if ((e = bilinear_exact(px, py, pu, tx, ty, &u))) return e;
  if ((e = bilinear_exact(px, py, pv, tx, ty, &v))) return e;
  out[0] = static_cast<double>(u);
  out[1] = static_cast<double>(v);
  out[2] = (u_se - u_sw) / c.xspace;
  out[3] = (u_nw - u_sw) / c.yspace;
  out[4] = (v_se - v_sw) / c.xspace;
  out[5] = (v_nw - v_sw) / c.yspace;
  return RHS_OK;
}

// WaveRayPath::odes (src/wave_ray_path.rs:118-150) with group_velocity
// (:177-188) and dkdt_bathy (:207-216) inlined in the reference's order.
__device__ __forceinline__ int odes_exact(const BathyDev &b, const CurrentDev &c, double x,
                                          double y, double kx, double ky, double out[4]) {
  float hg[3];
  int e = depth_and_gradient_exact(b, __double2float_rn(x), __double2float_rn(y), hg);
  if (e) return e;
  const double h = static_cast<double>(hg[0]);
  const double dhdx = static_cast<double>(hg[1]);
  const double dhdy = static_cast<double>(hg[2]);
  double cur[6];
  e = current_and_gradient_exact(c, x, y, cur);
  if (e) return e;
  const double k = sqrt(kx * kx + ky * ky);
  const double theta = atan2(ky, kx);
  double cg;
  if (h <= 0.0) {
    cg = __longlong_as_double(0x7ff8000000000000ll);
  } else {
    if (k <= 0.0) return RHS_ARGUMENT_OUT_OF_BOUNDS;
    const double kh = k * h;
    const double ch = cosh(kh);
    const double th = tanh(kh);
    cg = (kG / 2.0) * ((th + kh / (ch * ch)) / sqrt(k * kG * th));
  }
  const double cgx = cg * cos(theta) + cur[0];
  const double cgy = cg * sin(theta) + cur[1];
  const double kh = k * h;
  const double f = (-0.5) * k * 1.0 / sinh(kh) * 1.0 / cosh(kh) * sqrt(kG * k * tanh(kh));
  out[0] = cgx;
  out[1] = cgy;
  out[2] = f * dhdx - kx * cur[2] - ky * cur[4];
  out[3] = f * dhdy - kx * cur[3] - ky * cur[5];
  return RHS_OK;
}

// impl System::system (src/wave_ray_path.rs:220-234): errors become NaN.
__device__ __forceinline__ void system_exact(const BathyDev &b, const CurrentDev &c,
                                             const double s[4], double ds[4]) {
  if (odes_exact(b, c, s[0], s[1], s[2], s[3], ds) != RHS_OK) {
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    ds[0] = ds[1] = ds[2] = ds[3] = nan;
  }
}

__device__ __forceinline__ bool all_nan4(const double v[4]) {
  return isnan(v[0]) && isnan(v[1]) && isnan(v[2]) && isnan(v[3]);
}

}  // namespace mr
