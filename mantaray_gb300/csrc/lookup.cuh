// lookup.cuh -- field lookups of the reference, bit for bit, on the GPU.
//
// depth_and_gradient (src/bathymetry/cartesian_netcdf3.rs:98-135 and the
// analytic fields) and current_and_gradient
// (src/current/cartesian_current.rs:487-542).  Index arithmetic, corner
// rules, the coincident-corner shortcut and the f32 bilinear form follow the
// reference operation for operation; values and cell gradients come from the
// handle's tables (fields.h), which hold exactly what the reference computes.
// Translation units including this file are compiled with -fmad=false.
#pragma once

#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "fields.h"

namespace mr {

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

__device__ __forceinline__ float f32_nan() { return __int_as_float(0x7fffffff); }
__device__ __forceinline__ double f64_nan() { return __longlong_as_double(0x7ff8000000000000ll); }

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

// interpolator::bilinear for the corner quad the lookups build,
// [(ax1,ay1), (ax1,ay2), (ax2,ay2), (ax2,ay1)], for NV value sets on the same
// corners (depth; or u and v, which then share every step up to the
// normalised coordinates, as they are the same operations on the same
// inputs).  With finite corner coordinates and edges, bt0 = ax1 - ax1 and
// dt1 = ay1 - ay1 are +0, so bt0*dt1 = +0, det = +0 - dt0*bt1, and the
// diagonal of the inverse, +0/det, is +0 for det > 0 and -0 for det < 0
// (det is never NaN there); everything else is the reference's operations in
// its order (src/interpolator.rs:46-83).  Other quads take bilinear_exact.
template <int NV>
__device__ __forceinline__ int bilinear_cell(float ax1, float ax2, float ay1, float ay2,
                                             const float (&pv)[NV][4], float tx, float ty,
                                             float (&out)[NV]) {
  const float px[4] = {ax1, ax1, ax2, ax2};
  const float py[4] = {ay1, ay2, ay2, ay1};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (tx == px[i] && ty == py[i]) {  // :46-50 coincident corner
#pragma unroll
      for (int v = 0; v < NV; ++v) out[v] = pv[v][i];
      return RHS_OK;
    }
  }
  const float bt1 = __fsub_rn(ay2, ay1);
  const float dt0 = __fsub_rn(ax2, ax1);
  if (!(isfinite(ax1) && isfinite(ay1) && isfinite(bt1) && isfinite(dt0))) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int e = bilinear_exact(px, py, pv[v], tx, ty, &out[v]);
      if (e) return e;
    }
    return RHS_OK;
  }
  const float tt0 = __fsub_rn(tx, ax1), tt1 = __fsub_rn(ty, ay1);
  const float det = __fsub_rn(0.0f, __fmul_rn(dt0, bt1));  // :64 with bt0*dt1 = +0
  if (det == 0.0f) return RHS_INVALID_ARGUMENT;
  const float m00 = det > 0.0f ? 0.0f : -0.0f;  // dt1 / det and bt0 / det
  const float m01 = -__fdiv_rn(dt0, det);
  const float m10 = -__fdiv_rn(bt1, det);
  const float x = __fadd_rn(__fmul_rn(m00, tt0), __fmul_rn(m01, tt1));  // :74
  const float y = __fadd_rn(__fmul_rn(m10, tt0), __fmul_rn(m00, tt1));  // :75
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const float a00 = pv[v][0];
    const float a10 = __fsub_rn(pv[v][1], pv[v][0]);
    const float a01 = __fsub_rn(pv[v][3], pv[v][0]);
    const float a11 = __fsub_rn(__fsub_rn(__fsub_rn(pv[v][2], pv[v][0]), a10), a01);
    out[v] = __fadd_rn(__fadd_rn(__fadd_rn(a00, __fmul_rn(a10, x)), __fmul_rn(a01, y)),
                       __fmul_rn(__fmul_rn(a11, x), y));  // :83, left to right
  }
  return RHS_OK;
}

// What bilinear_cell computes from a regular cell alone, kept so that the
// next lookups in the same cell skip the loads and the two divisions: corner
// coordinates, the inverse's entries and each value set's coefficients.
// x1 == kNoCell: empty.
constexpr uint32_t kNoCell = 0xffffffffu;
template <int NV>
struct CellWeights {
  uint32_t x1 = kNoCell, y1 = kNoCell;
  float ax1, ax2, ay1, ay2;
  float m00, m01, m10;
  float a00[NV], a10[NV], a01[NV], a11[NV];
};

// Fills W when bilinear_cell's fast path applies to the corners (finite
// coordinates and edges, det != 0); false otherwise.
template <int NV>
__device__ __forceinline__ bool cell_prepare(float ax1, float ax2, float ay1, float ay2,
                                             const float (&pv)[NV][4], CellWeights<NV> &W) {
  const float bt1 = __fsub_rn(ay2, ay1);
  const float dt0 = __fsub_rn(ax2, ax1);
  if (!(isfinite(ax1) && isfinite(ay1) && isfinite(bt1) && isfinite(dt0))) return false;
  const float det = __fsub_rn(0.0f, __fmul_rn(dt0, bt1));
  if (det == 0.0f) return false;
  W.ax1 = ax1; W.ax2 = ax2; W.ay1 = ay1; W.ay2 = ay2;
  W.m00 = det > 0.0f ? 0.0f : -0.0f;
  W.m01 = -__fdiv_rn(dt0, det);
  W.m10 = -__fdiv_rn(bt1, det);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    W.a00[v] = pv[v][0];
    W.a10[v] = __fsub_rn(pv[v][1], pv[v][0]);
    W.a01[v] = __fsub_rn(pv[v][3], pv[v][0]);
    W.a11[v] = __fsub_rn(__fsub_rn(__fsub_rn(pv[v][2], pv[v][0]), W.a10[v]), W.a01[v]);
  }
  return true;
}

// bilinear_cell from prepared weights, the same operations in the same
// order; false when the target is a corner (the full path returns it).
template <int NV>
__device__ __forceinline__ bool cell_apply(const CellWeights<NV> &W, float tx, float ty,
                                           float (&out)[NV]) {
  if ((tx == W.ax1 || tx == W.ax2) && (ty == W.ay1 || ty == W.ay2)) return false;
  const float tt0 = __fsub_rn(tx, W.ax1), tt1 = __fsub_rn(ty, W.ay1);
  const float x = __fadd_rn(__fmul_rn(W.m00, tt0), __fmul_rn(W.m01, tt1));
  const float y = __fadd_rn(__fmul_rn(W.m10, tt0), __fmul_rn(W.m00, tt1));
#pragma unroll
  for (int v = 0; v < NV; ++v)
    out[v] = __fadd_rn(__fadd_rn(__fadd_rn(W.a00[v], __fmul_rn(W.a10[v], x)),
                                 __fmul_rn(W.a01[v], y)),
                       __fmul_rn(__fmul_rn(W.a11[v], x), y));
  return true;
}

// Lookup caches: NoCache does nothing; LookupCache keeps the cells a lane
// looked up last (bathymetry and current) for the next lookups in them.  On
// a hit the loads and divisions that depend on the cell alone are skipped:
// shorter dependent chains for calls too small to hide them; for large
// calls the FP64 pipe bounds the plain kernel and the extra registers do not
// pay, so the kernel takes NoCache there.
struct NoCache {};
struct LookupCache {
  CellWeights<1> b;
  CellWeights<2> c;
};

// nearest + the edge/on-grid/interior corner rule (cartesian_netcdf3.rs:274-390
// in f32, cartesian_current.rs:231-339 in f64).  a0/sp/high are the host
// precomputed a[0], |a[1]-a[0]| and (n-1) as T; n >= 2.
template <typename T>
__device__ __forceinline__ int corner_pair(T target, T a0, T sp, T high, uint64_t *lo,
                                           uint64_t *hi) {
  const T idx = (target - a0) / sp;
  if (idx < T(0) || idx > high) return RHS_INDEX_OUT_OF_BOUNDS;
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

// corner_pair<double> with the division replaced by a multiplication where
// that provably gives the same answer.  q = (target - a0) * (1/sp) lies within
// two ulps of the reference's idx = (target - a0) / sp.  When q is more than a
// few ulps away from every integer, idx has the same floor, is not an integer,
// and lies on the same side of 0 and of high, so the corner pair follows from
// floor(q) alone; otherwise (grid lines, NaN, infinities) the exact rule runs.
__device__ __forceinline__ int corner_pair_f64(double target, double a0, double sp,
                                               double inv_sp, double high, uint64_t *lo,
                                               uint64_t *hi) {
  const double a = target - a0;
  const double q = a * inv_sp;
  const double n = floor(q);
  const double fr = q - n;  // exact for |q| < 2^52
  const double tol = fabs(q) * 0x1p-48 + 0x1p-1000;
  if (fr > tol && fr < 1.0 - tol) {
    if (n < 0.0 || n >= high) return RHS_INDEX_OUT_OF_BOUNDS;
    *lo = static_cast<uint64_t>(n);
    *hi = *lo + 1;
    return RHS_OK;
  }
  return corner_pair<double>(target, a0, sp, high, lo, hi);
}

// The corner pair of corner_pair<double> from the axis thresholds of
// fields.h, without FP64 arithmetic: with key = order_key(target),
// idx(target) >= j exactly when key >= thr[j], so idx < 0 (key < thr[0]) and
// idx > high (key >= thr[n]) are out of bounds, and otherwise the pair is
// (i, i+1) for the i with thr[i] <= key < thr[i+1], except (high-1, high)
// when idx == high -- the reference's edge, on-grid and interior rules
// (cartesian_current.rs:283-339) all reduce to that.  An f32 estimate of idx
// picks i; it is corrected by up to two cells (the estimate is within a
// small fraction of a cell) and checked.  Returns RHS_OK or
// RHS_INDEX_OUT_OF_BOUNDS, or -1 when the caller must use the exact rule
// (NaN target, estimate not confirmed).
__device__ __forceinline__ int corner_pair_thr(double target, float target32, float a0f,
                                               float inv_spf, const long long *thr,
                                               uint64_t n, uint64_t *lo, uint64_t *hi) {
  const long long bits = __double_as_longlong(target);
  if ((bits & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) return -1;  // NaN
  const long long key = order_key_bits(bits);
  const int high = static_cast<int>(n) - 1;
  if (key < __ldg(thr) || key >= __ldg(thr + n)) return RHS_INDEX_OUT_OF_BOUNDS;
  float g = (target32 - a0f) * inv_spf;
  g = fminf(fmaxf(g, 0.0f), static_cast<float>(high));  // NaN estimate -> 0
  int i = __float2int_rz(g);
  // thr[0] <= key < thr[n]: every step below stays inside 0..high.
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    if (key < __ldg(thr + i))
      --i;
    else if (key >= __ldg(thr + i + 1))
      ++i;
  }
  if (key < __ldg(thr + i) || key >= __ldg(thr + i + 1)) return -1;
  const int c = i < high ? i : high - 1;
  *lo = static_cast<uint64_t>(c);
  *hi = static_cast<uint64_t>(c) + 1;
  return RHS_OK;
}

// BathymetryData::depth_and_gradient for every kind.  out = (h, dh/dx, dh/dy).
template <typename Cache = NoCache>
__device__ __forceinline__ int depth_and_gradient(const BathyDev &b, float x, float y,
                                                  float out[3], Cache *L = nullptr) {
  constexpr bool kCache = std::is_same<Cache, LookupCache>::value;
  if (b.kind == BATHY_GRID) {
    // cartesian_netcdf3.rs:98-135
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = f32_nan();
      return RHS_OK;
    }
    uint64_t x1, x2, y1, y2;
    int e = corner_pair<float>(x, b.x0, b.xsp, b.xhigh, &x1, &x2);
    if (e) return e;
    e = corner_pair<float>(y, b.y0, b.ysp, b.yhigh, &y1, &y2);
    if (e) return e;
    const bool regular = x2 == x1 + 1 && y2 == y1 + 1;
    float depth[1];
    if constexpr (kCache) {
      if (regular && x1 == L->b.x1 && y1 == L->b.y1 && cell_apply<1>(L->b, x, y, depth)) {
        const uint64_t sw = b.nx * y1 + x1;
        out[0] = depth[0];
        out[1] = __ldg(b.gx + sw);
        out[2] = __ldg(b.gy + sw);
        return RHS_OK;
      }
    }
    // depth_at_indexes checks every corner's flat index against the array
    // length (:465-471); the largest of them is nx*y2 + x2.
    uint64_t sw, nw, ne, se;
    if (regular) {
      sw = b.nx * y1 + x1; nw = sw + b.nx; se = sw + 1; ne = nw + 1;
    } else {
      sw = b.nx * y1 + x1; nw = b.nx * y2 + x1; ne = b.nx * y2 + x2; se = b.nx * y1 + x2;
    }
    if (ne >= b.depth_len) return RHS_INDEX_OUT_OF_BOUNDS;
    const float pv[1][4] = {{__ldg(b.depth32 + sw), __ldg(b.depth32 + nw),
                             __ldg(b.depth32 + ne), __ldg(b.depth32 + se)}};
    const float ax1 = __ldg(b.x + x1), ax2 = __ldg(b.x + x2);
    const float ay1 = __ldg(b.y + y1), ay2 = __ldg(b.y + y2);
    e = bilinear_cell<1>(ax1, ax2, ay1, ay2, pv, x, y, depth);
    if (e) return e;
    out[0] = depth[0];
    if (regular) {
      out[1] = __ldg(b.gx + sw);
      out[2] = __ldg(b.gy + sw);
      if constexpr (kCache) {
        if (x1 < kNoCell && y1 < kNoCell && cell_prepare<1>(ax1, ax2, ay1, ay2, pv, L->b)) {
          L->b.x1 = static_cast<uint32_t>(x1);
          L->b.y1 = static_cast<uint32_t>(y1);
        }
      }
    } else {  // degenerate corners (NaN index): the reference's own expression
      const double d_sw = __ldg(b.depth + sw);
      out[1] = __double2float_rn((__ldg(b.depth + se) - d_sw) / b.xspace);
      out[2] = __double2float_rn((__ldg(b.depth + nw) - d_sw) / b.yspace);
    }
    return RHS_OK;
  }
  if (b.kind == BATHY_CONSTANT) {
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = f32_nan();
    } else {
      out[0] = b.h; out[1] = 0.0f; out[2] = 0.0f;
    }
    return RHS_OK;
  }
  if (b.kind == BATHY_SLOPE) {
    if (isnan(x) || isnan(y)) {
      out[0] = out[1] = out[2] = f32_nan();
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
    out[0] = out[1] = out[2] = f32_nan();
  } else {
    out[0] = __ldg(b.arr + i * b.an + j); out[1] = 0.0f; out[2] = 0.0f;
  }
  return RHS_OK;
}

// CurrentData::current_and_gradient.  out = (u, v, du/dx, du/dy, dv/dx, dv/dy).
template <typename Cache = NoCache>
__device__ __forceinline__ int current_and_gradient(const CurrentDev &c, double x, double y,
                                                    double out[6], Cache *L = nullptr) {
  constexpr bool kCache = std::is_same<Cache, LookupCache>::value;
  if (c.kind == CURRENT_CONSTANT) {
    out[0] = c.cu; out[1] = c.cv;
    out[2] = out[3] = out[4] = out[5] = 0.0;
    return RHS_OK;
  }
  // cartesian_current.rs:487-542
  uint64_t x1, x2, y1, y2;
  const float tx = d2f(x), ty = d2f(y);
  int e = -1;
  if (c.xthr) e = corner_pair_thr(x, tx, c.x0f, c.inv_xspf, c.xthr, c.nx, &x1, &x2);
  if (e < 0) e = corner_pair_f64(x, c.x0, c.xsp, c.inv_xsp, c.xhigh, &x1, &x2);
  if (e) return e;
  e = -1;
  if (c.ythr) e = corner_pair_thr(y, ty, c.y0f, c.inv_yspf, c.ythr, c.ny, &y1, &y2);
  if (e < 0) e = corner_pair_f64(y, c.y0, c.ysp, c.inv_ysp, c.yhigh, &y1, &y2);
  if (e) return e;
  const bool regular = x2 == x1 + 1 && y2 == y1 + 1;
  float uv[2];
  if constexpr (kCache) {
    if (regular && x1 == L->c.x1 && y1 == L->c.y1 && cell_apply<2>(L->c, tx, ty, uv)) {
      const uint64_t sw = c.nx * y1 + x1;
      out[0] = f2d(uv[0]);
      out[1] = f2d(uv[1]);
      out[2] = __ldg(c.dudx + sw);
      out[3] = __ldg(c.dudy + sw);
      out[4] = __ldg(c.dvdx + sw);
      out[5] = __ldg(c.dvdy + sw);
      return RHS_OK;
    }
  }
  uint64_t sw, nw, ne, se;
  if (regular) {
    sw = c.nx * y1 + x1; nw = sw + c.nx; se = sw + 1; ne = nw + 1;
  } else {
    sw = c.nx * y1 + x1; nw = c.nx * y2 + x1; ne = c.nx * y2 + x2; se = c.nx * y1 + x2;
  }
  // val_from_arr (:421-427) on u, then v: the largest flat index is ne.
  if (ne >= c.u_len || ne >= c.v_len) return RHS_INDEX_OUT_OF_BOUNDS;
  const float pv[2][4] = {
      {__ldg(c.u32 + sw), __ldg(c.u32 + nw), __ldg(c.u32 + ne), __ldg(c.u32 + se)},
      {__ldg(c.v32 + sw), __ldg(c.v32 + nw), __ldg(c.v32 + ne), __ldg(c.v32 + se)}};
  const float ax1 = __ldg(c.x32 + x1), ax2 = __ldg(c.x32 + x2);
  const float ay1 = __ldg(c.y32 + y1), ay2 = __ldg(c.y32 + y2);
  if ((e = bilinear_cell<2>(ax1, ax2, ay1, ay2, pv, tx, ty, uv))) return e;
  out[0] = f2d(uv[0]);
  out[1] = f2d(uv[1]);
  if (regular) {
    out[2] = __ldg(c.dudx + sw);
    out[3] = __ldg(c.dudy + sw);
    out[4] = __ldg(c.dvdx + sw);
    out[5] = __ldg(c.dvdy + sw);
    if constexpr (kCache) {
      if (x1 < kNoCell && y1 < kNoCell && cell_prepare<2>(ax1, ax2, ay1, ay2, pv, L->c)) {
        L->c.x1 = static_cast<uint32_t>(x1);
        L->c.y1 = static_cast<uint32_t>(y1);
      }
    }
  } else {
    const double u_sw = __ldg(c.u + sw), v_sw = __ldg(c.v + sw);
    out[2] = (__ldg(c.u + se) - u_sw) / c.xspace;
    out[3] = (__ldg(c.u + nw) - u_sw) / c.yspace;
    out[4] = (__ldg(c.v + se) - v_sw) / c.xspace;
    out[5] = (__ldg(c.v + nw) - v_sw) / c.yspace;
  }
  return RHS_OK;
}

}  // namespace mr
