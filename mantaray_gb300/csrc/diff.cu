// diff.cu -- K3 (discrete adjoint) and K4 (tangent-linear) of the RK4 ray
// integrator, with its forward pass (checkpoints every C steps).
//
// The differentiated map is the reference's RK4 step (ode_solvers 0.4.0, as
// restated for the plain form) over the reference's equations
// (src/wave_ray_path.rs:118-216) with the grid lookups in the working
// precision T, without the reference's f32 casts (those make the map a
// staircase at the ulp level, below any finite-difference step): bilinear
// depth / current inside the cell that holds the point (the reference's
// corner rule), and cell-constant forward-difference gradients
// (src/bathymetry/cartesian_netcdf3.rs:119-134,
// src/current/cartesian_current.rs:515-536).  Inside a cell the map is smooth;
// cell-constant gradients jump across cell edges, where it is not
// differentiable.
//
// Right-hand side F(s; D, U, V) with s = (x, y, kx, ky), k = |(kx, ky)|,
// c = kx/k, s_ = ky/k, a = k h, and the group velocity q(k, h) and refraction
// factor f(k, h) = -k sigma / sinh(2a), sigma = sqrt(g k tanh a):
//   F0 = q c + u,  F1 = q s_ + v,
//   F2 = f hx - kx ux - ky vx,  F3 = f hy - kx uy - ky vy.
// Its partial derivatives are written out by hand below (q_k, q_h, f_k, f_h
// from sigma and n(a) = 1 + 2a / sinh(2a), with exp(-2a) forms that stay finite
// in deep water); the tangent-linear step applies them forward (JVP), the
// adjoint step backward (VJP), both through the four RK4 stages.
//
// Adjoint pass per ray: the forward stored the state every C steps; each
// segment is recomputed from its checkpoint into a scratch buffer (every
// step's four stage states) and walked backward, evaluating each stage's
// partials where its transpose is applied.  Gradients with respect to grid nodes are accumulated per ray
// while the ray stays in one cell, then added to the node arrays with FP64
// atomics, aggregated across the lanes of a warp that flush the same cell.
// The per-cell accumulation runs in the working precision; only the
// accumulation onto the node arrays is FP64.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/mantaray_gpu.h"
#include "handles.h"

namespace mr {
namespace {

template <typename T>
struct DGrid {
  const T *a;     // depth (bathymetry) or u (current)
  const T *b;     // v (current), null for bathymetry
  int nx, ny;
  T x0, y0, inv_dx, inv_dy;
};

template <typename T>
struct DiffArgs {
  DGrid<T> bg, cg;
  int same_grid;        // the current on the bathymetry's grid: one cell location serves both
  int64_t n;
  const T *x0, *y0, *kx0, *ky0;
  T dt;
  int64_t steps, ck_every, n_ck;
  T *ckpt;              // [n_ck][4][n]
  T *end_state;         // [4][n]
  uint8_t *status;      // [n]
  // adjoint
  const T *grad_end;    // [4][n]
  T *seg;               // [ck_every][16][n]: y and the stage states Y2, Y3, Y4
  T *grad_state0;       // [4][n]
  double *grad_depth;   // [bny*bnx]
  double *grad_u, *grad_v;  // [cny*cnx]
  // tangent
  const T *dstate0;     // [4][n]
  const T *d_depth, *d_u, *d_v;
  T *d_end;             // [4][n]
};

// Fast math helpers per precision.
__device__ __forceinline__ double t_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float t_expm1(float x) { return expm1f(x); }
__device__ __forceinline__ double t_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float t_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double t_floor(double x) { return floor(x); }
__device__ __forceinline__ float t_floor(float x) { return floorf(x); }

template <typename T>
struct Cell {
  int i, j;
  T fx, fy;
};

// Cell holding (x, y): the reference's corner rule (index in [0, n-1], the
// last cell for index n-1).  False outside the grid or for NaN.
template <typename T>
__device__ __forceinline__ bool locate(const DGrid<T> &g, T x, T y, Cell<T> *c) {
  const T ix = (x - g.x0) * g.inv_dx, iy = (y - g.y0) * g.inv_dy;
  if (!(ix >= T(0) && ix <= T(g.nx - 1) && iy >= T(0) && iy <= T(g.ny - 1))) return false;
  T fi = t_floor(ix), fj = t_floor(iy);
  if (fi > T(g.nx - 2)) fi = T(g.nx - 2);
  if (fj > T(g.ny - 2)) fj = T(g.ny - 2);
  c->i = static_cast<int>(fi);
  c->j = static_cast<int>(fj);
  c->fx = ix - fi;
  c->fy = iy - fj;
  return true;
}

// Bilinear value, its spatial derivatives (already divided by the spacing)
// and the cell forward differences of field `a` in cell c.
template <typename T>
struct Interp {
  T val, dxp, dyp;  // value, d/dx, d/dy of the bilinear surface
  T gx, gy;         // cell forward differences (cell-constant gradient)
};

template <typename T>
__device__ __forceinline__ Interp<T> interp(const T *a, const DGrid<T> &g, const Cell<T> &c) {
  const int64_t base = static_cast<int64_t>(c.j) * g.nx + c.i;
  const T v00 = __ldg(a + base), v10 = __ldg(a + base + 1);
  const T v01 = __ldg(a + base + g.nx), v11 = __ldg(a + base + g.nx + 1);
  const T ex = v10 - v00, ey = v01 - v00, exy = ((v11 - v10) - v01) + v00;
  Interp<T> r;
  r.val = ((v00 + ex * c.fx) + ey * c.fy) + exy * c.fx * c.fy;
  r.dxp = (ex + exy * c.fy) * g.inv_dx;
  r.dyp = (ey + exy * c.fx) * g.inv_dy;
  r.gx = ex * g.inv_dx;
  r.gy = ey * g.inv_dy;
  return r;
}

// Everything the RHS and its derivatives need at one state.
template <typename T>
struct Point {
  Cell<T> cb, cc;
  Interp<T> h, u, v;
  T k, rk, c, s;         // |k|, 1/|k|, kx/k, ky/k
  T q, q_k, q_h;         // group velocity and its partials
  T f, f_k, f_h;         // refraction factor and its partials
};

constexpr double kG = 9.8;

// Evaluates F at s; false when the reference would produce NaN there
// (outside a grid, depth <= 0, k <= 0, non-finite).
template <typename T>
__device__ __forceinline__ bool eval(const DiffArgs<T> &A, const T s[4], Point<T> &P, T F[4]) {
  if (!locate(A.bg, s[0], s[1], &P.cb)) return false;
  if (A.same_grid)
    P.cc = P.cb;
  else if (!locate(A.cg, s[0], s[1], &P.cc))
    return false;
  P.h = interp(A.bg.a, A.bg, P.cb);
  P.u = interp(A.cg.a, A.cg, P.cc);
  P.v = interp(A.cg.b, A.cg, P.cc);
  const T h = P.h.val;
  const T k2 = s[2] * s[2] + s[3] * s[3];
  if (!(h > T(0)) || !(k2 > T(0))) return false;
  const T g = T(kG);
  // one expm1, one reciprocal and two rsqrt: m4 = 1 - exp(-4a) = m2 (2 - m2),
  // w = 1 / m4, and 1/k, 1/sigma from rsqrt (exact identities)
  const T rk = t_rsqrt(k2);
  const T k = k2 * rk;
  P.k = k;
  P.rk = rk;
  P.c = s[2] * rk;
  P.s = s[3] * rk;
  const T a = k * h;
  const T m2 = -t_expm1(T(-2) * a);  // 1 - exp(-2a)
  const T E = T(1) - m2;             // exp(-2a)
  const T p = T(2) - m2;             // 1 + exp(-2a)
  const T m4 = m2 * p;               // 1 - exp(-4a)
  const T w = T(1) / m4;
  const T rp = m2 * w;               // 1 / p
  const T th = m2 * rp;              // tanh(a)
  const T sech2 = T(4) * E * rp * rp;
  const T isinh2 = T(2) * E * w;     // 1/sinh(2a)
  const T coth2 = (T(2) - m4) * w;   // coth(2a)
  const T gkt = g * k * th;
  const T rsig = t_rsqrt(gkt);
  const T sigma = gkt * rsig;
  const T hrsig = T(0.5) * rsig;     // 1 / (2 sigma)
  const T hrk = T(0.5) * rk;         // 1 / (2 k)
  const T nfac = T(1) + T(2) * a * isinh2;
  const T dsig_dk = g * (th + a * sech2) * hrsig;
  const T dsig_dh = g * k * k * sech2 * hrsig;
  const T dn_da = T(2) * isinh2 - T(4) * a * coth2 * isinh2;
  P.q = sigma * hrk * nfac;
  P.q_k = hrk * ((dsig_dk - sigma * rk) * nfac + sigma * dn_da * h);
  P.q_h = hrk * (dsig_dh * nfac + sigma * dn_da * k);
  P.f = -k * sigma * isinh2;
  P.f_k = -sigma * isinh2 - k * dsig_dk * isinh2 + T(2) * k * sigma * h * coth2 * isinh2;
  P.f_h = -k * dsig_dh * isinh2 + T(2) * k * k * sigma * coth2 * isinh2;
  F[0] = P.q * P.c + P.u.val;
  F[1] = P.q * P.s + P.v.val;
  F[2] = P.f * P.h.gx - s[2] * P.u.gx - s[3] * P.v.gx;
  F[3] = P.f * P.h.gy - s[2] * P.u.gy - s[3] * P.v.gy;
  const bool ok = isfinite(F[0]) && isfinite(F[1]) && isfinite(F[2]) && isfinite(F[3]);
  return ok;
}

template <typename T>
__device__ __forceinline__ bool rk4(const DiffArgs<T> &A, T y[4]) {
  Point<T> P;
  T k1[4], k2[4], k3[4], k4[4], t[4];
  const T half = A.dt * T(0.5);
  if (!eval(A, y, P, k1)) return false;
#pragma unroll
  for (int q = 0; q < 4; ++q) t[q] = y[q] + k1[q] * half;
  if (!eval(A, t, P, k2)) return false;
#pragma unroll
  for (int q = 0; q < 4; ++q) t[q] = y[q] + k2[q] * half;
  if (!eval(A, t, P, k3)) return false;
#pragma unroll
  for (int q = 0; q < 4; ++q) t[q] = y[q] + k3[q] * A.dt;
  if (!eval(A, t, P, k4)) return false;
  const T sixth = A.dt / T(6);
#pragma unroll
  for (int q = 0; q < 4; ++q) y[q] = y[q] + (((k1[q] + k2[q] * T(2)) + k3[q] * T(2)) + k4[q]) * sixth;
  return true;
}

// ---------------------------------------------------------------- JVP --

template <typename T>
__device__ __forceinline__ T bilin_d(const T *d, const DGrid<T> &g, const Cell<T> &c, T *dgx,
                                     T *dgy) {
  const int64_t base = static_cast<int64_t>(c.j) * g.nx + c.i;
  const T v00 = __ldg(d + base), v10 = __ldg(d + base + 1);
  const T v01 = __ldg(d + base + g.nx), v11 = __ldg(d + base + g.nx + 1);
  *dgx = (v10 - v00) * g.inv_dx;
  *dgy = (v01 - v00) * g.inv_dy;
  return ((v00 + (v10 - v00) * c.fx) + (v01 - v00) * c.fy) + (((v11 - v10) - v01) + v00) * c.fx * c.fy;
}

// dF for the state tangent ds and the field tangents of A (d_depth, d_u, d_v).
template <typename T>
__device__ __forceinline__ void jvp(const DiffArgs<T> &A, const T s[4], const Point<T> &P,
                                    const T ds[4], T dF[4]) {
  T ddx = 0, ddy = 0, dux = 0, duy = 0, dvx = 0, dvy = 0, dD = 0, dU = 0, dV = 0;
  if (A.d_depth) dD = bilin_d(A.d_depth, A.bg, P.cb, &ddx, &ddy);
  if (A.d_u) dU = bilin_d(A.d_u, A.cg, P.cc, &dux, &duy);
  if (A.d_v) dV = bilin_d(A.d_v, A.cg, P.cc, &dvx, &dvy);
  const T dh = P.h.dxp * ds[0] + P.h.dyp * ds[1] + dD;
  const T du = P.u.dxp * ds[0] + P.u.dyp * ds[1] + dU;
  const T dv = P.v.dxp * ds[0] + P.v.dyp * ds[1] + dV;
  const T dk = P.c * ds[2] + P.s * ds[3];
  const T dc = (P.s * P.s * ds[2] - P.c * P.s * ds[3]) * P.rk;
  const T dsn = (-P.c * P.s * ds[2] + P.c * P.c * ds[3]) * P.rk;
  const T dq = P.q_k * dk + P.q_h * dh;
  const T df = P.f_k * dk + P.f_h * dh;
  dF[0] = dq * P.c + P.q * dc + du;
  dF[1] = dq * P.s + P.q * dsn + dv;
  dF[2] = df * P.h.gx + P.f * ddx - ds[2] * P.u.gx - s[2] * dux - ds[3] * P.v.gx - s[3] * dvx;
  dF[3] = df * P.h.gy + P.f * ddy - ds[2] * P.u.gy - s[2] * duy - ds[3] * P.v.gy - s[3] * dvy;
}

// ---------------------------------------------------------------- VJP --

// Per-ray accumulator of node gradients for one bathymetry cell and one
// current cell, in the working precision; flushed to the FP64 node arrays
// when the ray moves on.
template <typename T>
struct NodeAcc {
  int64_t bkey, ckey;   // flat index of the cells' south-west nodes, -1: empty
  T d[4];               // depth nodes (00, 10, 01, 11)
  T u[4], v[4];
};

// Adds `vals[4]` to nodes (base, base+1, base+nx, base+nx+1) of `arr` in
// FP64, summed first across the active lanes of the warp that flush the same
// base.  Each group's lowest lane (its leader) adds its peers' values in
// ascending lane order; the loop runs once per member of the largest group
// (all active lanes take part in every shuffle, each reading the next member
// of its own group), so lanes flushing distinct cells cost no shuffle at all.
template <typename T>
__device__ __forceinline__ void scatter4(double *arr, int64_t base, int nx, const T vals[4]) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, base);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  const unsigned largest = __reduce_max_sync(active, static_cast<unsigned>(__popc(peers)));
  double v[4] = {double(vals[0]), double(vals[1]), double(vals[2]), double(vals[3])};
  unsigned rest = peers & (peers - 1u);  // the group without its leader
  for (unsigned it = 1; it < largest; ++it) {
    const int src = rest ? __ffs(rest) - 1 : lane;
    rest &= rest - 1u;
    T o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = __shfl_sync(active, vals[q], src);
    if (lane == leader && src != lane) {
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] += double(o[q]);
    }
  }
  if (lane == leader) {
    atomicAdd(arr + base, v[0]);
    atomicAdd(arr + base + 1, v[1]);
    atomicAdd(arr + base + nx, v[2]);
    atomicAdd(arr + base + nx + 1, v[3]);
  }
}

template <typename T>
__device__ __forceinline__ void flush_bathy(const DiffArgs<T> &A, NodeAcc<T> &acc) {
  if (acc.bkey >= 0) scatter4(A.grad_depth, acc.bkey, A.bg.nx, acc.d);
  acc.bkey = -1;
#pragma unroll
  for (int q = 0; q < 4; ++q) acc.d[q] = T(0);
}

template <typename T>
__device__ __forceinline__ void flush_current(const DiffArgs<T> &A, NodeAcc<T> &acc) {
  if (acc.ckey >= 0) {
    scatter4(A.grad_u, acc.ckey, A.cg.nx, acc.u);
    scatter4(A.grad_v, acc.ckey, A.cg.nx, acc.v);
  }
  acc.ckey = -1;
#pragma unroll
  for (int q = 0; q < 4; ++q) acc.u[q] = acc.v[q] = T(0);
}

// r = J(s)^T w, and the node gradients of w . F added to acc.
template <typename T>
__device__ __forceinline__ void vjp(const DiffArgs<T> &A, const T s[4], const Point<T> &P,
                                    const T w[4], T r[4], NodeAcc<T> &acc) {
  const T c = P.c, sn = P.s;
  const T g_h = (w[0] * c + w[1] * sn) * P.q_h + (w[2] * P.h.gx + w[3] * P.h.gy) * P.f_h;
  r[0] = P.h.dxp * g_h + w[0] * P.u.dxp + w[1] * P.v.dxp;
  r[1] = P.h.dyp * g_h + w[0] * P.u.dyp + w[1] * P.v.dyp;
  const T qrk = P.q * P.rk;
  const T cs_k = qrk * c * sn;
  r[2] = w[0] * (P.q_k * c * c + qrk * sn * sn) + w[1] * (P.q_k * c * sn - cs_k) +
         w[2] * (P.f_k * c * P.h.gx - P.u.gx) + w[3] * (P.f_k * c * P.h.gy - P.u.gy);
  r[3] = w[0] * (P.q_k * sn * c - cs_k) + w[1] * (P.q_k * sn * sn + qrk * c * c) +
         w[2] * (P.f_k * sn * P.h.gx - P.v.gx) + w[3] * (P.f_k * sn * P.h.gy - P.v.gy);
  // bathymetry nodes of the cell
  {
    const int64_t key = static_cast<int64_t>(P.cb.j) * A.bg.nx + P.cb.i;
    if (key != acc.bkey) {
      flush_bathy(A, acc);
      acc.bkey = key;
    }
    const T fx = P.cb.fx, fy = P.cb.fy;
    const T hxw = w[2] * P.f * A.bg.inv_dx, hyw = w[3] * P.f * A.bg.inv_dy;
    acc.d[0] += g_h * (T(1) - fx) * (T(1) - fy) - hxw - hyw;
    acc.d[1] += g_h * fx * (T(1) - fy) + hxw;
    acc.d[2] += g_h * (T(1) - fx) * fy + hyw;
    acc.d[3] += g_h * fx * fy;
  }
  // current nodes of the cell
  {
    const int64_t key = static_cast<int64_t>(P.cc.j) * A.cg.nx + P.cc.i;
    if (key != acc.ckey) {
      flush_current(A, acc);
      acc.ckey = key;
    }
    const T fx = P.cc.fx, fy = P.cc.fy;
    const T w00 = (T(1) - fx) * (T(1) - fy), w10 = fx * (T(1) - fy), w01 = (T(1) - fx) * fy,
            w11 = fx * fy;
    const T ix = A.cg.inv_dx, iy = A.cg.inv_dy;
    const T kxw2 = s[2] * w[2] * ix, kxw3 = s[2] * w[3] * iy;
    const T kyw2 = s[3] * w[2] * ix, kyw3 = s[3] * w[3] * iy;
    acc.u[0] += w[0] * w00 + kxw2 + kxw3;
    acc.u[1] += w[0] * w10 - kxw2;
    acc.u[2] += w[0] * w01 - kxw3;
    acc.u[3] += w[0] * w11;
    acc.v[0] += w[1] * w00 + kyw2 + kyw3;
    acc.v[1] += w[1] * w10 - kyw2;
    acc.v[2] += w[1] * w01 - kyw3;
    acc.v[3] += w[1] * w11;
  }
}

// ------------------------------------------------------------- kernels --

template <typename T>
__global__ void __launch_bounds__(64) diff_forward_kernel(DiffArgs<T> A) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  T y[4] = {A.x0[i], A.y0[i], A.kx0[i], A.ky0[i]};
  bool ok = true;
  for (int64_t s = 0; s < A.steps; ++s) {
    if (s % A.ck_every == 0) {
#pragma unroll
      for (int q = 0; q < 4; ++q) A.ckpt[((s / A.ck_every) * 4 + q) * A.n + i] = y[q];
    }
    if (!rk4(A, y)) {
      ok = false;
      break;
    }
  }
  const T nan = T(NAN);
#pragma unroll
  for (int q = 0; q < 4; ++q) A.end_state[q * A.n + i] = ok ? y[q] : nan;
  A.status[i] = ok ? 0 : 1;
}

template <typename T>
__global__ void __launch_bounds__(64) diff_tangent_kernel(DiffArgs<T> A) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  T y[4] = {A.x0[i], A.y0[i], A.kx0[i], A.ky0[i]};
  T dy[4] = {A.dstate0[i], A.dstate0[A.n + i], A.dstate0[2 * A.n + i], A.dstate0[3 * A.n + i]};
  bool ok = true;
  const T half = A.dt * T(0.5), sixth = A.dt / T(6);
  for (int64_t s = 0; s < A.steps && ok; ++s) {
    Point<T> P;
    T k1[4], k2[4], k3[4], k4[4], d1[4], d2[4], d3[4], d4[4], t[4], dt_[4];
    ok = eval(A, y, P, k1);
    if (ok) jvp(A, y, P, dy, d1);
#pragma unroll
    for (int q = 0; q < 4; ++q) { t[q] = y[q] + k1[q] * half; dt_[q] = dy[q] + d1[q] * half; }
    ok = ok && eval(A, t, P, k2);
    if (ok) jvp(A, t, P, dt_, d2);
#pragma unroll
    for (int q = 0; q < 4; ++q) { t[q] = y[q] + k2[q] * half; dt_[q] = dy[q] + d2[q] * half; }
    ok = ok && eval(A, t, P, k3);
    if (ok) jvp(A, t, P, dt_, d3);
#pragma unroll
    for (int q = 0; q < 4; ++q) { t[q] = y[q] + k3[q] * A.dt; dt_[q] = dy[q] + d3[q] * A.dt; }
    ok = ok && eval(A, t, P, k4);
    if (ok) {
      jvp(A, t, P, dt_, d4);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        y[q] = y[q] + (((k1[q] + k2[q] * T(2)) + k3[q] * T(2)) + k4[q]) * sixth;
        dy[q] = dy[q] + (((d1[q] + d2[q] * T(2)) + d3[q] * T(2)) + d4[q]) * sixth;
      }
    }
  }
  const T nan = T(NAN);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    A.end_state[q * A.n + i] = ok ? y[q] : nan;
    A.d_end[q * A.n + i] = ok ? dy[q] : nan;
  }
  A.status[i] = ok ? 0 : 1;
}

// FP32: capped at 96 registers (10 blocks of 64 per SM; measured fastest of
// 8 / 10 / 12); FP64 uses what it needs (242).
template <typename T>
__global__ void __launch_bounds__(64, sizeof(T) == 4 ? 10 : 1) diff_adjoint_kernel(DiffArgs<T> A) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  if (A.status[i] != 0) {  // no gradient through a ray that stopped
#pragma unroll
    for (int q = 0; q < 4; ++q) A.grad_state0[q * A.n + i] = T(0);
    return;
  }
  T lam[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) lam[q] = A.grad_end[q * A.n + i];
  NodeAcc<T> acc;
  acc.bkey = acc.ckey = -1;
#pragma unroll
  for (int q = 0; q < 4; ++q) acc.d[q] = acc.u[q] = acc.v[q] = T(0);
  const T half = A.dt * T(0.5), h = A.dt, sixth = A.dt / T(6);
  for (int64_t seg = A.n_ck - 1; seg >= 0; --seg) {
    const int64_t first = seg * A.ck_every;
    const int64_t last = min(first + A.ck_every, A.steps);  // steps [first, last)
    // recompute the segment from its checkpoint, keeping every step's four
    // stage states (y, Y2, Y3, Y4) in the scratch
    T y[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) y[q] = A.ckpt[(seg * 4 + q) * A.n + i];
    for (int64_t s = first; s < last; ++s) {
      Point<T> P;
      T k1[4], k2[4], k3[4], k4[4], Y2[4], Y3[4], Y4[4];
      eval(A, y, P, k1);
#pragma unroll
      for (int q = 0; q < 4; ++q) Y2[q] = y[q] + k1[q] * half;
      eval(A, Y2, P, k2);
#pragma unroll
      for (int q = 0; q < 4; ++q) Y3[q] = y[q] + k2[q] * half;
      eval(A, Y3, P, k3);
#pragma unroll
      for (int q = 0; q < 4; ++q) Y4[q] = y[q] + k3[q] * h;
      T *row = A.seg + (s - first) * 16 * A.n + i;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        row[q * A.n] = y[q];
        row[(4 + q) * A.n] = Y2[q];
        row[(8 + q) * A.n] = Y3[q];
        row[(12 + q) * A.n] = Y4[q];
      }
      if (s + 1 < last) {
        eval(A, Y4, P, k4);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          y[q] = y[q] + (((k1[q] + k2[q] * T(2)) + k3[q] * T(2)) + k4[q]) * sixth;
      }
    }
    // walk it backward: each stage's partials are evaluated where its
    // transpose is applied (one live Point)
    for (int64_t s = last - 1; s >= first; --s) {
      const T *row = A.seg + (s - first) * 16 * A.n + i;
      Point<T> P;
      T Ys[4], kd[4], w[4], r4[4], r3[4], r2[4], r1[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) Ys[q] = row[(12 + q) * A.n];
      eval(A, Ys, P, kd);
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = lam[q] * (h / T(6));
      vjp(A, Ys, P, w, r4, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) Ys[q] = row[(8 + q) * A.n];
      eval(A, Ys, P, kd);
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = lam[q] * (h / T(3)) + h * r4[q];
      vjp(A, Ys, P, w, r3, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) Ys[q] = row[(4 + q) * A.n];
      eval(A, Ys, P, kd);
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = lam[q] * (h / T(3)) + half * r3[q];
      vjp(A, Ys, P, w, r2, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) Ys[q] = row[q * A.n];
      eval(A, Ys, P, kd);
#pragma unroll
      for (int q = 0; q < 4; ++q) w[q] = lam[q] * (h / T(6)) + half * r2[q];
      vjp(A, Ys, P, w, r1, acc);
#pragma unroll
      for (int q = 0; q < 4; ++q) lam[q] = lam[q] + r1[q] + r2[q] + r3[q] + r4[q];
    }
  }
  flush_bathy(A, acc);
  flush_current(A, acc);
#pragma unroll
  for (int q = 0; q < 4; ++q) A.grad_state0[q * A.n + i] = lam[q];
}

constexpr int kDiffBlock = 64;

template <typename T>
int make_args(const mr_diff_grid *bgrid, const void *depth, const mr_diff_grid *cgrid,
              const void *u, const void *v, size_t n, const void *x0, const void *y0,
              const void *kx0, const void *ky0, double dt, int64_t steps, int64_t ck_every,
              DiffArgs<T> *A) {
  if (!bgrid || !cgrid || !depth || !u || !v)
    return fail(MR_ERR_INVALID_ARGUMENT, "null grid or field");
  if (bgrid->nx < 2 || bgrid->ny < 2 || cgrid->nx < 2 || cgrid->ny < 2 ||
      bgrid->nx > INT32_MAX || bgrid->ny > INT32_MAX || cgrid->nx > INT32_MAX ||
      cgrid->ny > INT32_MAX)
    return fail(MR_ERR_INVALID_ARGUMENT, "grids need 2 to 2^31-1 points per axis");
  if (!(bgrid->dx > 0) || !(bgrid->dy > 0) || !(cgrid->dx > 0) || !(cgrid->dy > 0))
    return fail(MR_ERR_INVALID_ARGUMENT, "grid spacing must be positive");
  if (n > 0 && (!x0 || !y0 || !kx0 || !ky0)) return fail(MR_ERR_INVALID_ARGUMENT, "null rays");
  if (steps < 0 || ck_every < 1 || !(dt > 0.0))
    return fail(MR_ERR_INVALID_ARGUMENT, "steps >= 0, checkpoint_every >= 1, dt > 0 needed");
  *A = DiffArgs<T>{};
  A->bg = DGrid<T>{static_cast<const T *>(depth), nullptr, static_cast<int>(bgrid->nx),
                   static_cast<int>(bgrid->ny), T(bgrid->x0), T(bgrid->y0), T(1.0 / bgrid->dx),
                   T(1.0 / bgrid->dy)};
  A->cg = DGrid<T>{static_cast<const T *>(u), static_cast<const T *>(v), static_cast<int>(cgrid->nx),
                   static_cast<int>(cgrid->ny), T(cgrid->x0), T(cgrid->y0), T(1.0 / cgrid->dx),
                   T(1.0 / cgrid->dy)};
  A->same_grid = bgrid->nx == cgrid->nx && bgrid->ny == cgrid->ny && bgrid->x0 == cgrid->x0 &&
                 bgrid->y0 == cgrid->y0 && bgrid->dx == cgrid->dx && bgrid->dy == cgrid->dy;
  A->n = static_cast<int64_t>(n);
  A->x0 = static_cast<const T *>(x0);
  A->y0 = static_cast<const T *>(y0);
  A->kx0 = static_cast<const T *>(kx0);
  A->ky0 = static_cast<const T *>(ky0);
  A->dt = T(dt);
  A->steps = steps;
  A->ck_every = ck_every;
  A->n_ck = steps == 0 ? 0 : (steps + ck_every - 1) / ck_every;
  return MR_OK;
}

unsigned blocks_for(size_t n) { return static_cast<unsigned>((n + kDiffBlock - 1) / kDiffBlock); }

}  // namespace
}  // namespace mr

using mr::cuda_fail;
using mr::fail;

extern "C" {

int mr_diff_forward(int precision, const mr_diff_grid *bgrid, const void *depth,
                    const mr_diff_grid *cgrid, const void *u, const void *v, size_t n,
                    const void *x0, const void *y0, const void *kx0, const void *ky0, double dt,
                    int64_t steps, int64_t checkpoint_every, void *checkpoints, void *end_state,
                    uint8_t *status, void *stream) {
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  if (n > 0 && (!end_state || !status || (steps > 0 && !checkpoints)))
    return fail(MR_ERR_INVALID_ARGUMENT, "null output");
  if (precision == 64) {
    mr::DiffArgs<double> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps,
                           checkpoint_every, &A);
    if (rc) return rc;
    if (n == 0) return MR_OK;
    A.ckpt = static_cast<double *>(checkpoints);
    A.end_state = static_cast<double *>(end_state);
    A.status = status;
    mr::diff_forward_kernel<double><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else if (precision == 32) {
    mr::DiffArgs<float> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps,
                           checkpoint_every, &A);
    if (rc) return rc;
    if (n == 0) return MR_OK;
    A.ckpt = static_cast<float *>(checkpoints);
    A.end_state = static_cast<float *>(end_state);
    A.status = status;
    mr::diff_forward_kernel<float><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else {
    return fail(MR_ERR_INVALID_ARGUMENT, "precision must be 64 or 32");
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MR_OK : cuda_fail(e, "diff_forward launch");
}

int mr_diff_backward(int precision, const mr_diff_grid *bgrid, const void *depth,
                     const mr_diff_grid *cgrid, const void *u, const void *v, size_t n,
                     const void *x0, const void *y0, const void *kx0, const void *ky0, double dt,
                     int64_t steps, int64_t checkpoint_every, const void *checkpoints,
                     const uint8_t *status, const void *grad_end, void *segment,
                     void *grad_state0, double *grad_depth, double *grad_u, double *grad_v,
                     void *stream) {
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  if (!grad_depth || !grad_u || !grad_v) return fail(MR_ERR_INVALID_ARGUMENT, "null gradient array");
  if (n > 0 && (!status || !grad_end || !grad_state0 || (steps > 0 && (!checkpoints || !segment))))
    return fail(MR_ERR_INVALID_ARGUMENT, "null argument");
  const size_t bnodes = bgrid ? bgrid->nx * bgrid->ny : 0;
  const size_t cnodes = cgrid ? cgrid->nx * cgrid->ny : 0;
  cudaError_t e = cudaSuccess;
  if (precision == 64) {
    mr::DiffArgs<double> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps,
                           checkpoint_every, &A);
    if (rc) return rc;
    A.ckpt = const_cast<double *>(static_cast<const double *>(checkpoints));
    A.status = const_cast<uint8_t *>(status);
    A.grad_end = static_cast<const double *>(grad_end);
    A.seg = static_cast<double *>(segment);
    A.grad_state0 = static_cast<double *>(grad_state0);
    A.grad_depth = grad_depth; A.grad_u = grad_u; A.grad_v = grad_v;
    e = cudaMemsetAsync(grad_depth, 0, bnodes * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_u, 0, cnodes * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_v, 0, cnodes * sizeof(double), s);
    if (e == cudaSuccess && n > 0)
      mr::diff_adjoint_kernel<double><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else if (precision == 32) {
    mr::DiffArgs<float> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps,
                           checkpoint_every, &A);
    if (rc) return rc;
    A.ckpt = const_cast<float *>(static_cast<const float *>(checkpoints));
    A.status = const_cast<uint8_t *>(status);
    A.grad_end = static_cast<const float *>(grad_end);
    A.seg = static_cast<float *>(segment);
    A.grad_state0 = static_cast<float *>(grad_state0);
    A.grad_depth = grad_depth; A.grad_u = grad_u; A.grad_v = grad_v;
    e = cudaMemsetAsync(grad_depth, 0, bnodes * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_u, 0, cnodes * sizeof(double), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(grad_v, 0, cnodes * sizeof(double), s);
    if (e == cudaSuccess && n > 0)
      mr::diff_adjoint_kernel<float><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else {
    return fail(MR_ERR_INVALID_ARGUMENT, "precision must be 64 or 32");
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? MR_OK : cuda_fail(e, "diff_adjoint launch");
}

int mr_diff_tangent(int precision, const mr_diff_grid *bgrid, const void *depth,
                    const mr_diff_grid *cgrid, const void *u, const void *v, size_t n,
                    const void *x0, const void *y0, const void *kx0, const void *ky0,
                    const void *dstate0, const void *d_depth, const void *d_u, const void *d_v,
                    double dt, int64_t steps, void *end_state, void *d_end, uint8_t *status,
                    void *stream) {
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  if (n > 0 && (!dstate0 || !end_state || !d_end || !status))
    return fail(MR_ERR_INVALID_ARGUMENT, "null argument");
  if (precision == 64) {
    mr::DiffArgs<double> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps, 1, &A);
    if (rc) return rc;
    if (n == 0) return MR_OK;
    A.dstate0 = static_cast<const double *>(dstate0);
    A.d_depth = static_cast<const double *>(d_depth);
    A.d_u = static_cast<const double *>(d_u);
    A.d_v = static_cast<const double *>(d_v);
    A.end_state = static_cast<double *>(end_state);
    A.d_end = static_cast<double *>(d_end);
    A.status = status;
    mr::diff_tangent_kernel<double><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else if (precision == 32) {
    mr::DiffArgs<float> A;
    int rc = mr::make_args(bgrid, depth, cgrid, u, v, n, x0, y0, kx0, ky0, dt, steps, 1, &A);
    if (rc) return rc;
    if (n == 0) return MR_OK;
    A.dstate0 = static_cast<const float *>(dstate0);
    A.d_depth = static_cast<const float *>(d_depth);
    A.d_u = static_cast<const float *>(d_u);
    A.d_v = static_cast<const float *>(d_v);
    A.end_state = static_cast<float *>(end_state);
    A.d_end = static_cast<float *>(d_end);
    A.status = status;
    mr::diff_tangent_kernel<float><<<mr::blocks_for(n), mr::kDiffBlock, 0, s>>>(A);
  } else {
    return fail(MR_ERR_INVALID_ARGUMENT, "precision must be 64 or 32");
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MR_OK : cuda_fail(e, "diff_tangent launch");
}

}  // extern "C"
