// rk4_f64.cu -- K1, the plain FP64 ray integrator (the drop-in form).
//
// One ray per thread.  Each thread runs the reference stepper
// (ode_solvers 0.4.0 Rk4, called from src/ray.rs:198-213) on the reference
// right-hand side (ray_exact.cuh).  Trajectories are written time-major per
// variable, traj[v][row][ray] (v = t, x, y, kx, ky), which is the
// (time_step, ray) layout of the reference's xarray result
// (python/mantaray/core.py:114-125): at every step a warp stores 32
// consecutive doubles per variable (fully coalesced 256-byte rows).  Rows after
// a ray's last row are NaN, as the Python wrapper pads them.
//
// The right-hand side is a template parameter (RhsLibm: the reference's
// transcendental calls; RhsIdentity: the same quantities from fewer FP64
// instructions, see ray_exact.cuh).  Compiled with -fmad=false: nothing is
// contracted implicitly; with RhsIdentity the RK4 update uses explicit FMAs.
// A second template parameter picks the lookups' cache (lookup.cuh): small
// calls keep each lane's last bathymetry and current cells in registers,
// which gives the same values with shorter dependent chains.

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "kernels.h"
#include "ray_exact.cuh"

namespace mr {

namespace {

__device__ __forceinline__ void store_row(double *traj, uint64_t plane, uint64_t n,
                                          uint64_t row, uint64_t i, double t,
                                          const double y[4]) {
  double *p = traj + row * n + i;
  p[0] = t;
  p[plane] = y[0];
  p[2 * plane] = y[1];
  p[3 * plane] = y[2];
  p[4 * plane] = y[3];
}

__device__ __forceinline__ void store_nan_row(double *traj, uint64_t plane, uint64_t n,
                                              uint64_t row, uint64_t i) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  double *p = traj + row * n + i;
#pragma unroll
  for (int v = 0; v < 5; ++v) p[v * plane] = nan;
}

// One RK4 step as four right-hand-side evaluations in a rolled loop (one copy
// of the inlined right-hand side in the kernel, which keeps it in the
// instruction cache): stages 0-2 evaluate at y + k h/2, y + k h/2, y + k h
// and accumulate acc = k1 + k2*2 + k3*2 + k4 in the reference's left-to-right
// order; stage 3 forms y' = y + acc * (h/6) and evaluates there, which is
// the next step's first stage and the FRESH stop-rule derivative (system()
// does not depend on t).  With FMA (RhsIdentity) the same sums are FMAs.
template <bool FMA>
__device__ __forceinline__ double axpy(double y, double k, double h) {
  return FMA ? fma(k, h, y) : y + k * h;
}

template <int STOP_RULE, typename Rhs, typename Cache>
__global__ void __launch_bounds__(kK1Block) rk4_f64_kernel(BathyDev b, CurrentDev c,
                                                           TraceArgs a) {
  constexpr bool F = Rhs::kFma;
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool valid = i < a.n;
  // lanes present in this warp (blocks may be smaller than a warp)
  const unsigned warp_mask = blockDim.x >= 32 ? 0xffffffffu : (1u << blockDim.x) - 1u;
  Cache L;  // the lane's last cells (LookupCache) or nothing (NoCache)
  const uint64_t plane = a.rows_cap * a.n;
  double y[4] = {0.0, 0.0, 0.0, 0.0};
  double k1[4] = {0.0, 0.0, 0.0, 0.0};
  double t = a.t0;
  bool alive = valid;
  uint64_t rows = 0;
  if (valid) {
    y[0] = a.x0[i]; y[1] = a.y0[i]; y[2] = a.kx0[i]; y[3] = a.ky0[i];
    store_row(a.traj, plane, a.n, 0, i, t, y);
    rows = 1;
    system<Rhs, Cache>(b, c, y, k1, &L);
  }
  const double half = a.dt / 2.0;
  const double sixth = a.dt / 6.0;
  uint64_t s = 0;
  for (; s < a.nsteps; ++s) {
    // Once every lane of the warp has stopped, the rest is NaN padding.
    if (__all_sync(warp_mask, !alive)) break;
    if (alive) {
      double acc[4], kc[4], yn[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { acc[q] = k1[q]; kc[q] = k1[q]; }
#pragma unroll 1
      for (int st = 0; st < 4; ++st) {
        double in[4];
        if (st < 3) {
          const double hs = st == 2 ? a.dt : half;
#pragma unroll
          for (int q = 0; q < 4; ++q) in[q] = axpy<F>(y[q], kc[q], hs);
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) { yn[q] = axpy<F>(y[q], acc[q], sixth); in[q] = yn[q]; }
        }
        system<Rhs, Cache>(b, c, in, kc, &L);
        if (st < 2) {
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[q] = axpy<F>(acc[q], kc[q], 2.0);
        } else if (st == 2) {
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[q] = acc[q] + kc[q];
        }
      }
      t = t + a.dt;
      store_row(a.traj, plane, a.n, s + 1, i, t, yn);
      ++rows;
      const bool stop = STOP_RULE == 1 ? (all_nan4(kc) || all_nan4(yn))
                                       : (all_nan4(k1) || all_nan4(yn));
#pragma unroll
      for (int q = 0; q < 4; ++q) { y[q] = yn[q]; k1[q] = kc[q]; }
      if (stop) alive = false;
    } else if (valid) {
      store_nan_row(a.traj, plane, a.n, s + 1, i);
    }
  }
  if (valid) {
    for (uint64_t row = rows > s + 1 ? rows : s + 1; row < a.rows_cap; ++row)
      store_nan_row(a.traj, plane, a.n, row, i);
    a.n_rows[i] = static_cast<int32_t>(rows);
    a.status[i] = alive ? 0 : 1;
  }
}

}  // namespace

// Resident blocks per SM of the cached build, by stop rule, arithmetic and
// block size (8, 16, 32, 64), queried once; 0 when the query fails (no
// cache).
static int cached_resident(int stop_rule, int identity_math, int block) {
  static std::atomic<int> known[2][2][4];
  const int slot = block >= 64 ? 3 : block >= 32 ? 2 : block >= 16 ? 1 : 0;
  std::atomic<int> &k = known[stop_rule == 1][identity_math != 0][slot];
  int r = k.load(std::memory_order_relaxed);
  if (r) return r < 0 ? 0 : r;
  const void *fn =
      stop_rule == 1
          ? (identity_math ? reinterpret_cast<const void *>(&rk4_f64_kernel<1, RhsIdentity, LookupCache>)
                           : reinterpret_cast<const void *>(&rk4_f64_kernel<1, RhsLibm, LookupCache>))
          : (identity_math ? reinterpret_cast<const void *>(&rk4_f64_kernel<0, RhsIdentity, LookupCache>)
                           : reinterpret_cast<const void *>(&rk4_f64_kernel<0, RhsLibm, LookupCache>));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, fn, block, 0) != cudaSuccess || r < 1) {
    (void)cudaGetLastError();
    r = -1;
  }
  k.store(r, std::memory_order_relaxed);
  return r < 0 ? 0 : r;
}

template <typename Rhs, typename Cache>
static void launch_k1(int stop_rule, unsigned grid, int block, const BathyDev &b,
                      const CurrentDev &c, const TraceArgs &a, cudaStream_t stream) {
  if (stop_rule == 1)
    rk4_f64_kernel<1, Rhs, Cache><<<grid, block, 0, stream>>>(b, c, a);
  else
    rk4_f64_kernel<0, Rhs, Cache><<<grid, block, 0, stream>>>(b, c, a);
}

cudaError_t launch_rk4_f64(const BathyDev &b, const CurrentDev &c, const TraceArgs &a,
                           int stop_rule, int identity_math, cudaStream_t stream) {
  if (a.n == 0) return cudaSuccess;
  // Blocks of 64 rays, or fewer when that leaves SMs without a block: on
  // GB300 an SM issues 2 FP64 lanes per clock, so a small call runs fastest
  // with its rays spread over as many SMs as possible (down to 8 per block).
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  int block = kK1Block;
  while (block > 8 && (a.n + block - 1) / block < static_cast<uint64_t>(sms)) block /= 2;
  const unsigned grid = static_cast<unsigned>((a.n + block - 1) / block);
  // The lookup cache shortens the rays' dependent chains (1,024-16,384 rays:
  // 6-18% faster; the 65,536-ray seamount, identity arithmetic: 2.09 ->
  // 2.15 G ray-steps/s, bit-identical) but takes registers (identity 128 a
  // thread, libm 148, against 96 and 116).  It pays while every block of the
  // call is resident at once: a second wave of blocks costs more than the
  // cache saves (65,536 rays, libm: 26% slower).
  const bool cache = grid <= static_cast<unsigned>(cached_resident(stop_rule, identity_math, block)) *
                                 static_cast<unsigned>(sms);
  if (identity_math) {
    if (cache)
      launch_k1<RhsIdentity, LookupCache>(stop_rule, grid, block, b, c, a, stream);
    else
      launch_k1<RhsIdentity, NoCache>(stop_rule, grid, block, b, c, a, stream);
  } else {
    if (cache)
      launch_k1<RhsLibm, LookupCache>(stop_rule, grid, block, b, c, a, stream);
    else
      launch_k1<RhsLibm, NoCache>(stop_rule, grid, block, b, c, a, stream);
  }
  return cudaGetLastError();
}

}  // namespace mr
