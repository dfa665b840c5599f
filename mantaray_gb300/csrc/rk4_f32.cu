// rk4_f32.cu -- K2, the batched FP32 ray integrator, and K5, its grid prep.
//
// K5 (pack_*_cells): repacks a bathymetry / current grid of the plain form
// (f64 values in HBM) into the cell records of batch.h, one thread per cell.
//
// K2 (rk4_f32_kernel_1 / _1r / _2, device code in k2.cuh): a persistent
// kernel, grid = SMs x blocks per SM.  Each lane holds 1 or 2 rays (_2); one
// ray per lane has an uncapped and a 72-register build (_1r), chosen by the
// launch shape, and their sweep forms (_1s / _1rs: each launch advances its
// rays by at most sweep_steps steps, the rays still running re-sorted by
// position between launches; batch_api.cu queues the sequence).  Each build
// has two scenario-table forms (instantiated here) and two single-scenario
// forms (rk4_f32_one.cu).  A lane whose ray has ended
// refills from a device work queue: the warp ballots its empty slots, one lane reserves
// that many ray indices with a single atomicAdd and the indices are handed out
// by rank within the ballot, so lanes never idle while work remains and rays
// of very different lifetimes (domain exits, dry cells) keep every lane busy.
// There is no waiting on other blocks or threads anywhere in the kernel.
//
// Precision: the right-hand side and the interpolation run in FP32 (the
// identity form of the RHS, see ray_exact.cuh, in single precision).  Each
// ray's position is an FP32 offset from an FP64 origin; offsets and
// wavenumbers are accumulated with Kahan compensation, and every
// `rebase_interval` steps the offset is folded into the FP64 origin, which
// keeps the offsets (and their rounding) small over tens of thousands of
// steps.  FP64 is used only for that rebase and for the stored positions.
//
// Memory: each lane keeps the cell records it read last in registers and
// reuses them while its ray stays in that cell; when the current is gridded
// on the bathymetry's grid one cell lookup serves both fields.  The queue may
// be taken in a spatial order (order.cu).
//
// Compiled with -fmad=false and every fused multiply-add written as fmaf, so
// each ray's arithmetic is fixed by the source: results are bit-identical for
// every launch shape (block size, blocks per SM, rays per lane, ordering)
// and both register builds.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <atomic>

#include "batch.h"
#include "fields.h"
#include "kernels.h"

namespace mr {

namespace {

// ---------------------------------------------------------------- K5 prep --

// The bilinear of corners (v00, v10, v01, v11) as v00 + c1 fx + c2 fy +
// c3 fx fy, the coefficients formed in FP64 and rounded once each.
__device__ __forceinline__ float4 bilinear_coefficients(double v00, double v10, double v01,
                                                        double v11) {
  return make_float4(__double2float_rn(v00), __double2float_rn(v10 - v00),
                     __double2float_rn(v01 - v00), __double2float_rn((v11 - v10) - (v01 - v00)));
}

__global__ void pack_bathy_cells(BathyDev b, float4 *cells) {
  const int64_t ncx = static_cast<int64_t>(b.nx) - 1, ncy = static_cast<int64_t>(b.ny) - 1;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= ncx * ncy) return;
  const int64_t i = c % ncx, j = c / ncx;
  const uint64_t sw = b.nx * j + i, se = sw + 1, nw = sw + b.nx, ne = nw + 1;
  float4 r0, r1;
  if (ne < b.depth_len) {
    const double d00 = b.depth[sw], d10 = b.depth[se], d01 = b.depth[nw], d11 = b.depth[ne];
    r0 = bilinear_coefficients(d00, d10, d01, d11);
    r1 = make_float4(__double2float_rn((d10 - d00) / b.xspace),
                     __double2float_rn((d01 - d00) / b.yspace), 0.0f, 0.0f);
  } else {  // corners past the end of the depth array: no water
    const float nan = __int_as_float(0x7fffffff);
    r0 = make_float4(nan, nan, nan, nan);
    r1 = make_float4(nan, nan, 0.0f, 0.0f);
  }
  cells[2 * c] = r0;
  cells[2 * c + 1] = r1;
}

__global__ void pack_current_cells(CurrentDev cu, float4 *cells) {
  const int64_t ncx = static_cast<int64_t>(cu.nx) - 1, ncy = static_cast<int64_t>(cu.ny) - 1;
  const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= ncx * ncy) return;
  const int64_t i = c % ncx, j = c / ncx;
  const uint64_t sw = cu.nx * j + i, se = sw + 1, nw = sw + cu.nx, ne = nw + 1;
  float4 r0, r1, r2;
  if (ne < cu.u_len && ne < cu.v_len) {
    const double u00 = cu.u[sw], u10 = cu.u[se], u01 = cu.u[nw], u11 = cu.u[ne];
    const double v00 = cu.v[sw], v10 = cu.v[se], v01 = cu.v[nw], v11 = cu.v[ne];
    r0 = bilinear_coefficients(u00, u10, u01, u11);
    r1 = bilinear_coefficients(v00, v10, v01, v11);
    r2 = make_float4(__double2float_rn((u10 - u00) / cu.xspace),
                     __double2float_rn((u01 - u00) / cu.yspace),
                     __double2float_rn((v10 - v00) / cu.xspace),
                     __double2float_rn((v01 - v00) / cu.yspace));
  } else {
    const float nan = __int_as_float(0x7fffffff);
    r0 = r1 = r2 = make_float4(nan, nan, nan, nan);
  }
  cells[3 * c] = r0;
  cells[3 * c + 1] = r1;
  cells[3 * c + 2] = r2;
}

}  // namespace

}  // namespace mr

#include "k2.cuh"

namespace mr {

cudaError_t launch_pack_bathy(const BathyDev &b, float4 *cells, cudaStream_t stream) {
  const int64_t ncell = static_cast<int64_t>(b.nx - 1) * static_cast<int64_t>(b.ny - 1);
  if (ncell <= 0) return cudaSuccess;
  pack_bathy_cells<<<static_cast<unsigned>((ncell + 255) / 256), 256, 0, stream>>>(b, cells);
  return cudaGetLastError();
}

cudaError_t launch_pack_current(const CurrentDev &c, float4 *cells, cudaStream_t stream) {
  const int64_t ncell = static_cast<int64_t>(c.nx - 1) * static_cast<int64_t>(c.ny - 1);
  if (ncell <= 0) return cudaSuccess;
  pack_current_cells<<<static_cast<unsigned>((ncell + 255) / 256), 256, 0, stream>>>(c, cells);
  return cudaGetLastError();
}

// NaN fill of the decimated rows (a kernel, so that it writes page-locked
// host buffers through their device mapping as well as device memory).
namespace {
__global__ void fill_nan_kernel(float *p, int64_t count) {
  const float nan = __int_as_float(0x7fffffff);
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < count;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    p[i] = nan;
}
}  // namespace

cudaError_t launch_fill_nan(float *p, int64_t count, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int64_t blocks = (count + 255) / 256;
  const unsigned grid = static_cast<unsigned>(blocks < 8ll * sms ? blocks : 8ll * sms);
  fill_nan_kernel<<<grid, 256, 0, stream>>>(p, count);
  return cudaGetLastError();
}

// The builds of each table mode: [0] one ray per lane, uncapped; [1] the
// same capped at 72 registers; [2] two rays per lane; [3] and [4] the sweep
// form of [0] and [1].  Row 0: mode 0, row 1: mode 3 (every current on its
// bathymetry's grid).
static const void *table_builds[2][5] = {
    {reinterpret_cast<const void *>(&rk4_f32_kernel_1<0>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1r<0>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_2<0>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1s<0>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1rs<0>)},
    {reinterpret_cast<const void *>(&rk4_f32_kernel_1<3>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1r<3>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_2<3>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1s<3>),
     reinterpret_cast<const void *>(&rk4_f32_kernel_1rs<3>)}};

// Resident blocks per SM of each mode's uncapped one-ray build (plain and
// sweep form) by block size (multiples of 32 up to 256), queried once; 0:
// not yet known.
static std::atomic<int> g_resident_1[2][4][9];

size_t rk4_f32_tile_smem(int block) {
  return static_cast<size_t>(block / 32) * (kTileBytes + 8);
}

const void *rk4_f32_function(int rays_per_lane, int block, int blocks_per_sm, int n_scenarios,
                             int same_grid, int staging, int sweep) {
  const int mode = n_scenarios == 1 ? (same_grid ? 2 : 1) : (same_grid ? 3 : 0);
  if (sweep && (staging != 0 || rays_per_lane != 1)) return nullptr;
  if (staging == 1) return (mode == 2 && rays_per_lane == 1) ? rk4_f32_one_function(3, 1) : nullptr;
  if (staging == 2) {
    if (rays_per_lane != 1) return nullptr;
    if (mode == 2) return rk4_f32_one_function(4, 1);
    if (mode == 3) return reinterpret_cast<const void *>(&rk4_f32_kernel_1a<3>);
    return nullptr;
  }
  // [0] uncapped, [1] capped, [2] two rays per lane; the sweep form of [0]
  // and [1] in their place
  static const int kOneBuild[2][3] = {{0, 1, 2}, {5, 6, 2}};
  static const int kTableBuild[2][3] = {{0, 1, 2}, {3, 4, 2}};
  const int sw = sweep ? 1 : 0;
  const void *fn[3];
  for (int k = 0; k < 3; ++k)
    fn[k] = (mode == 1 || mode == 2) ? rk4_f32_one_function(kOneBuild[sw][k], mode == 2)
                                     : table_builds[mode == 3][kTableBuild[sw][k]];
  if (rays_per_lane == 2) return fn[2];
  const int slot = (block >= 32 && block <= 256 && block % 32 == 0) ? block / 32 : 0;
  int resident = slot ? g_resident_1[sw][mode][slot].load(std::memory_order_relaxed) : 0;
  if (resident == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fn[0], block, 0) !=
            cudaSuccess ||
        resident < 1) {
      (void)cudaGetLastError();
      resident = blocks_per_sm;  // unknown: the uncapped build
    } else if (slot) {
      g_resident_1[sw][mode][slot].store(resident, std::memory_order_relaxed);
    }
  }
  return resident < blocks_per_sm ? fn[1] : fn[0];
}

cudaError_t launch_rk4_f32(const BatchArgs &a, int block, int blocks_per_sm, int rays_per_lane,
                           cudaStream_t stream) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const unsigned grid = static_cast<unsigned>(sms * blocks_per_sm);
  void *args[] = {const_cast<BatchArgs *>(&a)};
  const void *fn = rk4_f32_function(rays_per_lane, block, blocks_per_sm, a.n_scenarios,
                                    a.all_same_grid, a.staging, a.sweep_steps > 0);
  if (!fn) return cudaErrorInvalidValue;
  const size_t smem = a.staging == 1 ? rk4_f32_tile_smem(block)
                      : a.staging == 2 ? static_cast<size_t>(block) * 80 : 0;
  return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, stream);
}

}  // namespace mr
