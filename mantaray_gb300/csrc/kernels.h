// kernels.h -- launch interfaces of the device kernels (internal to the
// library; the public C ABI is include/mantaray_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "batch.h"
#include "fields.h"

namespace mr {

constexpr int kK1Block = 64;

// Arguments of one trace launch.  All pointers are device-visible.
struct TraceArgs {
  uint64_t n;                 // rays
  const double *x0, *y0, *kx0, *ky0;
  double t0, dt;
  uint64_t nsteps;            // ceil((t_end - t0) / dt) as usize
  uint64_t rows_cap;          // rows per ray in traj (>= nsteps + 1)
  double *traj;               // [5][rows_cap][n]: t, x, y, kx, ky
  int32_t *n_rows;            // [n]
  uint8_t *status;            // [n]
};

cudaError_t launch_rk4_f64(const BathyDev &b, const CurrentDev &c, const TraceArgs &a,
                           int stop_rule, int identity_math, cudaStream_t stream);

// Batched FP32 form: cell packing of one field (one thread per cell) and the
// persistent integrator (grid = SMs x blocks_per_sm).
cudaError_t launch_pack_bathy(const BathyDev &b, float4 *cells, cudaStream_t stream);
cudaError_t launch_pack_current(const CurrentDev &c, float4 *cells, cudaStream_t stream);
cudaError_t launch_rk4_f32(const BatchArgs &a, int block, int blocks_per_sm, int rays_per_lane,
                           cudaStream_t stream);
// The integrator build a launch of this shape runs, for n_scenarios
// scenarios (same_grid: every scenario's current is gridded on its
// bathymetry's grid; staging: MR_STAGING_*; sweep: the sweep form; null where
// that build does not exist); a graph's kernel node is found by it.
const void *rk4_f32_function(int rays_per_lane, int block, int blocks_per_sm, int n_scenarios,
                             int same_grid, int staging, int sweep);
// Dynamic shared memory of the tile build for blocks of `block` threads.
size_t rk4_f32_tile_smem(int block);
// The single-scenario builds (rk4_f32_one.cu): 0 one ray per lane, 1 the same
// capped at 72 registers, 2 two rays per lane, 3 the tile build, 4 the ahead
// build (3 and 4: same grid only, else null), 5 and 6 the sweep form of 0
// and 1.
const void *rk4_f32_one_function(int build, int same_grid);
cudaError_t launch_fill_nan(float *p, int64_t count, cudaStream_t stream);

// Spatial ordering of a batched call's rays (K6): sorts by key in `passes`
// 8-bit digits; the order is then o.vals[passes & 1].  Grids are sized for
// n_max >= o.n.
int order_tiles(int64_t n_max);
cudaError_t launch_order(const OrderArgs &o, int64_t n_max, int passes, cudaStream_t stream);
const void *order_keys_function();
// Between two sweeps: *n_dev = *next_count, then the list counter and the
// work-queue head back to zero (one thread).
cudaError_t launch_sweep_next(int64_t *n_dev, unsigned long long *next_count,
                              unsigned long long *queue, cudaStream_t stream);

}  // namespace mr
