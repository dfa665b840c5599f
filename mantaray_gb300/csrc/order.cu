// order.cu -- K6, the spatial ordering of a batched call's rays.
//
// The persistent batched kernel (K2) takes rays from its work queue in queue
// order.  When the caller's rays come in no spatial order, the 32 lanes of a
// warp read 32 unrelated cell records at every stage.  K6 sorts the rays by
// a key -- scenario, Morton code of the starting cell on the scenario's
// bathymetry grid, direction of the wavenumber -- with a stable LSD radix
// sort on 8-bit digits, and K2 then takes queue slot q to ray order[q]: the
// rays of a warp start in the same or neighbouring cells with close
// directions and stay close for many steps, so their cell reads are shared.
// Each ray's result is unchanged: its arithmetic does not depend on its lane,
// its neighbours or when it is taken; only the order of the queue changes.
// The sweep form sorts the rays still running between two launches the same
// way, by keys the batched kernel wrote when it stopped them (the Morton code
// of their current 2 x 2-cell block): order_keys does not run, the first
// pass reads those keys, and sweep_next moves their count into n_dev.
//
// All kernels run over grids sized for a capacity n_max, so one captured
// graph replays them for any n <= n_max: order_keys takes n as its argument
// and stores it in device memory, where the later kernels read it.
//   order_keys     one thread per ray: key and identity value
//   order_hist     one block per tile of kTile rays: digit counts, [digit][tile]
//   order_scan     one block per digit: exclusive scan of its counts over the
//                  tiles, and its total
//   order_scatter  one block per tile: stable scatter of (key, value) by digit
// Stability within a tile: rounds of 256 consecutive rays; inside a round a
// ray's rank among equal digits is its rank within its warp
// (__match_any_sync) plus the counts of the earlier warps and earlier rounds.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "batch.h"
#include "kernels.h"

namespace mr {

namespace {

constexpr int kOrderThreads = 256;
constexpr int kOrderWarps = kOrderThreads / 32;
constexpr int kScanThreads = 256;

// Bits 0-15 of v spread to the even bits of the result.
__device__ __forceinline__ uint32_t spread16(uint32_t v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// Cell coordinate of v on an axis (first value v0, spacing sp), clamped to
// 0..65535; NaN gives 0.
__device__ __forceinline__ uint32_t cell_coord(double v, double v0, double sp) {
  const double c = floor((v - v0) / sp);
  if (!(c > 0.0)) return 0u;
  return c >= 65535.0 ? 65535u : static_cast<uint32_t>(c);
}

__device__ __forceinline__ uint64_t order_key(const OrderArgs &o, int s, double x, double y,
                                              float kx, float ky) {
  if (s >= o.n_scenarios) s = 0;  // as the batched kernel maps it
  const PackedGrid &g = o.scen[s].bathy;
  const uint32_t cx = cell_coord(x, g.x0, g.sp_x);
  const uint32_t cy = cell_coord(y, g.y0, g.sp_y);
  const uint32_t morton = spread16(cx) | (spread16(cy) << 1);
  const float th = atan2f(ky, kx);
  float tb = (th + 3.14159265f) * (256.0f / 6.28318531f);
  tb = fminf(fmaxf(tb, 0.0f), 255.0f);  // NaN -> 0
  return (static_cast<uint64_t>(s) << o.scen_shift) | (static_cast<uint64_t>(morton) << 8) |
         static_cast<uint64_t>(tb);
}

// The n rays by their initial states, n stored for the later kernels;
// grid-stride over a fixed grid.
__global__ void order_keys(OrderArgs o) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *o.n_dev = o.n;
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; r < o.n;
       r += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int s = o.ray_scenario ? static_cast<int>(o.ray_scenario[r]) : 0;
    o.keys[0][r] = order_key(o, s, o.x0[r], o.y0[r], static_cast<float>(o.kx0[r]),
                             static_cast<float>(o.ky0[r]));
    o.vals[0][r] = static_cast<uint32_t>(r);
  }
}

__global__ void __launch_bounds__(kOrderThreads) order_hist(OrderArgs o, int pass) {
  __shared__ unsigned h[256];
  const int t = threadIdx.x;
  h[t] = 0u;
  __syncthreads();
  const int64_t n = *o.n_dev;
  const int shift = 8 * pass;
  const uint64_t *keys = (pass == 0 && o.in_keys) ? o.in_keys : o.keys[pass & 1];
  const int64_t start = static_cast<int64_t>(blockIdx.x) * kOrderTile;
  for (int i = t; i < kOrderTile; i += kOrderThreads) {
    const int64_t e = start + i;
    if (e >= n) break;
    atomicAdd(&h[(keys[e] >> shift) & 0xffu], 1u);
  }
  __syncthreads();
  o.counts[static_cast<int64_t>(t) * o.tiles + blockIdx.x] = h[t];
}

// Exclusive scan in place of one digit's counts over the tiles that hold
// rays (the first ceil(n / kOrderTile) of its row of counts [256][tiles]),
// one block per digit, and the digit's total to totals[digit].  The scatter
// adds the digits' own offsets (a scan of the 256 totals).
__global__ void __launch_bounds__(kScanThreads) order_scan(OrderArgs o) {
  __shared__ unsigned warp_sum[kScanThreads / 32];
  __shared__ unsigned carry_s;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int64_t n = *o.n_dev;
  const int used = static_cast<int>((n + kOrderTile - 1) / kOrderTile);
  uint32_t *row = o.counts + static_cast<int64_t>(blockIdx.x) * o.tiles;
  if (t == 0) carry_s = 0u;
  __syncthreads();
  for (int i0 = 0; i0 < used; i0 += kScanThreads) {
    const int i = i0 + t;
    const unsigned v = i < used ? row[i] : 0u;
    unsigned incl = v;  // inclusive scan across the warp
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned up = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += up;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
      const unsigned ws = lane < kScanThreads / 32 ? warp_sum[lane] : 0u;
      unsigned wi = ws;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned up = __shfl_up_sync(0xffffffffu, wi, d);
        if (lane >= d) wi += up;
      }
      if (lane < kScanThreads / 32) warp_sum[lane] = wi - ws;  // exclusive prefix of the warp sums
    }
    __syncthreads();
    const unsigned before = carry_s + warp_sum[w] + (incl - v);
    if (i < used) row[i] = before;
    __syncthreads();
    if (t == kScanThreads - 1) carry_s = before + v;
    __syncthreads();
  }
  if (t == 0) o.totals[blockIdx.x] = carry_s;
}

__global__ void __launch_bounds__(kOrderThreads) order_scatter(OrderArgs o, int pass) {
  __shared__ unsigned base[256], run[256];
  __shared__ unsigned wcnt[kOrderWarps][256];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const int64_t n = *o.n_dev;
  const int shift = 8 * pass;
  const uint64_t *kin = (pass == 0 && o.in_keys) ? o.in_keys : o.keys[pass & 1];
  const uint32_t *vin = (pass == 0 && o.in_keys) ? o.in_vals : o.vals[pass & 1];
  uint64_t *kout = o.keys[(pass & 1) ^ 1];
  uint32_t *vout = o.vals[(pass & 1) ^ 1];
  const int64_t start = static_cast<int64_t>(blockIdx.x) * kOrderTile;
  if (start >= n) return;  // uniform in the block
  {
    // where digit t starts: the totals of the smaller digits (an exclusive
    // scan of the 256 totals, the same in every block) plus this tile's
    // offset within the digit
    const unsigned v = o.totals[t];
    unsigned incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned up = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += up;
    }
    if (lane == 31) wcnt[0][w] = incl;
    __syncthreads();
    unsigned before = incl - v;
    for (int q = 0; q < w; ++q) before += wcnt[0][q];
    base[t] = before + o.counts[static_cast<int64_t>(t) * o.tiles + blockIdx.x];
    run[t] = 0u;
    __syncthreads();
  }
  for (int j = 0; j < kOrderTile / kOrderThreads; ++j) {
    if (start + static_cast<int64_t>(j) * kOrderThreads >= n) break;  // uniform in the block
#pragma unroll
    for (int q = 0; q < kOrderWarps; ++q) wcnt[q][t] = 0u;
    __syncthreads();
    const int64_t e = start + static_cast<int64_t>(j) * kOrderThreads + t;
    const bool valid = e < n;
    uint64_t key = 0;
    uint32_t val = 0, d = 0, rank = 0;
    const unsigned active = __ballot_sync(0xffffffffu, valid);
    if (valid) {
      key = kin[e];
      val = vin[e];
      d = static_cast<uint32_t>((key >> shift) & 0xffu);
      const unsigned peers = __match_any_sync(active, d);
      rank = __popc(peers & lt);
      if (rank == 0) wcnt[w][d] = __popc(peers);
    }
    __syncthreads();
    if (valid) {
      unsigned before = run[d] + rank;
      for (int q = 0; q < w; ++q) before += wcnt[q][d];
      const int64_t pos = static_cast<int64_t>(base[d]) + before;
      kout[pos] = key;
      vout[pos] = val;
    }
    __syncthreads();
    unsigned add = 0u;
#pragma unroll
    for (int q = 0; q < kOrderWarps; ++q) add += wcnt[q][t];
    run[t] += add;
  }
}

// The rays the last sweep left running become the next sweep's work; the
// list counter and the work-queue head start again from zero.
__global__ void sweep_next(int64_t *n_dev, unsigned long long *next_count,
                           unsigned long long *queue) {
  *n_dev = static_cast<int64_t>(*next_count);
  *next_count = 0ull;
  *queue = 0ull;
}

}  // namespace

cudaError_t launch_sweep_next(int64_t *n_dev, unsigned long long *next_count,
                              unsigned long long *queue, cudaStream_t stream) {
  sweep_next<<<1, 1, 0, stream>>>(n_dev, next_count, queue);
  return cudaGetLastError();
}

int order_tiles(int64_t n_max) {
  return static_cast<int>((n_max + kOrderTile - 1) / kOrderTile);
}

cudaError_t launch_order(const OrderArgs &o, int64_t n_max, int passes, cudaStream_t stream) {
  if (n_max <= 0) return cudaSuccess;
  if (!o.in_keys) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int64_t blocks = (n_max + kOrderThreads - 1) / kOrderThreads;
    const unsigned kgrid = static_cast<unsigned>(blocks < 8ll * sms ? blocks : 8ll * sms);
    order_keys<<<kgrid, kOrderThreads, 0, stream>>>(o);
  }
  for (int p = 0; p < passes; ++p) {
    order_hist<<<o.tiles, kOrderThreads, 0, stream>>>(o, p);
    order_scan<<<256, kScanThreads, 0, stream>>>(o);
    order_scatter<<<o.tiles, kOrderThreads, 0, stream>>>(o, p);
  }
  return cudaGetLastError();
}

const void *order_keys_function() { return reinterpret_cast<const void *>(&order_keys); }

}  // namespace mr
