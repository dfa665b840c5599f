// k2.cuh -- the batched FP32 integrator's device code (K2), included by the
// two translation units that instantiate its kernels: rk4_f32.cu (the
// scenario-table builds: MODE 0, and MODE 3 when every scenario's current is
// gridded on its bathymetry's grid) and rk4_f32_one.cu (the single-scenario
// builds, compiled with FP32 subnormals flushed: MODE 1, and MODE 2 when the
// current is gridded on the bathymetry's grid).  The design notes are at the
// top of rk4_f32.cu.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "batch.h"

namespace mr {

namespace {

// ------------------------------------------------------------------ K2 --

constexpr unsigned kFull = 0xffffffffu;
constexpr float kGf = 9.8f;

// Single-precision approximations of the special-function unit (PTX ISA:
// rcp.approx has at most 1 ulp of error, rsqrt.approx and ex2.approx a
// relative error near 2^-22), with subnormal inputs and results flushed to
// zero.  The same instruction in every build gives the same bits in every
// build, whatever its -ftz setting.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// m = 1 - exp(x) and q = exp(x) for x = -2kh <= 0.  Below -0.5, exp(x) is at
// most 0.61, so 1 - exp(x) keeps its relative accuracy: q = 2^(x log2 e) on
// the special-function unit.  From -0.5 to 0, m = -(e^x - 1) by the Taylor
// series of e^x - 1 to the x^8 / 8! term, evaluated by Horner's rule (the
// remainder is below 0.5^9 / 9! = 5.4e-9, relative 1.4e-8 at x = -0.5 and
// smaller toward 0), so m stays relatively accurate in shallow water where
// it tends to 2kh.
__device__ __forceinline__ void one_minus_exp(float x, float &m, float &q) {
  if (x < -0.5f) {
    q = ex2_approx(x * 1.44269504088896341f);
    m = 1.0f - q;
  } else {
    float p = fmaf(x, 1.0f / 40320.0f, 1.0f / 5040.0f);
    p = fmaf(x, p, 1.0f / 720.0f);
    p = fmaf(x, p, 1.0f / 120.0f);
    p = fmaf(x, p, 1.0f / 24.0f);
    p = fmaf(x, p, 1.0f / 6.0f);
    p = fmaf(x, p, 0.5f);
    p = fmaf(x, p, 1.0f);
    m = -(x * p);
    q = 1.0f - m;
  }
}

// Position of a lane on one grid: the cell of its origin (integral floats:
// exact, grids have fewer than 2^24 points per axis) plus the origin's
// fractional cell offset.
struct GridPos {
  float fi0, fj0;
  float f0, g0;
};

__device__ __forceinline__ GridPos grid_pos(const PackedGrid &g, double ox, double oy) {
  GridPos p;
  const double ux = (ox - g.x0) * g.inv_sp_xd, uy = (oy - g.y0) * g.inv_sp_yd;
  const double fx = floor(ux), fy = floor(uy);
  // clamp far-away origins (+-1e9 is exact in FP32); such a lane fails the
  // in-range test of its first lookup
  p.fi0 = static_cast<float>(fmin(fmax(fx, -1.0e9), 1.0e9));
  p.fj0 = static_cast<float>(fmin(fmax(fy, -1.0e9), 1.0e9));
  p.f0 = static_cast<float>(ux - fx);
  p.g0 = static_cast<float>(uy - fy);
  if (!(ux == ux) || !(uy == uy)) { p.fi0 = -2.0e9f; p.f0 = 0.0f; }
  return p;
}

// Cell index and in-cell fractions at offset (px, py) from the origin; false
// when outside the grid's cells (or at a NaN position), and the index is then
// meaningless.  The cell's coordinates are integral floats (exact sums),
// tested against the grid's bounds.  Cells are indexed in 32 bits (the
// batch refuses grids of 2^31 cells or more).
// ix, iy: the cell's column and row (meaningful when inside).
__device__ __forceinline__ bool locate(const PackedGrid &g, const GridPos &p, float px, float py,
                                       int *cell, float *fx, float *fy, int *ix, int *iy) {
  const float ux = fmaf(px, g.inv_sp_x, p.f0);
  const float uy = fmaf(py, g.inv_sp_y, p.g0);
  const float flx = floorf(ux), fly = floorf(uy);
  const float cx = p.fi0 + flx, cy = p.fj0 + fly;
  // saturating conversions and unsigned arithmetic: defined for any position
  *ix = __float2int_rz(cx);
  *iy = __float2int_rz(cy);
  *cell = static_cast<int>(static_cast<unsigned>(*iy) * static_cast<unsigned>(g.nx - 1) +
                           static_cast<unsigned>(*ix));
  *fx = ux - flx;
  *fy = uy - fly;
  // cx, cy are integral: for finite ones the unsigned test of their
  // (saturated) conversions is the bounds test 0 <= cx <= nx - 2.  A NaN
  // position converts to cell (0, 0) and passes it, but its fractions and
  // so its depth are NaN: the stage fails all the same, with the same
  // status (out of domain), and cell 0 is a valid load.
  return static_cast<unsigned>(*ix) <= static_cast<unsigned>(g.nx - 2) &&
         static_cast<unsigned>(*iy) <= static_cast<unsigned>(g.ny - 2);
}

__device__ __forceinline__ bool locate(const PackedGrid &g, const GridPos &p, float px, float py,
                                       int *cell, float *fx, float *fy) {
  int ix, iy;
  return locate(g, p, px, py, cell, fx, fy, &ix, &iy);
}

// c = the cell's bilinear coefficients (batch.h): c.x + c.y fx + c.z fy +
// c.w fx fy in three FMAs.
__device__ __forceinline__ float bilin(const float4 &c, float fx, float fy) {
  return fmaf(fy, fmaf(fx, c.w, c.z), fmaf(fx, c.y, c.x));
}

// The cell records a lane read last, kept in registers: a ray stays in one
// cell for several steps, so most stage lookups reuse them instead of
// loading them again (same values, no memory latency on the dependent chain).
struct CellCache {
  int bkey, ckey;         // cell indices held, -1: none
  float4 b0;              // depth's bilinear coefficients
  float bx, by;           // dh/dx, dh/dy
  float4 c0, c1, c2;      // u's and v's coefficients, the current's gradients
};

// The cell a lane's ray is heading into (the ahead build): its records are
// copied a step before the ray enters it into the lane's 80-byte slot of
// shared memory (5 float4: bathymetry 2, current 3).
struct NextCell {
  int key;                // cell index copied (or in flight), -1: none
};

extern __shared__ __align__(128) float4 k2_ahead_smem[];

struct RayLane {
  int64_t ray;      // -1: empty slot, -2: no work left
  int scen;
  double ox, oy;    // FP64 origin
  GridPos pb, pc;   // origin on the bathymetry and current grids
  float px, py, kx, ky;      // offsets and wavenumber
  float cpx, cpy, ckx, cky;  // Kahan compensations
  int32_t step;       // steps taken (max_steps < 2^31)
  int32_t saved;
  int32_t to_save;    // steps until the next decimated row (no 64-bit modulo per step)
  int32_t to_rebase;  // steps until the next origin rebase
  int32_t limit;      // the sweep form: the step at which the ray leaves this launch
  CellCache cache;
  NextCell next;      // the ahead build only
};

// The ray equations in FP32 from the looked-up fields (bx, by: dh/dx,
// dh/dy): the identity form of the right-hand side in single precision,
// with a = kh, q = exp(-2a), m = 1 - q:
//   tanh a = m / (2 - m),  a / cosh^2 a = 4 a q / (2 - m)^2,
//   1 / (sinh a cosh a) = 4 q / (m (2 - m)),
//   c_g = (g/2) (tanh a + a / cosh^2 a) / sqrt(g k tanh a),
//   dk/dt from the depth = -(k/2) sqrt(g k tanh a) / (sinh a cosh a) grad h;
// beyond a = 23 (deep water) c_g = (g/2) / sqrt(g k) and no refraction.
__device__ __forceinline__ void ray_equations(float h, float u, float v, float dudx, float dudy,
                                              float dvdx, float dvdy, float bx, float by,
                                              float kx, float ky, float k2, float d[4]) {
  const float rk = rsqrt_approx(k2);
  const float k = k2 * rk;
  const float kh = k * h;
  float cg, f;
  if (kh > 23.0f) {
    // deep water: exp(-2kh) < 1e-20, so tanh(kh) = 1 and the terms in
    // exp(-2kh) (kh / cosh^2, the refraction factor) vanish
    cg = (0.5f * kGf) * rsqrt_approx(kGf * k);
    f = 0.0f;
  } else {
    float m, q;
    one_minus_exp(-2.0f * kh, m, q);
    const float inv_d = rcp_approx(m * (2.0f - m));  // 1 / (m (2 - m))
    const float r = m * inv_d;            // 1 / (2 - m)
    const float th = m * r;               // tanh(kh)
    const float gkt = kGf * k * th;
    const float rs = rsqrt_approx(gkt);
    const float q4 = 4.0f * q;
    cg = (0.5f * kGf) * (fmaf(kh * q4, r * r, th) * rs);
    f = (-0.5f * k) * ((q4 * inv_d) * (gkt * rs));
  }
  const float cgk = cg * rk;            // c_g / k: c_g cos(theta) = cgk kx
  d[0] = fmaf(cgk, kx, u);
  d[1] = fmaf(cgk, ky, v);
  d[2] = fmaf(-ky, dvdx, fmaf(-kx, dudx, f * bx));
  d[3] = fmaf(-ky, dvdy, fmaf(-kx, dudy, f * by));
}

// The records of bathymetry cell cb, unless the lane holds them.
__device__ __forceinline__ void load_bathy_cell(const ScenarioDev &s, CellCache &C, int cb) {
  if (cb != C.bkey) {
    C.b0 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2);
    const float4 b1 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2 + 1);
    C.bx = b1.x;
    C.by = b1.y;
    C.bkey = cb;
  }
}

// The records of current cell cc, unless the lane holds them.
__device__ __forceinline__ void load_current_cell(const ScenarioDev &s, CellCache &C, int cc) {
  if (cc != C.ckey) {
    C.c0 = __ldg(s.current.cells + static_cast<int64_t>(cc) * 3);
    C.c1 = __ldg(s.current.cells + static_cast<int64_t>(cc) * 3 + 1);
    C.c2 = __ldg(s.current.cells + static_cast<int64_t>(cc) * 3 + 2);
    C.ckey = cc;
  }
}

// The records of cell cb of both fields when the current is gridded on the
// bathymetry's grid (modes 2 and 3), unless the lane holds them.
__device__ __forceinline__ void load_same_grid_cell(const ScenarioDev &s, CellCache &C, int cb) {
  if (cb != C.bkey) {
    C.b0 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2);
    const float4 b1 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2 + 1);
    C.bx = b1.x;
    C.by = b1.y;
    C.c0 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3);
    C.c1 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3 + 1);
    C.c2 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3 + 2);
    C.bkey = cb;
  }
}

// The ahead build's copies: cp.async (asynchronous global -> shared copies,
// 16 bytes each, cached in L2 only), committed as one group per cell; a lane
// waits only for its own groups.
__device__ __forceinline__ void cp_async16(uint32_t dst, const float4 *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// The records of cell cb of both fields (modes 2 and 3, the ahead build),
// unless the lane holds them: from its shared-memory slot when the ray
// entered the cell it was predicted to enter (after waiting for the copy,
// issued a step or more earlier), else from global memory.
__device__ __forceinline__ void load_same_grid_cell_ahead(const ScenarioDev &s, CellCache &C,
                                                          const NextCell &N, int cb) {
  if (cb != C.bkey) {
    if (cb == N.key) {
      cp_async_wait_all();
      const float4 *slot = k2_ahead_smem + threadIdx.x * 5;
      C.b0 = slot[0];
      const float4 b1 = slot[1];
      C.bx = b1.x;
      C.by = b1.y;
      C.c0 = slot[2];
      C.c1 = slot[3];
      C.c2 = slot[4];
      C.bkey = cb;
    } else {
      load_same_grid_cell(s, C, cb);
    }
  }
}

// The ahead build's prediction, once a step after the first stage: the
// neighbour cell the ray leaves its cell into at velocity (vx, vy) (the
// nearer of its x and y exits), whose records are copied into the lane's
// shared-memory slot now; they are first read when the ray enters that
// cell, a step or more later, so the copy's latency passes while the lane
// computes.
template <int MODE>
__device__ __forceinline__ void load_ahead(const ScenarioDev &s, RayLane &L, float vx, float vy) {
  int cb, ix, iy;
  float fx, fy;
  if (!locate(s.bathy, L.pb, L.px, L.py, &cb, &fx, &fy, &ix, &iy)) return;
  const float ux = vx * s.bathy.inv_sp_x, uy = vy * s.bathy.inv_sp_y;  // cells per second
  const float tx = ux > 0.0f ? (1.0f - fx) * rcp_approx(ux)
                             : (ux < 0.0f ? fx * rcp_approx(-ux) : 3.0e38f);
  const float ty = uy > 0.0f ? (1.0f - fy) * rcp_approx(uy)
                             : (uy < 0.0f ? fy * rcp_approx(-uy) : 3.0e38f);
  int ni = ix, nj = iy;
  if (tx < ty)
    ni += ux > 0.0f ? 1 : -1;
  else
    nj += uy > 0.0f ? 1 : -1;
  if (static_cast<unsigned>(ni) > static_cast<unsigned>(s.bathy.nx - 2) ||
      static_cast<unsigned>(nj) > static_cast<unsigned>(s.bathy.ny - 2))
    return;
  const int key = nj * (s.bathy.nx - 1) + ni;
  NextCell &N = L.next;
  if (key == N.key || key == L.cache.bkey) return;
  cp_async_wait_all();  // the slot's previous copy has landed before it is overwritten
  const uint32_t slot = static_cast<uint32_t>(__cvta_generic_to_shared(k2_ahead_smem)) +
                        threadIdx.x * 80u;
  const float4 *b = s.bathy.cells + static_cast<int64_t>(key) * 2;
  const float4 *c = s.current.cells + static_cast<int64_t>(key) * 3;
  cp_async16(slot, b);
  cp_async16(slot + 16, b + 1);
  cp_async16(slot + 32, c);
  cp_async16(slot + 48, c + 1);
  cp_async16(slot + 64, c + 2);
  cp_async_commit();
  N.key = key;
}

// ---------------------------------------------------- shared-memory tiles --
// The tile build (mode 2, BatchArgs::tile): each warp holds kTileCells^2
// cells of both fields' records in shared memory, a box of the cell arrays
// that the tensor memory accelerator copies in (one cp.async.bulk.tensor per
// field, completion counted on the warp's mbarrier).  A lane entering a cell
// of the tile reads its records there instead of from global memory; the
// values are the same, so results are bit-identical to the build without
// tiles.  Every 4 steps the warp moves its tile onto an outside lane's cell
// when most of its live lanes are outside it.  Waits are bounded: a copy
// that does not complete within kTileWaitPolls polls turns the warp's tiles
// off for the rest of the launch (global memory serves every lane).

constexpr int kTileWaitPolls = 1 << 22;

struct WarpTile {
  int ti, tj;          // tile origin (cell column and row)
  bool valid;          // the tile holds those cells
  bool off;            // tiles turned off (a copy timed out)
  bool pending;        // a timed-out copy may still be in flight
  uint32_t phase;      // parity of the mbarrier phase the next copy completes
  uint32_t smem;       // shared-memory address of this warp's tile
  uint32_t mbar;       // shared-memory address of this warp's mbarrier
  const float4 *tb;    // the tile's bathymetry records (then the current's)
};

extern __shared__ __align__(128) unsigned char k2_tile_smem[];

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
  for (int i = 0; i < kTileWaitPolls; ++i)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
}

// The warp's tile and mbarrier (lane 0 initialises the barrier: one arrival
// per phase, lane 0's, plus the copies' byte count).
__device__ __forceinline__ WarpTile tile_init() {
  WarpTile W;
  const int warp = threadIdx.x >> 5;
  const int warps = blockDim.x >> 5;
  W.smem = static_cast<uint32_t>(__cvta_generic_to_shared(k2_tile_smem)) + warp * kTileBytes;
  W.mbar = static_cast<uint32_t>(__cvta_generic_to_shared(k2_tile_smem)) + warps * kTileBytes +
           warp * 8;
  W.tb = reinterpret_cast<const float4 *>(k2_tile_smem + warp * kTileBytes);
  W.ti = W.tj = 0;
  W.valid = W.off = W.pending = false;
  W.phase = 0;
  if ((threadIdx.x & 31) == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(W.mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  return W;
}

// Copies the tile with origin (ti, tj) in, waits for it (bounded).  Called by
// the whole warp at the same point; the warp's earlier reads of the old tile
// are complete (ordered before the copy by __syncwarp and the proxy fence).
__device__ __forceinline__ void tile_load(const BatchArgs &a, WarpTile &W, int ti, int tj) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(W.mbar),
                 "r"(kTileBytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(W.smem),
        "l"(reinterpret_cast<uint64_t>(&a.tmap_bathy)), "r"(0), "r"(ti), "r"(tj), "r"(W.mbar)
        : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(W.smem + kTileBathyBytes),
        "l"(reinterpret_cast<uint64_t>(&a.tmap_current)), "r"(0), "r"(ti), "r"(tj),
        "r"(W.mbar)
        : "memory");
  }
  const bool done = __all_sync(kFull, mbar_wait_bounded(W.mbar, W.phase));
  W.phase ^= 1u;
  if (done) {
    W.ti = ti;
    W.tj = tj;
    W.valid = true;
  } else {
    W.valid = false;
    W.off = true;
    W.pending = true;
  }
}

// Before the warp exits: a copy that timed out gets one more bounded wait,
// so that none lands in shared memory after the block has left.
__device__ __forceinline__ void tile_finish(const WarpTile &W) {
  if (W.pending) (void)mbar_wait_bounded(W.mbar, W.phase ^ 1u);
}

// The records of cell cb (column ix, row iy) of both fields, mode 2, unless
// the lane holds them: from the warp's tile when the cell is in it.
__device__ __forceinline__ void load_same_grid_cell_tile(const ScenarioDev &s, CellCache &C,
                                                         const WarpTile &W, int cb, int ix,
                                                         int iy) {
  if (cb != C.bkey) {
    const unsigned dx = static_cast<unsigned>(ix - W.ti), dy = static_cast<unsigned>(iy - W.tj);
    if (W.valid && dx < static_cast<unsigned>(kTileCells) &&
        dy < static_cast<unsigned>(kTileCells)) {
      const int c = static_cast<int>(dy) * kTileCells + static_cast<int>(dx);
      const float4 *tb = W.tb;
      const float4 *tc = tb + kTileCells * kTileCells * 2;
      C.b0 = tb[2 * c];
      const float4 b1 = tb[2 * c + 1];
      C.bx = b1.x;
      C.by = b1.y;
      C.c0 = tc[3 * c];
      C.c1 = tc[3 * c + 1];
      C.c2 = tc[3 * c + 2];
    } else {
      C.b0 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2);
      const float4 b1 = __ldg(s.bathy.cells + static_cast<int64_t>(cb) * 2 + 1);
      C.bx = b1.x;
      C.by = b1.y;
      C.c0 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3);
      C.c1 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3 + 1);
      C.c2 = __ldg(s.current.cells + static_cast<int64_t>(cb) * 3 + 2);
    }
    C.bkey = cb;
  }
}

// One right-hand side in FP32 at offset (px, py), wavenumber (kx, ky).
// The fields come from the lane's cell records (loaded when the lane does not
// hold the cell; a point outside a grid loads nothing and uses the records
// held, whatever they are, and a NaN point reads cell 0's: its depth is NaN
// all the same).  With EXACT, returns the stage's BatchStatus: out
// of domain (outside a grid, or depth NaN: a cell past the depth array), dry
// (depth <= 0), bad wavenumber (k^2 not in (0, 3e38)), else complete;
// without, BATCH_COMPLETE or not (the same test, no status code).  d is
// meaningful only when complete.  Written without early returns so that the
// four stages of a step run with no branch between them.  MODE 2 and 3: the
// current is gridded on the bathymetry's grid, so one cell (one key, one
// test) serves both fields.  STAGE (MR_STAGING_*): 1 (mode 2), records from
// the warp's tile when the cell is in it; 2 (modes 2, 3), from the registers
// loaded ahead when the ray entered the predicted cell.
template <int MODE, bool EXACT, int STAGE>
__device__ __forceinline__ int rhs_f32(const ScenarioDev &s, RayLane &L, const WarpTile &W,
                                       float px, float py, float kx, float ky, float d[4]) {
  CellCache &C = L.cache;
  int cb, ix, iy;
  float fx, fy;
  bool inside = locate(s.bathy, L.pb, px, py, &cb, &fx, &fy, &ix, &iy);
  float u, v, dudx, dudy, dvdx, dvdy;
  if (MODE == 2 || MODE == 3) {
    if (STAGE == 1)
      load_same_grid_cell_tile(s, C, W, inside ? cb : C.bkey, ix, iy);
    else if (STAGE == 2)
      load_same_grid_cell_ahead(s, C, L.next, inside ? cb : C.bkey);
    else
      load_same_grid_cell(s, C, inside ? cb : C.bkey);
    u = bilin(C.c0, fx, fy);
    v = bilin(C.c1, fx, fy);
    dudx = C.c2.x; dudy = C.c2.y; dvdx = C.c2.z; dvdy = C.c2.w;
  } else {
    load_bathy_cell(s, C, inside ? cb : C.bkey);
    if (s.current.kind == 0) {
      int cc = cb;
      float gx = fx, gy = fy;  // the same cell when the grids coincide (same origin, same arithmetic)
      if (!s.same_grid) inside &= locate(s.current, L.pc, px, py, &cc, &gx, &gy);
      load_current_cell(s, C, inside ? cc : C.ckey);
      u = bilin(C.c0, gx, gy);
      v = bilin(C.c1, gx, gy);
      dudx = C.c2.x; dudy = C.c2.y; dvdx = C.c2.z; dvdy = C.c2.w;
    } else {
      u = s.current.cu;
      v = s.current.cv;
      dudx = dudy = dvdx = dvdy = 0.0f;
    }
  }
  const float h = bilin(C.b0, fx, fy);
  const float k2 = fmaf(kx, kx, ky * ky);
  ray_equations(h, u, v, dudx, dudy, dvdx, dvdy, C.bx, C.by, kx, ky, k2, d);
  const bool wet = h > 0.0f;
  // 0 < k2 < 3e38 on the bit pattern (k2 = kx^2 + ky^2 is +0, positive,
  // +inf or NaN; 3e38 is 0x7f61b1e6): one integer compare
  const bool kok = static_cast<unsigned>(__float_as_int(k2)) - 1u < 0x7f61b1e5u;
  if (!EXACT) return (inside && wet && kok) ? BATCH_COMPLETE : BATCH_OUT_OF_DOMAIN;
  if (inside && wet && kok) return BATCH_COMPLETE;
  if (!inside || (!(h <= 0.0f) && !wet)) return BATCH_OUT_OF_DOMAIN;
  return !wet ? BATCH_DRY : BATCH_BAD_WAVENUMBER;
}

__device__ __forceinline__ void kahan_add(float &sum, float &comp, float inc) {
  const float y = inc - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

__device__ __forceinline__ void rebase(const ScenarioDev &s, RayLane &L) {
  L.ox += static_cast<double>(L.px) - static_cast<double>(L.cpx);
  L.oy += static_cast<double>(L.py) - static_cast<double>(L.cpy);
  L.px = L.py = L.cpx = L.cpy = 0.0f;
  L.pb = grid_pos(s.bathy, L.ox, L.oy);
  L.pc = s.same_grid ? L.pb : grid_pos(s.current, L.ox, L.oy);
}

__device__ __forceinline__ void save_row(const BatchArgs &a, const RayLane &L) {
  if (L.saved >= a.save_cap) return;
  const int64_t plane = a.save_cap * a.n_stride;
  float *p = a.saved + static_cast<int64_t>(L.saved) * a.n_stride + L.ray;
  p[0] = static_cast<float>(a.t0 + static_cast<double>(L.step) * a.dt);
  p[plane] = static_cast<float>(L.ox + (static_cast<double>(L.px) - static_cast<double>(L.cpx)));
  p[2 * plane] = static_cast<float>(L.oy + (static_cast<double>(L.py) - static_cast<double>(L.cpy)));
  p[3 * plane] = L.kx - L.ckx;
  p[4 * plane] = L.ky - L.cky;
}

__device__ __forceinline__ void finish(const BatchArgs &a, RayLane &L, int status) {
  const int64_t r = L.ray;
  a.end_state[r] = a.t0 + static_cast<double>(L.step) * a.dt;
  a.end_state[a.n_stride + r] = L.ox + (static_cast<double>(L.px) - static_cast<double>(L.cpx));
  a.end_state[2 * a.n_stride + r] = L.oy + (static_cast<double>(L.py) - static_cast<double>(L.cpy));
  a.end_state[3 * a.n_stride + r] = static_cast<double>(L.kx) - static_cast<double>(L.ckx);
  a.end_state[4 * a.n_stride + r] = static_cast<double>(L.ky) - static_cast<double>(L.cky);
  a.n_steps[r] = L.step;
  a.n_saved[r] = L.saved;
  a.status[r] = static_cast<uint8_t>(status);
  L.ray = -1;
}

// The decimation as a step countdown.  A ray takes at most max_steps <
// 2^31 - 1 steps, so a countdown from 2^31 - 1 never reaches zero: that is
// the period when nothing is decimated (decimation 0), and when the
// decimation is larger (no row after step 0 either way).
__device__ __forceinline__ int32_t save_period(const BatchArgs &a) {
  return (a.decimation <= 0 || a.decimation > 0x7fffffff) ? 0x7fffffff
                                                          : static_cast<int32_t>(a.decimation);
}

// A lane's scenario: from the kernel's parameters in the single-scenario
// builds (MODE 1, 2), else from the device table (MODE 0, 3).
template <int MODE>
__device__ __forceinline__ const ScenarioDev &scenario(const BatchArgs &a, int s) {
  return (MODE == 1 || MODE == 2) ? a.scen0 : a.scen[s];
}

template <int MODE>
__device__ __forceinline__ void start(const BatchArgs &a, RayLane &L, int64_t r) {
  L.ray = r;
  L.scen = ((MODE == 0 || MODE == 3) && a.ray_scenario) ? static_cast<int>(a.ray_scenario[r])
                                                         : 0;
  if (L.scen >= a.n_scenarios) L.scen = 0;
  const ScenarioDev &s = scenario<MODE>(a, L.scen);
  L.ox = a.x0[r];
  L.oy = a.y0[r];
  L.px = L.py = L.cpx = L.cpy = L.ckx = L.cky = 0.0f;
  L.kx = static_cast<float>(a.kx0[r]);
  L.ky = static_cast<float>(a.ky0[r]);
  L.pb = grid_pos(s.bathy, L.ox, L.oy);
  L.pc = s.same_grid ? L.pb : grid_pos(s.current, L.ox, L.oy);
  L.step = 0;
  L.saved = 0;
  // no cell held; the records are defined values until the first load
  CellCache &C = L.cache;
  C.bkey = C.ckey = -1;
  C.b0 = C.c0 = C.c1 = C.c2 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  C.bx = C.by = 0.0f;
  L.to_save = save_period(a);
  L.to_rebase = a.rebase_interval;
  if (a.decimation > 0) {
    save_row(a, L);
    L.saved = 1;
  }
}

// The sweep form: a ray taken up again from the state a previous launch
// left, with no cell held -- the lane a launch that traced it without
// stopping would hold, as the cell records are a cache of immutable values
// and the origin's grid positions a function of the origin.
template <int MODE>
__device__ __forceinline__ void resume(const BatchArgs &a, RayLane &L, int64_t r) {
  L.ray = r;
  L.scen = ((MODE == 0 || MODE == 3) && a.ray_scenario) ? static_cast<int>(a.ray_scenario[r])
                                                         : 0;
  if (L.scen >= a.n_scenarios) L.scen = 0;
  const ScenarioDev &s = scenario<MODE>(a, L.scen);
  const float4 *p = reinterpret_cast<const float4 *>(a.sweep + r);
  const double2 o = *reinterpret_cast<const double2 *>(p);
  const float4 q = p[1], c = p[2];
  const int4 k = *reinterpret_cast<const int4 *>(p + 3);
  L.ox = o.x; L.oy = o.y;
  L.px = q.x; L.py = q.y; L.kx = q.z; L.ky = q.w;
  L.cpx = c.x; L.cpy = c.y; L.ckx = c.z; L.cky = c.w;
  L.step = k.x; L.saved = k.y; L.to_save = k.z; L.to_rebase = k.w;
  L.pb = grid_pos(s.bathy, L.ox, L.oy);
  L.pc = s.same_grid ? L.pb : grid_pos(s.current, L.ox, L.oy);
  CellCache &C = L.cache;
  C.bkey = C.ckey = -1;
  C.b0 = C.c0 = C.c1 = C.c2 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  C.bx = C.by = 0.0f;
  const int64_t lim = static_cast<int64_t>(L.step) + a.sweep_steps;
  L.limit = static_cast<int32_t>(lim < a.max_steps ? lim : a.max_steps);
}

// Bits 0-15 of v spread to the even bits of the result.
__device__ __forceinline__ uint32_t spread_even16(uint32_t v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}

// The 2 x 2-cell block of v on an axis (first value v0, 1 / spacing inv),
// clamped to 0..lim; NaN gives 0.  Only an ordering key: no exactness needed.
__device__ __forceinline__ uint32_t sweep_block(double v, double v0, double inv, uint32_t lim) {
  const double c = floor((v - v0) * inv);
  if (!(c > 0.0)) return 0u;
  const double b = c * 0.5;
  return b >= static_cast<double>(lim) ? lim : static_cast<uint32_t>(b);
}

// The sweep form's sort key of a running ray: the Morton code of its 2 x 2
// block of bathymetry cells, its scenario above it (BatchArgs::sweep_*).
__device__ __forceinline__ uint64_t sweep_key(const BatchArgs &a, const ScenarioDev &s,
                                              const RayLane &L) {
  const PackedGrid &g = s.bathy;
  const uint32_t lim = (1u << a.sweep_cell_bits) - 1u;
  const uint32_t bx = sweep_block(L.ox + (static_cast<double>(L.px) - static_cast<double>(L.cpx)),
                                  g.x0, g.inv_sp_xd, lim);
  const uint32_t by = sweep_block(L.oy + (static_cast<double>(L.py) - static_cast<double>(L.cpy)),
                                  g.y0, g.inv_sp_yd, lim);
  return (static_cast<uint64_t>(L.scen) << a.sweep_key_shift) |
         static_cast<uint64_t>(spread_even16(bx) | (spread_even16(by) << 1));
}

__device__ __forceinline__ void store_sweep(const BatchArgs &a, const RayLane &L) {
  float4 *p = reinterpret_cast<float4 *>(a.sweep + L.ray);
  *reinterpret_cast<double2 *>(p) = make_double2(L.ox, L.oy);
  p[1] = make_float4(L.px, L.py, L.kx, L.ky);
  p[2] = make_float4(L.cpx, L.cpy, L.ckx, L.cky);
  *reinterpret_cast<int4 *>(p + 3) = make_int4(L.step, L.saved, L.to_save, L.to_rebase);
}

// The status of a step whose four stages did not all succeed: the stages
// again, in order, up to the first that fails (the same arithmetic on the
// same inputs, so the same values and the same first failure).  Taken once
// per ray at most: the ray ends there.  One stage in a loop: little code.
template <int MODE, int STAGE>
__device__ __forceinline__ int step_status(const ScenarioDev &s, RayLane &L, const WarpTile &W,
                                           float dt, float half) {
  float k[4], x[4] = {L.px, L.py, L.kx, L.ky};
#pragma unroll 1
  for (int st = 0; st < 4; ++st) {
    const int r = rhs_f32<MODE, true, STAGE>(s, L, W, x[0], x[1], x[2], x[3], k);
    if (r != BATCH_COMPLETE) return r;
    const float w = st == 2 ? dt : half;
    x[0] = fmaf(w, k[0], L.px);
    x[1] = fmaf(w, k[1], L.py);
    x[2] = fmaf(w, k[2], L.kx);
    x[3] = fmaf(w, k[3], L.ky);
  }
  // not reached: the same four stages failed a moment ago.  Ending the ray
  // all the same keeps every ray's step count bounded.
  return BATCH_OUT_OF_DOMAIN;
}

// One RK4 step of lane L.  Returns BATCH_COMPLETE while the ray goes on.
// The four stages run without branches between them (each stage's outcome
// is one bit, tested once for all four); a failed step is redone by
// step_status for the status of its first failing stage, and the ray keeps
// the state it had before the step.  The increment k1 + 2 k2 + 2 k3 + k4 is
// summed as the stages complete, so only the sum and the latest stage's
// derivative stay live (register pressure, not arithmetic, bounds how many
// warps an SM holds).
template <int MODE, int STAGE>
__device__ __forceinline__ int advance(const BatchArgs &a, RayLane &L, const WarpTile &W) {
  const ScenarioDev &s = scenario<MODE>(a, L.scen);
  // step constants in FP32 from the host (a conversion here would run on the
  // FP64 pipe, and the compiler re-derives such values under register pressure)
  const float dt = a.dt_f;
  const float half = a.half_f;
  float k[4], sum[4];
  int fails = rhs_f32<MODE, false, STAGE>(s, L, W, L.px, L.py, L.kx, L.ky, k);
#pragma unroll
  for (int q = 0; q < 4; ++q) sum[q] = k[q];
  if (STAGE == 2) load_ahead<MODE>(s, L, k[0], k[1]);
  fails |= rhs_f32<MODE, false, STAGE>(s, L, W, fmaf(half, k[0], L.px), fmaf(half, k[1], L.py),
                                fmaf(half, k[2], L.kx), fmaf(half, k[3], L.ky), k);
#pragma unroll
  for (int q = 0; q < 4; ++q) sum[q] = fmaf(2.0f, k[q], sum[q]);
  fails |= rhs_f32<MODE, false, STAGE>(s, L, W, fmaf(half, k[0], L.px), fmaf(half, k[1], L.py),
                                fmaf(half, k[2], L.kx), fmaf(half, k[3], L.ky), k);
#pragma unroll
  for (int q = 0; q < 4; ++q) sum[q] = fmaf(2.0f, k[q], sum[q]);
  fails |= rhs_f32<MODE, false, STAGE>(s, L, W, fmaf(dt, k[0], L.px), fmaf(dt, k[1], L.py),
                                fmaf(dt, k[2], L.kx), fmaf(dt, k[3], L.ky), k);
  if (fails != BATCH_COMPLETE) return step_status<MODE, STAGE>(s, L, W, dt, half);
  const float sixth = a.sixth_f;
  kahan_add(L.px, L.cpx, sixth * (sum[0] + k[0]));
  kahan_add(L.py, L.cpy, sixth * (sum[1] + k[1]));
  kahan_add(L.kx, L.ckx, sixth * (sum[2] + k[2]));
  kahan_add(L.ky, L.cky, sixth * (sum[3] + k[3]));
  ++L.step;
  if (--L.to_save == 0) {
    L.to_save = save_period(a);
    save_row(a, L);
    ++L.saved;
  }
  if (--L.to_rebase == 0) {
    L.to_rebase = a.rebase_interval;
    rebase(s, L);
  }
  return BATCH_COMPLETE;
}

// The tile build's upkeep, every 4 steps: when most of the warp's live
// lanes are in cells outside its tile, the tile moves so that the first such
// lane's cell sits at its centre.
template <int MODE>
__device__ __forceinline__ void tile_refresh(const BatchArgs &a, const RayLane &L, WarpTile &W) {
  const ScenarioDev &s = scenario<MODE>(a, L.scen);
  int cb = 0, ix = 0, iy = 0;
  float fx, fy;
  const bool in_grid = L.ray >= 0 && locate(s.bathy, L.pb, L.px, L.py, &cb, &fx, &fy, &ix, &iy);
  const bool in_tile = W.valid && static_cast<unsigned>(ix - W.ti) < kTileCells &&
                       static_cast<unsigned>(iy - W.tj) < kTileCells;
  const unsigned live = __ballot_sync(kFull, in_grid);
  const unsigned out = __ballot_sync(kFull, in_grid && !in_tile);
  if (W.off || 2 * __popc(out) <= __popc(live)) return;
  const int src = __ffs(out) - 1;
  const int ti = __shfl_sync(kFull, ix, src) - kTileCells / 2;
  const int tj = __shfl_sync(kFull, iy, src) - kTileCells / 2;
  tile_load(a, W, ti, tj);
}

template <int RPT, int MODE, int STAGE, bool SWEEP = false>
__device__ __forceinline__ void k2_body(const BatchArgs &a) {
  static_assert(!SWEEP || (RPT == 1 && STAGE == 0), "the sweep form traces one ray per lane");
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int64_t n = SWEEP ? *a.n_dev : a.n;
  const int32_t max_steps = static_cast<int32_t>(a.max_steps);
  RayLane L[RPT];
#pragma unroll
  for (int j = 0; j < RPT; ++j) L[j].ray = -1;
  WarpTile W;
  if (STAGE == 1) W = tile_init();
  int iter = 0;
  while (true) {
    if (SWEEP) {
      // rays at the end of this launch's sweep: state out, listed with
      // their sort key for the next launch (one atomic per warp)
      const bool out = L[0].ray >= 0 && L[0].step >= L[0].limit && L[0].step < max_steps;
      const unsigned leaving = __ballot_sync(kFull, out);
      if (leaving) {
        const int leader = __ffs(leaving) - 1;
        unsigned long long base = 0;
        if (lane == leader)
          base = atomicAdd(a.next_count, static_cast<unsigned long long>(__popc(leaving)));
        base = __shfl_sync(kFull, base, leader);
        if (out) {
          store_sweep(a, L[0]);
          const unsigned long long pos = base + __popc(leaving & lt_mask);
          a.next_list[pos] = static_cast<uint32_t>(L[0].ray);
          a.next_keys[pos] = sweep_key(a, scenario<MODE>(a, L[0].scen), L[0]);
          L[0].ray = -1;
        }
      }
    }
    // refill empty slots from the work queue, one atomic per warp and slot
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
      const unsigned need = __ballot_sync(kFull, L[j].ray == -1);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(a.queue, static_cast<unsigned long long>(__popc(need)));
        base = __shfl_sync(kFull, base, leader);
        if (L[j].ray == -1) {
          const int64_t r = static_cast<int64_t>(base) + __popc(need & lt_mask);
          if (r < n) {
            const int64_t ray = a.order ? static_cast<int64_t>(__ldg(a.order + r)) : r;
            if (SWEEP && !a.sweep_first) {
              resume<MODE>(a, L[j], ray);
            } else {
              start<MODE>(a, L[j], ray);
              if (SWEEP) L[j].limit = a.sweep_steps < a.max_steps ? a.sweep_steps
                                                                  : static_cast<int32_t>(a.max_steps);
            }
            if (STAGE == 2) L[j].next.key = -1;
          } else {
            L[j].ray = -2;
          }
        }
      }
    }
    bool live = false;
#pragma unroll
    for (int j = 0; j < RPT; ++j) live |= L[j].ray >= 0;
    if (!__any_sync(kFull, live)) break;
    if (STAGE == 1 && (iter++ & 3) == 0) tile_refresh<MODE>(a, L[0], W);
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
      if (L[j].ray < 0) continue;
      if (L[j].step >= max_steps) {
        finish(a, L[j], BATCH_COMPLETE);
        continue;
      }
      if (RPT == 1 && STAGE == 0) {
        // Up to eight steps per pass of the loop, which cuts the refill,
        // sweep and termination votes to one per eight steps (8,192^2 case
        // in sweeps: +4-6% with two steps, +5-6% more with four, +3.6%
        // more with eight).  A ray stops early when it fails, reaches
        // max_steps or its sweep's end; the next pass then finishes or
        // suspends it as before, so each ray takes the same steps.
        const int32_t stop = SWEEP ? L[j].limit : max_steps;
        int st = BATCH_COMPLETE;
#pragma unroll 1
        for (int u = 0; u < 8; ++u) {
          st = advance<MODE, STAGE>(a, L[j], W);
          if (st != BATCH_COMPLETE || L[j].step >= stop) break;
        }
        if (st != BATCH_COMPLETE) finish(a, L[j], st);
      } else {
        const int st = advance<MODE, STAGE>(a, L[j], W);
        if (st != BATCH_COMPLETE) finish(a, L[j], st);
      }
    }
  }
  if (STAGE == 1) tile_finish(W);
  if (STAGE == 2) cp_async_wait_all();  // no copy lands after the block has left
}

// One ray per lane, two builds.  rk4_f32_kernel_1 takes the compiler's
// register count (~100: 4 blocks of 128 threads, 16 warps, per SM).
// rk4_f32_kernel_1r is capped at 72 registers (28 warps per SM; 80 B
// spilled to L1).  The kernel is issue- and latency-bound; when a call has
// rays for more warps than the first keeps resident, the extra warps hide
// more of the dependent FP32 chains than the spills cost (4,096^2
// shelf-slope, 2^20 rays: 30.6 -> 32.7 G ray-steps/s at 128 x 8; caps of
// 80 / 64 / 56 registers gave 32.0 / 32.7 / 31.5); with fewer rays than
// lanes the spills only add latency (65,536-ray seamount: 22.2 -> 19.3).
// The launcher takes the capped build when the launch asks for more blocks
// per SM than the uncapped one holds.
// Each comes in four modes: 0 reads the lane's scenario from the device
// table; 1 (one scenario) takes the scenario's fields from the kernel's
// parameters (operands of the instructions instead of loads at every
// lookup); 2 is mode 1 and 3 is mode 0 with the current gridded on the
// bathymetry's grid (every scenario's, for 3).
template <int MODE>
__global__ void __launch_bounds__(256) rk4_f32_kernel_1(BatchArgs a) { k2_body<1, MODE, 0>(a); }
template <int MODE>
__global__ void __maxnreg__(72) rk4_f32_kernel_1r(BatchArgs a) { k2_body<1, MODE, 0>(a); }
// The sweep form of both: each launch advances its rays by at most
// sweep_steps steps, the first from their initial states (sweep_first), the
// later ones from the states the previous launch left.
template <int MODE>
__global__ void __launch_bounds__(256) rk4_f32_kernel_1s(BatchArgs a) {
  k2_body<1, MODE, 0, true>(a);
}
template <int MODE>
__global__ void __maxnreg__(72) rk4_f32_kernel_1rs(BatchArgs a) { k2_body<1, MODE, 0, true>(a); }
// Two rays per lane hold twice the lane state: no cap.
template <int MODE>
__global__ void __launch_bounds__(256) rk4_f32_kernel_2(BatchArgs a) { k2_body<2, MODE, 0>(a); }
// The tile build (mode 2): one ray per lane (the compiler's register count,
// 80; capped at 72 it spilled), each warp's tile in dynamic
// shared memory (kTileBytes per warp, then 8 bytes of mbarrier per warp); the
// arguments stay in the parameter space (__grid_constant__) because the
// copies read the tensor maps from there.
template <int MODE>
__global__ void __launch_bounds__(256) rk4_f32_kernel_1t(const __grid_constant__ BatchArgs a) {
  k2_body<1, MODE, 1>(a);
}
// The ahead build (modes 2 and 3): one ray per lane, with the records of the
// cell each ray heads into copied a step early into the lane's 80-byte slot
// of dynamic shared memory.
template <int MODE>
__global__ void __launch_bounds__(256) rk4_f32_kernel_1a(BatchArgs a) { k2_body<1, MODE, 2>(a); }

}  // namespace

}  // namespace mr
