// batch.h -- device structures of the batched FP32 form.
//
// A scenario is one (bathymetry, current) pair.  For the FP32 form each field
// is repacked once, on the device, into cells: one cell per grid square,
// indexed by its south-west corner (i, j), holding everything a lookup
// inside that square needs, so a lookup is a few 16-byte loads from one
// contiguous record:
//   bathymetry cell (8 floats, 32 B):  h's bilinear coefficients c0 c1 c2 c3
//                                      dh/dx dh/dy 0 0
//   current cell (12 floats, 48 B):    u's coefficients x4, v's x4,
//                                      du/dx du/dy dv/dx dv/dy
// where a field inside the cell is c0 + c1 fx + c2 fy + c3 fx fy at the
// cell fractions (fx, fy): c0 = v(i,j), c1 = v(i+1,j) - v(i,j),
// c2 = v(i,j+1) - v(i,j), c3 = v(i+1,j+1) - v(i+1,j) - v(i,j+1) + v(i,j),
// formed in FP64 from the grid and rounded once each.
// The gradients are the reference's cell forward differences
// (src/bathymetry/cartesian_netcdf3.rs:119-134,
// src/current/cartesian_current.rs:515-536), so the FP32 form integrates the
// same equations as the plain form, in single precision.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace mr {

struct PackedGrid {
  const float4 *cells;   // [(ny-1)*(nx-1)] records of `vec4` float4s
  int nx, ny;            // grid points
  double x0, y0;         // first axis values
  double sp_x, sp_y;     // axis spacing (a[1] - a[0])
  float inv_sp_x, inv_sp_y;
  double inv_sp_xd, inv_sp_yd;  // 1 / spacing in FP64 (origin rebase)
  int kind;              // 0 grid, 1 constant (current only)
  float cu, cv;          // constant current
};

struct ScenarioDev {
  PackedGrid bathy;      // 2 float4 per cell
  PackedGrid current;    // 3 float4 per cell
  int same_grid;         // gridded current on the bathymetry's grid: one cell lookup serves both
};

// Per-ray termination status of the batched form.
enum BatchStatus : uint8_t {
  BATCH_COMPLETE = 0,      // all max_steps steps taken
  BATCH_OUT_OF_DOMAIN = 1, // a stage left the bathymetry or current grid
  BATCH_DRY = 2,           // depth <= 0
  BATCH_BAD_WAVENUMBER = 3,// k <= 0 or non-finite state
};

// Shared-memory tile of one warp (the tile build): kTileCells x kTileCells
// cells of both fields' records, bathymetry first.
constexpr int kTileCells = 8;
constexpr int kTileBathyBytes = kTileCells * kTileCells * 2 * 16;
constexpr int kTileBytes = kTileCells * kTileCells * 5 * 16;

// A running ray between two sweeps of the sweep form: the lane state that
// carries from one step to the next (the rest -- grid positions of the
// origin, cell records -- follows from it), 64 bytes.
struct __align__(16) SweepRay {
  double ox, oy;                 // FP64 origin
  float px, py, kx, ky;          // offsets and wavenumber
  float cpx, cpy, ckx, cky;      // Kahan compensations
  int32_t step, saved, to_save, to_rebase;
};

struct BatchArgs {
  // tensor maps of scenario 0's cell records (the tile build): bathymetry
  // [ny-1][nx-1][8 floats], current [ny-1][nx-1][12 floats]
  CUtensorMap tmap_bathy;
  CUtensorMap tmap_current;
  int staging;               // MR_STAGING_* (the tile and ahead builds)
  const ScenarioDev *scen;   // [n_scenarios]
  ScenarioDev scen0;         // scen[0] by value: the single-scenario build reads it from
                             // the kernel's parameters, with no load
  int all_same_grid;         // every scenario's current is gridded on its bathymetry's grid
  int n_scenarios;
  const uint8_t *ray_scenario;  // [n] scenario per ray, or null (all scenario 0)
  int64_t n;                 // rays of this call
  const double *x0, *y0, *kx0, *ky0;  // [n] initial states
  double t0, dt;
  float dt_f, half_f, sixth_f;  // (float)dt, dt/2, dt/6 as the integrator uses them
  int64_t max_steps;
  int64_t decimation;        // store every `decimation`-th step (0: endpoints only)
  int64_t save_cap;          // rows of `saved` per ray
  int64_t n_stride;          // ray stride of `saved` (>= n; the buffer's capacity)
  int rebase_interval;       // steps between FP64 origin rebases
  float *saved;              // [5][save_cap][n_stride] f32 t, x, y, kx, ky
  double *end_state;         // [5][n_stride] f64 t, x, y, kx, ky of the last valid state
  int32_t *n_steps;          // [n] steps taken
  int32_t *n_saved;          // [n] rows stored in `saved`
  uint8_t *status;           // [n] BatchStatus
  unsigned long long *queue; // work-queue head (scratch, zeroed before the launch)
  const uint32_t *order;     // [n] ray taken at each queue slot, or null (slot = ray)
  // The sweep form (sweep_steps > 0): a launch advances each ray it takes by
  // at most sweep_steps steps; a ray still running then leaves its state in
  // sweep[ray], and its index and sort key in next_list / next_keys at
  // position *next_count (counted up) for the next launch.  Every launch
  // takes *n_dev rays in the order `order` (the first: the call's n rays;
  // the later ones: the list, sorted by key).  The key: the Morton code of
  // the ray's 2 x 2-cell block on its scenario's bathymetry grid (sweep_cell_bits
  // bits per axis), the scenario above it (bit sweep_key_shift up).
  int32_t sweep_steps;
  int32_t sweep_first;             // 1: the call's first launch (rays from x0, y0, kx0, ky0)
  int32_t sweep_cell_bits;
  int32_t sweep_key_shift;
  SweepRay *sweep;                 // [n_stride]
  uint32_t *next_list;             // [n_stride]
  uint64_t *next_keys;             // [n_stride]
  unsigned long long *next_count;
  const int64_t *n_dev;
};

// Spatial ordering of the rays (order.cu): keys [2][n_max] and values
// [2][n_max] ping-pong buffers, per-tile digit counts [256][tiles], digit
// totals [256].
constexpr int kOrderTile = 4096;
struct OrderArgs {
  const ScenarioDev *scen;
  int n_scenarios;
  const uint8_t *ray_scenario;
  const double *x0, *y0, *kx0, *ky0;
  int64_t n;                 // rays of this call (<= the capacity the grids are sized for)
  int64_t *n_dev;            // device copy of n for the kernels after order_keys
  uint64_t *keys[2];
  uint32_t *vals[2];
  uint32_t *counts;
  uint32_t *totals;          // [256] rays per digit of the current pass
  int tiles;                 // ceil(capacity / kOrderTile)
  int scen_shift;            // bit position of the scenario in the key
  // keys and values sorted by the first pass when order_keys does not run
  // (the sweep form: the keys the batched kernel wrote); null: keys[0], vals[0]
  const uint64_t *in_keys;
  const uint32_t *in_vals;
};

}  // namespace mr
