// fields.h -- device-side descriptions of the bathymetry and current fields.
//
// Plain structs passed by value as kernel parameters.  Grid arrays live in
// device memory (HBM) with the reference's flat layout, index nx*j + i
// (src/bathymetry/cartesian_netcdf3.rs:465-471,
// src/current/cartesian_current.rs:421-427).  Besides the reference's own
// arrays (f32 axes + f64 depth; f64 axes, u, v) a handle holds tables derived
// from them once, on the host, with the reference's own operations, so a
// lookup reads the values it needs instead of recomputing them per call:
//  - f32 copies of every value the reference casts to f32 before bilinear
//    interpolation (depth, u, v, current axes: `as f32`, round to nearest);
//  - per-cell forward differences, indexed by the cell's south-west corner:
//    bathymetry (d[j][i+1] - d[j][i]) / x_space cast to f32 and
//    (d[j+1][i] - d[j][i]) / y_space cast to f32 (cartesian_netcdf3.rs:119-134),
//    current du/dx, du/dy, dv/dx, dv/dy in f64 (cartesian_current.rs:515-536).
// Each table entry is bit-identical to the value the reference computes at
// lookup time.
#pragma once

#include <stdint.h>

#include "bits.h"

namespace mr {

enum BathyKind : int {
  BATHY_GRID = 0,      // CartesianNetcdf3
  BATHY_CONSTANT = 1,  // ConstantDepth (constant_depth.rs:98-129)
  BATHY_SLOPE = 2,     // ConstantSlope (constant_slope.rs:28-77)
  BATHY_ARRAY = 3      // ArrayDepth test field (array_depth.rs:9-35)
};

enum CurrentKind : int {
  CURRENT_GRID = 0,     // CartesianCurrent
  CURRENT_CONSTANT = 1  // ConstantCurrent (constant_current.rs:50-108)
};

struct BathyDev {
  int kind;
  uint64_t nx, ny;
  const float *x;        // [nx] axis (f32, as the reference stores it)
  const float *y;        // [ny]
  const double *depth;   // [depth_len] f64 depth, flat nx*j + i
  const float *depth32;  // [depth_len] depth as f32
  const float *gx;       // [depth_len] f32 cell gradient d/dx, by south-west corner
  const float *gy;       // [depth_len] f32 cell gradient d/dy
  uint64_t depth_len;
  // nearest(): spacing = |a[1] - a[0]| (f32), high = (n - 1) as f32
  float x0, xsp, xhigh;
  float y0, ysp, yhigh;
  // gradient denominators: a[1] as f64 - a[0] as f64 (cartesian_netcdf3.rs:119-120)
  double xspace, yspace;
  // analytic fields
  float h;                                  // constant depth
  float s_h0, s_x0, s_y0, s_dhdx, s_dhdy;   // constant slope
  uint64_t an;                              // array depth: an x an
  const float *arr;                         // arr[i*an + j] = array[i][j]
};

struct CurrentDev {
  int kind;
  uint64_t nx, ny;
  const double *x;   // [nx] f64 axes
  const double *y;   // [ny]
  const double *u;   // [u_len] f64 values
  const double *v;   // [v_len]
  const float *x32;  // [nx] axes as f32
  const float *y32;  // [ny]
  const float *u32;  // [u_len] values as f32
  const float *v32;  // [v_len]
  const double *dudx, *dudy, *dvdx, *dvdy;  // [min(u_len, v_len)] cell gradients
  uint64_t u_len, v_len;
  double x0, xsp, xhigh;   // nearest() in f64
  double y0, ysp, yhigh;
  double inv_xsp, inv_ysp; // 1 / spacing (fast path of the index, lookup.cuh)
  // Cell thresholds of each axis (lookup.cuh, corner_pair_thr): thr[j] is the
  // order key (order_key below) of the smallest double t whose index
  // (t - a0) / spacing, computed as the reference computes it, is >= j, for
  // j = 0..n-1; thr[n] that of the smallest t whose index is > n - 1.  Null
  // when an axis has fewer than two points or a spacing that is not finite
  // and positive.
  const long long *xthr, *ythr;
  float x0f, inv_xspf;     // f32 first guess of the cell (any error is corrected)
  float y0f, inv_yspf;
  double xspace, yspace;   // a[1] - a[0] (cartesian_current.rs:515-516)
  double cu, cv;           // constant current
};

// Error values of src/error.rs:7-37 that the right-hand side can produce.
enum RhsError : int {
  RHS_OK = 0,
  RHS_ARGUMENT_OUT_OF_BOUNDS = 1,
  RHS_INVALID_ARGUMENT = 2,
  RHS_INDEX_OUT_OF_BOUNDS = 3
};

}  // namespace mr
