// fields.h -- device-side descriptions of the bathymetry and current fields.
//
// Plain structs passed by value as kernel parameters.  Grid arrays live in
// device memory (HBM) in the reference's own precisions and flat layout
// (src/bathymetry/cartesian_netcdf3.rs:35-43: f32 axes + f64 depth;
// src/current/cartesian_current.rs:18-27: f64 axes, u, v), flat index
// nx*j + i (cartesian_netcdf3.rs:465-471, cartesian_current.rs:421-427).
// Host-precomputed scalars repeat the reference's own per-call arithmetic
// (same operands, same precision), so they are bit-identical to it.
#pragma once

#include <stdint.h>

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
  const float *x;        // [nx]
  const float *y;        // [ny]
  const double *depth;   // [depth_len], flat nx*j + i
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
  const double *x;   // [nx]
  const double *y;   // [ny]
  const double *u;   // [u_len]
  const double *v;   // [v_len]
  uint64_t u_len, v_len;
  double x0, xsp, xhigh;   // nearest() in f64
  double y0, ysp, yhigh;
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
