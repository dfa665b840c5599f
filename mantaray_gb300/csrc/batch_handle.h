// batch_handle.h -- the mr_batch handle (internal).
#pragma once

#include <stdint.h>

#include <vector>

#include "batch.h"

// Device scratch of the spatial ordering (order.cu) for up to `cap` rays:
// one allocation holding n_dev, keys [2][cap], vals [2][cap], counts
// [256][tiles], totals [256]; and for the sweep form, for up to `sweep_cap` rays, another
// holding the list counter, the running rays' states [sweep_cap], the list
// [sweep_cap] and its sort keys [sweep_cap].
struct mr_order_buffers {
  void *mem = nullptr;
  size_t cap = 0;
  int tiles = 0;
  int64_t *n_dev = nullptr;
  uint64_t *keys[2] = {nullptr, nullptr};
  uint32_t *vals[2] = {nullptr, nullptr};
  uint32_t *counts = nullptr;
  uint32_t *totals = nullptr;
  void *sweep_mem = nullptr;
  size_t sweep_cap = 0;
  unsigned long long *count = nullptr;
  mr::SweepRay *sweep = nullptr;
  uint32_t *list = nullptr;
  uint64_t *list_keys = nullptr;
};

struct mr_batch {
  int device = 0;
  int n_scenarios = 0;
  std::vector<mr::ScenarioDev> host_scen;
  mr::ScenarioDev *scen = nullptr;   // device copy of host_scen
  std::vector<void *> mem;           // packed cells
  unsigned long long *queue = nullptr;  // work-queue head (device scratch)
  mr_order_buffers ord;              // ordering scratch of direct calls, grown on demand
  int order_scen_shift = 8;          // key layout of the ordering (order.cu)
  int order_passes = 1;
  int sweep_cell_bits = 0;           // key layout of the sweep form's orderings (k2.cuh)
  int sweep_key_shift = 0;
  int sweep_passes = 1;
  // tensor maps of the cell records for the tile build (one scenario with its
  // current on the bathymetry's grid), made at creation
  CUtensorMap tmap_bathy{};
  CUtensorMap tmap_current{};
  bool has_tmaps = false;
};

// 1 when every scenario's current is gridded on its bathymetry's grid (the
// batched kernel then takes one cell lookup for both fields).
inline int all_same_grid(const mr_batch *b) {
  for (const auto &sc : b->host_scen)
    if (!sc.same_grid) return 0;
  return 1;
}

struct mr_batch_config;

namespace mr {

// Checks the arguments of a batched call for n rays over buffers of n_stride
// rays and fills the kernel's arguments (batch_api.cu).  Outputs may be
// device memory or page-locked host memory (taken through its device
// mapping); anything else fails with MR_ERR_INVALID_ARGUMENT before any work
// is queued.  a->scen and a->queue are the batch's own device table and
// work-queue head.  Allocates nothing.
int batch_fill_args(mr_batch *b, size_t n, size_t n_stride, const uint8_t *ray_scenario,
                    const double *x0, const double *y0, const double *kx0, const double *ky0,
                    double t0, double dt, int64_t max_steps, int64_t decimation,
                    size_t save_cap, float *saved, double *end_state, int32_t *n_steps,
                    int32_t *n_saved, uint8_t *status, const mr_batch_config *cfg,
                    BatchArgs *a);

}  // namespace mr
