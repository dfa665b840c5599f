// batch_handle.h -- the mr_batch handle (internal).
#pragma once

#include <vector>

#include "batch.h"

struct mr_batch {
  int device = 0;
  int n_scenarios = 0;
  std::vector<mr::ScenarioDev> host_scen;
  mr::ScenarioDev *scen = nullptr;   // device copy of host_scen
  std::vector<void *> mem;           // packed cells
  unsigned long long *queue = nullptr;  // work-queue head (device scratch)
};
