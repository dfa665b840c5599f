// batch_static.cu -- mr_batch_trace_device_static: the batched FP32 trace
// with no device allocation of its own.
//
// Who needs it: callers that cannot call cudaMalloc when they trace -- a host
// application whose device memory is owned by another runtime's pool (a
// framework that reserved the GPU's memory up front, an embedding engine
// with a fixed budget), or a real-time loop that must not allocate or free on
// its hot path because allocation can synchronise the device.  They build
// their mr_batch (which does allocate: it packs the fields) once, at set-up,
// and then trace as often as they like without any further allocation,
// through this entry point.
//
// Its scratch -- the work-queue head the persistent kernel hands rays out
// from, and this call's copy of the scenario table -- lives in the file-scope
// array below instead of in memory the library allocates.  Every GPU that
// loads the library holds that array (16 KiB) until the process exits.

#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <vector>

#include "../../include/mantaray_gpu.h"
#include "batch.h"
#include "batch_handle.h"
#include "handles.h"
#include "kernels.h"

namespace {

using mr::cuda_fail;
using mr::DeviceGuard;
using mr::fail;

constexpr size_t kStaticScratchBytes = 16384;  // 16 KiB in all
constexpr size_t kQueueBytes = 256;            // the work-queue head, first 256 bytes
constexpr int kStaticMaxScenarios = MR_BATCH_STATIC_MAX_SCENARIOS;
static_assert(kQueueBytes + kStaticMaxScenarios * sizeof(mr::ScenarioDev) <= kStaticScratchBytes,
              "the scenario table must fit in the static scratch");

// The scratch.  Host code must not use this name as an address: on the host
// it is only a stand-in for the device variable.  Its device address comes
// from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_batch_scratch[kStaticScratchBytes];

std::mutex g_scratch_mu;
std::vector<unsigned char *> g_scratch_addr;  // per device ordinal; null until set up

// Device address of g_batch_scratch on `device`, which must be current.
// Looked up on the first call on each device.
int scratch_address(int device, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (device < 0) return fail(MR_ERR_INVALID_ARGUMENT, "bad device ordinal %d", device);
  if (static_cast<size_t>(device) >= g_scratch_addr.size())
    g_scratch_addr.resize(static_cast<size_t>(device) + 1, nullptr);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_batch_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static batch scratch)");
    g_scratch_addr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_scratch_addr[device];
  return MR_OK;
}

}  // namespace

extern "C" int mr_batch_trace_device_static(
    mr_batch *b, size_t n, const uint8_t *ray_scenario, const double *x0, const double *y0,
    const double *kx0, const double *ky0, double t0, double dt, int64_t max_steps,
    int64_t decimation, size_t save_cap, float *saved, double *end_state, int32_t *n_steps,
    int32_t *n_saved, uint8_t *status, const mr_batch_config *cfg, void *stream) {
  if (!b) return fail(MR_ERR_INVALID_ARGUMENT, "null batch");
  if (b->n_scenarios > kStaticMaxScenarios)
    return fail(MR_ERR_CAPACITY,
                "%d scenarios exceed the static scratch of mr_batch_trace_device_static "
                "(at most %d scenarios); use mr_batch_trace_device",
                b->n_scenarios, kStaticMaxScenarios);
  if (!cfg) return fail(MR_ERR_INVALID_ARGUMENT, "null config");
  if (cfg->block < 32 || cfg->block > 256 || cfg->block % 32 || cfg->blocks_per_sm < 1 ||
      cfg->blocks_per_sm > 32 || (cfg->rays_per_lane != 1 && cfg->rays_per_lane != 2) ||
      cfg->rebase_interval < 1)
    return fail(MR_ERR_INVALID_ARGUMENT, "bad launch configuration");
  if (cfg->order != 0)
    return fail(MR_ERR_INVALID_ARGUMENT,
                "ray ordering needs scratch memory; use mr_batch_trace_device");
  if (n > 0 && (!x0 || !y0 || !kx0 || !ky0 || !end_state || !n_steps || !n_saved || !status))
    return fail(MR_ERR_INVALID_ARGUMENT, "null array argument");
  if (decimation < 0 || max_steps < 0 || max_steps >= INT32_MAX)
    return fail(MR_ERR_INVALID_ARGUMENT, "bad max_steps or decimation");
  if (decimation > 0 && (!saved || static_cast<int64_t>(save_cap) < max_steps / decimation + 1))
    return fail(MR_ERR_CAPACITY, "saved buffer too small for max_steps / decimation + 1 rows");
  if (!(dt > 0.0) || !isfinite(t0)) return fail(MR_ERR_INVALID_ARGUMENT, "dt must be > 0");
  if (n == 0) return MR_OK;

  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the batch's device");
  unsigned char *scratch = nullptr;
  int rc = scratch_address(b->device, &scratch);
  if (rc) return rc;
  unsigned long long *queue = reinterpret_cast<unsigned long long *>(scratch);
  mr::ScenarioDev *table = reinterpret_cast<mr::ScenarioDev *>(scratch + kQueueBytes);

  mr::BatchArgs a{};
  a.scen = table;
  a.scen0 = b->host_scen[0];
  a.all_same_grid = all_same_grid(b);
  a.n_scenarios = b->n_scenarios;
  a.ray_scenario = ray_scenario;
  a.n = static_cast<int64_t>(n);
  a.x0 = x0; a.y0 = y0; a.kx0 = kx0; a.ky0 = ky0;
  a.t0 = t0;
  a.dt = dt;
  a.dt_f = static_cast<float>(dt);
  a.half_f = 0.5f * a.dt_f;
  a.sixth_f = a.dt_f * (1.0f / 6.0f);
  a.max_steps = max_steps;
  a.decimation = decimation;
  a.save_cap = static_cast<int64_t>(save_cap);
  a.n_stride = static_cast<int64_t>(n);
  a.rebase_interval = cfg->rebase_interval;
  a.saved = saved;
  a.end_state = end_state;
  a.n_steps = n_steps;
  a.n_saved = n_saved;
  a.status = status;
  a.queue = queue;

  // The scratch keeps the previous call's contents: the queue head must start
  // at zero, and the scenario table is rewritten for this batch.
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  cudaError_t e = cudaMemcpyAsync(table, b->host_scen.data(),
                                  b->host_scen.size() * sizeof(mr::ScenarioDev),
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess && decimation > 0)
    e = cudaMemsetAsync(saved, 0xFF, sizeof(float) * 5 * save_cap * n, s);
  if (e == cudaSuccess)
    e = mr::launch_rk4_f32(a, cfg->block, cfg->blocks_per_sm, cfg->rays_per_lane, s);
  if (e != cudaSuccess) return cuda_fail(e, "rk4_f32 launch (static scratch)");
  return MR_OK;
}
