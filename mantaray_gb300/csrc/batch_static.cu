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
  if (cfg && cfg->order != 0)
    return fail(MR_ERR_INVALID_ARGUMENT,
                "ray ordering needs scratch memory; use mr_batch_trace_device");
  // The same checks as mr_batch_trace_device, with the same messages:
  // outputs must be device memory or page-locked host memory (written
  // through its device mapping); pageable host memory is refused here,
  // before anything is queued.
  mr::BatchArgs a{};
  int rc = mr::batch_fill_args(b, n, n, ray_scenario, x0, y0, kx0, ky0, t0, dt, max_steps,
                               decimation, save_cap, saved, end_state, n_steps, n_saved, status,
                               cfg, &a);
  if (rc) return rc;
  if (n == 0) return MR_OK;

  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the batch's device");
  unsigned char *scratch = nullptr;
  rc = scratch_address(b->device, &scratch);
  if (rc) return rc;
  unsigned long long *queue = reinterpret_cast<unsigned long long *>(scratch);
  mr::ScenarioDev *table = reinterpret_cast<mr::ScenarioDev *>(scratch + kQueueBytes);
  a.scen = table;
  a.queue = queue;

  // The scratch keeps the previous call's contents: the queue head must start
  // at zero, and the scenario table is rewritten for this batch from the
  // batch's own device copy (a device-to-device copy: no host staging).  The
  // single-scenario builds take their scenario from the kernel's parameters
  // and never read the table, so one scenario needs no copy.
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  cudaError_t e = cudaSuccess;
  if (b->n_scenarios > 1)
    e = cudaMemcpyAsync(table, b->scen, static_cast<size_t>(b->n_scenarios) * sizeof(mr::ScenarioDev),
                        cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  // rows a ray does not reach: the same NaN as mr_batch_trace_device writes
  if (e == cudaSuccess && decimation > 0 && save_cap > 0)
    e = mr::launch_fill_nan(a.saved, 5 * static_cast<int64_t>(save_cap) * a.n_stride, s);
  if (e == cudaSuccess)
    e = mr::launch_rk4_f32(a, cfg->block, cfg->blocks_per_sm, cfg->rays_per_lane, s);
  if (e != cudaSuccess) return cuda_fail(e, "rk4_f32 launch (static scratch)");
  return MR_OK;
}
