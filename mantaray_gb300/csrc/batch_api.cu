// batch_api.cu -- C ABI of the batched FP32 form (include/mantaray_gpu.h):
// scenario packing, device-buffer tracing, and CUDA-graph replay.

#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/mantaray_gpu.h"
#include "batch.h"
#include "batch_handle.h"
#include "handles.h"
#include "kernels.h"


struct mr_batch_graph {
  mr_batch *batch = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t kernel_node = nullptr;   // the batched kernel
  cudaKernelNodeParams params{};
  mr::BatchArgs args{};
  cudaGraphNode_t order_node = nullptr;    // order_keys, when the rays are ordered
  cudaKernelNodeParams order_params{};
  mr::OrderArgs oargs{};
  mr_order_buffers ord;                    // the graph's own ordering scratch
  size_t n_max = 0;
  bool sweep = false;                      // the sweep form: every launch reads n from the device
};

namespace {

using mr::cuda_fail;
using mr::DeviceGuard;
using mr::fail;

int pack_bathy(mr_batch *b, const mr_bathymetry *h, mr::PackedGrid *g, cudaStream_t s) {
  if (h->dev.kind != mr::BATHY_GRID)
    return fail(MR_ERR_INVALID_ARGUMENT, "the batched form needs gridded bathymetry");
  if (h->one_point_axis)
    return fail(MR_ERR_INVALID_ARGUMENT, "a bathymetry axis has a single point");
  if (!(h->dev.xspace > 0.0) || !(h->dev.yspace > 0.0))
    return fail(MR_ERR_INVALID_ARGUMENT, "the batched form needs ascending, evenly spaced axes");
  const size_t ncell = (h->dev.nx - 1) * (h->dev.ny - 1);
  if (ncell > 0x7fffffffull)
    return fail(MR_ERR_INVALID_ARGUMENT, "the batched form indexes fewer than 2^31 cells");
  void *cells = nullptr;
  MR_CUDA(cudaMalloc(&cells, ncell * 2 * sizeof(float4)));
  b->mem.push_back(cells);
  MR_CUDA(mr::launch_pack_bathy(h->dev, static_cast<float4 *>(cells), s));
  g->cells = static_cast<const float4 *>(cells);
  g->nx = static_cast<int>(h->dev.nx);
  g->ny = static_cast<int>(h->dev.ny);
  g->x0 = static_cast<double>(h->dev.x0);
  g->y0 = static_cast<double>(h->dev.y0);
  g->sp_x = h->dev.xspace;
  g->sp_y = h->dev.yspace;
  g->inv_sp_x = static_cast<float>(1.0 / h->dev.xspace);
  g->inv_sp_y = static_cast<float>(1.0 / h->dev.yspace);
  g->inv_sp_xd = 1.0 / h->dev.xspace;
  g->inv_sp_yd = 1.0 / h->dev.yspace;
  g->kind = 0;
  return MR_OK;
}

int pack_current(mr_batch *b, const mr_current *c, mr::PackedGrid *g, cudaStream_t s) {
  if (c->dev.kind == mr::CURRENT_CONSTANT) {
    g->kind = 1;
    g->cu = static_cast<float>(c->dev.cu);
    g->cv = static_cast<float>(c->dev.cv);
    g->cells = nullptr;
    g->nx = g->ny = 2;
    g->x0 = g->y0 = 0.0;
    g->sp_x = g->sp_y = 1.0;
    g->inv_sp_x = g->inv_sp_y = 1.0f;
    g->inv_sp_xd = g->inv_sp_yd = 1.0;
    return MR_OK;
  }
  if (c->one_point_axis) return fail(MR_ERR_INVALID_ARGUMENT, "a current axis has a single point");
  if (!(c->dev.xspace > 0.0) || !(c->dev.yspace > 0.0))
    return fail(MR_ERR_INVALID_ARGUMENT, "the batched form needs ascending, evenly spaced axes");
  const size_t ncell = (c->dev.nx - 1) * (c->dev.ny - 1);
  if (ncell > 0x7fffffffull)
    return fail(MR_ERR_INVALID_ARGUMENT, "the batched form indexes fewer than 2^31 cells");
  void *cells = nullptr;
  MR_CUDA(cudaMalloc(&cells, ncell * 3 * sizeof(float4)));
  b->mem.push_back(cells);
  MR_CUDA(mr::launch_pack_current(c->dev, static_cast<float4 *>(cells), s));
  g->cells = static_cast<const float4 *>(cells);
  g->nx = static_cast<int>(c->dev.nx);
  g->ny = static_cast<int>(c->dev.ny);
  g->x0 = c->dev.x0;
  g->y0 = c->dev.y0;
  g->sp_x = c->dev.xspace;
  g->sp_y = c->dev.yspace;
  g->inv_sp_x = static_cast<float>(1.0 / c->dev.xspace);
  g->inv_sp_y = static_cast<float>(1.0 / c->dev.yspace);
  g->inv_sp_xd = 1.0 / c->dev.xspace;
  g->inv_sp_yd = 1.0 / c->dev.yspace;
  g->kind = 0;
  return MR_OK;
}

// A tensor map of a packed cell array (ny-1 rows of nx-1 cells of
// `floats` FP32 values) with boxes of kTileCells x kTileCells cells, for the
// tile build's copies.  cuTensorMapEncodeTiled comes from the driver through
// the runtime's entry-point query (the library links no driver library).
int encode_cells(CUtensorMap *m, const float4 *cells, int nx, int ny, int floats) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      fn = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return fail(MR_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[3] = {static_cast<cuuint64_t>(floats), static_cast<cuuint64_t>(nx - 1),
                              static_cast<cuuint64_t>(ny - 1)};
  const cuuint64_t strides[2] = {static_cast<cuuint64_t>(floats) * 4,
                                 static_cast<cuuint64_t>(nx - 1) * floats * 4};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>(floats), mr::kTileCells, mr::kTileCells};
  const cuuint32_t step[3] = {1, 1, 1};
  const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                            const_cast<float4 *>(cells), dims, strides, box, step,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(MR_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", int(r));
  return MR_OK;
}

void order_free(mr_order_buffers *o) {
  if (o->mem) cudaFree(o->mem);
  if (o->sweep_mem) cudaFree(o->sweep_mem);
  *o = mr_order_buffers();
}

// Makes the sweep scratch hold at least n rays (the ordering scratch is
// reserved separately; cudaFree waits for work that still uses the old one).
cudaError_t sweep_reserve(mr_order_buffers *o, size_t n) {
  if (n <= o->sweep_cap && o->sweep_mem) return cudaSuccess;
  if (o->sweep_mem) cudaFree(o->sweep_mem);
  o->sweep_mem = nullptr;
  o->sweep_cap = 0;
  auto up = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
  const size_t states = up(n * sizeof(mr::SweepRay)), keys = up(n * sizeof(uint64_t));
  char *p = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p),
                             256 + states + keys + up(n * sizeof(uint32_t)));
  if (e != cudaSuccess) return e;
  o->sweep_mem = p;
  o->sweep_cap = n;
  o->count = reinterpret_cast<unsigned long long *>(p);
  o->sweep = reinterpret_cast<mr::SweepRay *>(p + 256);
  o->list_keys = reinterpret_cast<uint64_t *>(p + 256 + states);
  o->list = reinterpret_cast<uint32_t *>(p + 256 + states + keys);
  return cudaSuccess;
}

// Makes the ordering scratch hold at least n rays (the old contents are not
// kept; cudaFree waits for work that still uses them).
cudaError_t order_reserve(mr_order_buffers *o, size_t n) {
  if (n <= o->cap && o->mem) return cudaSuccess;
  order_free(o);
  const int tiles = mr::order_tiles(static_cast<int64_t>(n));
  auto up = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
  const size_t keys = up(n * sizeof(uint64_t)), vals = up(n * sizeof(uint32_t));
  const size_t counts = up(256ull * tiles * sizeof(uint32_t));
  char *p = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p),
                             256 + 2 * keys + 2 * vals + counts + 256 * sizeof(uint32_t));
  if (e != cudaSuccess) return e;
  o->mem = p;
  o->cap = n;
  o->tiles = tiles;
  o->n_dev = reinterpret_cast<int64_t *>(p);
  o->keys[0] = reinterpret_cast<uint64_t *>(p + 256);
  o->keys[1] = reinterpret_cast<uint64_t *>(p + 256 + keys);
  o->vals[0] = reinterpret_cast<uint32_t *>(p + 256 + 2 * keys);
  o->vals[1] = reinterpret_cast<uint32_t *>(p + 256 + 2 * keys + vals);
  o->counts = reinterpret_cast<uint32_t *>(p + 256 + 2 * keys + 2 * vals);
  o->totals = reinterpret_cast<uint32_t *>(p + 256 + 2 * keys + 2 * vals + counts);
  return cudaSuccess;
}

mr::OrderArgs order_args(const mr_batch *b, const mr::BatchArgs &a, const mr_order_buffers &o) {
  mr::OrderArgs r{};
  r.scen = a.scen;
  r.n_scenarios = a.n_scenarios;
  r.ray_scenario = a.ray_scenario;
  r.x0 = a.x0; r.y0 = a.y0; r.kx0 = a.kx0; r.ky0 = a.ky0;
  r.n = a.n;
  r.n_dev = o.n_dev;
  r.keys[0] = o.keys[0]; r.keys[1] = o.keys[1];
  r.vals[0] = o.vals[0]; r.vals[1] = o.vals[1];
  r.counts = o.counts;
  r.totals = o.totals;
  r.tiles = o.tiles;
  r.scen_shift = b->order_scen_shift;
  return r;
}

int check_config(const mr_batch_config *cfg) {
  if (!cfg) return fail(MR_ERR_INVALID_ARGUMENT, "null config");
  if (cfg->block < 32 || cfg->block > 256 || cfg->block % 32)
    return fail(MR_ERR_INVALID_ARGUMENT, "block must be a multiple of 32 in [32, 256]");
  if (cfg->blocks_per_sm < 1 || cfg->blocks_per_sm > 32)
    return fail(MR_ERR_INVALID_ARGUMENT, "blocks_per_sm must be in [1, 32]");
  if (cfg->rays_per_lane != 1 && cfg->rays_per_lane != 2)
    return fail(MR_ERR_INVALID_ARGUMENT, "rays_per_lane must be 1 or 2");
  if (cfg->rebase_interval < 1)
    return fail(MR_ERR_INVALID_ARGUMENT, "rebase_interval must be >= 1");
  if (cfg->order != 0 && cfg->order != 1)
    return fail(MR_ERR_INVALID_ARGUMENT, "order must be 0 or 1");
  if (cfg->staging < MR_STAGING_NONE || cfg->staging > MR_STAGING_AHEAD)
    return fail(MR_ERR_INVALID_ARGUMENT, "staging must be 0, 1 or 2");
  if (cfg->staging && cfg->rays_per_lane != 1)
    return fail(MR_ERR_INVALID_ARGUMENT, "staging traces one ray per lane");
  if (cfg->sweep_steps < 0) return fail(MR_ERR_INVALID_ARGUMENT, "sweep_steps must be >= 0");
  if (cfg->sweep_steps > 0 && (cfg->order != 1 || cfg->rays_per_lane != 1 || cfg->staging))
    return fail(MR_ERR_INVALID_ARGUMENT,
                "sweeps need order = 1, one ray per lane and no staging");
  return MR_OK;
}

// The device address of an output buffer: device memory as given,
// page-locked host memory through its device mapping; null for pageable host
// memory (not writable from the kernel).
template <typename T>
T *device_view(T *p) {
  if (!p) return p;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return p;
  if (attr.type == cudaMemoryTypeHost && attr.devicePointer)
    return static_cast<T *>(attr.devicePointer);
  return nullptr;
}

int fill_args(mr_batch *b, size_t n, size_t n_stride, const uint8_t *ray_scenario,
              const double *x0, const double *y0, const double *kx0, const double *ky0, double t0,
              double dt, int64_t max_steps, int64_t decimation, size_t save_cap, float *saved,
              double *end_state, int32_t *n_steps, int32_t *n_saved, uint8_t *status,
              const mr_batch_config *cfg, mr::BatchArgs *a) {
  if (!b) return fail(MR_ERR_INVALID_ARGUMENT, "null batch");
  int rc = check_config(cfg);
  if (rc) return rc;
  if (n > n_stride) return fail(MR_ERR_INVALID_ARGUMENT, "n exceeds the buffers' capacity");
  if (cfg->order && n_stride > 0xffffffffull)
    return fail(MR_ERR_INVALID_ARGUMENT, "ray ordering handles at most 2^32 - 1 rays per call");
  if (n_stride > 0 && (!x0 || !y0 || !kx0 || !ky0 || !end_state || !n_steps || !n_saved || !status))
    return fail(MR_ERR_INVALID_ARGUMENT, "null array argument");
  if (decimation < 0 || max_steps < 0 || max_steps >= INT32_MAX)
    return fail(MR_ERR_INVALID_ARGUMENT, "bad max_steps or decimation");
  if (decimation > 0) {
    if (!saved) return fail(MR_ERR_INVALID_ARGUMENT, "null saved buffer with decimation > 0");
    if (static_cast<int64_t>(save_cap) < max_steps / decimation + 1)
      return fail(MR_ERR_CAPACITY, "save_cap %zu < max_steps / decimation + 1 = %lld", save_cap,
                  static_cast<long long>(max_steps / decimation + 1));
  }
  if (!(dt > 0.0) || !isfinite(t0)) return fail(MR_ERR_INVALID_ARGUMENT, "dt must be > 0");
  if (cfg->staging == MR_STAGING_TILE && !b->has_tmaps)
    return fail(MR_ERR_INVALID_ARGUMENT,
                "tile staging needs one scenario with its current gridded on the bathymetry's "
                "grid");
  if (cfg->staging == MR_STAGING_AHEAD && !all_same_grid(b))
    return fail(MR_ERR_INVALID_ARGUMENT,
                "staging ahead needs every scenario's current gridded on its bathymetry's grid");
  a->staging = cfg->staging;
  if (b->has_tmaps) {
    a->tmap_bathy = b->tmap_bathy;
    a->tmap_current = b->tmap_current;
  }
  a->scen = b->scen;
  a->scen0 = b->host_scen[0];
  a->all_same_grid = all_same_grid(b);
  a->n_scenarios = b->n_scenarios;
  a->ray_scenario = ray_scenario;
  a->n = static_cast<int64_t>(n);
  a->x0 = x0; a->y0 = y0; a->kx0 = kx0; a->ky0 = ky0;
  a->t0 = t0;
  a->dt = dt;
  a->dt_f = static_cast<float>(dt);
  a->half_f = 0.5f * a->dt_f;
  a->sixth_f = a->dt_f * (1.0f / 6.0f);
  a->max_steps = max_steps;
  a->decimation = decimation;
  a->save_cap = static_cast<int64_t>(save_cap);
  a->n_stride = static_cast<int64_t>(n_stride);
  a->rebase_interval = cfg->rebase_interval;
  // outputs: device memory or page-locked host memory (written in place)
  a->saved = decimation > 0 ? device_view(saved) : saved;
  a->end_state = device_view(end_state);
  a->n_steps = device_view(n_steps);
  a->n_saved = device_view(n_saved);
  a->status = device_view(status);
  if (n_stride > 0 && (!a->end_state || !a->n_steps || !a->n_saved || !a->status ||
                       (decimation > 0 && !a->saved)))
    return fail(MR_ERR_INVALID_ARGUMENT,
                "outputs must be device memory or page-locked host memory");
  a->queue = b->queue;
  return MR_OK;
}

// Stream work of one batched call: reset the queue, NaN-fill the saved rows
// (rows a ray does not reach stay NaN, as the reference pads them), order
// the rays when cfg->order (into `ord`, sized for n_stride rays), launch.
// The sweep form launches ceil(max_steps / sweep_steps) times (at least
// once), the running rays listed, counted and re-ordered between launches,
// all on the stream: the host never waits.  *a gets the arguments of the
// (first) launch.
cudaError_t enqueue(const mr_batch *b, mr::BatchArgs *a, const mr_batch_config *cfg,
                    const mr_order_buffers *ord, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a->queue, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (a->decimation > 0 && a->save_cap > 0) {
    e = mr::launch_fill_nan(a->saved, 5 * a->save_cap * a->n_stride, s);
    if (e != cudaSuccess) return e;
  }
  a->order = nullptr;
  mr::OrderArgs o{};
  if (cfg->order) {
    o = order_args(b, *a, *ord);
    e = mr::launch_order(o, a->n_stride, b->order_passes, s);
    if (e != cudaSuccess) return e;
    a->order = ord->vals[b->order_passes & 1];
  }
  if (cfg->sweep_steps <= 0)
    return mr::launch_rk4_f32(*a, cfg->block, cfg->blocks_per_sm, cfg->rays_per_lane, s);
  e = cudaMemsetAsync(ord->count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  a->sweep_steps = cfg->sweep_steps;
  a->sweep_first = 1;
  a->sweep_cell_bits = b->sweep_cell_bits;
  a->sweep_key_shift = b->sweep_key_shift;
  a->sweep = ord->sweep;
  a->next_list = ord->list;
  a->next_keys = ord->list_keys;
  a->next_count = ord->count;
  a->n_dev = ord->n_dev;
  e = mr::launch_rk4_f32(*a, cfg->block, cfg->blocks_per_sm, cfg->rays_per_lane, s);
  if (e != cudaSuccess) return e;
  // later launches: the list sorted by the keys the kernel wrote
  mr::BatchArgs later = *a;
  later.sweep_first = 0;
  later.order = ord->vals[b->sweep_passes & 1];
  mr::OrderArgs ol = o;
  ol.in_keys = ord->list_keys;
  ol.in_vals = ord->list;
  const int64_t sweeps = (a->max_steps + cfg->sweep_steps - 1) / cfg->sweep_steps;
  for (int64_t k = 1; k < sweeps; ++k) {
    e = mr::launch_sweep_next(ord->n_dev, ord->count, a->queue, s);
    if (e == cudaSuccess) e = mr::launch_order(ol, a->n_stride, b->sweep_passes, s);
    if (e == cudaSuccess)
      e = mr::launch_rk4_f32(later, cfg->block, cfg->blocks_per_sm, cfg->rays_per_lane, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

namespace mr {

int batch_fill_args(mr_batch *b, size_t n, size_t n_stride, const uint8_t *ray_scenario,
                    const double *x0, const double *y0, const double *kx0, const double *ky0,
                    double t0, double dt, int64_t max_steps, int64_t decimation,
                    size_t save_cap, float *saved, double *end_state, int32_t *n_steps,
                    int32_t *n_saved, uint8_t *status, const mr_batch_config *cfg,
                    BatchArgs *a) {
  return fill_args(b, n, n_stride, ray_scenario, x0, y0, kx0, ky0, t0, dt, max_steps,
                   decimation, save_cap, saved, end_state, n_steps, n_saved, status, cfg, a);
}

}  // namespace mr

extern "C" {

int mr_batch_default_config(mr_batch_config *cfg) {
  if (!cfg) return fail(MR_ERR_INVALID_ARGUMENT, "null config");
  cfg->block = 128;
  cfg->blocks_per_sm = 4;
  cfg->rays_per_lane = 1;
  cfg->rebase_interval = 32;
  cfg->order = 0;
  cfg->staging = MR_STAGING_NONE;
  return MR_OK;
}

int mr_batch_create(size_t n_scenarios, const mr_bathymetry *const *bathy,
                    const mr_current *const *current, mr_batch **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  *out = nullptr;
  if (n_scenarios == 0 || n_scenarios > 256 || !bathy || !current)
    return fail(MR_ERR_INVALID_ARGUMENT, "1 to 256 scenarios are needed");
  for (size_t i = 0; i < n_scenarios; ++i) {
    if (!bathy[i] || !current[i]) return fail(MR_ERR_INVALID_ARGUMENT, "null field handle");
    if (bathy[i]->device != bathy[0]->device || current[i]->device != bathy[0]->device)
      return fail(MR_ERR_INVALID_ARGUMENT, "fields live on different devices");
  }
  DeviceGuard g(bathy[0]->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the fields' device");
  mr_batch *b = new mr_batch();
  b->device = bathy[0]->device;
  b->n_scenarios = static_cast<int>(n_scenarios);
  b->host_scen.resize(n_scenarios);
  cudaStream_t s = cudaStreamPerThread;
  int rc = MR_OK;
  for (size_t i = 0; i < n_scenarios && rc == MR_OK; ++i) {
    rc = pack_bathy(b, bathy[i], &b->host_scen[i].bathy, s);
    if (rc == MR_OK) rc = pack_current(b, current[i], &b->host_scen[i].current, s);
    if (rc == MR_OK) {
      const mr::PackedGrid &gb = b->host_scen[i].bathy, &gc = b->host_scen[i].current;
      b->host_scen[i].same_grid =
          gc.kind == 0 && gb.nx == gc.nx && gb.ny == gc.ny && gb.x0 == gc.x0 &&
          gb.y0 == gc.y0 && gb.sp_x == gc.sp_x && gb.sp_y == gc.sp_y &&
          gb.inv_sp_x == gc.inv_sp_x && gb.inv_sp_y == gc.inv_sp_y &&
          gb.inv_sp_xd == gc.inv_sp_xd && gb.inv_sp_yd == gc.inv_sp_yd;
    }
  }
  cudaError_t e = cudaSuccess;
  if (rc == MR_OK) e = cudaMalloc(reinterpret_cast<void **>(&b->scen), n_scenarios * sizeof(mr::ScenarioDev));
  if (rc == MR_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(b->scen, b->host_scen.data(), n_scenarios * sizeof(mr::ScenarioDev),
                        cudaMemcpyHostToDevice, s);
  if (rc == MR_OK && e == cudaSuccess)
    e = cudaMalloc(reinterpret_cast<void **>(&b->queue), sizeof(unsigned long long));
  if (rc == MR_OK) {
    // ordering key: direction in bits 0-7, the Morton code of the starting
    // cell (cbits per axis) above it, the scenario above that
    int cmax = 1;
    for (const auto &sc : b->host_scen)
      cmax = std::max(cmax, std::max(sc.bathy.nx - 1, sc.bathy.ny - 1));
    int cbits = 0;
    while (cbits < 16 && (1 << cbits) < cmax) ++cbits;
    int sbits = 0;
    while ((1 << sbits) < b->n_scenarios) ++sbits;
    b->order_scen_shift = 8 + 2 * cbits;
    b->order_passes = (b->order_scen_shift + sbits + 7) / 8;
    // the sweep form's key: the Morton code of the 2 x 2-cell block (no
    // direction), the scenario above it
    int bbits = 0;
    while (bbits < 15 && (1 << bbits) < (cmax + 1) / 2) ++bbits;
    b->sweep_cell_bits = bbits;
    b->sweep_key_shift = 2 * bbits;
    b->sweep_passes = std::max(1, (2 * bbits + sbits + 7) / 8);
  }
  if (rc == MR_OK && e == cudaSuccess && n_scenarios == 1 && b->host_scen[0].same_grid) {
    const mr::ScenarioDev &sc = b->host_scen[0];
    rc = encode_cells(&b->tmap_bathy, sc.bathy.cells, sc.bathy.nx, sc.bathy.ny, 8);
    if (rc == MR_OK)
      rc = encode_cells(&b->tmap_current, sc.current.cells, sc.current.nx, sc.current.ny, 12);
    // without the driver's encoder the batch still traces, without tiles
    if (rc != MR_OK) rc = MR_OK;
    else b->has_tmaps = true;
  }
  if (rc == MR_OK && e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (rc == MR_OK && e != cudaSuccess) rc = cuda_fail(e, "building the batched scenarios");
  if (rc != MR_OK) {
    mr_batch_destroy(b);
    return rc;
  }
  *out = b;
  return MR_OK;
}

void mr_batch_destroy(mr_batch *b) {
  if (!b) return;
  DeviceGuard g(b->device);
  for (void *p : b->mem) cudaFree(p);
  if (b->scen) cudaFree(b->scen);
  if (b->queue) cudaFree(b->queue);
  order_free(&b->ord);
  delete b;
}

int mr_batch_trace_device(mr_batch *b, size_t n, const uint8_t *ray_scenario, const double *x0,
                          const double *y0, const double *kx0, const double *ky0, double t0,
                          double dt, int64_t max_steps, int64_t decimation, size_t save_cap,
                          float *saved, double *end_state, int32_t *n_steps, int32_t *n_saved,
                          uint8_t *status, const mr_batch_config *cfg, void *stream) {
  mr::BatchArgs a{};
  int rc = fill_args(b, n, n, ray_scenario, x0, y0, kx0, ky0, t0, dt, max_steps, decimation,
                     save_cap, saved, end_state, n_steps, n_saved, status, cfg, &a);
  if (rc) return rc;
  if (n == 0) return MR_OK;
  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the batch's device");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  cudaError_t e = cudaSuccess;
  if (cfg->order) {
    // the scratch may be in use by earlier calls on this stream: order them first
    if (n > b->ord.cap || (cfg->sweep_steps > 0 && n > b->ord.sweep_cap))
      e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = order_reserve(&b->ord, n);
    if (e == cudaSuccess && cfg->sweep_steps > 0) e = sweep_reserve(&b->ord, n);
    if (e != cudaSuccess) return cuda_fail(e, "ordering scratch");
  }
  e = enqueue(b, &a, cfg, &b->ord, s);
  if (e != cudaSuccess) return cuda_fail(e, "rk4_f32 launch");
  return MR_OK;
}

int mr_batch_graph_create(mr_batch *b, size_t n_max, const uint8_t *ray_scenario,
                          const double *x0, const double *y0, const double *kx0,
                          const double *ky0, double t0, double dt, int64_t max_steps,
                          int64_t decimation, size_t save_cap, float *saved, double *end_state,
                          int32_t *n_steps, int32_t *n_saved, uint8_t *status,
                          const mr_batch_config *cfg, mr_batch_graph **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  *out = nullptr;
  mr::BatchArgs a{};
  int rc = fill_args(b, n_max, n_max, ray_scenario, x0, y0, kx0, ky0, t0, dt, max_steps,
                     decimation, save_cap, saved, end_state, n_steps, n_saved, status, cfg, &a);
  if (rc) return rc;
  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the batch's device");
  mr_batch_graph *gr = new mr_batch_graph();
  gr->batch = b;
  gr->args = a;
  gr->n_max = n_max;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaSuccess;
  gr->sweep = cfg->sweep_steps > 0;
  if (cfg->order) {
    e = order_reserve(&gr->ord, n_max);
    if (e == cudaSuccess && gr->sweep) e = sweep_reserve(&gr->ord, n_max);
    gr->oargs = order_args(b, a, gr->ord);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  // the integrator build for this shape, chosen (an occupancy query) before
  // the capture begins
  const void *k2 = mr::rk4_f32_function(cfg->rays_per_lane, cfg->block, cfg->blocks_per_sm,
                                        b->n_scenarios, all_same_grid(b), cfg->staging,
                                        gr->sweep);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    // the kernel node's arguments as captured (queue order included), for
    // the launches that change n
    cudaError_t le = enqueue(b, &gr->args, cfg, &gr->ord, s);
    e = cudaStreamEndCapture(s, &gr->graph);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&gr->exec, gr->graph, 0);
  size_t count = 0;
  if (e == cudaSuccess) e = cudaGraphGetNodes(gr->graph, nullptr, &count);
  std::vector<cudaGraphNode_t> nodes(count);
  if (e == cudaSuccess && count) e = cudaGraphGetNodes(gr->graph, nodes.data(), &count);
  for (size_t i = 0; e == cudaSuccess && i < count; ++i) {
    cudaGraphNodeType type;
    e = cudaGraphNodeGetType(nodes[i], &type);
    if (e == cudaSuccess && type == cudaGraphNodeTypeKernel) {
      cudaKernelNodeParams p{};
      e = cudaGraphKernelNodeGetParams(nodes[i], &p);
      if (e != cudaSuccess) break;
      // the ordering of the call's rays (a sweep form's later orderings
      // sort the keys its kernel wrote: no order_keys)
      if (p.func == mr::order_keys_function()) {
        gr->order_node = nodes[i];
        gr->order_params = p;
      } else if (p.func == k2 && !gr->kernel_node) {
        gr->kernel_node = nodes[i];
        gr->params = p;
      }
    }
  }
  if (e == cudaSuccess && cfg->order && !gr->order_node) e = cudaErrorInvalidValue;
  if (s) cudaStreamDestroy(s);
  if (e == cudaSuccess && !gr->kernel_node) e = cudaErrorInvalidValue;
  if (e != cudaSuccess) {
    mr_batch_graph_destroy(gr);
    return cuda_fail(e, "capturing the batched graph");
  }
  *out = gr;
  return MR_OK;
}

int mr_batch_graph_launch(mr_batch_graph *gr, size_t n, void *stream) {
  if (!gr) return fail(MR_ERR_INVALID_ARGUMENT, "null graph");
  if (n > gr->n_max) return fail(MR_ERR_CAPACITY, "n %zu exceeds the graph's capacity %zu", n, gr->n_max);
  DeviceGuard g(gr->batch->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the batch's device");
  // n is a kernel argument: the executable graph's kernel node takes the new
  // value for this and later launches (launches already queued keep theirs).
  // (The sweep form's launches read n from the device, where the first
  // ordering kernel puts it.)
  gr->args.n = static_cast<int64_t>(n);
  void *kargs[1] = {&gr->args};
  cudaKernelNodeParams p = gr->params;
  p.kernelParams = kargs;
  p.extra = nullptr;
  cudaError_t e = cudaSuccess;
  if (!gr->sweep) e = cudaGraphExecKernelNodeSetParams(gr->exec, gr->kernel_node, &p);
  if (e == cudaSuccess && gr->order_node) {
    gr->oargs.n = static_cast<int64_t>(n);
    void *oargs[1] = {&gr->oargs};
    cudaKernelNodeParams q = gr->order_params;
    q.kernelParams = oargs;
    q.extra = nullptr;
    e = cudaGraphExecKernelNodeSetParams(gr->exec, gr->order_node, &q);
  }
  if (e == cudaSuccess)
    e = cudaGraphLaunch(gr->exec, stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread);
  if (e != cudaSuccess) return cuda_fail(e, "launching the batched graph");
  return MR_OK;
}

void mr_batch_graph_destroy(mr_batch_graph *gr) {
  if (!gr) return;
  DeviceGuard g(gr->batch ? gr->batch->device : 0);
  if (gr->exec) cudaGraphExecDestroy(gr->exec);
  if (gr->graph) cudaGraphDestroy(gr->graph);
  order_free(&gr->ord);
  delete gr;
}

}  // extern "C"
