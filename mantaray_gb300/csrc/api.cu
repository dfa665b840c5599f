// api.cu -- the C ABI of libmantaray_gpu.so (include/mantaray_gpu.h).
//
// Host side of the drop-in: field handles staged once into HBM, argument
// checking, the reference's step count, launches of the plain FP64 kernel,
// and the file-path entry points of src/ffi.rs.

#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mantaray_gpu.h"
#include "fields.h"
#include "handles.h"
#include "kernels.h"
#include "netcdf3.h"

namespace mr {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(e == cudaErrorMemoryAllocation ? MR_ERR_OUT_OF_MEMORY : MR_ERR_CUDA, "%s: %s (%s)",
              what, cudaGetErrorString(e), cudaGetErrorName(e));
}

}  // namespace mr

using mr::cuda_fail;
using mr::DeviceGuard;
using mr::fail;

namespace {

// Device copy of a host array, owned (and freed) by the handle.
template <typename T>
cudaError_t upload(const T *src, size_t count, std::vector<void *> *owner, const T **dst) {
  *dst = nullptr;
  if (count == 0) return cudaSuccess;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T));
  if (e != cudaSuccess) return e;
  owner->push_back(p);
  *dst = static_cast<const T *>(p);
  return cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice);
}

void free_mem(std::vector<void *> &mem) {
  for (void *p : mem) cudaFree(p);
  mem.clear();
}

constexpr int kOptionsMask = MR_STOP_FRESH | MR_MATH_LIBM;
// Options of the reference-shaped entry points (mr_single_ray, the file
// forms): the default arithmetic, within 1e-9 of the reference like libm's.
constexpr int kDropInOptions = MR_STOP_STAGE1 | MR_MATH_IDENTITY;

// Keep freed stream-ordered allocations pooled across calls (set once per
// device); mr_trace's staging buffers are then reused instead of remapped.
void keep_pool(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lock(mu);
  for (int d : done)
    if (d == device) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t threshold = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  done.push_back(device);
}

uint64_t rust_ceil_as_usize(double v) {
  const double c = ceil(v);
  if (!(c > 0.0)) return 0;
  if (c >= 18446744073709551616.0) return UINT64_MAX;
  return static_cast<uint64_t>(c);
}

int check_trace_args(const mr_bathymetry *b, const mr_current *c, size_t n, const void *x0,
                     const void *y0, const void *kx0, const void *ky0, double t0, double t_end,
                     double dt, int options, size_t rows_cap, const void *traj,
                     const void *n_rows, const void *status, uint64_t *nsteps) {
  if (!b || !c) return fail(MR_ERR_INVALID_ARGUMENT, "null field handle");
  if (b->one_point_axis || c->one_point_axis)
    return fail(MR_ERR_INVALID_ARGUMENT,
                "a grid axis has a single point (the reference panics on its first lookup)");
  if (b->device != c->device)
    return fail(MR_ERR_INVALID_ARGUMENT, "bathymetry and current live on different devices");
  if (options & ~kOptionsMask)
    return fail(MR_ERR_INVALID_ARGUMENT, "unknown option bits 0x%x", options & ~kOptionsMask);
  if (n > 0 && (!x0 || !y0 || !kx0 || !ky0 || !traj || !n_rows || !status))
    return fail(MR_ERR_INVALID_ARGUMENT, "null array argument");
  *nsteps = mr_num_steps(t0, t_end, dt);
  if (*nsteps >= static_cast<uint64_t>(INT32_MAX))
    return fail(MR_ERR_CAPACITY, "%llu steps exceed the row counter range",
                static_cast<unsigned long long>(*nsteps));
  if (rows_cap < *nsteps + 1)
    return fail(MR_ERR_CAPACITY, "rows_cap %zu < %llu steps + 1", rows_cap,
                static_cast<unsigned long long>(*nsteps));
  return MR_OK;
}

// Device-visible alias of a host buffer when it is page-locked, else null.
void *mapped_host(void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (attr.type == cudaMemoryTypeHost && attr.devicePointer) return attr.devicePointer;
  return nullptr;
}

void fill_bathy_grid_scalars(mr_bathymetry *h, const float *x, const float *y, size_t nx,
                             size_t ny) {
  mr::BathyDev &d = h->dev;
  d.nx = nx;
  d.ny = ny;
  h->one_point_axis = nx < 2 || ny < 2;
  if (h->one_point_axis) return;
  // nearest(), cartesian_netcdf3.rs:287-291 (f32)
  d.x0 = x[0];
  d.xsp = fabsf(x[1] - x[0]);
  d.xhigh = static_cast<float>(nx - 1);
  d.y0 = y[0];
  d.ysp = fabsf(y[1] - y[0]);
  d.yhigh = static_cast<float>(ny - 1);
  // gradient spacing, cartesian_netcdf3.rs:119-120 (f64)
  d.xspace = static_cast<double>(x[1]) - static_cast<double>(x[0]);
  d.yspace = static_cast<double>(y[1]) - static_cast<double>(y[0]);
}

int make_bathy_grid(size_t nx, size_t ny, const float *x, const float *y, const double *depth,
                    size_t depth_len, mr_bathymetry **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  *out = nullptr;
  if (nx == 0 || ny == 0 || !x || !y || (depth_len && !depth))
    return fail(MR_ERR_INVALID_ARGUMENT, "empty axis or null array");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_bathymetry *h = new mr_bathymetry();
  h->dev.kind = mr::BATHY_GRID;
  h->device = device;
  fill_bathy_grid_scalars(h, x, y, nx, ny);
  // Tables (fields.h): depth as f32, and the f32 cell gradients of
  // cartesian_netcdf3.rs:119-134 for every cell whose corners are in range.
  std::vector<float> d32(depth_len), gx(depth_len, 0.0f), gy(depth_len, 0.0f);
  for (size_t i = 0; i < depth_len; ++i) d32[i] = static_cast<float>(depth[i]);
  if (!h->one_point_axis) {
    for (size_t j = 0; j + 1 < ny; ++j) {
      for (size_t i = 0; i + 1 < nx; ++i) {
        const size_t sw = nx * j + i;
        if (nx * (j + 1) + i + 1 >= depth_len) continue;
        gx[sw] = static_cast<float>((depth[sw + 1] - depth[sw]) / h->dev.xspace);
        gy[sw] = static_cast<float>((depth[sw + nx] - depth[sw]) / h->dev.yspace);
      }
    }
  }
  cudaError_t e;
  if ((e = upload(x, nx, &h->mem, &h->dev.x)) != cudaSuccess ||
      (e = upload(y, ny, &h->mem, &h->dev.y)) != cudaSuccess ||
      (e = upload(depth, depth_len, &h->mem, &h->dev.depth)) != cudaSuccess ||
      (e = upload(d32.data(), depth_len, &h->mem, &h->dev.depth32)) != cudaSuccess ||
      (e = upload(gx.data(), depth_len, &h->mem, &h->dev.gx)) != cudaSuccess ||
      (e = upload(gy.data(), depth_len, &h->mem, &h->dev.gy)) != cudaSuccess) {
    free_mem(h->mem);
    delete h;
    return cuda_fail(e, "staging bathymetry grid");
  }
  h->dev.depth_len = depth_len;
  *out = h;
  return MR_OK;
}

// Cell thresholds of one current axis (fields.h): thr[j] = key of the smallest
// double t with idx(t) >= j (j < n), thr[n] = key of the smallest t with
// idx(t) > n - 1, where idx(t) = (t - a0) / sp exactly as
// cartesian_current.rs:244-246 computes it.  idx is non-decreasing in t
// (rounded subtraction and division by sp > 0 are monotone), so each
// threshold is found by bisection over the ordered keys from -inf to +inf,
// where idx(+inf) = +inf satisfies every predicate.
std::vector<long long> current_axis_thresholds(double a0, double sp, size_t n) {
  auto value = [](long long key) {
    const long long bits = mr::order_key_bits(key);  // the key map is an involution
    double t;
    std::memcpy(&t, &bits, sizeof t);
    return t;
  };
  auto key_of = [](double t) {
    long long bits;
    std::memcpy(&bits, &t, sizeof bits);
    return mr::order_key_bits(bits);
  };
  const double high = static_cast<double>(n - 1);
  std::vector<long long> thr(n + 1);
  for (size_t j = 0; j <= n; ++j) {
    const bool strict = j == n;
    const double bound = strict ? high : static_cast<double>(j);
    long long lo = key_of(-INFINITY), hi = key_of(INFINITY);
    while (lo < hi) {
      const long long mid =
          lo + static_cast<long long>((static_cast<unsigned long long>(hi) -
                                       static_cast<unsigned long long>(lo)) / 2);
      const double idx = (value(mid) - a0) / sp;
      if (strict ? idx > bound : idx >= bound)
        hi = mid;
      else
        lo = mid + 1;
    }
    thr[j] = lo;
  }
  return thr;
}

int make_current_grid(size_t nx, size_t ny, const double *x, const double *y, const double *u,
                      size_t u_len, const double *v, size_t v_len, mr_current **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  *out = nullptr;
  if (nx == 0 || ny == 0 || !x || !y || (u_len && !u) || (v_len && !v))
    return fail(MR_ERR_INVALID_ARGUMENT, "empty axis or null array");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_current *h = new mr_current();
  h->dev.kind = mr::CURRENT_GRID;
  h->device = device;
  mr::CurrentDev &d = h->dev;
  d.u_len = u_len;
  d.v_len = v_len;
  d.nx = nx;
  d.ny = ny;
  h->one_point_axis = nx < 2 || ny < 2;
  if (!h->one_point_axis) {
    // nearest(), cartesian_current.rs:244-248 and gradient spacing :515-516
    d.x0 = x[0];
    d.xsp = fabs(x[1] - x[0]);
    d.xhigh = static_cast<double>(nx - 1);
    d.y0 = y[0];
    d.ysp = fabs(y[1] - y[0]);
    d.yhigh = static_cast<double>(ny - 1);
    d.xspace = x[1] - x[0];
    d.yspace = y[1] - y[0];
    d.inv_xsp = 1.0 / d.xsp;
    d.inv_ysp = 1.0 / d.ysp;
  }
  const bool use_thr = !h->one_point_axis && std::isfinite(d.x0) && std::isfinite(d.y0) &&
                       std::isfinite(d.xsp) && std::isfinite(d.ysp) && d.xsp > 0.0 &&
                       d.ysp > 0.0 && nx < (1u << 30) && ny < (1u << 30);
  std::vector<long long> xthr, ythr;
  if (use_thr) {
    xthr = current_axis_thresholds(d.x0, d.xsp, nx);
    ythr = current_axis_thresholds(d.y0, d.ysp, ny);
    d.x0f = static_cast<float>(d.x0);
    d.y0f = static_cast<float>(d.y0);
    d.inv_xspf = static_cast<float>(d.inv_xsp);
    d.inv_yspf = static_cast<float>(d.inv_ysp);
  }
  // Tables (fields.h): axes and values as f32 (interpolate, :375-396) and
  // the f64 cell gradients of :522-536.
  const size_t len = u_len < v_len ? u_len : v_len;
  std::vector<float> x32(nx), y32(ny), u32(u_len), v32(v_len);
  std::vector<double> dudx(len, 0.0), dudy(len, 0.0), dvdx(len, 0.0), dvdy(len, 0.0);
  for (size_t i = 0; i < nx; ++i) x32[i] = static_cast<float>(x[i]);
  for (size_t i = 0; i < ny; ++i) y32[i] = static_cast<float>(y[i]);
  for (size_t i = 0; i < u_len; ++i) u32[i] = static_cast<float>(u[i]);
  for (size_t i = 0; i < v_len; ++i) v32[i] = static_cast<float>(v[i]);
  if (!h->one_point_axis) {
    for (size_t j = 0; j + 1 < ny; ++j) {
      for (size_t i = 0; i + 1 < nx; ++i) {
        const size_t sw = nx * j + i;
        if (nx * (j + 1) + i + 1 >= len) continue;
        dudx[sw] = (u[sw + 1] - u[sw]) / d.xspace;
        dudy[sw] = (u[sw + nx] - u[sw]) / d.yspace;
        dvdx[sw] = (v[sw + 1] - v[sw]) / d.xspace;
        dvdy[sw] = (v[sw + nx] - v[sw]) / d.yspace;
      }
    }
  }
  cudaError_t e;
  if ((e = upload(x, nx, &h->mem, &d.x)) != cudaSuccess ||
      (e = upload(y, ny, &h->mem, &d.y)) != cudaSuccess ||
      (e = upload(u, u_len, &h->mem, &d.u)) != cudaSuccess ||
      (e = upload(v, v_len, &h->mem, &d.v)) != cudaSuccess ||
      (e = upload(x32.data(), nx, &h->mem, &d.x32)) != cudaSuccess ||
      (e = upload(y32.data(), ny, &h->mem, &d.y32)) != cudaSuccess ||
      (e = upload(u32.data(), u_len, &h->mem, &d.u32)) != cudaSuccess ||
      (e = upload(v32.data(), v_len, &h->mem, &d.v32)) != cudaSuccess ||
      (e = upload(dudx.data(), len, &h->mem, &d.dudx)) != cudaSuccess ||
      (e = upload(dudy.data(), len, &h->mem, &d.dudy)) != cudaSuccess ||
      (e = upload(dvdx.data(), len, &h->mem, &d.dvdx)) != cudaSuccess ||
      (e = upload(dvdy.data(), len, &h->mem, &d.dvdy)) != cudaSuccess ||
      (use_thr && (e = upload(xthr.data(), nx + 1, &h->mem, &d.xthr)) != cudaSuccess) ||
      (use_thr && (e = upload(ythr.data(), ny + 1, &h->mem, &d.ythr)) != cudaSuccess)) {
    free_mem(h->mem);
    delete h;
    return cuda_fail(e, "staging current grid");
  }
  *out = h;
  return MR_OK;
}

int launch(const mr_bathymetry *b, const mr_current *c, size_t n, const double *x0,
           const double *y0, const double *kx0, const double *ky0, double t0, double dt,
           uint64_t nsteps, int options, size_t rows_cap, double *traj, int32_t *n_rows,
           uint8_t *status, cudaStream_t stream) {
  mr::TraceArgs a;
  a.n = n;
  a.x0 = x0; a.y0 = y0; a.kx0 = kx0; a.ky0 = ky0;
  a.t0 = t0;
  a.dt = dt;
  a.nsteps = nsteps;
  a.rows_cap = rows_cap;
  a.traj = traj;
  a.n_rows = n_rows;
  a.status = status;
  cudaError_t e = mr::launch_rk4_f64(b->dev, c->dev, a, options & MR_STOP_FRESH,
                                     (options & MR_MATH_LIBM) == 0, stream);
  if (e != cudaSuccess) return cuda_fail(e, "rk4_f64 launch");
  return MR_OK;
}

}  // namespace

extern "C" {

const char *mr_last_error(void) { return mr::g_last_error.c_str(); }

int mr_version(void) { return 100; }

uint64_t mr_num_steps(double t0, double t_end, double dt) {
  return rust_ceil_as_usize((t_end - t0) / dt);
}

int mr_bathymetry_grid(size_t nx, size_t ny, const float *x, const float *y, const double *depth,
                       size_t depth_len, mr_bathymetry **out) {
  return make_bathy_grid(nx, ny, x, y, depth, depth_len, out);
}

int mr_bathymetry_open(const char *path, const char *x_name, const char *y_name,
                       const char *depth_name, mr_bathymetry **out) {
  if (!path || !x_name || !y_name || !depth_name || !out)
    return fail(MR_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> xd, yd, depth;
  std::vector<float> x, y;
  int type = 0;
  mr::nc3::Result r = mr::nc3::read_variable(path, x_name, &xd, &type, &x);
  if (!r.code) r = mr::nc3::read_variable(path, y_name, &yd, &type, &y);
  if (!r.code) r = mr::nc3::read_variable(path, depth_name, &depth, &type);
  if (r.code) return fail(r.code, "%s", r.message.c_str());
  return make_bathy_grid(x.size(), y.size(), x.data(), y.data(), depth.data(), depth.size(), out);
}

int mr_bathymetry_constant(float h, mr_bathymetry **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_bathymetry *b = new mr_bathymetry();
  b->device = device;
  b->dev.kind = mr::BATHY_CONSTANT;
  b->dev.h = h;
  *out = b;
  return MR_OK;
}

int mr_bathymetry_slope(float h0, float x0, float y0, float dhdx, float dhdy,
                        mr_bathymetry **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_bathymetry *b = new mr_bathymetry();
  b->device = device;
  b->dev.kind = mr::BATHY_SLOPE;
  b->dev.s_h0 = h0; b->dev.s_x0 = x0; b->dev.s_y0 = y0;
  b->dev.s_dhdx = dhdx; b->dev.s_dhdy = dhdy;
  *out = b;
  return MR_OK;
}

int mr_bathymetry_array(size_t n, const float *arr, mr_bathymetry **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  *out = nullptr;
  if (n && !arr) return fail(MR_ERR_INVALID_ARGUMENT, "null array");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_bathymetry *b = new mr_bathymetry();
  b->device = device;
  b->dev.kind = mr::BATHY_ARRAY;
  b->dev.an = n;
  cudaError_t e = upload(arr, n * n, &b->mem, &b->dev.arr);
  if (e != cudaSuccess) {
    free_mem(b->mem);
    delete b;
    return cuda_fail(e, "staging array depth");
  }
  *out = b;
  return MR_OK;
}

void mr_bathymetry_destroy(mr_bathymetry *b) {
  if (!b) return;
  DeviceGuard g(b->device);
  free_mem(b->mem);
  delete b;
}

int mr_current_grid(size_t nx, size_t ny, const double *x, const double *y, const double *u,
                    size_t u_len, const double *v, size_t v_len, mr_current **out) {
  return make_current_grid(nx, ny, x, y, u, u_len, v, v_len, out);
}

int mr_current_open(const char *path, const char *x_name, const char *y_name, const char *u_name,
                    const char *v_name, mr_current **out) {
  if (!path || !x_name || !y_name || !u_name || !v_name || !out)
    return fail(MR_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> x, y, u, v;
  int type = 0;
  mr::nc3::Result r = mr::nc3::read_variable(path, x_name, &x, &type);
  if (!r.code) r = mr::nc3::read_variable(path, y_name, &y, &type);
  if (!r.code) r = mr::nc3::read_variable(path, u_name, &u, &type);
  if (!r.code) r = mr::nc3::read_variable(path, v_name, &v, &type);
  if (r.code) return fail(r.code, "%s", r.message.c_str());
  return make_current_grid(x.size(), y.size(), x.data(), y.data(), u.data(), u.size(), v.data(),
                           v.size(), out);
}

int mr_current_constant(double u, double v, mr_current **out) {
  if (!out) return fail(MR_ERR_INVALID_ARGUMENT, "null output handle pointer");
  int device = 0;
  MR_CUDA(cudaGetDevice(&device));
  mr_current *c = new mr_current();
  c->device = device;
  c->dev.kind = mr::CURRENT_CONSTANT;
  c->dev.cu = u;
  c->dev.cv = v;
  *out = c;
  return MR_OK;
}

void mr_current_destroy(mr_current *c) {
  if (!c) return;
  DeviceGuard g(c->device);
  free_mem(c->mem);
  delete c;
}

int mr_trace_device(const mr_bathymetry *b, const mr_current *c, size_t n, const double *x0,
                    const double *y0, const double *kx0, const double *ky0, double t0,
                    double t_end, double dt, int options, size_t rows_cap, double *traj,
                    int32_t *n_rows, uint8_t *status, void *stream) {
  uint64_t nsteps = 0;
  int rc = check_trace_args(b, c, n, x0, y0, kx0, ky0, t0, t_end, dt, options, rows_cap, traj,
                            n_rows, status, &nsteps);
  if (rc) return rc;
  if (n == 0) return MR_OK;
  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select device %d", b->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  return launch(b, c, n, x0, y0, kx0, ky0, t0, dt, nsteps, options, rows_cap, traj, n_rows,
                status, s);
}

int mr_trace(const mr_bathymetry *b, const mr_current *c, size_t n, const double *x0,
             const double *y0, const double *kx0, const double *ky0, double t0, double t_end,
             double dt, int options, size_t rows_cap, double *traj, int32_t *n_rows,
             uint8_t *status) {
  uint64_t nsteps = 0;
  int rc = check_trace_args(b, c, n, x0, y0, kx0, ky0, t0, t_end, dt, options, rows_cap, traj,
                            n_rows, status, &nsteps);
  if (rc) return rc;
  if (n == 0) return MR_OK;
  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select device %d", b->device);
  keep_pool(b->device);
  cudaStream_t s = cudaStreamPerThread;
  const size_t traj_bytes = 5 * rows_cap * n * sizeof(double);
  // Inputs: one staging block for the four initial-state arrays.
  double *d_in = nullptr;
  MR_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&d_in), 4 * n * sizeof(double), s));
  const double *srcs[4] = {x0, y0, kx0, ky0};
  for (int q = 0; q < 4; ++q) {
    cudaError_t e = cudaMemcpyAsync(d_in + q * n, srcs[q], n * sizeof(double),
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      cudaFreeAsync(d_in, s);
      return cuda_fail(e, "copying initial states to the device");
    }
  }
  // Outputs: written in place when the caller's buffers are page-locked,
  // else through device buffers copied back after the launch.
  double *d_traj = static_cast<double *>(mapped_host(traj));
  int32_t *d_rows = static_cast<int32_t *>(mapped_host(n_rows));
  uint8_t *d_status = static_cast<uint8_t *>(mapped_host(status));
  const bool own_traj = !d_traj, own_rows = !d_rows, own_status = !d_status;
  cudaError_t e = cudaSuccess;
  if (own_traj) e = cudaMallocAsync(reinterpret_cast<void **>(&d_traj), traj_bytes, s);
  if (e == cudaSuccess && own_rows)
    e = cudaMallocAsync(reinterpret_cast<void **>(&d_rows), n * sizeof(int32_t), s);
  if (e == cudaSuccess && own_status) e = cudaMallocAsync(reinterpret_cast<void **>(&d_status), n, s);
  if (e == cudaSuccess) {
    rc = launch(b, c, n, d_in, d_in + n, d_in + 2 * n, d_in + 3 * n, t0, dt, nsteps, options,
                rows_cap, d_traj, d_rows, d_status, s);
  } else {
    rc = cuda_fail(e, "allocating device output buffers");
  }
  if (rc == MR_OK && own_traj) e = cudaMemcpyAsync(traj, d_traj, traj_bytes, cudaMemcpyDeviceToHost, s);
  if (rc == MR_OK && e == cudaSuccess && own_rows)
    e = cudaMemcpyAsync(n_rows, d_rows, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
  if (rc == MR_OK && e == cudaSuccess && own_status)
    e = cudaMemcpyAsync(status, d_status, n, cudaMemcpyDeviceToHost, s);
  if (rc == MR_OK && e != cudaSuccess) rc = cuda_fail(e, "copying trajectories to the host");
  cudaError_t se = cudaStreamSynchronize(s);
  if (rc == MR_OK && se != cudaSuccess) rc = cuda_fail(se, "rk4_f64 execution");
  cudaFreeAsync(d_in, s);
  if (own_traj && d_traj) cudaFreeAsync(d_traj, s);
  if (own_rows && d_rows) cudaFreeAsync(d_rows, s);
  if (own_status && d_status) cudaFreeAsync(d_status, s);
  return rc;
}

int mr_single_ray(const mr_bathymetry *b, const mr_current *c, double x0, double y0, double kx0,
                  double ky0, double duration, double step_size, size_t rows_cap, double *rows,
                  int32_t *n_rows) {
  if (!rows || !n_rows) return fail(MR_ERR_INVALID_ARGUMENT, "null output");
  std::vector<double> traj(5 * rows_cap);
  uint8_t status = 0;
  int rc = mr_trace(b, c, 1, &x0, &y0, &kx0, &ky0, 0.0, duration, step_size, kDropInOptions,
                    rows_cap, traj.data(), n_rows, &status);
  if (rc) return rc;
  for (size_t r = 0; r < rows_cap; ++r)
    for (int v = 0; v < 5; ++v) rows[r * 5 + v] = traj[v * rows_cap + r];
  return MR_OK;
}

int mr_single_ray_files(const char *bathymetry_path, const char *current_path, double x0,
                        double y0, double kx0, double ky0, double duration, double step_size,
                        size_t rows_cap, double *rows, int32_t *n_rows) {
  mr_bathymetry *b = nullptr;
  mr_current *c = nullptr;
  int rc = mr_bathymetry_open(bathymetry_path, "x", "y", "depth", &b);
  if (!rc) rc = mr_current_open(current_path, "x", "y", "u", "v", &c);
  if (!rc) rc = mr_single_ray(b, c, x0, y0, kx0, ky0, duration, step_size, rows_cap, rows, n_rows);
  mr_bathymetry_destroy(b);
  mr_current_destroy(c);
  return rc;
}

int mr_ray_tracing_files(const char *bathymetry_path, const char *current_path, size_t n,
                         const double *x0, const double *y0, const double *kx0,
                         const double *ky0, double duration, double step_size, size_t rows_cap,
                         double *traj, int32_t *n_rows, uint8_t *status) {
  mr_bathymetry *b = nullptr;
  mr_current *c = nullptr;
  int rc = mr_bathymetry_open(bathymetry_path, "x", "y", "depth", &b);
  if (!rc) rc = mr_current_open(current_path, "x", "y", "u", "v", &c);
  if (!rc)
    rc = mr_trace(b, c, n, x0, y0, kx0, ky0, 0.0, duration, step_size, kDropInOptions, rows_cap,
                  traj, n_rows, status);
  mr_bathymetry_destroy(b);
  mr_current_destroy(c);
  return rc;
}

int mr_netcdf3_read_f64(const char *path, const char *name, double *out, size_t cap, size_t *len,
                        int *nc_type) {
  if (!path || !name || !len) return fail(MR_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> v;
  int type = 0;
  mr::nc3::Result r = mr::nc3::read_variable(path, name, &v, &type);
  if (r.code) return fail(r.code, "%s", r.message.c_str());
  *len = v.size();
  if (nc_type) *nc_type = type;
  if (out) memcpy(out, v.data(), (cap < v.size() ? cap : v.size()) * sizeof(double));
  return MR_OK;
}

}  // extern "C"
