// seed.cu -- K7, initial ray states on the device (include/mantaray_gpu.h,
// mr_seed_point_sources / mr_seed_line).
//
// One thread per ray: launch point, direction and period from the ray index
// (SplitMix64, Steele, Lea and Flood 2014, of seed + index: two 53-bit
// uniforms per ray), the depth at the launch point from the bathymetry
// handle's lookup (the integrator's own, lookup.cuh), and |k| from the
// dispersion relation (2 pi / T)^2 = g k tanh(k h) by Newton iteration in
// FP64 from the larger of the deep- and shallow-water values, at most 60
// iterations, stopping when the step is below 1e-15 of k.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/mantaray_gpu.h"
#include "handles.h"
#include "lookup.cuh"

namespace mr {
namespace {

constexpr double kSeedG = 9.8;  // src/wave_ray_path.rs:23

__device__ __forceinline__ double unit_hash(uint64_t seed, uint64_t i) {
  uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return static_cast<double>(z >> 11) * 0x1.0p-53;
}

__device__ double dispersion_k(double period, double h) {
  const double two_pi = 6.283185307179586;
  const double w = two_pi / period;
  const double w2 = w * w;
  if (!(h > 0.0) || !(period > 0.0)) return f64_nan();
  double k = fmax(w2 / kSeedG, sqrt(w2 / (kSeedG * h)));
  for (int it = 0; it < 60; ++it) {
    const double th = tanh(k * h);
    const double f = kSeedG * k * th - w2;
    const double df = kSeedG * th + kSeedG * k * h * (1.0 - th * th);
    const double step = f / df;
    k = k - step;
    if (fabs(step) <= 1e-15 * fabs(k)) break;
  }
  return k;
}

struct SeedArgs {
  BathyDev b;
  int64_t n;
  int64_t per;                 // rays per source (point sources); n (line)
  const double *sx, *sy;       // point sources, or null for a line
  double xa, ya, xb, yb;       // line
  double theta0, theta1, period0, period1;
  uint64_t seed;
  int flags;
  double *x0, *y0, *kx0, *ky0;
};

__global__ void seed_kernel(SeedArgs a) {
  const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= a.n) return;
  const int64_t s = r / a.per, j = r % a.per;
  double x, y;
  if (a.sx) {
    x = a.sx[s];
    y = a.sy[s];
  } else if (a.n > 1) {  // numpy.linspace: start + i * step, the last point exact
    const double t = static_cast<double>(r);
    const double den = static_cast<double>(a.n - 1);
    x = r == a.n - 1 ? a.xb : a.xa + t * ((a.xb - a.xa) / den);
    y = r == a.n - 1 ? a.yb : a.ya + t * ((a.yb - a.ya) / den);
  } else {
    x = a.xa;
    y = a.ya;
  }
  const double u = (a.flags & MR_SEED_EVEN_DIRECTIONS)
                       ? (static_cast<double>(j) + 0.5) / static_cast<double>(a.per)
                       : unit_hash(a.seed, 2 * static_cast<uint64_t>(r));
  const double v = unit_hash(a.seed, 2 * static_cast<uint64_t>(r) + 1);
  const double theta = a.theta0 + (a.theta1 - a.theta0) * u;
  const double period = a.period0 + (a.period1 - a.period0) * v;
  float hg[3];
  double k = f64_nan();
  if (depth_and_gradient(a.b, __double2float_rn(x), __double2float_rn(y), hg) == RHS_OK)
    k = dispersion_k(period, static_cast<double>(hg[0]));
  a.x0[r] = x;
  a.y0[r] = y;
  a.kx0[r] = k * cos(theta);
  a.ky0[r] = k * sin(theta);
}

int launch_seed(const mr_bathymetry *b, SeedArgs &a, void *stream) {
  if (!b) return fail(MR_ERR_INVALID_ARGUMENT, "null bathymetry");
  if (a.n > 0 && (!a.x0 || !a.y0 || !a.kx0 || !a.ky0))
    return fail(MR_ERR_INVALID_ARGUMENT, "null output array");
  if (!isfinite(a.theta0) || !isfinite(a.theta1) || !(a.period0 > 0.0) || !(a.period1 > 0.0))
    return fail(MR_ERR_INVALID_ARGUMENT, "directions must be finite and periods > 0");
  if (a.n == 0) return MR_OK;
  DeviceGuard g(b->device);
  if (!g.ok()) return fail(MR_ERR_CUDA, "cannot select the bathymetry's device");
  a.b = b->dev;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : cudaStreamPerThread;
  seed_kernel<<<static_cast<unsigned>((a.n + 127) / 128), 128, 0, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "seed launch");
  return MR_OK;
}

}  // namespace
}  // namespace mr

extern "C" {

int mr_seed_point_sources(const mr_bathymetry *b, size_t n_sources, const double *sx,
                          const double *sy, size_t rays_per_source, double theta0,
                          double theta1, double period0, double period1, uint64_t seed,
                          int flags, double *x0, double *y0, double *kx0, double *ky0,
                          void *stream) {
  if (n_sources && rays_per_source && (!sx || !sy))
    return mr::fail(MR_ERR_INVALID_ARGUMENT, "null source arrays");
  mr::SeedArgs a{};
  a.n = static_cast<int64_t>(n_sources * rays_per_source);
  a.per = rays_per_source ? static_cast<int64_t>(rays_per_source) : 1;
  a.sx = sx; a.sy = sy;
  a.theta0 = theta0; a.theta1 = theta1; a.period0 = period0; a.period1 = period1;
  a.seed = seed; a.flags = flags;
  a.x0 = x0; a.y0 = y0; a.kx0 = kx0; a.ky0 = ky0;
  return mr::launch_seed(b, a, stream);
}

int mr_seed_line(const mr_bathymetry *b, double xa, double ya, double xb, double yb, size_t n,
                 double theta0, double theta1, double period0, double period1, uint64_t seed,
                 int flags, double *x0, double *y0, double *kx0, double *ky0, void *stream) {
  mr::SeedArgs a{};
  a.n = static_cast<int64_t>(n);
  a.per = n ? static_cast<int64_t>(n) : 1;
  a.xa = xa; a.ya = ya; a.xb = xb; a.yb = yb;
  a.theta0 = theta0; a.theta1 = theta1; a.period0 = period0; a.period1 = period1;
  a.seed = seed; a.flags = flags;
  a.x0 = x0; a.y0 = y0; a.kx0 = kx0; a.ky0 = ky0;
  return mr::launch_seed(b, a, stream);
}

}  // extern "C"
