// bits.h -- exact float / double conversions and tests on bit patterns.
//
// GB300 issues two FP64 lanes per SM per clock, and the conversions between
// float and double run on that pipe; these do the same conversions with
// 32-bit integer operations for the common cases (normal numbers, zeros) and
// leave the rest (subnormal results, overflow, infinities, NaN) to the
// conversion instruction.  Results equal the IEEE conversions bit for bit.
// Host and device code: the host build is what the CPU tests check.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MR_HD __host__ __device__ __forceinline__
#else
#define MR_HD inline
#endif

namespace mr {

MR_HD uint64_t bits_of(double v) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(v));
#else
  uint64_t b;
  memcpy(&b, &v, sizeof b);
  return b;
#endif
}

MR_HD double double_of(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
  return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
#else
  const uint64_t b = (static_cast<uint64_t>(hi) << 32) | lo;
  double v;
  memcpy(&v, &b, sizeof v);
  return v;
#endif
}

MR_HD uint32_t bits_of(float v) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(v);
#else
  uint32_t b;
  memcpy(&b, &v, sizeof b);
  return b;
#endif
}

MR_HD float float_of(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float v;
  memcpy(&v, &b, sizeof v);
  return v;
#endif
}

// Key of a double under which signed integer order is the double order
// (-0 just below +0; NaN outside -inf..+inf).  Its own inverse.
MR_HD long long order_key_bits(long long bits) {
  return bits ^ ((bits >> 63) & 0x7fffffffffffffffll);
}

// static_cast<double>(f): re-biased exponent, mantissa shifted into place.
MR_HD double f2d(float f) {
  const uint32_t u = bits_of(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e - 1u < 0xfeu)  // normal
    return double_of((u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xfffffu), u << 29);
  if ((u & 0x7fffffffu) == 0u) return double_of(u & 0x80000000u, 0u);  // +-0
  return static_cast<double>(f);
}

// static_cast<float>(d), round to nearest even: for doubles whose float is
// normal or rounds to the next binade (exponent 897..1150), the top 23
// mantissa bits plus the rounding increment of the 29 dropped bits; a carry
// out of the mantissa raises the exponent, and out of the largest binade it
// gives infinity, as the IEEE conversion does.
MR_HD float d2f(double d) {
  const uint64_t b = bits_of(d);
  const uint32_t hi = static_cast<uint32_t>(b >> 32), lo = static_cast<uint32_t>(b);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1fffffffu;
    uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    f += (rem > 0x10000000u) | ((rem == 0x10000000u) & (m & 1u));
    return float_of(f);
  }
  return static_cast<float>(d);
}

// isnan for doubles on the integer pipe.
MR_HD bool nan_bits(double v) {
  return (bits_of(v) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}

}  // namespace mr
