// rk4_f32_one.cu -- the single-scenario builds of the batched FP32
// integrator (K2, k2.cuh in modes 1 and 2: the scenario's fields are
// operands from the kernel's parameters; mode 2 when the current is gridded
// on the bathymetry's grid).  Compiled with -ftz=true: FP32 subnormals
// flush to zero, so the reciprocal square roots and reciprocals need no
// subnormal handling (the 65,536-ray seamount, the shelf bump and the
// 4,096^2 shelf-slope case ran 4-5% faster with the same endpoint errors).
// Only values below 1.2e-38 change, such as exp(-2kh) in very deep water,
// where the refraction term it scales is far below one ulp of k.  The
// scenario-table builds (rk4_f32.cu) keep subnormals: flushed there, the
// 8-scenario multi-source case ran 8% slower.

#include "k2.cuh"
#include "kernels.h"

namespace mr {

template <int MODE>
static const void *one_build(int build) {
  switch (build) {
    case 0: return reinterpret_cast<const void *>(&rk4_f32_kernel_1<MODE>);
    case 1: return reinterpret_cast<const void *>(&rk4_f32_kernel_1r<MODE>);
    case 5: return reinterpret_cast<const void *>(&rk4_f32_kernel_1s<MODE>);
    case 6: return reinterpret_cast<const void *>(&rk4_f32_kernel_1rs<MODE>);
    default: return reinterpret_cast<const void *>(&rk4_f32_kernel_2<MODE>);
  }
}

const void *rk4_f32_one_function(int build, int same_grid) {
  if (build == 3) return same_grid ? reinterpret_cast<const void *>(&rk4_f32_kernel_1t<2>) : nullptr;
  if (build == 4) return same_grid ? reinterpret_cast<const void *>(&rk4_f32_kernel_1a<2>) : nullptr;
  return same_grid ? one_build<2>(build) : one_build<1>(build);
}

}  // namespace mr
