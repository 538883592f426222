// norms.cuh - per-sample terms of the misfit norms of libs/libinv/Norm.f90
// (fct_compute :12-81, gdt_compute :83-141) for the thresholded and L1
// norms, in FP32 with the reference's operation order.  The caller sums the
// terms in sample order; the L2 norm (FP64 products) is written out where it
// is used.
#pragma once

#include "../../include/swave.h"

namespace swave {

// One term of fct_compute for SW_NRM_L1, SW_NRM_HUBER, SW_NRM_CAUCHY or
// SW_NRM_HYPERBOLIC with threshold g.
__device__ __forceinline__ float nrm_term(int ntype, float d, float g) {
  switch (ntype) {
    case SW_NRM_L1:
      return fabsf(d);
    case SW_NRM_HUBER: {
      const float ad = fabsf(d);
      return ad > g ? ad - g / 2.0f : d * d / (2.0f * g);
    }
    case SW_NRM_CAUCHY: {
      const float q = d / g;
      return logf(1.0f + q * q) / 2.0f;
    }
    default:
      return sqrtf(g * g + d * d) - g;
  }
}

// gdt_compute of one sample for every norm (SW_NRM_L2 is the identity).
__device__ __forceinline__ float nrm_gdt(int ntype, float e, float g) {
  switch (ntype) {
    case SW_NRM_L2:
      return e;
    case SW_NRM_L1:
      return e < 0.0f ? -1.0f : (e > 0.0f ? 1.0f : 0.0f);
    case SW_NRM_HUBER:
      return fmaxf(-1.0f, fminf(1.0f, e / g));
    case SW_NRM_CAUCHY:
      return e / (g * g + e * e);
    default:
      return (e / g) / sqrtf(1.0f + e * e / (g * g));
  }
}

}  // namespace swave
