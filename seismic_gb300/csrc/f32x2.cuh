// f32x2.cuh - packed pairs of FP32 values for sm_100-family arithmetic.
//
// add/sub/mul.rn.f32x2 apply the IEEE round-to-nearest operation to each
// lane independently, so a pair computes what two scalar instructions with
// the same operands compute.  Measured on sm_103a with CUDA 13.0: a packed
// mul.rn whose only use is a packed add.rn or sub.rn is fused into one
// rounding by the assembler, even with --fmad=false, while a scalar
// mul.rn feeding a packed add (or a packed mul feeding scalar adds) keeps
// both roundings.  So every product that feeds a sum is formed with
// scalar multiplies (s_mul); packed multiplies only feed other multiplies
// or stores.  Fewer FP instructions matter to the fused step kernels, whose
// arithmetic has to follow the reference's evaluation order without FMA.
#pragma once

namespace swave {

struct P2 {
  float x, y;
};

__device__ __forceinline__ P2 p2(float a, float b) { return P2{a, b}; }
__device__ __forceinline__ P2 p2s(float a) { return P2{a, a}; }

__device__ __forceinline__ P2 p_add(P2 a, P2 b) {
  P2 r;
  asm("{.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2,%3};\n\t"
      "mov.b64 rb, {%4,%5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\t"
      "mov.b64 {%0,%1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

__device__ __forceinline__ P2 p_sub(P2 a, P2 b) {
  P2 r;
  asm("{.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2,%3};\n\t"
      "mov.b64 rb, {%4,%5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\t"
      "mov.b64 {%0,%1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

__device__ __forceinline__ P2 p_mul(P2 a, P2 b) {
  P2 r;
  asm("{.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2,%3};\n\t"
      "mov.b64 rb, {%4,%5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\t"
      "mov.b64 {%0,%1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

// c * x lane by lane with scalar IEEE multiplies (safe to feed a sum).
__device__ __forceinline__ P2 s_mul(float c, P2 x) {
  return P2{__fmul_rn(c, x.x), __fmul_rn(c, x.y)};
}
__device__ __forceinline__ P2 s_mul(P2 c, P2 x) {
  return P2{__fmul_rn(c.x, x.x), __fmul_rn(c.y, x.y)};
}

__device__ __forceinline__ P2 lo2(const float4 &a) { return P2{a.x, a.y}; }
__device__ __forceinline__ P2 hi2(const float4 &a) { return P2{a.z, a.w}; }

}  // namespace swave
