// st3d_p4.cuh -- four points of a lane as two packed FP32 pairs, and the
// 16-bit word conversions the 16-bit storage kernels share.
//
// add.rn.f32x2 / mul.rn.f32x2 / fma.rn.f32x2 (__fadd2_rn, __fmul2_rn,
// __ffma2_rn) give per component exactly __fadd_rn, __fmul_rn and __fmaf_rn,
// so packed arithmetic keeps the scalar operation sequence bit for bit.
// KIND selects the word type: 0 FP16, 1 BF16.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace st3d {

struct P4 {
  float2 a, b;
};
__device__ __forceinline__ float2 splat(float x) { return make_float2(x, x); }
__device__ __forceinline__ P4 add4(const P4& x, const P4& y) {
  return {__fadd2_rn(x.a, y.a), __fadd2_rn(x.b, y.b)};
}
__device__ __forceinline__ P4 mul4(const P4& x, float2 c) { return {__fmul2_rn(x.a, c), __fmul2_rn(x.b, c)}; }
__device__ __forceinline__ P4 fma4(float2 c, const P4& x, const P4& y) {
  return {__ffma2_rn(c, x.a, y.a), __ffma2_rn(c, x.b, y.b)};
}
__device__ __forceinline__ float p4c(const P4& x, int c) {
  return c == 0 ? x.a.x : c == 1 ? x.a.y : c == 2 ? x.b.x : x.b.y;
}

// two packed words <-> two floats (round to nearest even on the way in)
template <int KIND>
__device__ __forceinline__ float2 w2_to_f2(uint32_t w) {
  if (KIND == 0) return __half22float2(*reinterpret_cast<const __half2*>(&w));
  return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
}
template <int KIND>
__device__ __forceinline__ uint32_t f2_to_w2(float2 x) {
  if (KIND == 0) {
    const __half2 h = __floats2half2_rn(x.x, x.y);
    return *reinterpret_cast<const uint32_t*>(&h);
  }
  const __nv_bfloat162 h = __floats2bfloat162_rn(x.x, x.y);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// 4 words -> 4 floats, unscaled
template <int KIND>
__device__ __forceinline__ P4 words4(uint2 w) {
  return {w2_to_f2<KIND>(w.x), w2_to_f2<KIND>(w.y)};
}
// 4 words -> 4 floats times the plane scale sc = 2^E (exact)
template <int KIND>
__device__ __forceinline__ P4 decode4(uint2 w, float sc) {
  return {__fmul2_rn(w2_to_f2<KIND>(w.x), splat(sc)), __fmul2_rn(w2_to_f2<KIND>(w.y), splat(sc))};
}
// 4 floats -> 4 words at the plane scale (inv = 2^-E)
template <int KIND>
__device__ __forceinline__ uint2 encode4(const P4& x, float inv) {
  return make_uint2(f2_to_w2<KIND>(__fmul2_rn(x.a, splat(inv))), f2_to_w2<KIND>(__fmul2_rn(x.b, splat(inv))));
}

}  // namespace st3d
