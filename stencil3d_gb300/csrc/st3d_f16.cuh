// st3d_f16.cuh -- the 16-bit storage forms: encoding, decoding and the
// per-plane scale rule, shared by the kernels (device) and the context code
// (host).
//
// A field in 16-bit storage keeps, per i-plane, a power-of-two scale 2^E:
// the value x of a point is stored as h = rn16(x * 2^-E) (FP16 or BF16,
// round to nearest even).  The compensated form (ST3D_F16_HILO) adds a signed
// byte q per point holding the rounding residual in units of 1/256 of h's
// last place:
//     r  = x*2^-E - h                    (exact)
//     q  = clamp(rint(r / ulp256(h)), -127, 127),  ulp256(h) = ulp(h) / 256
//     x' = (h + q*ulp256(h)) * 2^E       (every step exact)
// which carries ~19 significant bits for 3 bytes.  Decoding is exact; only
// the encoder rounds.
//
// Scale rule (one step lag with a proven bound): the plane i of U^{n+1}
// written by step n gets E = floor(log2(B_i)) - 13 with
//     B_i = 3*max(M_u[i], M_v[i]) + k4*max_{|d|<=R} M_u[i+d] + c2*(M_s[i] + |a_n|*[i == src_i])
// where M_* are the plane maxima of |U^n|, |U^{n-1}|, |s| and k4 = 4*c1*sum(w).
// |v_new| <= B_i, so the scaled plane stays below 2^14, under FP16's 65504,
// whatever the wave does in one step.  Planes with B_i = 0 use E = -100.
// The halos must be zero (a zero Dirichlet boundary): they are never
// rewritten, so they could not follow a plane's scale.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace st3d {

constexpr int kScaleMin = -100;
constexpr int kScaleMax = 100;
constexpr int kScaleTop = 13;  // E = floor(log2 B) - kScaleTop

__host__ __device__ inline int scale_exponent(float bound) {
  if (!(bound > 0.0f) || !(bound < 3.0e38f)) return kScaleMin;
  uint32_t bits;
#ifdef __CUDA_ARCH__
  bits = __float_as_uint(bound);
#else
  __builtin_memcpy(&bits, &bound, 4);
#endif
  const int e = (int)((bits >> 23) & 0xff);
  if (e == 0) return kScaleMin;  // subnormal bound
  int E = (e - 127) - kScaleTop;
  return E < kScaleMin ? kScaleMin : (E > kScaleMax ? kScaleMax : E);
}

// 2^e as a float, e in [-126, 127].
__host__ __device__ inline float exp2i(int e) {
  const uint32_t bits = (uint32_t)(e + 127) << 23;
#ifdef __CUDA_ARCH__
  return __uint_as_float(bits);
#else
  float f;
  __builtin_memcpy(&f, &bits, 4);
  return f;
#endif
}

// ulp(h)/256 for an FP16 bit pattern: 2^(max(e,1) - 25 - 8).
__host__ __device__ inline float ulp256_f16(uint16_t hbits) {
  int e = (hbits >> 10) & 0x1f;
  if (e == 0) e = 1;
  return exp2i(e - 33);
}

}  // namespace st3d
