// st3d_kernels_copy.cu -- host-boundary layout conversion on the device.
//
// The caller's arrays use the reference layout (IDX = ijk_ofs + k +
// j*jmult + i*imult, stencils.h:5, grid.cpp:20-24); the kernels use the
// library layout (st3d_internal.h).  A strided host<->device copy of ~1M rows
// of a few KB each runs far below the link rate, so transfers go through a
// staging buffer in the reference layout instead:
//   upload:   one contiguous host->device copy of the whole host array, then
//             k_ref_to_dev scatters the region the stencil can read (interior
//             plus up to 4 halo planes/rows and up to `pk` halo points along
//             k) into the library layout;
//   download: k_dev_to_ref gathers every interior row together with its k
//             halo into the staging buffer, then one 2-D copy moves, per
//             i-plane, the span of the interior rows (ys rows of jmult
//             points) back to the host.  The j-halo rows and i-halo planes of
//             the host array are not written; the k-halo points inside the
//             span are written with the values uploaded for them.
#include "st3d_internal.h"

namespace st3d {

namespace {

// Each thread moves kRowUnroll points of a row, blockDim apart, loads first:
// the host-link path (the source or destination a pinned host array) needs
// several transfers in flight per thread to cover its latency.
constexpr int kRowUnroll = 4;
constexpr int kRowBlock = 256;

template <typename T>
__global__ void k_ref_to_dev(Layout L, RefGeom R, const T* __restrict__ stage, T* __restrict__ dst,
                             int hx, int hy, int hz) {
  const int klen = R.zs + 2 * hz;
  const int k0 = blockIdx.x * (kRowBlock * kRowUnroll) + threadIdx.x;
  const int j = (int)blockIdx.y - hy;
  const int i = (int)blockIdx.z - hx;
  const long long srow = R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult - hz;
  const long long drow = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (int)L.pk - hz;
  T x[kRowUnroll];
#pragma unroll
  for (int m = 0; m < kRowUnroll; ++m) {
    const int kk = k0 + m * kRowBlock;
    if (kk < klen) x[m] = stage[srow + kk];
  }
#pragma unroll
  for (int m = 0; m < kRowUnroll; ++m) {
    const int kk = k0 + m * kRowBlock;
    if (kk < klen) dst[drow + kk] = x[m];
  }
}

template <typename T>
__global__ void k_dev_to_ref(Layout L, RefGeom R, const T* __restrict__ src, T* __restrict__ stage,
                             int hz) {
  const int klen = R.zs + 2 * hz;
  const int k0 = blockIdx.x * (kRowBlock * kRowUnroll) + threadIdx.x;
  const int j = (int)blockIdx.y;
  const int i = (int)blockIdx.z;
  const long long srow = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (int)L.pk - hz;
  const long long drow = R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult - hz;
  T x[kRowUnroll];
#pragma unroll
  for (int m = 0; m < kRowUnroll; ++m) {
    const int kk = k0 + m * kRowBlock;
    if (kk < klen) x[m] = src[srow + kk];
  }
#pragma unroll
  for (int m = 0; m < kRowUnroll; ++m) {
    const int kk = k0 + m * kRowBlock;
    if (kk < klen) stage[drow + kk] = x[m];
  }
}

}  // namespace

cudaError_t launch_ref_to_dev(int eb, const Layout& L, const RefGeom& R, const void* stage,
                              void* dst, int hx, int hy, int hz, cudaStream_t stream) {
  dim3 block(kRowBlock);
  dim3 grid((R.zs + 2 * hz + kRowBlock * kRowUnroll - 1) / (kRowBlock * kRowUnroll), R.ys + 2 * hy,
            R.xs + 2 * hx);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (eb == 4)
    k_ref_to_dev<float><<<grid, block, 0, stream>>>(L, R, (const float*)stage, (float*)dst, hx, hy, hz);
  else if (eb == 8)
    k_ref_to_dev<double><<<grid, block, 0, stream>>>(L, R, (const double*)stage, (double*)dst, hx, hy, hz);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_dev_to_ref(int eb, const Layout& L, const RefGeom& R, const void* src,
                              void* stage, int hz, cudaStream_t stream) {
  dim3 block(kRowBlock);
  dim3 grid((R.zs + 2 * hz + kRowBlock * kRowUnroll - 1) / (kRowBlock * kRowUnroll), R.ys, R.xs);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (eb == 4)
    k_dev_to_ref<float><<<grid, block, 0, stream>>>(L, R, (const float*)src, (float*)stage, hz);
  else if (eb == 8)
    k_dev_to_ref<double><<<grid, block, 0, stream>>>(L, R, (const double*)src, (double*)stage, hz);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace st3d

// ---------------------------------------------------------------------------
// 16-bit storage (st3d_f16.cuh): host arrays stay float; the device keeps a
// 16-bit word per point (plus a low byte in the compensated form) and a
// power-of-two scale per i-plane.
// ---------------------------------------------------------------------------
#include "st3d_f16.cuh"

namespace st3d {

namespace {

template <int KIND>
__device__ __forceinline__ float word_to_float(uint16_t b) {
  if (KIND == 0) return __half2float(__ushort_as_half(b));
  return __uint_as_float((uint32_t)b << 16);
}
template <int KIND>
__device__ __forceinline__ uint16_t float_to_word(float x) {
  if (KIND == 0) return __half_as_ushort(__float2half_rn(x));
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

// Per-plane maxima of |x| over the interior (float bits, atomicMax) and the
// maximum over the halo points the stencil reads; x = stage - stage2 when
// stage2 is given (the halo check then covers both arrays).
__global__ void k_plane_max_ref(RefGeom R, const float* __restrict__ stage,
                                const float* __restrict__ stage2, uint32_t* __restrict__ M,
                                uint32_t* __restrict__ halo_max, int hx, int hy, int hz) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = (int)blockIdx.y - hy;
  const int i = (int)blockIdx.z - hx;
  const int k = kk - hz;
  float m_in = 0.0f, m_halo = 0.0f;
  if (kk < R.zs + 2 * hz) {
    const long long s = R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k;
    const float a = stage[s];
    const float b = stage2 ? stage2[s] : 0.0f;
    const bool inner = i >= 0 && i < R.xs && j >= 0 && j < R.ys && k >= 0 && k < R.zs;
    if (inner) m_in = fabsf(a - b); else m_halo = fmaxf(fabsf(a), fabsf(b));
  }
  const uint32_t a = __reduce_max_sync(0xffffffffu, __float_as_uint(m_in));
  const uint32_t b = __reduce_max_sync(0xffffffffu, __float_as_uint(m_halo));
  if ((threadIdx.x & 31) == 0) {
    if (a && i >= 0 && i < R.xs) atomicMax(&M[i], a);
    if (b) atomicMax(halo_max, b);
  }
}

// Scatter + encode: staging (reference layout, float) -> words (+ low bytes)
// in the library layout, the plane's scale from its maximum.
// With lo16 (FP16 words), the lo word of the hi/lo pair: fp16(xs - hi).
template <int KIND, bool HILO>
__global__ void k_ref_to_dev16(Layout L, RefGeom R, const float* __restrict__ stage,
                               const float* __restrict__ stage2, uint16_t* __restrict__ hi,
                               int8_t* __restrict__ lo, const uint32_t* __restrict__ M,
                               int* __restrict__ E, int hx, int hy, int hz,
                               uint16_t* __restrict__ lo16) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= R.zs + 2 * hz) return;
  const int j = (int)blockIdx.y - hy;
  const int i = (int)blockIdx.z - hx;
  const int k = kk - hz;
  const bool plane_in = i >= 0 && i < R.xs;
  const int e = plane_in ? scale_exponent(__uint_as_float(M[i])) : 0;
  if (plane_in && kk == 0 && blockIdx.y == 0) E[i] = e;
  const long long s = R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k;
  const float xs = (stage2 ? stage[s] - stage2[s] : stage[s]) * exp2i(-e);
  const long long d = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (k + (int)L.pk);
  const uint16_t w = float_to_word<KIND>(xs);
  hi[d] = w;
  if (lo16) lo16[d] = float_to_word<KIND>(xs - word_to_float<KIND>(w));
  if (HILO) {
    const float r = xs - word_to_float<KIND>(w);
    int eb = (w >> 10) & 0x1f;
    if (eb == 0) eb = 1;
    int q = __float2int_rn(r * exp2i(33 - eb));
    q = q > 127 ? 127 : (q < -127 ? -127 : q);
    lo[d] = (int8_t)q;
  }
}

// Gather + decode: words (+ low bytes) -> staging (reference layout, float),
// interior rows with their k halo.
template <int KIND, bool HILO>
__global__ void k_dev16_to_ref(Layout L, RefGeom R, const uint16_t* __restrict__ hi,
                               const int8_t* __restrict__ lo, const int* __restrict__ E,
                               float* __restrict__ stage, int hz) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= R.zs + 2 * hz) return;
  const int j = (int)blockIdx.y;
  const int i = (int)blockIdx.z;
  const int k = kk - hz;
  const long long s = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (k + (int)L.pk);
  const uint16_t w = hi[s];
  float x = word_to_float<KIND>(w);
  if (HILO) x = __fmaf_rn((float)lo[s], ulp256_f16(w), x);
  stage[R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k] = x * exp2i(E[i]);
}

// Delta form -> float: u = dec(U), or v = dec(U) - dec(D).
template <int KIND>
__global__ void k_delta_to_ref(Layout L, RefGeom R, const uint16_t* __restrict__ u,
                               const int* __restrict__ Eu, const uint16_t* __restrict__ d,
                               const int* __restrict__ Ed, bool minus_d, float* __restrict__ stage,
                               int hz, const uint16_t* __restrict__ ul) {
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= R.zs + 2 * hz) return;
  const int j = (int)blockIdx.y;
  const int i = (int)blockIdx.z;
  const int k = kk - hz;
  const long long s = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (k + (int)L.pk);
  float x = word_to_float<KIND>(u[s]);
  if (ul) x = x + word_to_float<KIND>(ul[s]);  // exact: the pair holds <= 22 bits
  x = x * exp2i(Eu[i]);
  if (minus_d) x = x - word_to_float<KIND>(d[s]) * exp2i(Ed[i]);
  stage[R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k] = x;
}

}  // namespace

cudaError_t launch_plane_max_ref(const RefGeom& R, const float* stage, uint32_t* M,
                                 uint32_t* halo_max, int hx, int hy, int hz, cudaStream_t stream,
                                 const float* stage2) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys + 2 * hy, R.xs + 2 * hx);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  k_plane_max_ref<<<grid, block, 0, stream>>>(R, stage, stage2, M, halo_max, hx, hy, hz);
  return cudaGetLastError();
}

cudaError_t launch_ref_to_dev16(int storage, const Layout& L, const RefGeom& R, const float* stage,
                                uint16_t* hi, int8_t* lo, const uint32_t* M, int* E, int hx, int hy,
                                int hz, cudaStream_t stream, const float* stage2, uint16_t* lo16) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys + 2 * hy, R.xs + 2 * hx);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (lo16 && storage != ST3D_F16) return cudaErrorInvalidValue;
  if (storage == ST3D_F16)
    k_ref_to_dev16<0, false><<<grid, block, 0, stream>>>(L, R, stage, stage2, hi, lo, M, E, hx, hy, hz, lo16);
  else if (storage == ST3D_BF16)
    k_ref_to_dev16<1, false><<<grid, block, 0, stream>>>(L, R, stage, stage2, hi, lo, M, E, hx, hy, hz, lo16);
  else if (storage == ST3D_F16_HILO)
    k_ref_to_dev16<0, true><<<grid, block, 0, stream>>>(L, R, stage, stage2, hi, lo, M, E, hx, hy, hz, lo16);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_delta_to_ref(int storage, const Layout& L, const RefGeom& R, const uint16_t* u,
                                const int* Eu, const uint16_t* d, const int* Ed, bool minus_d,
                                float* stage, int hz, cudaStream_t stream, const uint16_t* ul) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys, R.xs);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (ul && storage != ST3D_F16) return cudaErrorInvalidValue;
  if (storage == ST3D_F16)
    k_delta_to_ref<0><<<grid, block, 0, stream>>>(L, R, u, Eu, d, Ed, minus_d, stage, hz, ul);
  else if (storage == ST3D_BF16)
    k_delta_to_ref<1><<<grid, block, 0, stream>>>(L, R, u, Eu, d, Ed, minus_d, stage, hz, ul);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_dev16_to_ref(int storage, const Layout& L, const RefGeom& R, const uint16_t* hi,
                                const int8_t* lo, const int* E, float* stage, int hz,
                                cudaStream_t stream) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys, R.xs);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (storage == ST3D_F16)
    k_dev16_to_ref<0, false><<<grid, block, 0, stream>>>(L, R, hi, lo, E, stage, hz);
  else if (storage == ST3D_BF16)
    k_dev16_to_ref<1, false><<<grid, block, 0, stream>>>(L, R, hi, lo, E, stage, hz);
  else if (storage == ST3D_F16_HILO)
    k_dev16_to_ref<0, true><<<grid, block, 0, stream>>>(L, R, hi, lo, E, stage, hz);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace st3d
