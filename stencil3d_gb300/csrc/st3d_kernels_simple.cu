// st3d_kernels_simple.cu -- direct-load 2.5D streaming kernels.
//
// One thread owns one (j,k) column of the interior and streams along i (the
// slowest axis of the reference layout, grid.cpp:20-22) through a chunk of
// planes, holding u(i-R .. i+R) of its column in a register queue.  j and k
// neighbours are read straight from global memory (they hit L1/L2: the
// warp's neighbours read the same lines).  This kernel serves every storage
// type, the FP64 run that judges drift, and odd sizes; the TMA-staged kernel
// (st3d_kernels_tma.cu) is the fast FP32 path.
//
// Arithmetic per point, in the reference's pair order (Coefs::cf):
//   mode R (stencil_7.h:31-39, stencil_13.h:50-61, stencil_25.h:75-95):
//     st = coef0*u0; st = fma(cf_p, u[-r]+u[+r], st) ...;
//     v = fma(s0, st, fma(-K, u0, v0))
//   mode W (README.md:11-20, c0 = 2 - 2*c1*sum(w)), difference form, u2 = 2*u0:
//     lap = cf_0*((u[-r]+u[+r]) - u2); lap = fma(cf_p, (u[-r]+u[+r]) - u2, lap) ...;
//     v = fma(c2, s_eff, fma(c1, lap, u2 - v0))
//   Algebraically c0*u - v + c1*sum(w*(u[-r]+u[+r])) + c2*s; the difference
//   form keeps constant fields exactly constant, where the literal form's
//   separately rounded c0 lets the smoothest modes drift (about 5e-3 relative
//   L2 against FP64 after 1000 FP32 steps of a blob field, against 1e-5).
//   2 points (stencil_2.h:20-29): v = coef0*(u0 + u[k+1])
// The library is built with -fmad=false, so these are the only fused
// operations, the sequence oracle/st3d_oracle.c's fma flavour reproduces.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstring>
#include <type_traits>

#include "st3d_internal.h"

namespace st3d {

namespace {

template <typename T>
__device__ __forceinline__ T fma_t(T a, T b, T c);
template <>
__device__ __forceinline__ float fma_t<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fma_t<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

constexpr int kSimpleBX = 32;  // threads along k
constexpr int kSimpleBY = 8;   // threads along j

template <typename T, int P, int MODE>
__global__ void __launch_bounds__(kSimpleBX* kSimpleBY)
    k_simple(Geom g, Coefs<T> cf, T* __restrict__ v, const T* __restrict__ u,
             const T* __restrict__ s, int src_i, int src_j, int src_k, T amp, int ichunk) {
  constexpr int R = (P == 25) ? 4 : (P == 13) ? 2 : 1;
  constexpr int NP = npairs_of(P);
  const int k = blockIdx.x * kSimpleBX + threadIdx.x;
  const int j = blockIdx.y * kSimpleBY + threadIdx.y;
  if (k >= g.zs || j >= g.ys) return;
  const int i0 = blockIdx.z * ichunk;
  const int i1 = min(i0 + ichunk, g.xs);
  const long long col = g.org + (long long)j * g.sj + k;  // (0, j, k)
  const T* uc = u + col;
  T q[2 * R + 1];
#pragma unroll
  for (int m = 0; m < 2 * R; ++m) q[m] = __ldg(uc + (long long)(i0 - R + m) * g.si);
  for (int i = i0; i < i1; ++i) {
    q[2 * R] = __ldg(uc + (long long)(i + R) * g.si);
    const long long x = col + (long long)i * g.si;
    const T* c = u + x;
    const T u0 = q[R];
    T pr[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int ax = pair_axis(P, p);
      const int r = pair_r(P, p);
      T a, b;
      if (ax == 0) {
        a = q[R - r];
        b = q[R + r];
      } else if (ax == 1) {
        a = __ldg(c - (long long)r * g.sj);
        b = __ldg(c + (long long)r * g.sj);
      } else {
        a = __ldg(c - r);
        b = __ldg(c + r);
      }
      pr[p] = a + b;
    }
    const T v0 = v[x];
    T s0 = __ldg(s + x);
    T out;
    if (MODE == ST3D_MODE_REF) {
      T st = cf.coef0 * u0;
#pragma unroll
      for (int p = 0; p < NP; ++p) st = fma_t<T>(cf.cf[p], pr[p], st);
      out = fma_t<T>(s0, st, fma_t<T>(-cf.K, u0, v0));
    } else {
      if (i == src_i && j == src_j && k == src_k) s0 = s0 + amp;
      const T u2 = u0 + u0;
      T lap = cf.cf[0] * (pr[0] - u2);
#pragma unroll
      for (int p = 1; p < NP; ++p) lap = fma_t<T>(cf.cf[p], pr[p] - u2, lap);
      T t = u2 - v0;
      t = fma_t<T>(cf.c1, lap, t);
      out = fma_t<T>(cf.c2, s0, t);
    }
    v[x] = out;
#pragma unroll
    for (int m = 0; m < 2 * R; ++m) q[m] = q[m + 1];
  }
}

// 2 points: v = coef0*(u + u[k+1]) (stencil_2.h:20-29); u's k-halo supplies
// u[zs].
template <typename T>
__global__ void __launch_bounds__(kSimpleBX* kSimpleBY)
    k_two_point(Geom g, T coef0, T* __restrict__ v, const T* __restrict__ u, int ichunk) {
  const int k = blockIdx.x * kSimpleBX + threadIdx.x;
  const int j = blockIdx.y * kSimpleBY + threadIdx.y;
  if (k >= g.zs || j >= g.ys) return;
  const int i0 = blockIdx.z * ichunk;
  const int i1 = min(i0 + ichunk, g.xs);
  for (int i = i0; i < i1; ++i) {
    const long long x = g.org + (long long)i * g.si + (long long)j * g.sj + k;
    v[x] = coef0 * (__ldg(u + x) + __ldg(u + x + 1));
  }
}

// The same update with 16-byte accesses: a thread owns V = 16/sizeof(T)
// consecutive points of a row (aligned: rows start on 128-byte boundaries),
// takes u[k+V] with one more load, and walks its chunk of planes two at a
// time so that more loads are in flight.  Rows carry at least 32 floats of
// padding past zs, so the vector loads of a row's last points stay inside it.
template <typename T>
__global__ void __launch_bounds__(256)
    k_two_point_vec(Geom g, T coef0, T* __restrict__ v, const T* __restrict__ u, int ichunk) {
  constexpr int V = 16 / sizeof(T);
  using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) * V;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (k >= g.zs || j >= g.ys) return;
  const int i0 = blockIdx.z * ichunk;
  const int i1 = min(i0 + ichunk, g.xs);
  const long long row = g.org + (long long)j * g.sj + k;
  for (int i = i0; i < i1; i += 2) {
    const bool two = i + 1 < i1;
    const long long x0 = row + (long long)i * g.si, x1 = x0 + g.si;
    const VT a0 = __ldg(reinterpret_cast<const VT*>(u + x0));
    const T n0 = __ldg(u + x0 + V);
    VT a1;
    T n1 = T(0);
    if (two) {
      a1 = __ldg(reinterpret_cast<const VT*>(u + x1));
      n1 = __ldg(u + x1 + V);
    }
    T e0[V + 1], e1[V + 1];
    memcpy(e0, &a0, sizeof a0);
    e0[V] = n0;
    if (two) {
      memcpy(e1, &a1, sizeof a1);
      e1[V] = n1;
    }
    T o0[V], o1[V];
#pragma unroll
    for (int c = 0; c < V; ++c) {
      o0[c] = coef0 * (e0[c] + e0[c + 1]);
      o1[c] = two ? coef0 * (e1[c] + e1[c + 1]) : T(0);
    }
    if (k + V <= g.zs) {
      VT w0;
      memcpy(&w0, o0, sizeof w0);
      *reinterpret_cast<VT*>(v + x0) = w0;
      if (two) {
        VT w1;
        memcpy(&w1, o1, sizeof w1);
        *reinterpret_cast<VT*>(v + x1) = w1;
      }
    } else {
      for (int c = 0; c < V && k + c < g.zs; ++c) {
        v[x0 + c] = o0[c];
        if (two) v[x1 + c] = o1[c];
      }
    }
  }
}

template <typename T, int P, int MODE>
cudaError_t launch_t(const Geom& g, const void* coefs, void* v, const void* u, const void* s,
                     const Source& src, int ichunk, cudaStream_t stream) {
  const Coefs<T>& cf = *static_cast<const Coefs<T>*>(coefs);
  dim3 block(kSimpleBX, kSimpleBY, 1);
  dim3 grid((g.zs + kSimpleBX - 1) / kSimpleBX, (g.ys + kSimpleBY - 1) / kSimpleBY,
            (g.xs + ichunk - 1) / ichunk);
  if constexpr (P == 2) {
    // 16-byte accesses need 16-byte aligned rows (always: rows start on
    // 128-byte boundaries) and a 16-byte aligned base
    if (((uintptr_t)v | (uintptr_t)u) % 16 == 0) {
      constexpr int V = 16 / sizeof(T);
      dim3 vb(64, 4, 1);
      dim3 vg((g.zs + 64 * V - 1) / (64 * V), (g.ys + 3) / 4, (g.xs + ichunk - 1) / ichunk);
      k_two_point_vec<T><<<vg, vb, 0, stream>>>(g, cf.coef0, (T*)v, (const T*)u, ichunk);
    } else {
      k_two_point<T><<<grid, block, 0, stream>>>(g, cf.coef0, (T*)v, (const T*)u, ichunk);
    }
  } else {
    T amp = sizeof(T) == 8 ? (T)src.amp_d : (T)src.amp;
    k_simple<T, P, MODE><<<grid, block, 0, stream>>>(g, cf, (T*)v, (const T*)u, (const T*)s,
                                                      src.i, src.j, src.k, amp, ichunk);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_typed(int points, int mode, const Geom& g, const void* coefs, void* v,
                         const void* u, const void* s, const Source& src, int ichunk,
                         cudaStream_t stream) {
#define ST3D_CASE(PTS)                                                                   \
  case PTS:                                                                              \
    return mode == ST3D_MODE_REF                                                         \
               ? launch_t<T, PTS, ST3D_MODE_REF>(g, coefs, v, u, s, src, ichunk, stream) \
               : launch_t<T, PTS, ST3D_MODE_WAVE>(g, coefs, v, u, s, src, ichunk, stream);
  switch (points) {
    case 2:
      return launch_t<T, 2, ST3D_MODE_REF>(g, coefs, v, u, s, src, ichunk, stream);
      ST3D_CASE(7)
      ST3D_CASE(13)
      ST3D_CASE(25)
    default:
      return cudaErrorInvalidValue;
  }
#undef ST3D_CASE
}

}  // namespace

cudaError_t launch_simple(int points, int mode, int storage, const Geom& g, const void* coefs,
                          void* v, const void* u, const void* s, const Source& src, int ichunk,
                          cudaStream_t stream) {
  if (ichunk <= 0) ichunk = 64;
  if (storage == ST3D_F32)
    return launch_typed<float>(points, mode, g, coefs, v, u, s, src, ichunk, stream);
  if (storage == ST3D_F64)
    return launch_typed<double>(points, mode, g, coefs, v, u, s, src, ichunk, stream);
  return cudaErrorInvalidValue;
}

}  // namespace st3d
