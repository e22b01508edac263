// st3d_kernels_tma16.cu -- the compensated precision form: the leapfrog
// wave step on u and v stored as FP16 words with a power-of-two scale per
// i-plane plus a compensating low byte per point (FP16 + int8, ~19
// significant bits), arithmetic and accumulation in FP32.  (The FP16 / BF16
// forms without the low byte hold u and the time difference instead of v:
// st3d_kernels_delta16.cu.)  The kernel keeps the word type as a template
// parameter; only FP16 words are instantiated.
//
// Same structure as the FP32 kernel (st3d_kernels_tma.cu): persistent CTAs
// over (16-row x 128-point x ichunk-plane) work units, a producer warp
// streaming TMA tiles through an mbarrier pipeline, one consumer warp per
// row with 4 points per lane and a register queue of 2R+1 planes along i.
// What differs:
//   - tiles hold 16-bit words (the u tile keeps 8 words = 16 bytes of halo
//     either side along k); the compensated form adds byte tiles for the
//     centre plane of u and for v;
//   - values are decoded to FP32 on load (exact: h*2^E, plus q*ulp(h)/256*2^E
//     for the compensated form) and encoded on store (st3d_f16.cuh); the
//     neighbour terms use the 16-bit word, the centre u and v use the full
//     compensated value;
//   - the producer publishes each stage's plane scales in shared memory and
//     derives the scale of the plane being written from the per-plane maxima
//     of the previous two time levels (the bound in st3d_f16.cuh); consumers
//     fold |v_new| into a per-stage shared maximum that the producer adds to
//     the global per-plane maximum with one atomic per stage.
// The arithmetic on decoded values is the FP32 kernel's difference form, in
// the same operation order.
#include "st3d_f16.cuh"
#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

constexpr int kTK = 128;
constexpr int kKH16 = 8;               // 16-bit words of k halo either side (16 bytes)
constexpr int kUKW16 = kTK + 2 * kKH16;  // words per u-tile row

template <int KIND>
struct Word;
template <>
struct Word<0> {  // FP16
  static __device__ __forceinline__ float to_float(uint16_t b) {
    return __half2float(__ushort_as_half(b));
  }
  static __device__ __forceinline__ uint16_t from_float(float x) {
    return __half_as_ushort(__float2half_rn(x));
  }
};
// Producer-published scales of one stage.
struct StageInfo {
  int e_up;   // plane entering the queue (i + R)
  int e_uc;   // centre plane i of u
  int e_v;    // plane i of v
  int e_s;    // plane i of s
  int e_out;  // plane i of the field being written
  int pad[3];
};

template <int P>
struct Rad {
  static constexpr int value = (P == 25) ? 4 : (P == 13) ? 2 : 1;
};

struct Tma16Args {
  Geom g;
  Coefs<float> cf;
  uint16_t* vout;
  int8_t* vlo_out;
  const int* Eu;
  const int* Ev;
  const int* Es;
  const int* Eout;
  const uint32_t* Mu;
  const uint32_t* Mv;
  const uint32_t* Ms;
  uint32_t* Mout;
  uint32_t* Mzero;
  float k4;
  int ntk, ntjk, ichunk, units;
  Source src;
  uint64_t timeout_ns;
  uint32_t* status;
};

__device__ __forceinline__ float mx(const uint32_t* M, int i) { return __uint_as_float(M[i]); }

template <int KIND, bool HILO, int P, int TJ, int NV>
__global__ void __launch_bounds__((TJ + 1) * 32, 1)
    k_tma16(const __grid_constant__ CUtensorMap uhi, const __grid_constant__ CUtensorMap vhi,
            const __grid_constant__ CUtensorMap shi, const __grid_constant__ CUtensorMap ulo,
            const __grid_constant__ CUtensorMap vlo, const Tma16Args a) {
  using W = Word<KIND>;
  constexpr int R = Rad<P>::value;
  constexpr int QN = 2 * R + 1;
  constexpr int NU = NV + R;
  constexpr int NP = npairs_of(P);
  constexpr int USLOT = (kUKW16 * (TJ + 2 * R) * 2 + 127) / 128 * 128;  // bytes
  constexpr int VSLOT = kTK * TJ * 2;                                    // bytes
  constexpr int LSLOT = kTK * TJ;                                        // bytes
  constexpr uint32_t UBYTES = kUKW16 * (TJ + 2 * R) * 2;
  constexpr uint32_t STEP_BYTES = 2 * VSLOT + (HILO ? 2 * LSLOT : 0);

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* ur = smem;
  unsigned char* vr = ur + NU * USLOT;
  unsigned char* sr = vr + NV * VSLOT;
  unsigned char* ulr = sr + NV * VSLOT;                 // HILO: centre-plane low bytes of u
  unsigned char* vlr = ulr + (HILO ? NV * LSLOT : 0);   // HILO: low bytes of v
  // the rings end on a 128-byte boundary: barriers, then the stage records
  uint64_t* full = reinterpret_cast<uint64_t*>(vlr + (HILO ? NV * LSLOT : 0));
  uint64_t* empty = full + NV;
  StageInfo* info = reinterpret_cast<StageInfo*>(empty + NV);
  uint32_t* smax = reinterpret_cast<uint32_t*>(info + NV);
  int* splane = reinterpret_cast<int*>(smax + NV);

  const Geom& g = a.g;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TJ);
      smax[s] = 0u;
      splane[s] = -1;
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if (warp == TJ) {
    // ---------------- producer (whole warp; lane 0 drives the pipeline) -----
    if (lane == 0) {
      tma_prefetch_desc(&uhi);
      tma_prefetch_desc(&vhi);
      tma_prefetch_desc(&shi);
      if (HILO) {
        tma_prefetch_desc(&ulo);
        tma_prefetch_desc(&vlo);
      }
    }
    uint32_t h = 0;
    bool ok = true;
    for (int unit = blockIdx.x; unit < a.units && ok; unit += gridDim.x) {
      const int ic = unit / a.ntjk;
      const int rem = unit - ic * a.ntjk;
      const int jt = rem / a.ntk;
      const int kt = rem - jt * a.ntk;
      const int k0 = kt * kTK, j0 = jt * TJ;
      const int ia = ic * a.ichunk;
      const int ib = min(ia + a.ichunk, g.xs);
      const int nsteps = (ib - ia) + 2 * R;
      for (int n0 = 0; n0 < nsteps && ok; n0 += 32) {
        // lane L fetches the scales of step n0 + L, one load per array for
        // 32 steps, so no scale load sits on the per-stage path
        int e_up = 0, e_uc = 0, e_v = 0, e_s = 0, e_out = 0;
        {
          const int n = n0 + lane;
          const int p = ia - R + n;
          if (n < nsteps && p >= 0 && p < g.xs) e_up = a.Eu[p];
          if (n < nsteps && n >= 2 * R) {
            const int i = ia + n - 2 * R;
            e_uc = a.Eu[i];
            e_v = a.Ev[i];
            e_s = a.Es[i];
            e_out = a.Eout[i];
          }
        }
        const int cnt = min(32, nsteps - n0);
        for (int m = 0; m < cnt; ++m, ++h) {
          StageInfo si;
          si.e_up = __shfl_sync(0xffffffffu, e_up, m);
          si.e_uc = __shfl_sync(0xffffffffu, e_uc, m);
          si.e_v = __shfl_sync(0xffffffffu, e_v, m);
          si.e_s = __shfl_sync(0xffffffffu, e_s, m);
          si.e_out = __shfl_sync(0xffffffffu, e_out, m);
          const int n = n0 + m;
          const int stage = (int)(h % NV);
          int good = 1;
          if (lane == 0 && h >= (uint32_t)NV) {
            if (!mbar_wait_bounded(&empty[stage], ((h / NV) - 1) & 1u, a.timeout_ns)) {
              atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
              good = 0;
            } else {
              if (splane[stage] >= 0 && smax[stage] != 0u) atomicMax(&a.Mout[splane[stage]], smax[stage]);
              smax[stage] = 0u;
            }
          }
          good = __shfl_sync(0xffffffffu, good, 0);
          if (!good) {
            ok = false;
            break;
          }
          if (lane == 0) {
            const int p = ia - R + n;
            const bool has_vs = n >= 2 * R;
            splane[stage] = has_vs ? ia + n - 2 * R : -1;
            info[stage] = si;
            mbar_arrive_expect_tx(&full[stage], UBYTES + (has_vs ? STEP_BYTES : 0u));
            tma_load_3d(ur + (h % NU) * USLOT, &uhi, &full[stage], g.pk + k0 - kKH16, g.pj + j0 - R,
                        g.pi + p);
            if (has_vs) {
              const int i = ia + n - 2 * R;
              tma_load_3d(vr + stage * VSLOT, &vhi, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
              tma_load_3d(sr + stage * VSLOT, &shi, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
              if (HILO) {
                tma_load_3d(ulr + stage * LSLOT, &ulo, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
                tma_load_3d(vlr + stage * LSLOT, &vlo, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
              }
            }
          }
          __syncwarp();
        }
      }
    }
    // Drain: no copy in flight (full phases complete), every stage consumed,
    // maxima flushed.
    if (lane == 0) {
      for (uint32_t m = (h > (uint32_t)NV ? h - NV : 0u); m < h; ++m) {
        const int stage = (int)(m % NV);
        const bool landed = mbar_wait_bounded(&full[stage], (m / NV) & 1u, a.timeout_ns);
        if (!landed || !mbar_wait_bounded(&empty[stage], (m / NV) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          continue;
        }
        if (splane[stage] >= 0 && smax[stage] != 0u) atomicMax(&a.Mout[splane[stage]], smax[stage]);
      }
    }
    return;
  }

  // ---------------- consumers ----------------
  const int r = warp;
  uint32_t h = 0;
  bool failed = false;
  P4 q[QN];
  for (int unit = blockIdx.x; unit < a.units; unit += gridDim.x) {
    const int ic = unit / a.ntjk;
    const int rem = unit - ic * a.ntjk;
    const int jt = rem / a.ntk;
    const int kt = rem - jt * a.ntk;
    const int j = jt * TJ + r;
    const int k = kt * kTK + 4 * lane;
    const int ia = ic * a.ichunk;
    const int ib = min(ia + a.ichunk, g.xs);
    const int nsteps = (ib - ia) + 2 * R;
    const bool row_ok = j < g.ys;
    const long long rowoff = g.org + (long long)j * g.sj + k;
    for (int n0 = 0; n0 < nsteps; n0 += QN) {
#pragma unroll
      for (int ph = 0; ph < QN; ++ph) {
        const int n = n0 + ph;
        if (n >= nsteps) break;
        const uint32_t hh = h + (uint32_t)n;
        const int stage = (int)(hh % NV);
        // After a timed-out wait the warp stops waiting but keeps stepping and
        // arriving on the stages' empty barriers, so that the producer's
        // bounded waits end and the kernel returns (its results are then
        // void; the status word says so).
        if (!failed && !mbar_wait_bounded(&full[stage], (hh / NV) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutFull);
          failed = true;
        }
        const StageInfo si = info[stage];
        {
          const uint16_t* un = reinterpret_cast<const uint16_t*>(ur + (hh % NU) * USLOT) +
                               (r + R) * kUKW16 + kKH16 + 4 * lane;
          const float sc = exp2i(si.e_up);
          q[ph] = decode4<KIND>(*reinterpret_cast<const uint2*>(un), sc);
        }
        float vmax = 0.0f;
        if (n >= 2 * R) {
          const int i = ia + n - 2 * R;
          const uint16_t* uc = reinterpret_cast<const uint16_t*>(ur + ((hh - R) % NU) * USLOT) +
                               (r + R) * kUKW16;
          const float sc1 = exp2i(si.e_uc);
          const float2 sc = make_float2(sc1, sc1);
          // j and k neighbours straight from the 16-bit centre tile: the
          // pair terms run in units of the centre plane's scale (the words
          // themselves, 2u and the i-pair sums multiplied by the inverse
          // scale) and the sum is scaled once; power-of-two scaling commutes
          // with every rounding, so this is bit for bit the scaled sum.
          const float inv1 = exp2i(-si.e_uc);
          const uint16_t* row = uc + kKH16 + 4 * lane;
          const uint2 wl = *reinterpret_cast<const uint2*>(row - 4);
          const uint2 wc = *reinterpret_cast<const uint2*>(row);
          const uint2 wr = *reinterpret_cast<const uint2*>(row + 4);
          const P4 l4 = words4<KIND>(wl);
          const P4 c4 = words4<KIND>(wc);
          const P4 r4 = words4<KIND>(wr);
          const float w[12] = {l4.a.x, l4.a.y, l4.b.x, l4.b.y, c4.a.x, c4.a.y, c4.b.x, c4.b.y,
                               r4.a.x, r4.a.y, r4.b.x, r4.b.y};
          // centre values: the word, plus the low byte in the compensated form
          P4 u0 = mul4(c4, sc);
          if (HILO) {
            const uint32_t lb = *reinterpret_cast<const uint32_t*>(ulr + stage * LSLOT + r * kTK + 4 * lane);
            const uint16_t cb[4] = {(uint16_t)(wc.x & 0xffff), (uint16_t)(wc.x >> 16),
                                    (uint16_t)(wc.y & 0xffff), (uint16_t)(wc.y >> 16)};
            float uc4[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const float qv = (float)(int8_t)((lb >> (8 * c)) & 0xff);
              uc4[c] = __fmaf_rn(qv, ulp256_f16(cb[c]), W::to_float(cb[c])) * sc1;
            }
            u0 = {make_float2(uc4[0], uc4[1]), make_float2(uc4[2], uc4[3])};
          }
          const P4 u2 = add4(u0, u0);
          const float2 ninv = make_float2(-inv1, -inv1);
          const P4 nu2 = mul4(u2, ninv);  // -2u in the centre plane's units
          P4 acc;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const int ax = pair_axis(P, p);
            const int rr = pair_r(P, p);
            P4 sum;
            if (ax == 2 && (rr & 1)) {
              // odd offsets straddle register pairs: one point at a time
              sum = {make_float2(w[4 - rr] + w[4 + rr], w[5 - rr] + w[5 + rr]),
                     make_float2(w[6 - rr] + w[6 + rr], w[7 - rr] + w[7 + rr])};
            } else if (ax == 2) {
              sum = add4({make_float2(w[4 - rr], w[5 - rr]), make_float2(w[6 - rr], w[7 - rr])},
                         {make_float2(w[4 + rr], w[5 + rr]), make_float2(w[6 + rr], w[7 + rr])});
            } else if (ax == 1) {
              const uint2 A = *reinterpret_cast<const uint2*>(row - rr * kUKW16);
              const uint2 B = *reinterpret_cast<const uint2*>(row + rr * kUKW16);
              sum = add4(words4<KIND>(A), words4<KIND>(B));
            } else {
              sum = add4(q[(ph + 2 * QN - R - rr) % QN], q[(ph + QN - R + rr) % QN]);
            }
            P4 d;
            if (ax != 0) {
              d = add4(sum, nu2);
            } else if (p == 0) {
              // the 7-point order starts with its i pair: centre plane units
              d = add4(mul4(sum, make_float2(inv1, inv1)), nu2);
            } else {
              // the i pairs close the 13- and 25-point orders: the sum so far
              // is scaled before the first of them and they enter as they are
              if (pair_axis(P, p - 1) != 0) acc = mul4(acc, sc);
              d = add4(sum, {make_float2(-u2.a.x, -u2.a.y), make_float2(-u2.b.x, -u2.b.y)});
            }
            const float2 cf2 = make_float2(a.cf.cf[p], a.cf.cf[p]);
            acc = p == 0 ? mul4(d, cf2) : fma4(cf2, d, acc);
          }
          if (pair_axis(P, NP - 1) != 0) acc = mul4(acc, sc);
          // v and s of plane i
          const uint2 vw = *reinterpret_cast<const uint2*>(vr + stage * VSLOT + (r * kTK + 4 * lane) * 2);
          const uint2 sw = *reinterpret_cast<const uint2*>(sr + stage * VSLOT + (r * kTK + 4 * lane) * 2);
          const float scv1 = exp2i(si.e_v), scs1 = exp2i(si.e_s);
          P4 v0;
          if (HILO) {
            const uint32_t vlb = *reinterpret_cast<const uint32_t*>(vlr + stage * LSLOT + r * kTK + 4 * lane);
            const uint16_t vb[4] = {(uint16_t)(vw.x & 0xffff), (uint16_t)(vw.x >> 16),
                                    (uint16_t)(vw.y & 0xffff), (uint16_t)(vw.y >> 16)};
            float vv[4];
#pragma unroll
            for (int c = 0; c < 4; ++c)
              vv[c] = __fmaf_rn((float)(int8_t)((vlb >> (8 * c)) & 0xff), ulp256_f16(vb[c]),
                                W::to_float(vb[c])) * scv1;
            v0 = {make_float2(vv[0], vv[1]), make_float2(vv[2], vv[3])};
          } else {
            v0 = decode4<KIND>(vw, scv1);
          }
          P4 s0 = decode4<KIND>(sw, scs1);
          if (i == a.src.i && j == a.src.j && (unsigned)(a.src.k - k) < 4u) {
            const int c = a.src.k - k;
            if (c == 0) s0.a.x = s0.a.x + a.src.amp;
            if (c == 1) s0.a.y = s0.a.y + a.src.amp;
            if (c == 2) s0.b.x = s0.b.x + a.src.amp;
            if (c == 3) s0.b.y = s0.b.y + a.src.amp;
          }
          const P4 nv0 = {make_float2(-v0.a.x, -v0.a.y), make_float2(-v0.b.x, -v0.b.y)};
          P4 t = add4(u2, nv0);
          t = fma4(make_float2(a.cf.c1, a.cf.c1), acc, t);
          const P4 x = fma4(make_float2(a.cf.c2, a.cf.c2), s0, t);
          const float io = exp2i(-si.e_out);
          const P4 xs = mul4(x, make_float2(io, io));
          uint16_t ob[4];
          uint32_t olo = 0;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const float xsc = p4c(xs, c);
            ob[c] = W::from_float(xsc);
            if (HILO) {
              const float rres = xsc - W::to_float(ob[c]);
              int e = (ob[c] >> 10) & 0x1f;
              if (e == 0) e = 1;
              int qi = __float2int_rn(rres * exp2i(33 - e));
              qi = qi > 127 ? 127 : (qi < -127 ? -127 : qi);
              olo |= ((uint32_t)(qi & 0xff)) << (8 * c);
            }
            if (row_ok && k + c < g.zs) vmax = fmaxf(vmax, fabsf(p4c(x, c)));
          }
          if (row_ok) {
            const long long x0 = rowoff + (long long)i * g.si;
            if (k + 3 < g.zs) {
              *reinterpret_cast<uint2*>(a.vout + x0) =
                  make_uint2((uint32_t)ob[0] | ((uint32_t)ob[1] << 16), (uint32_t)ob[2] | ((uint32_t)ob[3] << 16));
              if (HILO) *reinterpret_cast<uint32_t*>(a.vlo_out + x0) = olo;
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (k + c < g.zs) {
                  a.vout[x0 + c] = ob[c];
                  if (HILO) a.vlo_out[x0 + c] = (int8_t)((olo >> (8 * c)) & 0xff);
                }
            }
          }
        }
        const uint32_t wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(vmax));
        if (lane == 0) {
          if (wmax != 0u) atomicMax(&smax[stage], wmax);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
      }
    }
    h += (uint32_t)nsteps;
  }
}

// Scales of the planes written by one step (the bound of st3d_f16.cuh) and
// the reset of the maxima two time levels ahead.
__global__ void k_scales16(int xs, int R, const uint32_t* __restrict__ Mu, const uint32_t* __restrict__ Mv,
                           const uint32_t* __restrict__ Ms, int* __restrict__ Eout,
                           uint32_t* __restrict__ Mzero, float k4, float c2, int src_i, float amp_abs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= xs) return;
  float nb = 0.0f;
  for (int d = -R; d <= R; ++d)
    if (i + d >= 0 && i + d < xs) nb = fmaxf(nb, mx(Mu, i + d));
  float B = 3.0f * fmaxf(mx(Mu, i), mx(Mv, i));
  B = B + k4 * nb;
  B = B + c2 * (mx(Ms, i) + (i == src_i ? amp_abs : 0.0f));
  Eout[i] = scale_exponent(B);
  Mzero[i] = 0u;
}

}  // namespace

size_t tma16_smem_bytes(int tj, int nv, int R, bool hilo) {
  const size_t uslot = ((size_t)kUKW16 * (tj + 2 * R) * 2 + 127) / 128 * 128;
  const size_t vslot = (size_t)kTK * tj * 2;
  const size_t lslot = (size_t)kTK * tj;
  return (size_t)(nv + R) * uslot + 2 * (size_t)nv * vslot + (hilo ? 2 * (size_t)nv * lslot : 0) +
         2 * (size_t)nv * 8 + (size_t)nv * sizeof(StageInfo) +
         2 * (size_t)nv * 4 + 128;
}

namespace {

template <int KIND, bool HILO, int P, int NV>
cudaError_t launch16_nv(const Tma16Plan& pl, const Tma16Args& args, const CUtensorMap* maps,
                        cudaStream_t stream, int* occupancy_out) {
  auto kern = k_tma16<KIND, HILO, P, 16, NV>;
  const int threads = 17 * 32;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  if (e != cudaSuccess) return e;
  if (occupancy_out) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy_out, kern, threads, pl.smem);
  }
  kern<<<pl.grid, threads, pl.smem, stream>>>(maps[0], maps[1], maps[2], maps[3], maps[4], args);
  return cudaGetLastError();
}

// Pipeline depth: a 16-bit stage carries half the bytes of an FP32 stage
// and is consumed in about half the time, so the ring needs about twice the
// stages to cover the same DRAM latency.
template <int KIND, bool HILO, int P>
cudaError_t launch16_p(const Tma16Plan& pl, const Tma16Args& args, const CUtensorMap* maps,
                       cudaStream_t stream, int* occupancy_out) {
  switch (pl.nv) {
    case 4: return launch16_nv<KIND, HILO, P, 4>(pl, args, maps, stream, occupancy_out);
    case 6: return launch16_nv<KIND, HILO, P, 6>(pl, args, maps, stream, occupancy_out);
    case 8: return launch16_nv<KIND, HILO, P, 8>(pl, args, maps, stream, occupancy_out);
    case 12: return launch16_nv<KIND, HILO, P, 12>(pl, args, maps, stream, occupancy_out);
    default: return cudaErrorInvalidConfiguration;
  }
}

template <int KIND, bool HILO>
cudaError_t launch16_k(int points, const Tma16Plan& pl, const Tma16Args& args, const CUtensorMap* maps,
                       cudaStream_t stream, int* occ) {
  switch (points) {
    case 7: return launch16_p<KIND, HILO, 7>(pl, args, maps, stream, occ);
    case 13: return launch16_p<KIND, HILO, 13>(pl, args, maps, stream, occ);
    case 25: return launch16_p<KIND, HILO, 25>(pl, args, maps, stream, occ);
    default: return cudaErrorInvalidValue;
  }
}

// FP16 / BF16 without the low byte run in the delta form
// (st3d_kernels_delta16.cu); this kernel serves the compensated form.
cudaError_t dispatch16(int storage, int points, const Tma16Plan& pl, const Tma16Args& args,
                       const CUtensorMap* maps, cudaStream_t stream, int* occ) {
  if (storage == ST3D_F16_HILO) return launch16_k<0, true>(points, pl, args, maps, stream, occ);
  return cudaErrorInvalidValue;
}

}  // namespace

int tma16_blocks_per_sm(int storage, int points, const Tma16Plan& pl) {
  Tma16Args dummy;
  int occ = 0;
  if (dispatch16(storage, points, pl, dummy, nullptr, nullptr, &occ) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

cudaError_t launch_tma16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                         const Coefs<float>& cf, const Tma16Step& st, const Source& src,
                         uint32_t* dev_status, cudaStream_t stream) {
  Tma16Args a;
  a.g = g;
  a.cf = cf;
  a.vout = st.vout;
  a.vlo_out = st.vlo_out;
  a.Eu = st.Eu;
  a.Ev = st.Ev;
  a.Es = st.Es;
  a.Eout = st.Eout;
  a.Mu = st.Mu;
  a.Mv = st.Mv;
  a.Ms = st.Ms;
  a.Mout = st.Mout;
  a.Mzero = st.Mzero;
  a.k4 = st.k4;
  a.ntk = pl.ntk;
  a.ntjk = pl.ntj * pl.ntk;
  a.ichunk = pl.ichunk;
  a.units = pl.units;
  a.src = src;
  a.timeout_ns = pl.timeout_ns;
  a.status = dev_status;
  const CUtensorMap maps[5] = {pl.uhi[st.ubuf], pl.vhi[st.vbuf], pl.vhi[2], pl.lo[st.ubuf],
                               pl.lo[st.vbuf]};
  k_scales16<<<(g.xs + 255) / 256, 256, 0, stream>>>(g.xs, pl.radius, st.Mu, st.Mv, st.Ms, st.Eout,
                                                     st.Mzero, st.k4, cf.c2, src.i, fabsf(src.amp));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return dispatch16(storage, points, pl, a, maps, stream, nullptr);
}

}  // namespace st3d
