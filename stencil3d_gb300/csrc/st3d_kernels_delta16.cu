// st3d_kernels_delta16.cu -- the FP16 / BF16 storage forms of the leapfrog
// wave step: u and the time difference d = u^n - u^{n-1} held in 16 bits with
// a power-of-two scale per i-plane, arithmetic in FP32.
//
// Why d and not u^{n-1}: the leapfrog velocity information is the small
// difference of two consecutive levels (|u^n - u^{n-1}| is ~1e-3 |u| for the
// blob workloads at CFL 0.075), which 11 significant bits of u^{n-1} cannot
// carry; the recurrence
//     d^{n+1} = d^n + c1 * lap(u^n) + c2 * (s + a_n delta_src)
//     u^{n+1} = u^n + d^{n+1}
// is the same leapfrog update (u^{n+1} = 2u^n - u^{n-1} + ...) with the
// difference stored at its own scale, so rounding affects u and d only
// relative to their own size.
//
// One step reads u (with its neighbours), d and s and writes u^{n+1} into the
// other u buffer and d^{n+1} in place: 10 bytes per point.  The kernel has
// the structure of the FP32 kernel (persistent CTAs over 16-row x 128-point x
// ichunk-plane units, a producer warp streaming TMA tiles through an mbarrier
// ring, one consumer warp per row, 4 points per lane, a register queue of
// 2R+1 planes along i) with these differences:
//   - the j and k neighbours are read as 16-bit words straight from the TMA
//     tile (64-bit loads, four words per lane) and converted in registers;
//     their sum runs in units of the centre plane's scale and is scaled once,
//     so no decoded tile and no barrier between the consumer warps is needed;
//   - lap = sum_p w_p (a_p + b_p) + m2s * u with m2s = -2 sum_p w_p, on
//     packed FP32 pairs (fma.rn.f32x2 / add.rn.f32x2, per component exactly
//     the scalar operations);
//   - d^{n+1} is encoded with the scale of its plane, decoded again, and the
//     decoded value is what u^{n+1} adds, so that the stored u and d stay
//     consistent;
//   - the producer publishes each stage's plane scales in shared memory and
//     adds the stage's maxima of |u^{n+1}| and |d^{n+1}| (folded by the
//     consumers into shared words) to the global per-plane maxima; a small
//     kernel before each step turns the maxima of the current levels into
//     the scales of the next ones (the bound is in st3d_f16.cuh).
#include "st3d_f16.cuh"
#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

constexpr int kTK = 128;
constexpr int kKH = 8;                  // 16-bit words of k halo either side (16 bytes)
constexpr int kUKW = kTK + 2 * kKH;     // words per u-tile row

template <int P>
struct RadD {
  static constexpr int value = (P == 25) ? 4 : (P == 13) ? 2 : 1;
};

// Producer-published plane scales of one stage (2^E, or 2^-E to encode).
struct StageScales {
  float up;     // plane entering the queue (i + R) of u
  float uc;     // centre plane i of u
  float d;      // plane i of d
  float s;      // plane i of s
  float inv_uo; // plane i of u^{n+1}
  float inv_do; // plane i of d^{n+1}
  float dq;     // plane i of d^{n+1} (decoding it back)
  float inv_uc; // 1 / uc
};

struct Delta16Args {
  Geom g;
  Coefs<float> cf;
  uint16_t* uout;
  uint16_t* d;
  const int *Eu, *Ed, *Es, *Eu_out, *Ed_out;
  uint32_t *Mu_out, *Md_out;
  float m2s;
  int ntk, ntjk, ichunk, units;
  Source src;
  uint64_t timeout_ns;
  uint32_t* status;
  uint16_t* lout;  // PAIR: lo words of u^{n+1}
};

__device__ __forceinline__ float amax4(const P4& x, bool c0, bool c1, bool c2, bool c3, float m) {
  if (c0) m = fmaxf(m, fabsf(x.a.x));
  if (c1) m = fmaxf(m, fabsf(x.a.y));
  if (c2) m = fmaxf(m, fabsf(x.b.x));
  if (c3) m = fmaxf(m, fabsf(x.b.y));
  return m;
}

// TJ = 16 or 20 rows: one CTA of 17 or 21 warps per SM; TJ = 8: two CTAs of
// 9 warps.  PAIR (the F16_HL form, FP16 words): u^n also has lo words (lmap,
// a third tile per stage for the centre plane); the centre u is hi + lo, the
// neighbours the hi words, and u^{n+1} is written as a pair.
template <int KIND, int P, int TJ, int NV, bool PAIR>
__global__ void __launch_bounds__((TJ + 1) * 32, TJ == 8 ? 2 : 1)
    k_delta16(const __grid_constant__ CUtensorMap umap, const __grid_constant__ CUtensorMap dmap,
              const __grid_constant__ CUtensorMap smap, const __grid_constant__ CUtensorMap lmap,
              const Delta16Args a) {
  constexpr int R = RadD<P>::value;
  constexpr int QN = 2 * R + 1;
  constexpr int NU = NV + R;
  constexpr int NP = npairs_of(P);
  constexpr int USLOT = (kUKW * (TJ + 2 * R) * 2 + 127) / 128 * 128;  // bytes
  constexpr int VSLOT = kTK * TJ * 2;                                  // bytes
  constexpr uint32_t UBYTES = kUKW * (TJ + 2 * R) * 2;

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* ur = smem;
  unsigned char* dr = ur + NU * USLOT;
  unsigned char* sr = dr + NV * VSLOT;
  unsigned char* lr = sr + NV * VSLOT;  // PAIR: lo words of the centre plane of u
  uint64_t* full = reinterpret_cast<uint64_t*>(lr + (PAIR ? NV * VSLOT : 0));
  uint64_t* empty = full + NV;
  StageScales* info = reinterpret_cast<StageScales*>(empty + NV);
  uint32_t* smax_u = reinterpret_cast<uint32_t*>(info + NV);
  uint32_t* smax_d = smax_u + NV;
  int* splane = reinterpret_cast<int*>(smax_d + NV);

  const Geom& g = a.g;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TJ);
      smax_u[s] = 0u;
      smax_d[s] = 0u;
      splane[s] = -1;
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if (warp == TJ) {
    // ---------------- producer (whole warp; lane 0 drives the pipeline) -----
    if (lane == 0) {
      tma_prefetch_desc(&umap);
      tma_prefetch_desc(&dmap);
      tma_prefetch_desc(&smap);
      if (PAIR) tma_prefetch_desc(&lmap);
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
        // lane L fetches the scales of step n0 + L: one load per array for
        // 32 steps, none on the per-stage path
        int e_up = 0, e_uc = 0, e_d = 0, e_s = 0, e_uo = 0, e_do = 0;
        {
          const int n = n0 + lane;
          const int p = ia - R + n;
          if (n < nsteps && p >= 0 && p < g.xs) e_up = a.Eu[p];
          if (n < nsteps && n >= 2 * R) {
            const int i = ia + n - 2 * R;
            e_uc = a.Eu[i];
            e_d = a.Ed[i];
            e_s = a.Es[i];
            e_uo = a.Eu_out[i];
            e_do = a.Ed_out[i];
          }
        }
        const int cnt = min(32, nsteps - n0);
        for (int m = 0; m < cnt; ++m, ++h) {
          StageScales si;
          si.up = exp2i(__shfl_sync(0xffffffffu, e_up, m));
          const int euc = __shfl_sync(0xffffffffu, e_uc, m);
          si.uc = exp2i(euc);
          si.inv_uc = exp2i(-euc);
          si.d = exp2i(__shfl_sync(0xffffffffu, e_d, m));
          si.s = exp2i(__shfl_sync(0xffffffffu, e_s, m));
          si.inv_uo = exp2i(-__shfl_sync(0xffffffffu, e_uo, m));
          const int edo = __shfl_sync(0xffffffffu, e_do, m);
          si.inv_do = exp2i(-edo);
          si.dq = exp2i(edo);
          const int n = n0 + m;
          const int stage = (int)(h % NV);
          int good = 1;
          if (lane == 0 && h >= (uint32_t)NV) {
            if (!mbar_wait_bounded(&empty[stage], ((h / NV) - 1) & 1u, a.timeout_ns)) {
              atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
              good = 0;
            } else if (splane[stage] >= 0) {
              if (smax_u[stage]) atomicMax(&a.Mu_out[splane[stage]], smax_u[stage]);
              if (smax_d[stage]) atomicMax(&a.Md_out[splane[stage]], smax_d[stage]);
              smax_u[stage] = 0u;
              smax_d[stage] = 0u;
            }
          }
          good = __shfl_sync(0xffffffffu, good, 0);
          if (!good) {
            ok = false;
            break;
          }
          if (lane == 0) {
            const int p = ia - R + n;
            const bool has_ds = n >= 2 * R;
            splane[stage] = has_ds ? ia + n - 2 * R : -1;
            info[stage] = si;
            mbar_arrive_expect_tx(&full[stage], UBYTES + (has_ds ? (PAIR ? 3u : 2u) * VSLOT : 0u));
            tma_load_3d(ur + (h % NU) * USLOT, &umap, &full[stage], g.pk + k0 - kKH, g.pj + j0 - R,
                        g.pi + p);
            if (has_ds) {
              const int i = ia + n - 2 * R;
              tma_load_3d(dr + stage * VSLOT, &dmap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
              tma_load_3d(sr + stage * VSLOT, &smap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
              if (PAIR)
                tma_load_3d(lr + stage * VSLOT, &lmap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
            }
          }
          __syncwarp();
        }
      }
    }
    // Drain: no copy in flight, every stage consumed, maxima flushed.
    if (lane == 0) {
      for (uint32_t m = (h > (uint32_t)NV ? h - NV : 0u); m < h; ++m) {
        const int stage = (int)(m % NV);
        const bool landed = mbar_wait_bounded(&full[stage], (m / NV) & 1u, a.timeout_ns);
        if (!landed || !mbar_wait_bounded(&empty[stage], (m / NV) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          continue;
        }
        if (splane[stage] >= 0) {
          if (smax_u[stage]) atomicMax(&a.Mu_out[splane[stage]], smax_u[stage]);
          if (smax_d[stage]) atomicMax(&a.Md_out[splane[stage]], smax_d[stage]);
        }
      }
    }
    return;
  }

  // ---------------- consumers ----------------
  const int r = warp;
  uint32_t h = 0;
  bool failed = false;
  const float2 c1 = splat(a.cf.c1), c2 = splat(a.cf.c2), m2s = splat(a.m2s);
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
    const bool k0ok = row_ok && k < g.zs, k1ok = row_ok && k + 1 < g.zs;
    const bool k2ok = row_ok && k + 2 < g.zs, k3ok = row_ok && k + 3 < g.zs;
    // the source point, if this lane holds it: its column in the lane
    const int src_c = (j == a.src.j && (unsigned)(a.src.k - k) < 4u) ? a.src.k - k : -1;
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
        const StageScales si = info[stage];
        q[ph] = decode4<KIND>(*reinterpret_cast<const uint2*>(
                                  reinterpret_cast<const uint16_t*>(ur + (hh % NU) * USLOT) +
                                  (r + R) * kUKW + kKH + 4 * lane),
                              si.up);
        float mu = 0.0f, md = 0.0f;
        if (n >= 2 * R) {
          const int i = ia + n - 2 * R;
          // Neighbours along j and k come straight from the 16-bit centre
          // tile; the sum runs in units of the centre plane's scale (the
          // words themselves) and is scaled once at the end, and the i pairs
          // (decoded with their own planes' scales) enter multiplied by the
          // inverse scale.  Power-of-two scaling commutes with every rounding,
          // so this is bit for bit the sum of scaled values.
          const uint16_t* row = reinterpret_cast<const uint16_t*>(ur + ((hh - R) % NU) * USLOT) +
                                (r + R) * kUKW + kKH + 4 * lane;
          const uint2 wl = *reinterpret_cast<const uint2*>(row - 4);
          const uint2 wc = *reinterpret_cast<const uint2*>(row);
          const uint2 wr = *reinterpret_cast<const uint2*>(row + 4);
          const float2 l01 = w2_to_f2<KIND>(wl.x), l23 = w2_to_f2<KIND>(wl.y);
          const float2 c01 = w2_to_f2<KIND>(wc.x), c23 = w2_to_f2<KIND>(wc.y);
          const float2 r01 = w2_to_f2<KIND>(wr.x), r23 = w2_to_f2<KIND>(wr.y);
          const float w[12] = {l01.x, l01.y, l23.x, l23.y, c01.x, c01.y, c23.x, c23.y,
                               r01.x, r01.y, r23.x, r23.y};
          P4 u0;
          if (PAIR) {
            // the whole pair: hi + lo is exact in float (at most 22 bits)
            const uint2 lw = *reinterpret_cast<const uint2*>(lr + stage * VSLOT + (r * kTK + 4 * lane) * 2);
            u0 = {__fmul2_rn(__fadd2_rn(c01, w2_to_f2<KIND>(lw.x)), splat(si.uc)),
                  __fmul2_rn(__fadd2_rn(c23, w2_to_f2<KIND>(lw.y)), splat(si.uc))};
          } else {
            u0 = {__fmul2_rn(c01, splat(si.uc)), __fmul2_rn(c23, splat(si.uc))};
          }
          P4 acc;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const int ax = pair_axis(P, p);
            const int rr = pair_r(P, p);
            P4 sum;
            if (ax == 2 && (rr & 1)) {
              // odd offsets: the operands straddle register pairs, so the
              // sums are formed one point at a time (same rounding)
              sum = {make_float2(w[4 - rr] + w[4 + rr], w[5 - rr] + w[5 + rr]),
                     make_float2(w[6 - rr] + w[6 + rr], w[7 - rr] + w[7 + rr])};
            } else if (ax == 2) {
              sum = add4({make_float2(w[4 - rr], w[5 - rr]), make_float2(w[6 - rr], w[7 - rr])},
                         {make_float2(w[4 + rr], w[5 + rr]), make_float2(w[6 + rr], w[7 + rr])});
            } else if (ax == 1) {
              const uint2 A = *reinterpret_cast<const uint2*>(row - rr * kUKW);
              const uint2 B = *reinterpret_cast<const uint2*>(row + rr * kUKW);
              sum = add4({w2_to_f2<KIND>(A.x), w2_to_f2<KIND>(A.y)},
                         {w2_to_f2<KIND>(B.x), w2_to_f2<KIND>(B.y)});
            } else {
              sum = add4(q[(ph + 2 * QN - R - rr) % QN], q[(ph + QN - R + rr) % QN]);
              // the i pairs close the 13- and 25-point orders: the sum so far
              // is scaled before the first of them, so they enter as they are;
              // the 7-point order starts with its i pair, which enters in the
              // centre plane's units
              if (p == 0) sum = mul4(sum, splat(si.inv_uc));
              else if (pair_axis(P, p - 1) != 0) acc = mul4(acc, splat(si.uc));
            }
            acc = p == 0 ? mul4(sum, splat(a.cf.cf[p])) : fma4(splat(a.cf.cf[p]), sum, acc);
          }
          if (pair_axis(P, NP - 1) != 0) acc = mul4(acc, splat(si.uc));
          const P4 lap = fma4(m2s, u0, acc);
          // d and s of plane i
          const uint2 dw = *reinterpret_cast<const uint2*>(dr + stage * VSLOT + (r * kTK + 4 * lane) * 2);
          const uint2 sw = *reinterpret_cast<const uint2*>(sr + stage * VSLOT + (r * kTK + 4 * lane) * 2);
          const P4 d0 = decode4<KIND>(dw, si.d);
          P4 s0 = decode4<KIND>(sw, si.s);
          if (i == a.src.i && src_c >= 0) {
            if (src_c == 0) s0.a.x = s0.a.x + a.src.amp;
            if (src_c == 1) s0.a.y = s0.a.y + a.src.amp;
            if (src_c == 2) s0.b.x = s0.b.x + a.src.amp;
            if (src_c == 3) s0.b.y = s0.b.y + a.src.amp;
          }
          const P4 dn = fma4(c2, s0, fma4(c1, lap, d0));
          // d^{n+1}: encode, decode back, add to u
          const uint2 dwo = encode4<KIND>(dn, si.inv_do);
          const P4 dq = decode4<KIND>(dwo, si.dq);
          const P4 un = add4(u0, dq);
          uint2 uwo, ulo = make_uint2(0u, 0u);
          if (PAIR) {
            // hi = fp16(t), lo = fp16(t - hi): t - hi is exact in float
            const float2 t01 = __fmul2_rn(un.a, splat(si.inv_uo));
            const float2 t23 = __fmul2_rn(un.b, splat(si.inv_uo));
            uwo = make_uint2(f2_to_w2<KIND>(t01), f2_to_w2<KIND>(t23));
            const float2 h01 = w2_to_f2<KIND>(uwo.x), h23 = w2_to_f2<KIND>(uwo.y);
            ulo = make_uint2(f2_to_w2<KIND>(__fadd2_rn(t01, make_float2(-h01.x, -h01.y))),
                             f2_to_w2<KIND>(__fadd2_rn(t23, make_float2(-h23.x, -h23.y))));
          } else {
            uwo = encode4<KIND>(un, si.inv_uo);
          }
          mu = amax4(un, k0ok, k1ok, k2ok, k3ok, mu);
          md = amax4(dn, k0ok, k1ok, k2ok, k3ok, md);
          if (row_ok) {
            const long long x0 = rowoff + (long long)i * g.si;
            if (k3ok) {
              *reinterpret_cast<uint2*>(a.uout + x0) = uwo;
              *reinterpret_cast<uint2*>(a.d + x0) = dwo;
              if (PAIR) *reinterpret_cast<uint2*>(a.lout + x0) = ulo;
            } else {
              const uint16_t uo[4] = {(uint16_t)(uwo.x & 0xffff), (uint16_t)(uwo.x >> 16),
                                      (uint16_t)(uwo.y & 0xffff), (uint16_t)(uwo.y >> 16)};
              const uint16_t do_[4] = {(uint16_t)(dwo.x & 0xffff), (uint16_t)(dwo.x >> 16),
                                       (uint16_t)(dwo.y & 0xffff), (uint16_t)(dwo.y >> 16)};
              const uint16_t lo_[4] = {(uint16_t)(ulo.x & 0xffff), (uint16_t)(ulo.x >> 16),
                                       (uint16_t)(ulo.y & 0xffff), (uint16_t)(ulo.y >> 16)};
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (k + c < g.zs) {
                  a.uout[x0 + c] = uo[c];
                  a.d[x0 + c] = do_[c];
                  if (PAIR) a.lout[x0 + c] = lo_[c];
                }
            }
          }
        }
        const uint32_t wu = __reduce_max_sync(0xffffffffu, __float_as_uint(mu));
        const uint32_t wd = __reduce_max_sync(0xffffffffu, __float_as_uint(md));
        if (lane == 0) {
          if (wu) atomicMax(&smax_u[stage], wu);
          if (wd) atomicMax(&smax_d[stage], wd);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
      }
    }
    h += (uint32_t)nsteps;
  }
}

// Scales of the planes written by one step and the reset of their maxima:
//   Bd = Md[i] + k4 * max_{|e|<=R} Mu[i+e] + c2 * (Ms[i] + |a_n| [i == src_i])
//   Bu = Mu[i] + Bd
// (|d^{n+1}| <= Bd and |u^{n+1}| <= Bu up to FP32 rounding, which the 2^14
// ceiling of the scaled values leaves room for).
__global__ void k_scales_delta(int xs, int R, const uint32_t* __restrict__ Mu, const uint32_t* __restrict__ Md,
                               const uint32_t* __restrict__ Ms, int* __restrict__ Eu_out,
                               int* __restrict__ Ed_out, uint32_t* __restrict__ Mu_out,
                               uint32_t* __restrict__ Md_out, float k4, float c2, int src_i,
                               float amp_abs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= xs) return;
  float nb = 0.0f;
  for (int e = -R; e <= R; ++e)
    if (i + e >= 0 && i + e < xs) nb = fmaxf(nb, __uint_as_float(Mu[i + e]));
  float Bd = __fmaf_rn(k4, nb, __uint_as_float(Md[i]));
  Bd = __fmaf_rn(c2, __uint_as_float(Ms[i]) + (i == src_i ? amp_abs : 0.0f), Bd);
  const float Bu = __uint_as_float(Mu[i]) + Bd;
  Ed_out[i] = scale_exponent(Bd);
  Eu_out[i] = scale_exponent(Bu);
  Mu_out[i] = 0u;
  Md_out[i] = 0u;
}

template <int KIND, int P, int TJ, int NV, bool PAIR>
cudaError_t launch_nv(const Tma16Plan& pl, const Delta16Args& args, const CUtensorMap* maps,
                      cudaStream_t stream, int* occupancy_out) {
  auto kern = k_delta16<KIND, P, TJ, NV, PAIR>;
  const int threads = (TJ + 1) * 32;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  if (e != cudaSuccess) return e;
  if (occupancy_out) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy_out, kern, threads, pl.smem);
  kern<<<pl.grid, threads, pl.smem, stream>>>(maps[0], maps[1], maps[2], maps[3], args);
  return cudaGetLastError();
}

// Pipeline depths per tile height: 8 and 16 rows take 4/6/8/12 stages; 20
// rows (21 warps, 80 registers) take 6/8/10, the depths that fit 227 KB.
// The pair form carries a third tile per stage: 4/6/8, and 6/8 on 20 rows.
template <int KIND, int P, int TJ, bool PAIR>
cudaError_t launch_tj(const Tma16Plan& pl, const Delta16Args& args, const CUtensorMap* maps,
                      cudaStream_t stream, int* occ) {
  if constexpr (PAIR && TJ == 20) {
    switch (pl.nv) {
      case 6: return launch_nv<KIND, P, TJ, 6, PAIR>(pl, args, maps, stream, occ);
      case 8: return launch_nv<KIND, P, TJ, 8, PAIR>(pl, args, maps, stream, occ);
      default: return cudaErrorInvalidConfiguration;
    }
  } else if constexpr (PAIR) {
    switch (pl.nv) {
      case 4: return launch_nv<KIND, P, TJ, 4, PAIR>(pl, args, maps, stream, occ);
      case 6: return launch_nv<KIND, P, TJ, 6, PAIR>(pl, args, maps, stream, occ);
      case 8: return launch_nv<KIND, P, TJ, 8, PAIR>(pl, args, maps, stream, occ);
      default: return cudaErrorInvalidConfiguration;
    }
  } else if constexpr (TJ == 20) {
    switch (pl.nv) {
      case 6: return launch_nv<KIND, P, TJ, 6, PAIR>(pl, args, maps, stream, occ);
      case 8: return launch_nv<KIND, P, TJ, 8, PAIR>(pl, args, maps, stream, occ);
      case 10: return launch_nv<KIND, P, TJ, 10, PAIR>(pl, args, maps, stream, occ);
      default: return cudaErrorInvalidConfiguration;
    }
  } else {
    switch (pl.nv) {
      case 4: return launch_nv<KIND, P, TJ, 4, PAIR>(pl, args, maps, stream, occ);
      case 6: return launch_nv<KIND, P, TJ, 6, PAIR>(pl, args, maps, stream, occ);
      case 8: return launch_nv<KIND, P, TJ, 8, PAIR>(pl, args, maps, stream, occ);
      case 12: return launch_nv<KIND, P, TJ, 12, PAIR>(pl, args, maps, stream, occ);
      default: return cudaErrorInvalidConfiguration;
    }
  }
}

template <int KIND, int P, bool PAIR>
cudaError_t launch_p(const Tma16Plan& pl, const Delta16Args& args, const CUtensorMap* maps,
                     cudaStream_t stream, int* occ) {
  if (pl.tj == 16) return launch_tj<KIND, P, 16, PAIR>(pl, args, maps, stream, occ);
  if (pl.tj == 20) return launch_tj<KIND, P, 20, PAIR>(pl, args, maps, stream, occ);
  if (pl.tj == 8) return launch_tj<KIND, P, 8, PAIR>(pl, args, maps, stream, occ);
  return cudaErrorInvalidConfiguration;
}

template <int KIND, bool PAIR>
cudaError_t launch_k(int points, const Tma16Plan& pl, const Delta16Args& args, const CUtensorMap* maps,
                     cudaStream_t stream, int* occ) {
  switch (points) {
    case 7: return launch_p<KIND, 7, PAIR>(pl, args, maps, stream, occ);
    case 13: return launch_p<KIND, 13, PAIR>(pl, args, maps, stream, occ);
    case 25: return launch_p<KIND, 25, PAIR>(pl, args, maps, stream, occ);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch(int storage, int points, const Tma16Plan& pl, const Delta16Args& args,
                     const CUtensorMap* maps, cudaStream_t stream, int* occ) {
  if (storage == ST3D_F16) return launch_k<0, false>(points, pl, args, maps, stream, occ);
  if (storage == ST3D_BF16) return launch_k<1, false>(points, pl, args, maps, stream, occ);
  if (storage == ST3D_F16_HL) return launch_k<0, true>(points, pl, args, maps, stream, occ);
  return cudaErrorInvalidValue;
}

}  // namespace

size_t delta16_smem_bytes(int tj, int nv, int R, bool pair) {
  const size_t uslot = ((size_t)kUKW * (tj + 2 * R) * 2 + 127) / 128 * 128;
  const size_t vslot = (size_t)kTK * tj * 2;
  return (size_t)(nv + R) * uslot + (pair ? 3 : 2) * (size_t)nv * vslot +
         2 * (size_t)nv * 8 + (size_t)nv * sizeof(StageScales) + 3 * (size_t)nv * 4 + 128;
}

int delta16_blocks_per_sm(int storage, int points, const Tma16Plan& pl) {
  Delta16Args dummy;
  int occ = 0;
  if (dispatch(storage, points, pl, dummy, nullptr, nullptr, &occ) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

cudaError_t launch_delta16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                           const Coefs<float>& cf, const Delta16Step& st, const Source& src,
                           uint32_t* dev_status, cudaStream_t stream) {
  Delta16Args a;
  a.g = g;
  a.cf = cf;
  a.uout = st.uout;
  a.d = st.d;
  a.Eu = st.Eu;
  a.Ed = st.Ed;
  a.Es = st.Es;
  a.Eu_out = st.Eu_out;
  a.Ed_out = st.Ed_out;
  a.Mu_out = st.Mu_out;
  a.Md_out = st.Md_out;
  a.m2s = st.m2s;
  a.ntk = pl.ntk;
  a.ntjk = pl.ntj * pl.ntk;
  a.ichunk = pl.ichunk;
  a.units = pl.units;
  a.src = src;
  a.timeout_ns = pl.timeout_ns;
  a.status = dev_status;
  a.lout = st.lout;
  if (pl.pair != (st.lout != nullptr)) return cudaErrorInvalidValue;
  const CUtensorMap maps[4] = {pl.uhi[st.ubuf], pl.dmap, pl.vhi[2], pl.lo[st.ubuf]};
  cudaError_t e = launch_scales_delta(g, pl.radius, st, cf.c2, src, stream);
  if (e != cudaSuccess) return e;
  return dispatch(storage, points, pl, a, maps, stream, nullptr);
}

cudaError_t launch_scales_delta(const Geom& g, int R, const Delta16Step& st, float c2, const Source& src,
                                cudaStream_t stream) {
  k_scales_delta<<<(g.xs + 255) / 256, 256, 0, stream>>>(g.xs, R, st.Mu, st.Md, st.Ms, st.Eu_out,
                                                         st.Ed_out, st.Mu_out, st.Md_out, st.k4, c2,
                                                         src.i, fabsf(src.amp));
  return cudaGetLastError();
}

}  // namespace st3d
