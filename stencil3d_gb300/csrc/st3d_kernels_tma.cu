// st3d_kernels_tma.cu -- the FP32 hot path: a TMA-staged 2.5D streaming
// stencil kernel for sm_103a.
//
// Replaces the traversal and per-point update of the reference's ITERATE
// (iterators.cpp:130-289 with stencil_{7,13,25}.h) for one time step.
//
// Work decomposition.  A work unit is a tile of TJ rows (j) x 128 points (k)
// and a chunk of `ichunk` planes along i, the slowest axis.  A persistent
// grid of at most (#SMs x resident CTAs) CTAs takes units round robin; the
// unit order runs over all tiles of one i-chunk before the next, so CTAs
// working at the same time hold neighbouring tiles and their halo rows meet
// in L2.
//
// Inside a CTA (warp specialised):
//   - one producer warp: lane 0 streams planes in with 3-D tiled TMA loads,
//     one pipeline stage per plane step: the u tile of plane i+R with its
//     halo (TJ+2R rows x 136 floats: 4 floats = 16 bytes either side along
//     k keep every TMA x-coordinate 16-byte aligned), and the v and s tiles
//     of plane i.  A stage completes on its `full` mbarrier by transaction
//     bytes; the producer reuses a stage once all consumer warps arrived on
//     its `empty` mbarrier.
//   - TJ consumer warps, one per row; each lane owns 4 consecutive k points
//     (one float4).  Along i a lane keeps u(i-R .. i+R) of its 4 points in a
//     register queue of 2R+1 float4 whose slot for local step n is n mod
//     (2R+1): the step loop is unrolled 2R+1 times so every queue index is a
//     compile-time constant and nothing is shifted.  j neighbours come from
//     the shared-memory u tile of plane i (kept for R+1 stages: the u ring has
//     nv+R slots), k neighbours from the same row (128-bit shared loads of
//     the left and right float4).  v and s come from their stage slots; the
//     new v leaves with a 128-bit coalesced store.
// Every wait is bounded (mbar_wait_bounded): on timeout the kernel records
// the reason in a device status word, so a broken pipeline ends as an error
// code instead of a hung GPU.  A consumer warp whose wait gave up does not
// return: it stops waiting but keeps stepping and arriving on the stages'
// empty barriers (its results are void; the status word says so), so the
// producer keeps going to the end of its units and its drain waits for the
// copies it issued last -- a CTA that left with bulk copies still in flight
// into its shared memory could fault the GPU (a mis-sized transaction count
// once did, with Xid 43).  Only a copy that never lands at all, which no
// kernel code can repair, ends the drain's bounded waits with copies in
// flight.
//
// Arithmetic: the same operation sequence as the direct-load kernel and the
// oracle's fma flavour (see st3d_kernels_simple.cu), on packed FP32 pairs
// (add/fma.rn.f32x2, per component the scalar operations; the k pairs of odd
// offset straddle register pairs and are added one point at a time).
#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

template <int P>
struct RadiusOf {
  static constexpr int value = (P == 25) ? 4 : (P == 13) ? 2 : 1;
};

template <int P, int MODE, int TJ, int NV>
__global__ void __launch_bounds__((TJ + 1) * 32, 1)
    k_tma(const __grid_constant__ CUtensorMap umap, const __grid_constant__ CUtensorMap vmap,
          const __grid_constant__ CUtensorMap smap, Geom g, Coefs<float> cf,
          float* __restrict__ vout, int ntk, int ntjk, int ichunk, int units, Source src,
          uint64_t timeout_ns, uint32_t* __restrict__ status) {
  constexpr int R = RadiusOf<P>::value;
  constexpr int QN = 2 * R + 1;
  constexpr int NU = NV + R;
  constexpr int NP = npairs_of(P);
  constexpr int TK = kTmaTK;
  constexpr int UKW = kTmaUKW;
  // Slots start on 128-byte boundaries (TMA shared-memory destinations);
  // the transaction counts are the boxes' bytes.
  constexpr int USLOT = (UKW * (TJ + 2 * R) + 31) / 32 * 32;  // floats
  constexpr int VSLOT = TK * TJ;                              // floats
  constexpr uint32_t UBYTES = UKW * (TJ + 2 * R) * 4;
  constexpr uint32_t VBYTES = VSLOT * 4;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* ur = reinterpret_cast<float*>(smem_raw);
  float* vr = ur + NU * USLOT;
  float* sr = vr + NV * VSLOT;
  uint64_t* full = reinterpret_cast<uint64_t*>(sr + NV * VSLOT);
  uint64_t* empty = full + NV;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TJ);
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if (warp == TJ) {
    // ---------------- producer ----------------
    if (lane == 0) {
      tma_prefetch_desc(&umap);
      tma_prefetch_desc(&vmap);
      tma_prefetch_desc(&smap);
      uint32_t h = 0;
      bool ok = true;
      for (int unit = blockIdx.x; unit < units && ok; unit += gridDim.x) {
        const int ic = unit / ntjk;
        const int rem = unit - ic * ntjk;
        const int jt = rem / ntk;
        const int kt = rem - jt * ntk;
        const int k0 = kt * TK, j0 = jt * TJ;
        const int ia = ic * ichunk;
        const int ib = min(ia + ichunk, g.xs);
        const int nsteps = (ib - ia) + 2 * R;
        for (int n = 0; n < nsteps; ++n, ++h) {
          const int stage = (int)(h % NV);
          if (h >= (uint32_t)NV) {
            if (!mbar_wait_bounded(&empty[stage], ((h / NV) - 1) & 1u, timeout_ns)) {
              atomicExch(status, (uint32_t)kDevTimeoutEmpty);
              ok = false;
              break;
            }
          }
          const bool has_vs = n >= 2 * R;
          mbar_arrive_expect_tx(&full[stage], UBYTES + (has_vs ? 2 * VBYTES : 0u));
          const int p = ia - R + n;  // u plane loaded at this step
          tma_load_3d(ur + (h % NU) * USLOT, &umap, &full[stage], g.pk + k0 - kTmaKHalo,
                      g.pj + j0 - R, g.pi + p);
          if (has_vs) {
            const int i = ia + n - 2 * R;
            tma_load_3d(vr + stage * VSLOT, &vmap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
            tma_load_3d(sr + stage * VSLOT, &smap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
          }
        }
      }
      // Leave no copy in flight: wait for the stages issued last.
      for (uint32_t m = (h > (uint32_t)NV ? h - NV : 0u); m < h; ++m)
        (void)mbar_wait_bounded(&full[m % NV], (m / NV) & 1u, timeout_ns);
    }
    return;
  }

  // ---------------- consumers ----------------
  const int r = warp;
  uint32_t h = 0;
  bool failed = false;
  float4 q[QN];
  for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int ic = unit / ntjk;
    const int rem = unit - ic * ntjk;
    const int jt = rem / ntk;
    const int kt = rem - jt * ntk;
    const int j = jt * TJ + r;
    const int k = kt * TK + 4 * lane;
    const int ia = ic * ichunk;
    const int ib = min(ia + ichunk, g.xs);
    const int nsteps = (ib - ia) + 2 * R;
    const bool row_ok = j < g.ys;
    float* vrow = vout + g.org + (long long)j * g.sj + k;
    for (int n0 = 0; n0 < nsteps; n0 += QN) {
#pragma unroll
      for (int ph = 0; ph < QN; ++ph) {
        const int n = n0 + ph;
        if (n >= nsteps) break;
        const uint32_t hh = h + (uint32_t)n;
        const int stage = (int)(hh % NV);
        if (!failed && !mbar_wait_bounded(&full[stage], (hh / NV) & 1u, timeout_ns)) {
          atomicExch(status, (uint32_t)kDevTimeoutFull);
          failed = true;
        }
        q[ph] = *reinterpret_cast<const float4*>(ur + (hh % NU) * USLOT + (r + R) * UKW +
                                                 kTmaKHalo + 4 * lane);
        if (n >= 2 * R) {
          const int i = ia + n - 2 * R;
          const float* uc = ur + ((hh - R) % NU) * USLOT + (r + R) * UKW;
          const float4 c4 = q[(ph + QN - R) % QN];
          const float4 l4 = *reinterpret_cast<const float4*>(uc + 4 * lane);
          const float4 r4 = *reinterpret_cast<const float4*>(uc + 2 * kTmaKHalo + 4 * lane);
          const float w[12] = {l4.x, l4.y, l4.z, l4.w, c4.x, c4.y, c4.z, c4.w,
                               r4.x, r4.y, r4.z, r4.w};
          const P4 cu = {make_float2(c4.x, c4.y), make_float2(c4.z, c4.w)};
          const P4 u2 = add4(cu, cu);
          const P4 nu2 = {make_float2(-u2.a.x, -u2.a.y), make_float2(-u2.b.x, -u2.b.y)};
          P4 acc;
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const int ax = pair_axis(P, p);
            const int rr = pair_r(P, p);
            P4 sum;
            if (ax == 2 && (rr & 1)) {
              sum = {make_float2(w[4 - rr] + w[4 + rr], w[5 - rr] + w[5 + rr]),
                     make_float2(w[6 - rr] + w[6 + rr], w[7 - rr] + w[7 + rr])};
            } else if (ax == 2) {
              sum = add4({make_float2(w[4 - rr], w[5 - rr]), make_float2(w[6 - rr], w[7 - rr])},
                         {make_float2(w[4 + rr], w[5 + rr]), make_float2(w[6 + rr], w[7 + rr])});
            } else if (ax == 1) {
              const float4 A = *reinterpret_cast<const float4*>(uc - rr * UKW + kTmaKHalo + 4 * lane);
              const float4 B = *reinterpret_cast<const float4*>(uc + rr * UKW + kTmaKHalo + 4 * lane);
              sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                         {make_float2(B.x, B.y), make_float2(B.z, B.w)});
            } else {
              const float4 A = q[(ph + 2 * QN - R - rr) % QN];
              const float4 B = q[(ph + QN - R + rr) % QN];
              sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                         {make_float2(B.x, B.y), make_float2(B.z, B.w)});
            }
            if (MODE == ST3D_MODE_REF) {
              acc = fma4(splat(cf.cf[p]), sum, p == 0 ? mul4(cu, splat(cf.coef0)) : acc);
            } else {
              const P4 d = add4(sum, nu2);
              acc = p == 0 ? mul4(d, splat(cf.cf[0])) : fma4(splat(cf.cf[p]), d, acc);
            }
          }
          const float4 v4 = *reinterpret_cast<const float4*>(vr + stage * VSLOT + r * TK + 4 * lane);
          const float4 s4 = *reinterpret_cast<const float4*>(sr + stage * VSLOT + r * TK + 4 * lane);
          const P4 vv = {make_float2(v4.x, v4.y), make_float2(v4.z, v4.w)};
          P4 ss = {make_float2(s4.x, s4.y), make_float2(s4.z, s4.w)};
          P4 x;
          if (MODE == ST3D_MODE_REF) {
            const P4 t = fma4(splat(-cf.K), cu, vv);
            x = {__ffma2_rn(ss.a, acc.a, t.a), __ffma2_rn(ss.b, acc.b, t.b)};
          } else {
            if (i == src.i && j == src.j && (unsigned)(src.k - k) < 4u) {
              const int c = src.k - k;
              if (c == 0) ss.a.x = ss.a.x + src.amp;
              if (c == 1) ss.a.y = ss.a.y + src.amp;
              if (c == 2) ss.b.x = ss.b.x + src.amp;
              if (c == 3) ss.b.y = ss.b.y + src.amp;
            }
            P4 t = add4(u2, {make_float2(-vv.a.x, -vv.a.y), make_float2(-vv.b.x, -vv.b.y)});
            t = fma4(splat(cf.c1), acc, t);
            x = fma4(splat(cf.c2), ss, t);
          }
          const float o[4] = {x.a.x, x.a.y, x.b.x, x.b.y};
          if (row_ok) {
            float* dst = vrow + (long long)i * g.si;
            if (k + 3 < g.zs) {
              *reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (k + c < g.zs) dst[c] = o[c];
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
      }
    }
    h += (uint32_t)nsteps;
  }
}

template <int P, int MODE, int TJ, int NV>
cudaError_t launch_cfg(const TmaPlan& plan, const Geom& g, const Coefs<float>& cf, float* v,
                       int ubuf, int vbuf, int sbuf, const Source& src, uint32_t* dev_status,
                       cudaStream_t stream) {
  auto kern = k_tma<P, MODE, TJ, NV>;
  cudaError_t e =
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plan.smem);
  if (e != cudaSuccess) return e;
  kern<<<plan.grid, (TJ + 1) * 32, plan.smem, stream>>>(
      plan.umap[ubuf], plan.vmap[vbuf], plan.vmap[sbuf], g, cf, v, plan.ntk, plan.ntj * plan.ntk,
      plan.ichunk, plan.units, src, plan.timeout_ns, dev_status);
  return cudaGetLastError();
}

template <int P, int MODE>
cudaError_t launch_mode(const TmaPlan& plan, const Geom& g, const Coefs<float>& cf, float* v,
                        int ubuf, int vbuf, int sbuf, const Source& src, uint32_t* dev_status,
                        cudaStream_t stream) {
  if (plan.tj == 16 && plan.nv == 3)
    return launch_cfg<P, MODE, 16, 3>(plan, g, cf, v, ubuf, vbuf, sbuf, src, dev_status, stream);
  if (plan.tj == 8 && plan.nv == 3)
    return launch_cfg<P, MODE, 8, 3>(plan, g, cf, v, ubuf, vbuf, sbuf, src, dev_status, stream);
  if (plan.tj == 8 && plan.nv == 4)
    return launch_cfg<P, MODE, 8, 4>(plan, g, cf, v, ubuf, vbuf, sbuf, src, dev_status, stream);
  if (plan.tj == 16 && plan.nv == 2)
    return launch_cfg<P, MODE, 16, 2>(plan, g, cf, v, ubuf, vbuf, sbuf, src, dev_status, stream);
  if (plan.tj == 16 && plan.nv == 4)
    return launch_cfg<P, MODE, 16, 4>(plan, g, cf, v, ubuf, vbuf, sbuf, src, dev_status, stream);
  return cudaErrorInvalidConfiguration;
}

template <int P, int MODE>
int occupancy_mode(int tj, int nv, size_t smem) {
  int n = 0;
  auto probe = [&](auto kern, int threads) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 0;
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, threads, smem) != cudaSuccess)
      return 0;
    return b;
  };
  if (tj == 16 && nv == 3) n = probe(k_tma<P, MODE, 16, 3>, 17 * 32);
  if (tj == 8 && nv == 3) n = probe(k_tma<P, MODE, 8, 3>, 9 * 32);
  if (tj == 8 && nv == 4) n = probe(k_tma<P, MODE, 8, 4>, 9 * 32);
  if (tj == 16 && nv == 2) n = probe(k_tma<P, MODE, 16, 2>, 17 * 32);
  if (tj == 16 && nv == 4) n = probe(k_tma<P, MODE, 16, 4>, 17 * 32);
  cudaGetLastError();
  return n;
}

}  // namespace

int tma_blocks_per_sm(int points, int mode, int tj, int nv, size_t smem) {
  const bool ref = mode == ST3D_MODE_REF;
  switch (points) {
    case 7: return ref ? occupancy_mode<7, ST3D_MODE_REF>(tj, nv, smem) : occupancy_mode<7, ST3D_MODE_WAVE>(tj, nv, smem);
    case 13: return ref ? occupancy_mode<13, ST3D_MODE_REF>(tj, nv, smem) : occupancy_mode<13, ST3D_MODE_WAVE>(tj, nv, smem);
    case 25: return ref ? occupancy_mode<25, ST3D_MODE_REF>(tj, nv, smem) : occupancy_mode<25, ST3D_MODE_WAVE>(tj, nv, smem);
    default: return 0;
  }
}

bool tma_config_supported(int tj, int nv) {
  return (tj == 16 && (nv == 2 || nv == 3 || nv == 4)) || (tj == 8 && (nv == 3 || nv == 4));
}

cudaError_t launch_tma(const TmaPlan& plan, int points, int mode, const Geom& g,
                       const Coefs<float>& cf, float* v, int ubuf, int vbuf, int sbuf,
                       const Source& src, uint32_t* dev_status, cudaStream_t stream) {
#define ST3D_TMA_CASE(PTS)                                                                  \
  case PTS:                                                                                 \
    return mode == ST3D_MODE_REF                                                            \
               ? launch_mode<PTS, ST3D_MODE_REF>(plan, g, cf, v, ubuf, vbuf, sbuf, src,     \
                                                 dev_status, stream)                        \
               : launch_mode<PTS, ST3D_MODE_WAVE>(plan, g, cf, v, ubuf, vbuf, sbuf, src,    \
                                                  dev_status, stream);
  switch (points) {
    ST3D_TMA_CASE(7)
    ST3D_TMA_CASE(13)
    ST3D_TMA_CASE(25)
    default:
      return cudaErrorInvalidValue;
  }
#undef ST3D_TMA_CASE
}

}  // namespace st3d
