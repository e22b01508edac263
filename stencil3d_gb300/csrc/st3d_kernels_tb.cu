// st3d_kernels_tb.cu -- temporal blocking of the FP32 wave update: T
// leapfrog steps fused into one pass over HBM.
//
// One pass reads U^n, U^{n-1} and s once and writes U^{n+T-1} and U^{n+T},
// the two levels that form the next state, so a pass moves 20 bytes per
// point for T steps instead of 16 bytes per step.  The levels are chained in
// a wavefront along i inside each CTA: when plane p of U^n arrives, level t
// (U^{n+t}) is computed at plane p - t*R from level t-1, whose planes the CTA
// computed in the previous R steps.  Each level keeps the planes its
// successor needs: i neighbours in a per-level register queue of 2R+1 float4
// per lane, j/k neighbours of the centre plane in a per-level shared-memory
// ring (one named barrier per step makes a level's tile visible to the warps
// of the neighbouring rows).  Level t at a plane also needs level t-2 there
// (the "v" of the leapfrog): U^{n-1} from its TMA tile for t = 1, the oldest
// entry of level t-2's queue above that.
//
// Tiles shrink by R per level: one consumer warp per row of a level-1 tile
// of tb_rows(P, T) rows (rows j0 - (T-1)R ..; 26 for 7 points T=2, 15 for 13
// points T=4 and 25 points T=2, else 18), 4 points per lane over 128 columns
// (k0 - KH .. k0 + 127 - KH, KH = tb_khalo(P, T) = 4 or 8); the pass writes
// the rows - 2(T-1)R middle rows and the 128 - 2 KH columns k0 .. k0 + 127 -
// 2 KH.  Level 1 is exact over its whole tile (the level-0 TMA tile carries R
// rows and 4 columns of halo); a level above reads zeros beyond its tile's
// edge, so level t is exact in all but (t-1)R rows and columns at either
// edge, which bounds (T-1)R by the KH margin columns: T = 2 or 4 for the 7-
// and 13-point stencils, T = 2 for the 25-point one.  Levels outside the grid
// interior are the zero halo (temporal blocking requires a zero boundary).
// Output goes to two other buffers (neighbouring tiles still read U^n and
// U^{n-1} while a tile writes), so a context that blocks in time holds four
// field buffers.
//
// Arithmetic per level point is the single-step kernels' difference form in
// the same order, so T fused steps give bit for bit the result of T plain
// steps.  It runs on packed FP32 pairs (add/fma.rn.f32x2, per component the
// scalar operations): the fused levels make the pass issue-bound, and the
// pairs raised 7 points T=4 from 510 to 531 and 13 points T=2 from 393 to
// 411 Gpts/s at 1024^3 (on 16-row tiles, before the taller ones).
#include <cstring>

#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

constexpr int kCols = 128;      // level columns per tile (32 lanes x 4)
constexpr int kW = kCols + 8;   // smem row width (4 floats of pad either side)

struct TbArgs {
  Geom g;
  Coefs<float> cf;
  float* out_prev;  // U^{n+T-1}
  float* out_new;   // U^{n+T}
  int ntk, ntjk, ichunk, units, rows_out;
  int src_i, src_j, src_k;
  float amp[4];     // source amplitude of each fused step
  uint64_t timeout_ns;
  uint32_t* status;
};

template <int P>
struct RadTB {
  static constexpr int value = (P == 25) ? 4 : (P == 13) ? 2 : 1;
};

// Pipeline stages: 13 points T=2 on 18 rows has room in shared memory for a
// fourth (203 KB; 460 against 453 Gpts/s at 1024^3 with 3); the other tiles
// fill it with 3.
template <int P, int T>
constexpr int tb_stages() { return (P == 13 && T == 2) ? 4 : 3; }

// Slots per level ring.  Level t writes its plane at step n into slot
// (n - tR) mod NL and level t+1 reads that slot at step n + R; the named
// barrier that ends every step orders each read before the slot's next
// write, which comes NL steps after the first, so NL = R + 1 suffices (a
// slot is never read and written in the same step: R mod (R+1) != 0).  13
// points T=4 takes R + 1 to fit 227 KB; the other depths keep R + 2.
template <int P, int T>
constexpr int tb_level_slots() { return RadTB<P>::value + ((P == 13 && T == 4) ? 1 : 2); }

template <int P, int T, int NV>
struct TbShape {
  static constexpr int R = RadTB<P>::value;
  static constexpr int kRows = tb_rows(P, T);  // level-1 rows per tile = consumer warps
  static constexpr int QN = 2 * R + 1;
  static constexpr int NU = NV + R;                       // level-0 ring (TMA u tiles)
  static constexpr int NS = NV + (T - 1) * R;             // s ring (kept for the later levels)
  static constexpr int NL = tb_level_slots<P, T>();       // slots per level ring
  static constexpr int KH = tb_khalo(P, T);               // k margin columns either side
  static constexpr int OUTC = kCols - 2 * KH;             // columns written per tile
  static constexpr int USLOT = (kW * (kRows + 2 * R) + 31) / 32 * 32;  // floats
  static constexpr int VSLOT = kCols * kRows;             // floats
  static constexpr int LSLOT = kW * kRows;                // floats
  static constexpr size_t smem() {
    return ((size_t)NU * USLOT + (size_t)NV * VSLOT + (size_t)NS * VSLOT +
            (size_t)(T - 1) * NL * LSLOT) * 4 + 2 * NV * 8 + 128;
  }
};

template <int P, int T, int NV>
__global__ void __launch_bounds__((tb_rows(P, T) + 1) * 32, 1)
    k_tb(const __grid_constant__ CUtensorMap umap, const __grid_constant__ CUtensorMap vmap,
         const __grid_constant__ CUtensorMap smap, const TbArgs a) {
  using S = TbShape<P, T, NV>;
  constexpr int R = S::R;
  constexpr int QN = S::QN;
  constexpr int kRows = S::kRows;
  constexpr int NP = npairs_of(P);
  constexpr int KH = S::KH;
  constexpr int OUTC = S::OUTC;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* ur = reinterpret_cast<float*>(smem_raw);
  float* vr = ur + S::NU * S::USLOT;
  float* sr = vr + NV * S::VSLOT;
  float* lr = sr + S::NS * S::VSLOT;  // level rings: (T-1) x NL slots
  uint64_t* full = reinterpret_cast<uint64_t*>(lr + (T - 1) * S::NL * S::LSLOT);
  uint64_t* empty = full + NV;

  const Geom& g = a.g;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kRows);
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  // zero the level rings once: their pad columns are read by edge lanes
  for (int x = threadIdx.x; x < (T - 1) * S::NL * S::LSLOT; x += blockDim.x) lr[x] = 0.0f;
  __syncthreads();

  if (warp == kRows) {
    // ---------------- producer ----------------
    if (lane != 0) return;
    uint32_t h = 0;
    bool ok = true;
    for (int unit = blockIdx.x; unit < a.units && ok; unit += gridDim.x) {
      const int ic = unit / a.ntjk;
      const int rem = unit - ic * a.ntjk;
      const int jt = rem / a.ntk;
      const int kt = rem - jt * a.ntk;
      const int k0 = kt * OUTC;
      const int jb = jt * a.rows_out - (T - 1) * R;  // first level-1 row
      const int ia = ic * a.ichunk;
      const int ib = min(ia + a.ichunk, g.xs);
      const int nsteps = (ib - ia) + 2 * T * R;
      for (int n = 0; n < nsteps; ++n, ++h) {
        const int stage = (int)(h % NV);
        if (h >= (uint32_t)NV &&
            !mbar_wait_bounded(&empty[stage], ((h / NV) - 1) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          ok = false;
          break;
        }
        const int p = ia - T * R + n;  // level-0 plane arriving
        const int p1 = p - R;          // level-1 plane of this step
        mbar_arrive_expect_tx(&full[stage], (uint32_t)(kW * (kRows + 2 * R) * 4 + 2 * S::VSLOT * 4));
        // level column c sits at k0 - KH + c, smem column 4 + c of a u row
        tma_load_3d(ur + (h % S::NU) * S::USLOT, &umap, &full[stage], g.pk + k0 - KH - 4,
                    g.pj + jb - R, g.pi + p);
        tma_load_3d(vr + stage * S::VSLOT, &vmap, &full[stage], g.pk + k0 - KH, g.pj + jb, g.pi + p1);
        tma_load_3d(sr + (h % S::NS) * S::VSLOT, &smap, &full[stage], g.pk + k0 - KH, g.pj + jb,
                    g.pi + p1);
      }
    }
    for (uint32_t m = (h > (uint32_t)NV ? h - NV : 0u); m < h; ++m) {
      (void)mbar_wait_bounded(&full[m % NV], (m / NV) & 1u, a.timeout_ns);
      (void)mbar_wait_bounded(&empty[m % NV], (m / NV) & 1u, a.timeout_ns);
    }
    return;
  }

  // ---------------- consumers ----------------
  const int r = warp;
  uint32_t h = 0;
  bool failed = false;
  float4 q[T][QN];  // q[t]: planes of level t around its newest plane
  for (int unit = blockIdx.x; unit < a.units; unit += gridDim.x) {
    const int ic = unit / a.ntjk;
    const int rem = unit - ic * a.ntjk;
    const int jt = rem / a.ntk;
    const int kt = rem - jt * a.ntk;
    const int k0 = kt * OUTC;
    const int jb = jt * a.rows_out - (T - 1) * R;
    const int j = jb + r;
    const int kc = k0 - KH + 4 * lane;  // first column of this lane
    const int ia = ic * a.ichunk;
    const int ib = min(ia + a.ichunk, g.xs);
    const int nsteps = (ib - ia) + 2 * T * R;
    const bool row_in = j >= 0 && j < g.ys;
    const bool out_row = r >= (T - 1) * R && r < kRows - (T - 1) * R && row_in;
    const bool out_col = lane >= KH / 4 && lane < 32 - KH / 4 && kc < g.zs;
    // interior columns of this lane, and the source's column in it (or -1)
    bool colv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) colv[c] = row_in && kc + c >= 0 && kc + c < g.zs;
    const int src_c = (j == a.src_j && (unsigned)(a.src_k - kc) < 4u) ? a.src_k - kc : -1;
    for (int n0 = 0; n0 < nsteps; n0 += QN) {
#pragma unroll
      for (int ph = 0; ph < QN; ++ph) {
        const int n = n0 + ph;
        if (n >= nsteps) break;
        const uint32_t hh = h + (uint32_t)n;
        const int stage = (int)(hh % NV);
        if (!failed && !mbar_wait_bounded(&full[stage], (hh / NV) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutFull);
          failed = true;
        }
        const int p = ia - T * R + n;
        // level 0 enters its queue
        q[0][ph] = *reinterpret_cast<const float4*>(ur + (hh % S::NU) * S::USLOT + (r + R) * kW + 4 + 4 * lane);
        // levels 1..T at planes p - t*R
#pragma unroll
        for (int t = 1; t <= T; ++t) {
          const int pt = p - t * R;
          const bool live = pt >= ia - (T - t) * R && pt < ib + (T - t) * R;
          // level t feeds the output only in rows (t-1)R .. kRows-1-(t-1)R;
          // the warps of the other rows skip it (their ring rows are never
          // read by a row that is computed)
          const bool needed = t == 1 || (r >= (t - 1) * R && r < kRows - (t - 1) * R);
          if (!live || !needed) continue;
          // centre row of level t-1 at plane pt, its j/k neighbours
          const float* base;
          int pitch_rows_off;
          // every level keeps plane x of the unit at queue slot / ring slot
          // (step at which level-0 plane x arrived) mod size: plane pt sits at
          // step n - t*R
          if (t == 1) {
            base = ur + ((hh - R) % S::NU) * S::USLOT;  // level-0 tile of plane p - R
            pitch_rows_off = R;                          // row 0 of the tile is level-1 row -R
          } else {
            const int slot = (int)((hh - (uint32_t)(t * R)) % S::NL);
            base = lr + ((t - 2) * S::NL + slot) * S::LSLOT;
            pitch_rows_off = 0;
          }
          const float* ctr = base + (r + pitch_rows_off) * kW;
          const float4 c4 = q[t - 1][(ph + 2 * QN - t * R) % QN];
          const float4 l4 = *reinterpret_cast<const float4*>(ctr + 4 * lane);
          const float4 r4 = *reinterpret_cast<const float4*>(ctr + 8 + 4 * lane);
          const float w[12] = {l4.x, l4.y, l4.z, l4.w, c4.x, c4.y, c4.z, c4.w,
                               r4.x, r4.y, r4.z, r4.w};
          const P4 cu = {make_float2(c4.x, c4.y), make_float2(c4.z, c4.w)};
          const P4 u2 = add4(cu, cu);
          const P4 nu2 = {make_float2(-u2.a.x, -u2.a.y), make_float2(-u2.b.x, -u2.b.y)};
          P4 acc;
#pragma unroll
          for (int pp = 0; pp < NP; ++pp) {
            const int ax = pair_axis(P, pp);
            const int rr = pair_r(P, pp);
            P4 sum;
            if (ax == 2 && (rr & 1)) {
              sum = {make_float2(w[4 - rr] + w[4 + rr], w[5 - rr] + w[5 + rr]),
                     make_float2(w[6 - rr] + w[6 + rr], w[7 - rr] + w[7 + rr])};
            } else if (ax == 2) {
              sum = add4({make_float2(w[4 - rr], w[5 - rr]), make_float2(w[6 - rr], w[7 - rr])},
                         {make_float2(w[4 + rr], w[5 + rr]), make_float2(w[6 + rr], w[7 + rr])});
            } else if (ax == 1) {
              // rows outside the level's tile read its neighbours' junk; only
              // rows whose result is discarded do that
              const int ra = r + pitch_rows_off - rr, rb = r + pitch_rows_off + rr;
              const int rows_avail = (t == 1) ? kRows + 2 * R : kRows;
              const float4 A = (ra >= 0) ? *reinterpret_cast<const float4*>(base + ra * kW + 4 + 4 * lane)
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
              const float4 B = (rb < rows_avail) ? *reinterpret_cast<const float4*>(base + rb * kW + 4 + 4 * lane)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
              sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                         {make_float2(B.x, B.y), make_float2(B.z, B.w)});
            } else {
              const float4 A = q[t - 1][(ph + 3 * QN - t * R - rr) % QN];
              const float4 B = q[t - 1][(ph + 2 * QN - t * R + rr) % QN];
              sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                         {make_float2(B.x, B.y), make_float2(B.z, B.w)});
            }
            const P4 d = add4(sum, nu2);
            acc = pp == 0 ? mul4(d, splat(a.cf.cf[0])) : fma4(splat(a.cf.cf[pp]), d, acc);
          }
          // level t-2 at plane pt: U^{n-1} for t = 1, else the oldest entry of
          // level t-2's queue
          float4 v4;
          if (t == 1) {
            v4 = *reinterpret_cast<const float4*>(vr + stage * S::VSLOT + r * kCols + 4 * lane);
          } else {
            v4 = q[t - 2][(ph + 2 * QN - t * R) % QN];
          }
          const float4 s4 = *reinterpret_cast<const float4*>(
              sr + ((hh - (t - 1) * R) % S::NS) * S::VSLOT + r * kCols + 4 * lane);
          P4 ss = {make_float2(s4.x, s4.y), make_float2(s4.z, s4.w)};
          const bool plane_in = pt >= 0 && pt < g.xs;
          if (pt == a.src_i && src_c >= 0) {
            if (src_c == 0) ss.a.x = ss.a.x + a.amp[t - 1];
            if (src_c == 1) ss.a.y = ss.a.y + a.amp[t - 1];
            if (src_c == 2) ss.b.x = ss.b.x + a.amp[t - 1];
            if (src_c == 3) ss.b.y = ss.b.y + a.amp[t - 1];
          }
          P4 tt = add4(u2, {make_float2(-v4.x, -v4.y), make_float2(-v4.z, -v4.w)});
          tt = fma4(splat(a.cf.c1), acc, tt);
          const P4 x = fma4(splat(a.cf.c2), ss, tt);
          float o[4] = {x.a.x, x.a.y, x.b.x, x.b.y};
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if (!(plane_in && colv[c])) o[c] = 0.0f;  // outside the interior a level is the zero halo
          const float4 o4 = make_float4(o[0], o[1], o[2], o[3]);
          if (t < T) {
            // level t: push into its queue and its ring (the ring slot of plane pt)
            q[t][(ph + 2 * QN - t * R) % QN] = o4;
            float* ring = lr + ((t - 1) * S::NL + (int)((hh - t * R) % S::NL)) * S::LSLOT;
            *reinterpret_cast<float4*>(ring + r * kW + 4 + 4 * lane) = o4;
          }
          if (t >= T - 1 && out_row && out_col && pt >= ia && pt < ib) {
            float* dst = (t == T ? a.out_new : a.out_prev) + g.org + (long long)pt * g.si +
                         (long long)j * g.sj + kc;
            if (kc + 3 < g.zs) {
              *reinterpret_cast<float4*>(dst) = o4;
            } else {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (kc + c < g.zs) dst[c] = o[c];
            }
          }
        }
        // the level tiles written this step become readable to all rows
        asm volatile("bar.sync 1, %0;" ::"r"(kRows * 32) : "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
      }
    }
    h += (uint32_t)nsteps;
  }
}

template <int P, int T>
cudaError_t launch_pt(const TbPlan& pl, const TbArgs& a, const CUtensorMap& u, const CUtensorMap& v,
                      const CUtensorMap& s, cudaStream_t stream, int* occ) {
  using Sh = TbShape<P, T, tb_stages<P, T>()>;
  auto kern = k_tb<P, T, tb_stages<P, T>()>;
  const size_t smem = Sh::smem();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, (Sh::kRows + 1) * 32, smem);
  if (pl.rows != Sh::kRows) return cudaErrorInvalidConfiguration;  // maps built for another height
  kern<<<pl.grid, (Sh::kRows + 1) * 32, smem, stream>>>(u, v, s, a);
  return cudaGetLastError();
}

cudaError_t dispatch_tb(int points, int T, const TbPlan& pl, const TbArgs& a, const CUtensorMap& u,
                        const CUtensorMap& v, const CUtensorMap& s, cudaStream_t stream, int* occ) {
  if (points == 7 && T == 2) return launch_pt<7, 2>(pl, a, u, v, s, stream, occ);
  if (points == 7 && T == 4) return launch_pt<7, 4>(pl, a, u, v, s, stream, occ);
  if (points == 13 && T == 2) return launch_pt<13, 2>(pl, a, u, v, s, stream, occ);
  if (points == 13 && T == 4) return launch_pt<13, 4>(pl, a, u, v, s, stream, occ);
  if (points == 25 && T == 2) return launch_pt<25, 2>(pl, a, u, v, s, stream, occ);
  return cudaErrorInvalidConfiguration;
}

}  // namespace

size_t tb_smem_bytes(int points, int T) {
  if (points == 7 && T == 2) return TbShape<7, 2, tb_stages<7, 2>()>::smem();
  if (points == 7 && T == 4) return TbShape<7, 4, tb_stages<7, 4>()>::smem();
  if (points == 13 && T == 2) return TbShape<13, 2, tb_stages<13, 2>()>::smem();
  if (points == 13 && T == 4) return TbShape<13, 4, tb_stages<13, 4>()>::smem();
  if (points == 25 && T == 2) return TbShape<25, 2, tb_stages<25, 2>()>::smem();
  return 0;
}

int tb_blocks_per_sm(int points, int T) {
  TbPlan pl;
  TbArgs a;
  CUtensorMap m;
  memset(&m, 0, sizeof m);
  int occ = 0;
  if (dispatch_tb(points, T, pl, a, m, m, m, nullptr, &occ) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

cudaError_t launch_tb(int points, int T, const TbPlan& pl, const Geom& g, const Coefs<float>& cf,
                      float* out_prev, float* out_new, int ubuf, int vbuf, const Source& src,
                      const float* amps, uint32_t* dev_status, cudaStream_t stream) {
  TbArgs a;
  a.g = g;
  a.cf = cf;
  a.out_prev = out_prev;
  a.out_new = out_new;
  a.ntk = pl.ntk;
  a.ntjk = pl.ntj * pl.ntk;
  a.ichunk = pl.ichunk;
  a.units = pl.units;
  a.rows_out = pl.rows_out;
  a.src_i = src.i;
  a.src_j = src.j;
  a.src_k = src.k;
  for (int t = 0; t < 4; ++t) a.amp[t] = t < T ? amps[t] : 0.0f;
  a.timeout_ns = pl.timeout_ns;
  a.status = dev_status;
  return dispatch_tb(points, T, pl, a, pl.umap[ubuf], pl.vmap[vbuf], pl.vmap[2], stream, nullptr);
}

}  // namespace st3d
