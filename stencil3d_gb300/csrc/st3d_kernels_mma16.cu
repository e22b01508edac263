// st3d_kernels_mma16.cu -- the 16-bit delta forms (FP16 / BF16, and the
// F16_HL pair form) with every linear term of the step on the tensor cores.
//
// The update is the delta form of st3d_kernels_delta16.cu:
//     lap     = sum_p w_p (a_p + b_p) + m2s * u
//     d^{n+1} = d^n + c1 * lap + c2 * (s + a_n delta_src)
//     u^{n+1} = u^n + dec(enc(d^{n+1}))
// with u, d and s held as 16-bit words at a power-of-two scale per i-plane.
// d^{n+1} is linear in the words of u (planes i-R .. i+R), d and s, so a
// 16x8 block of it (j rows x k columns) is a sum of mma.sync products on
// 16-bit operands with FP32 accumulators:
//   - Djk, the j and k sums and the centre term, in units of the centre
//     plane: the k sum and m2s*u as U[16 x 24] * Wk[24 x 8] (U = rows
//     j..j+15, columns k-8..k+15; Wk[c][n] = w_k(c - 8 - n), w_k(0) = m2s),
//     the j sum as Wj[16 x 24] * U[24 x 8] (U = rows j-R..j-R+23, the block's
//     columns; Wj[m][c] = w_j(c - R - m), w_j(0) = 0), constant band
//     matrices of w * 2^S held as 16-bit hi/lo pairs (S puts the largest
//     weight near 2^14; hi + lo carries a weight to ~22 bits, ~16 for BF16);
//   - Ds, d and s: [D | S] * [diag(v_d); diag(v_s)] with v_d = 2^(E_d - Y)
//     and v_s = c2 2^(E_s - Y) (hi/lo words; Y puts the larger in
//     [2^13, 2^14));
//   - Pr, the i pair at radius r: [U_{i-r} | U_{i+r}] * [diag(2^(E_{i-r}-X));
//     diag(2^(E_{i+r}-X))], the planes' scales relative to 2^X (X = the
//     largest of them less 15) as exact 16-bit powers of two, so the
//     products are exact and one mma per radius carries the pair;
//   - d^{n+1} = Djk * c1 2^(E_i - S) + Ds * 2^Y + sum_r (c1 w_r 2^X) * Pr in
//     FP32.
// The per-plane weights, 2^X-scaled factors c1 w_r 2^X, 2^Y and the step's
// other scales form one 128-byte record per plane, written before each step
// by k_mma_records and brought into the stage by the producer with one bulk
// copy.  The u planes i-R .. i+R all stay in the shared-memory ring (16 slots
// >= 8 stages + 2R), so no register queue along i is needed.  The centre u
// (and, for the pair form, its lo words) is decoded in FP32 for
// u^{n+1} = u + dec(enc(d)).
//
// The tensor cores sum the products in their own order and rounding, so this
// kernel is not bit-identical to the scalar one or to the oracle's
// restatement: a step agrees with them to FP32 rounding of the sum, and the
// 16-bit words of u and d to one unit in the last place where the sum falls
// near a rounding boundary.  A neighbour plane whose scale lies more than
// 2^39 below the largest of them (2^55 for BF16) takes a zero weight (the
// FP16 powers of two end at 2^-24 = 2^(39-15) below 2^X): its contribution
// is far below FP32 rounding of the sum.
//
// Structure (one CTA per SM, persistent over 16-row x 152-column x
// ichunk-plane units): a producer thread streams, per step, the u plane i+R
// (rows j0-R .. j0-R+23, columns k0-8 .. k0+159) and, for the centre plane
// i, d, s (the lo words of u) over columns k0 .. k0+151 and the plane's
// record, through an mbarrier ring of 8 stages (4 for the pair form); 19
// consumer warps each own one 16x8 block (20 warps with the producer: five
// on some schedulers, within the 96 registers a thread that leaves; the
// kernel takes 81-87).  The row pitches (336 and 304 bytes) put the eight
// rows of every ldmatrix in distinct banks.  Each warp writes its block of
// u^{n+1}, d^{n+1} (and the lo words) into the stage's s, d (and lo) slots, whose
// inputs it has read, with zero words at the points outside the grid; once
// every warp has released the stage the producer stores the three tiles with
// TMA (whole lines, clipped by the tensor maps' extents) and waits for the
// stores to read shared memory before it loads the slots again.  A store
// whose clipped row ends inside a 16-byte segment was seen to write the rest
// of that segment (the zero halo along k when zs is not a multiple of 8), so
// the outputs outside the grid are zeros, the value the halo holds.  Waits
// are bounded; after a timeout the consumers keep stepping and arriving
// without waiting, so that the producer's bounded drain ends and every CTA
// returns (the status word marks the results void).
#include <math.h>
#include <string.h>

#include "st3d_f16.cuh"
#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

constexpr int kMTJ = 16;         // rows per tile (one 16-row mma block)
constexpr int kMTK = kMmaTK;     // columns per tile (nineteen 8-column blocks)
constexpr int kMCW = kMmaTK / 8; // consumer warps, one 8-column block each
constexpr int kMUW = kMTK + 16;  // u tile row: k0-8 .. k0+159, 336 bytes
constexpr int kMVW = kMTK;       // d / s / lo tile row: k0 .. k0+151, 304 bytes
constexpr int kMUH = kMTJ + 8;   // u tile rows: j0-R .. j0-R+23
constexpr int kMNV = 8;          // pipeline stages (4 for the pair form, whose third tile per stage
                                 // would not fit 8)
constexpr int kMNU = 16;         // u ring slots (>= NV + 2R; a power of two)

template <int P>
struct RadM {
  static constexpr int value = (P == 25) ? 4 : (P == 13) ? 2 : 1;
};

struct Mma16Args {
  Geom g;
  Coefs<float> cf;
  const MmaRecord* rec;
  uint32_t *Mu_out, *Md_out;
  float wj[5], wk[5];  // band weights w * 2^S by offset 0..R (wj[0] = 0, wk[0] = m2s * 2^S)
  int need_lo;         // some band weight is not exact in one 16-bit word
  float c1m2s;         // PAIR: c1 * m2s (the centre's lo words)
  int ntk, ntjk, ichunk, units;
  Source src;
  uint64_t timeout_ns;
  uint32_t* status;
};

// ---- fragments ----------------------------------------------------------

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr)
               : "memory");
}
__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];"
               : "=r"(r0), "=r"(r1)
               : "r"(addr)
               : "memory");
}

// D += A (16x16) * B (16x8); D += A (16x8) * B (8x8); 16-bit operands of
// kind KIND (0 FP16, 1 BF16), FP32 accumulators.
template <int KIND>
__device__ __forceinline__ void mma_k16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                        uint32_t b0, uint32_t b1) {
  if constexpr (KIND == 0) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
        "{%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  } else {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
        "{%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
}
template <int KIND>
__device__ __forceinline__ void mma_k8(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t b0) {
  if constexpr (KIND == 0) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5}, {%6}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(b0));
  } else {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5}, {%6}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(b0));
  }
}

// One bulk copy (no tensor map) of `bytes` from global memory into shared
// memory, completing on `bar`; both addresses 16-byte aligned, bytes a
// multiple of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// 3-D tiled TMA store of the box at element coordinates (x, y, z) from
// shared memory (elements outside the tensor map's extent are not written),
// then commit / wait for the stores' reads of shared memory, or for their
// completion.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read1() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// w -> (hi, lo) 16-bit words with hi = rn16(w), lo = rn16(w - hi)
template <int KIND>
__device__ __forceinline__ void split16(float w, uint32_t& hi, uint32_t& lo) {
  if constexpr (KIND == 0) {
    const __half h = __float2half_rn(w);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn(w - __half2float(h)));
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(w);
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(__float2bfloat16_rn(w - __bfloat162float(h)));
  }
}

__device__ __forceinline__ float band_w(const float* wt, int e, int R) {
  const int m = e < 0 ? -e : e;
  return m <= R ? wt[m] : 0.0f;
}

// hi/lo words of the band fragments of lane (g, t):
//   wk: B of the k sum, rows c = 2t, 2t+1 | 2t+8, 2t+9 | 16+2t, 17+2t, column g;
//   wj: A of the j sum, (row, columns) = (g, 2t..) | (g+8, 2t..) | (g, 2t+8..) |
//       (g+8, 2t+8..) | (g, 16+2t..) | (g+8, 16+2t..).
template <int KIND>
__device__ void band_fragments(const Mma16Args& a, int R, int g, int t, uint32_t (&wkh)[3],
                               uint32_t (&wkl)[3], uint32_t (&wjh)[6], uint32_t (&wjl)[6]) {
  float wk[5], wj[5];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    wk[r] = a.wk[r];
    wj[r] = a.wj[r];
  }
  const int kc[3] = {2 * t, 2 * t + 8, 16 + 2 * t};
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    uint32_t h0, l0, h1, l1;
    split16<KIND>(band_w(wk, kc[f] - 8 - g, R), h0, l0);
    split16<KIND>(band_w(wk, kc[f] + 1 - 8 - g, R), h1, l1);
    wkh[f] = h0 | (h1 << 16);
    wkl[f] = l0 | (l1 << 16);
  }
  const int jm[6] = {g, g + 8, g, g + 8, g, g + 8};
  const int jc[6] = {2 * t, 2 * t, 2 * t + 8, 2 * t + 8, 16 + 2 * t, 16 + 2 * t};
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    uint32_t h0, l0, h1, l1;
    split16<KIND>(band_w(wj, jc[f] - R - jm[f], R), h0, l0);
    split16<KIND>(band_w(wj, jc[f] + 1 - R - jm[f], R), h1, l1);
    wjh[f] = h0 | (h1 << 16);
    wjl[f] = l0 | (l1 << 16);
  }
}

// max of |x| over the components whose bit is set in v
__device__ __forceinline__ float amax4m(const P4& x, uint32_t v) {
  float m = 0.0f;
  if (v & 1u) m = fmaxf(m, fabsf(x.a.x));
  if (v & 2u) m = fmaxf(m, fabsf(x.a.y));
  if (v & 4u) m = fmaxf(m, fabsf(x.b.x));
  if (v & 8u) m = fmaxf(m, fabsf(x.b.y));
  return m;
}

template <int KIND, int P, bool PAIR>
__global__ void __launch_bounds__((kMCW + 1) * 32, 1)
    k_mma16(const __grid_constant__ CUtensorMap umap, const __grid_constant__ CUtensorMap dmap,
            const __grid_constant__ CUtensorMap smap, const __grid_constant__ CUtensorMap lmap,
            const __grid_constant__ CUtensorMap uomap, const __grid_constant__ CUtensorMap lomap,
            const Mma16Args a) {
  constexpr int R = RadM<P>::value;
  constexpr int NV = PAIR ? kMNV / 2 : kMNV;
  constexpr int NU = kMNU;
  constexpr int CW = kMCW;
  constexpr uint32_t UBYTES = kMUW * kMUH * 2;
  constexpr uint32_t VBYTES = kMVW * kMTJ * 2;
  constexpr uint32_t RBYTES = sizeof(MmaRecord);
  constexpr int USLOT = (UBYTES + 127) / 128 * 128;
  constexpr int VSLOT = (VBYTES + 127) / 128 * 128;
  static_assert(NU >= NV + 2 * R && (NU & (NU - 1)) == 0 && (NV & (NV - 1)) == 0, "ring sizes");
  static_assert(sizeof(MmaRecord) % 128 == 0, "record size");

  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* ur = smem;
  unsigned char* dr = ur + NU * USLOT;
  unsigned char* sr = dr + NV * VSLOT;
  unsigned char* lr = sr + NV * VSLOT;
  MmaRecord* rec = reinterpret_cast<MmaRecord*>(lr + (PAIR ? NV * VSLOT : 0));
  uint64_t* full = reinterpret_cast<uint64_t*>(rec + NV);
  uint64_t* empty = full + NV;
  uint32_t* smax_u = reinterpret_cast<uint32_t*>(empty + NV);
  uint32_t* smax_d = smax_u + NV;
  int* splane = reinterpret_cast<int*>(smax_d + NV);
  int* sj0 = splane + NV;  // tile origin of the stage's step (its outputs' store)
  int* sk0 = sj0 + NV;

  const Geom& g = a.g;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CW * 32);
      smax_u[s] = 0u;
      smax_d[s] = 0u;
      splane[s] = -1;
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if (warp == CW) {
    // ---------------- producer (lane 0 drives the pipeline) -----------------
    if (lane != 0) return;
    // The outputs of a finished step sit in its stage's d (d^{n+1}), s
    // (u^{n+1}) and lo slots; they go out as tile stores, clipped to the
    // interior by the tensor maps.  A step is retired (its consumers done,
    // its stores issued, its maxima flushed) one step before its stage is
    // loaded again, so that by then the stores have read the slots and the
    // wait for that is short (7-point FP16 549 -> 613 Gpts/s at 1024^3); the
    // pair form's 4-stage ring retires a step just before the reload
    // instead (one step early it loses a quarter of its depth: 394 -> 351
    // at 25 points).
    uint32_t hr = 0;           // next step to retire
    bool stored = false;       // the last retired step issued stores
    auto retire = [&]() -> bool {
      const uint32_t m = hr++;
      const int stage = (int)(m & (NV - 1));
      if (!mbar_wait_bounded(&empty[stage], (m / NV) & 1u, a.timeout_ns)) {
        atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
        stored = false;
        return false;
      }
      stored = splane[stage] >= 0;
      if (stored) {
        const int i = splane[stage];
        const int x = g.pk + sk0[stage], y = g.pj + sj0[stage], z = g.pi + i;
        tma_store_3d(&uomap, sr + stage * VSLOT, x, y, z);
        tma_store_3d(&dmap, dr + stage * VSLOT, x, y, z);
        if (PAIR) tma_store_3d(&lomap, lr + stage * VSLOT, x, y, z);
        bulk_commit();
        if (smax_u[stage]) atomicMax(&a.Mu_out[i], smax_u[stage]);
        if (smax_d[stage]) atomicMax(&a.Md_out[i], smax_d[stage]);
        smax_u[stage] = 0u;
        smax_d[stage] = 0u;
      }
      return true;
    };
    tma_prefetch_desc(&umap);
    tma_prefetch_desc(&dmap);
    tma_prefetch_desc(&smap);
    if (PAIR) tma_prefetch_desc(&lmap);
    uint32_t h = 0;
    bool ok = true;
    for (int unit = blockIdx.x; unit < a.units && ok; unit += gridDim.x) {
      const int ic = unit / a.ntjk;
      const int rem = unit - ic * a.ntjk;
      const int jt = rem / a.ntk;
      const int kt = rem - jt * a.ntk;
      const int k0 = kt * kMTK, j0 = jt * kMTJ;
      const int ia = ic * a.ichunk;
      const int ib = min(ia + a.ichunk, g.xs);
      const int nsteps = (ib - ia) + 2 * R;
      for (int n = 0; n < nsteps; ++n, ++h) {
        const int stage = (int)(h & (NV - 1));
        if constexpr (NV >= 8) {
          // retire the step whose stage is loaded next (h + 1 - NV); the
          // stores of this stage's last step (h - NV) were issued one step
          // ago: wait until at most the group just issued still reads
          if (h + 1 >= (uint32_t)NV) {
            if (!retire()) {
              ok = false;
              break;
            }
            if (stored) bulk_wait_read1();
            else bulk_wait_read0();
          }
        } else {
          // a shallow ring (the pair form's 4 stages) keeps every stage in
          // flight: retire this stage's last step (h - NV) and wait for its
          // stores' reads
          if (h >= (uint32_t)NV) {
            if (!retire()) {
              ok = false;
              break;
            }
            bulk_wait_read0();
          }
        }
        const int p = ia - R + n;
        const bool has_ds = n >= 2 * R;
        const int i = ia + n - 2 * R;
        splane[stage] = has_ds ? i : -1;
        sj0[stage] = j0;
        sk0[stage] = k0;
        mbar_arrive_expect_tx(&full[stage], UBYTES + (has_ds ? (PAIR ? 3u : 2u) * VBYTES + RBYTES : 0u));
        tma_load_3d(ur + (h & (NU - 1)) * USLOT, &umap, &full[stage], g.pk + k0 - 8, g.pj + j0 - R,
                    g.pi + p);
        if (has_ds) {
          tma_load_3d(dr + stage * VSLOT, &dmap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
          tma_load_3d(sr + stage * VSLOT, &smap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
          if (PAIR) tma_load_3d(lr + stage * VSLOT, &lmap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
          bulk_load(&rec[stage], &a.rec[i], RBYTES, &full[stage]);
        }
      }
    }
    // Drain: no copy in flight, every step retired (stores issued, maxima
    // flushed), then every store complete.
    while (hr < h) {
      const uint32_t m = hr;
      if (!mbar_wait_bounded(&full[m & (NV - 1)], (m / NV) & 1u, a.timeout_ns)) {
        atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
        ++hr;
        continue;
      }
      retire();
    }
    bulk_wait_all();
    return;
  }

  // ---------------- consumers: one 16x8 block per warp ----------------
  const int g8 = lane >> 2, t4 = lane & 3;
  const int kb = warp;  // the warp's 8-column block
  uint32_t wkh[3], wkl[3], wjh[6], wjl[6];
  band_fragments<KIND>(a, R, g8, t4, wkh, wkl, wjh, wjl);
  const bool need_lo = a.need_lo != 0;
  // diagonal of an 8x8 block in the B fragment of this lane: (row 2t, column
  // g) in the low half, (row 2t+1, column g) in the high half
  const uint32_t dmask = (g8 == 2 * t4 ? 0x0000ffffu : 0u) | (g8 == 2 * t4 + 1 ? 0xffff0000u : 0u);
  // ldmatrix row addresses of this lane (the x2 loads use lanes 0..15, whose
  // column term (lane >> 4) * 8 is 0):
  //   abase: u rows R..R+15, columns 8kb + 0..15 (+32 bytes: 16..23);
  //   bbase: u rows 0..23 (x4.trans: 0-7, 8-15, 16-23, 16-23), the block's columns;
  //   pbase: u rows R..R+15, the block's columns, for the i planes (lanes
  //          0..15 the plane i-r, 16..31 the plane i+r);
  //   vbase: d rows 0..15 (lanes 0..15) and s rows 0..15 (lanes 16..31);
  //   lbase: the lo words of u, rows 0..15.
  const int lrow = (lane & 7) + ((lane >> 3) & 1) * 8;
  const uint32_t u0s = smem_u32(ur);
  const uint32_t abase = u0s + (uint32_t)(((R + lrow) * kMUW + kb * 8 + (lane >> 4) * 8) * 2);
  const uint32_t bbase = u0s + (uint32_t)((((lane & 7) + 8 * min(lane >> 3, 2)) * kMUW + kb * 8 + 8) * 2);
  const uint32_t pbase = u0s + (uint32_t)(((R + lrow) * kMUW + kb * 8 + 8) * 2);
  const uint32_t vbase = smem_u32(lane < 16 ? dr : sr) + (uint32_t)((lrow * kMVW + kb * 8) * 2);
  const uint32_t lbase = smem_u32(lr) + (uint32_t)((lrow * kMVW + kb * 8) * 2);
  const int rsign = lane < 16 ? -1 : 1;
  // this lane's output words in a d / s / lo slot: rows g and g+8, columns 8kb + 2t
  const uint32_t obase = (uint32_t)((g8 * kMVW + kb * 8 + 2 * t4) * 2);

  uint32_t h = 0;
  bool failed = false;
  for (int unit = blockIdx.x; unit < a.units; unit += gridDim.x) {
    const int ic = unit / a.ntjk;
    const int rem = unit - ic * a.ntjk;
    const int jt = rem / a.ntk;
    const int kt = rem - jt * a.ntk;
    const int j0 = jt * kMTJ, k0 = kt * kMTK;
    const int ia = ic * a.ichunk;
    const int ib = min(ia + a.ichunk, g.xs);
    const int nsteps = (ib - ia) + 2 * R;
    // this lane's points: rows jr0, jr0 + 8, columns kc, kc + 1
    const int jr0 = j0 + g8;
    const int kc = k0 + 8 * kb + 2 * t4;
    const bool r0 = jr0 < g.ys, r1 = jr0 + 8 < g.ys, c0ok = kc < g.zs, c1ok = kc + 1 < g.zs;
    const bool whole = j0 + kMTJ <= g.ys && k0 + kMTK <= g.zs;
    // points inside the grid (bit c: component c of the lane's P4) for the
    // plane maxima; the tile stores clip the rest
    const uint32_t vbits = (r0 && c0ok ? 1u : 0u) | (r0 && c1ok ? 2u : 0u) | (r1 && c0ok ? 4u : 0u) |
                           (r1 && c1ok ? 8u : 0u);
    // output words outside the grid are zero: a tile store that ends inside
    // a 16-byte row segment can write the rest of that segment, which along
    // k is the zero halo (and the zero row pad after it)
    const uint32_t cmask = (c0ok ? 0x0000ffffu : 0u) | (c1ok ? 0xffff0000u : 0u);
    const uint32_t om0 = r0 ? cmask : 0u, om1 = r1 ? cmask : 0u;
    const bool src_unit = a.src.i >= ia && a.src.i < ib && a.src.j >= j0 && a.src.j < j0 + kMTJ &&
                          a.src.k >= k0 && a.src.k < k0 + kMTK;
    for (int n = 0; n < nsteps; ++n) {
      const uint32_t hh = h + (uint32_t)n;
      const uint32_t stage = hh & (NV - 1);
      if (!failed && !mbar_wait_bounded(&full[stage], (hh / NV) & 1u, a.timeout_ns)) {
        atomicExch(a.status, (uint32_t)kDevTimeoutFull);
        failed = true;
      }
      if (n >= 2 * R) {
        const int i = ia + n - 2 * R;
        const MmaRecord& W = rec[stage];
        const uint32_t cs = ((hh - R) & (NU - 1)) * USLOT;
        uint32_t X[4], Y0, Y1, B[4], DS[4], lw0 = 0u, lw1 = 0u;
        ldsm_x4(X, abase + cs);
        ldsm_x2(Y0, Y1, abase + cs + 32u);
        ldsm_x4_t(B, bbase + cs);
        ldsm_x4(DS, vbase + stage * VSLOT);
        if (PAIR) ldsm_x2(lw0, lw1, lbase + stage * VSLOT);
        // Djk: [U | U] x [Wk_hi ; Wk_lo] and [Wj_hi | Wj_lo] x [U ; U] (K = 48),
        // the hi parts alone (K = 24) where every band weight is exact
        float Dk[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float Dj[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mma_k16<KIND>(Dk, X[0], X[1], X[2], X[3], wkh[0], wkh[1]);
        mma_k16<KIND>(Dj, wjh[0], wjh[1], wjh[2], wjh[3], B[0], B[1]);
        if (need_lo) {
          mma_k16<KIND>(Dk, Y0, Y1, X[0], X[1], wkh[2], wkl[0]);
          mma_k16<KIND>(Dj, wjh[4], wjh[5], wjl[0], wjl[1], B[2], B[0]);
          mma_k16<KIND>(Dk, X[2], X[3], Y0, Y1, wkl[1], wkl[2]);
          mma_k16<KIND>(Dj, wjl[2], wjl[3], wjl[4], wjl[5], B[1], B[2]);
        } else {
          mma_k8<KIND>(Dk, Y0, Y1, wkh[2]);
          mma_k8<KIND>(Dj, wjh[4], wjh[5], B[2]);
        }
        // d and s with the plane's weights, then the i pairs: per radius
        // [U_{i-r} | U_{i+r}] x [diag(2^(E_{i-r}-X)) ; diag(2^(E_{i+r}-X))]
        // (exact products) times c1 w_r 2^X in FP32
        float Ds[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        mma_k16<KIND>(Ds, DS[0], DS[1], DS[2], DS[3], W.wd & dmask, W.wsh & dmask);
        mma_k8<KIND>(Ds, DS[2], DS[3], W.wsl & dmask);
        const float2 ys2 = splat(W.ys2), c1s = splat(W.c1s);
        const float2 jk01 = __fadd2_rn(make_float2(Dk[0], Dk[1]), make_float2(Dj[0], Dj[1]));
        const float2 jk23 = __fadd2_rn(make_float2(Dk[2], Dk[3]), make_float2(Dj[2], Dj[3]));
        P4 dn = {__ffma2_rn(jk01, c1s, __fmul2_rn(make_float2(Ds[0], Ds[1]), ys2)),
                 __ffma2_rn(jk23, c1s, __fmul2_rn(make_float2(Ds[2], Ds[3]), ys2))};
#pragma unroll
        for (int r = 1; r <= R; ++r) {
          uint32_t Q[4];
          ldsm_x4(Q, pbase + ((hh - R + rsign * r) & (NU - 1)) * USLOT);
          float Pr[4] = {0.0f, 0.0f, 0.0f, 0.0f};
          mma_k16<KIND>(Pr, Q[0], Q[1], Q[2], Q[3], W.ipw[2 * r - 2] & dmask, W.ipw[2 * r - 1] & dmask);
          dn = fma4(splat(W.ci[r - 1]), P4{make_float2(Pr[0], Pr[1]), make_float2(Pr[2], Pr[3])}, dn);
        }
        // the centre u: the hi words (X[2], X[3]) and, for the pair form, the lo words
        P4 u0 = decode4<KIND>(make_uint2(X[2], X[3]), W.uc);
        if (PAIR) {
          const P4 ul = decode4<KIND>(make_uint2(lw0, lw1), W.uc);
          dn = fma4(splat(a.c1m2s), ul, dn);
          u0 = add4(u0, ul);
        }
        if (src_unit && i == a.src.i) {
          const int srcc = (a.src.j == jr0 ? 0 : a.src.j == jr0 + 8 ? 2 : 16) +
                           (a.src.k == kc ? 0 : a.src.k == kc + 1 ? 1 : 16);
          const float add = a.cf.c2 * a.src.amp;
          if (srcc == 0) dn.a.x = dn.a.x + add;
          if (srcc == 1) dn.a.y = dn.a.y + add;
          if (srcc == 2) dn.b.x = dn.b.x + add;
          if (srcc == 3) dn.b.y = dn.b.y + add;
        }
        const uint2 dwo = encode4<KIND>(dn, W.inv_do);
        const P4 dq = decode4<KIND>(dwo, W.dq);
        const P4 un = add4(u0, dq);
        uint2 uwo, ulo = make_uint2(0u, 0u);
        if (PAIR) {
          const float2 t01 = __fmul2_rn(un.a, splat(W.inv_uo));
          const float2 t23 = __fmul2_rn(un.b, splat(W.inv_uo));
          uwo = make_uint2(f2_to_w2<KIND>(t01), f2_to_w2<KIND>(t23));
          const float2 h01 = w2_to_f2<KIND>(uwo.x), h23 = w2_to_f2<KIND>(uwo.y);
          ulo = make_uint2(f2_to_w2<KIND>(__fadd2_rn(t01, make_float2(-h01.x, -h01.y))),
                           f2_to_w2<KIND>(__fadd2_rn(t23, make_float2(-h23.x, -h23.y))));
        } else {
          uwo = encode4<KIND>(un, W.inv_uo);
        }
        float mu, md;
        if (whole) {
          mu = fmaxf(fmaxf(fabsf(un.a.x), fabsf(un.a.y)), fmaxf(fabsf(un.b.x), fabsf(un.b.y)));
          md = fmaxf(fmaxf(fabsf(dn.a.x), fabsf(dn.a.y)), fmaxf(fabsf(dn.b.x), fabsf(dn.b.y)));
        } else {
          mu = amax4m(un, vbits);
          md = amax4m(dn, vbits);
        }
        // outputs into the stage's slots, whose inputs this lane's block no
        // longer needs: u^{n+1} over s, d^{n+1} over d, the lo words over lo
        {
          unsigned char* so = sr + stage * VSLOT + obase;
          unsigned char* dout = dr + stage * VSLOT + obase;
          *reinterpret_cast<uint32_t*>(so) = uwo.x & om0;
          *reinterpret_cast<uint32_t*>(so + 8 * kMVW * 2) = uwo.y & om1;
          *reinterpret_cast<uint32_t*>(dout) = dwo.x & om0;
          *reinterpret_cast<uint32_t*>(dout + 8 * kMVW * 2) = dwo.y & om1;
          if (PAIR) {
            unsigned char* lo = lr + stage * VSLOT + obase;
            *reinterpret_cast<uint32_t*>(lo) = ulo.x & om0;
            *reinterpret_cast<uint32_t*>(lo + 8 * kMVW * 2) = ulo.y & om1;
          }
          fence_proxy_async_smem();
        }
        const uint32_t wu = __reduce_max_sync(0xffffffffu, __float_as_uint(mu));
        const uint32_t wd = __reduce_max_sync(0xffffffffu, __float_as_uint(md));
        if (lane == 0) {
          atomicMax(&smax_u[stage], wu);
          atomicMax(&smax_d[stage], wd);
        }
      }
      // every consumer thread arrives after its own reads of the stage (and
      // lane 0 after its maxima)
      mbar_arrive(&empty[stage]);
    }
    h += (uint32_t)nsteps;
  }
}

// Before each step, per plane i (one thread each): the scales of the planes
// the step writes (the rule of k_scales_delta) and the plane's record.
template <int KIND>
__global__ void k_mma_records(int xs, int R, const int* __restrict__ Eu, const int* __restrict__ Ed,
                              const int* __restrict__ Es, const uint32_t* __restrict__ Mu,
                              const uint32_t* __restrict__ Md, const uint32_t* __restrict__ Ms,
                              int* __restrict__ Eu_out, int* __restrict__ Ed_out, uint32_t* __restrict__ Mu_out,
                              uint32_t* __restrict__ Md_out, float k4, float c1, float c2, float4 wi, int S,
                              int src_i, float amp_abs, MmaRecord* __restrict__ rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= xs) return;
  // scales of u^{n+1} and d^{n+1} (as k_scales_delta)
  float nb = 0.0f;
  for (int e = -R; e <= R; ++e)
    if (i + e >= 0 && i + e < xs) nb = fmaxf(nb, __uint_as_float(Mu[i + e]));
  float Bd = __fmaf_rn(k4, nb, __uint_as_float(Md[i]));
  Bd = __fmaf_rn(c2, __uint_as_float(Ms[i]) + (i == src_i ? amp_abs : 0.0f), Bd);
  const float Bu = __uint_as_float(Mu[i]) + Bd;
  const int edo = scale_exponent(Bd), euo = scale_exponent(Bu);
  Ed_out[i] = edo;
  Eu_out[i] = euo;
  Mu_out[i] = 0u;
  Md_out[i] = 0u;
  // the i planes: their scales relative to 2^X, X = the largest of them
  // less 15, as exact 16-bit powers of two (a plane more than 2^39 below the
  // largest, 2^55 for BF16, takes 0: its contribution is below FP32 rounding
  // of the sum)
  const float w[5] = {0.0f, wi.x, wi.y, wi.z, wi.w};
  int ep[8];
  int emax = -100000;
  for (int r = 1; r <= 4; ++r)
    for (int side = 0; side < 2; ++side) {
      const int p = side ? i + r : i - r;
      const bool in = r <= R && p >= 0 && p < xs;
      ep[2 * r - 2 + side] = in ? Eu[p] : -100000;
      if (in) emax = max(emax, Eu[p]);
    }
  const int X = emax == -100000 ? 0 : emax - 15;
  MmaRecord o;
  for (int m = 0; m < 8; ++m) {
    uint32_t p2 = 0u, unused;
    if (ep[m] != -100000 && ep[m] - X >= -40) split16<KIND>(ldexpf(1.0f, ep[m] - X), p2, unused);
    o.ipw[m] = p2 | (p2 << 16);
  }
  for (int r = 1; r <= 4; ++r) o.ci[r - 1] = ldexpf(c1 * w[r], X);
  // d and s relative to 2^Y, the larger of them in [2^13, 2^14)
  const float md = ldexpf(1.0f, Ed[i]), ms = ldexpf(c2, Es[i]);
  int e1 = 0, e2 = 0;
  frexpf(md, &e1);
  if (ms != 0.0f) frexpf(ms, &e2);
  const int Y = (ms != 0.0f ? max(e1, e2) : e1) - 14;
  uint32_t hi, lo;
  split16<KIND>(ldexpf(md, -Y), hi, lo);
  o.wd = hi | (hi << 16);
  split16<KIND>(ldexpf(ms, -Y), hi, lo);
  o.wsh = hi | (hi << 16);
  o.wsl = lo | (lo << 16);
  o.ys2 = ldexpf(1.0f, Y);
  o.c1s = ldexpf(c1, Eu[i] - S);
  o.uc = exp2i(Eu[i]);
  o.inv_uo = exp2i(-euo);
  o.inv_do = exp2i(-edo);
  o.dq = exp2i(edo);
  for (int m = 0; m < 11; ++m) o.pad[m] = 0u;
  rec[i] = o;
}

template <int KIND, int P, bool PAIR>
cudaError_t launch_p(const Tma16Plan& pl, const Mma16Args& args, const CUtensorMap* maps,
                     cudaStream_t stream, int* occupancy_out) {
  if (pl.nv != (PAIR ? kMNV / 2 : kMNV) || pl.nb != 1) return cudaErrorInvalidConfiguration;
  auto kern = k_mma16<KIND, P, PAIR>;
  const int threads = (kMCW + 1) * 32;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  if (e != cudaSuccess) return e;
  if (occupancy_out) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy_out, kern, threads, pl.smem);
  kern<<<pl.grid, threads, pl.smem, stream>>>(maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], args);
  return cudaGetLastError();
}

template <int KIND, bool PAIR>
cudaError_t launch_k(int points, const Tma16Plan& pl, const Mma16Args& args, const CUtensorMap* maps,
                     cudaStream_t stream, int* occ) {
  switch (points) {
    case 7: return launch_p<KIND, 7, PAIR>(pl, args, maps, stream, occ);
    case 13: return launch_p<KIND, 13, PAIR>(pl, args, maps, stream, occ);
    case 25: return launch_p<KIND, 25, PAIR>(pl, args, maps, stream, occ);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch(int storage, int points, const Tma16Plan& pl, const Mma16Args& args,
                     const CUtensorMap* maps, cudaStream_t stream, int* occ) {
  if (storage == ST3D_F16) return launch_k<0, false>(points, pl, args, maps, stream, occ);
  if (storage == ST3D_BF16) return launch_k<1, false>(points, pl, args, maps, stream, occ);
  if (storage == ST3D_F16_HL) return launch_k<0, true>(points, pl, args, maps, stream, occ);
  return cudaErrorInvalidValue;
}

// exact in one word of the storage's type
bool exact16(int storage, float w) {
  uint32_t b;
  memcpy(&b, &w, 4);
  if (storage == ST3D_BF16) return (b & 0xffffu) == 0u;
  if (w == 0.0f) return true;
  // FP16: 11 significant bits and a normal exponent
  const int e = (int)((b >> 23) & 0xff) - 127;
  return e >= -14 && e <= 15 && (b & 0x1fffu) == 0u;
}

}  // namespace

size_t mma16_smem_bytes(int nv, int R, bool pair) {
  (void)R;
  const size_t uslot = ((size_t)kMUW * kMUH * 2 + 127) / 128 * 128;
  const size_t vslot = ((size_t)kMVW * kMTJ * 2 + 127) / 128 * 128;
  return (size_t)kMNU * uslot + (pair ? 3 : 2) * (size_t)nv * vslot + (size_t)nv * sizeof(MmaRecord) +
         2 * (size_t)nv * 8 + 5 * (size_t)nv * 4 + 128;
}

int mma16_blocks_per_sm(int storage, int points, const Tma16Plan& pl) {
  Mma16Args dummy;
  int occ = 0;
  if (dispatch(storage, points, pl, dummy, nullptr, nullptr, &occ) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

cudaError_t launch_mma16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                         const Coefs<float>& cf, const Delta16Step& st, const Source& src,
                         uint32_t* dev_status, cudaStream_t stream) {
  if (!pl.mma || !pl.mma_rec || pl.pair != (st.lout != nullptr)) return cudaErrorInvalidValue;
  Mma16Args a;
  memset(&a, 0, sizeof a);
  a.g = g;
  a.cf = cf;
  a.rec = pl.mma_rec;
  a.Mu_out = st.Mu_out;
  a.Md_out = st.Md_out;
  const int P = points;
  const int R = pl.radius;
  float wi[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  float wmax = fabsf(st.m2s);
  for (int p = 0; p < npairs_of(P); ++p) {
    const int ax = pair_axis(P, p), r = pair_r(P, p);
    const float w = cf.cf[p];
    if (ax == 0) wi[r] = w;
    if (ax == 1) a.wj[r] = w;
    if (ax == 2) a.wk[r] = w;
    if (ax != 0) wmax = fmaxf(wmax, fabsf(w));
  }
  a.wk[0] = st.m2s;
  // S: the largest band weight times 2^S lies in [2^13, 2^14)
  int S = 0;
  if (wmax > 0.0f) {
    int e;
    frexpf(wmax, &e);  // wmax = f * 2^e, f in [0.5, 1)
    S = 14 - e;
  }
  bool lo = false;
  for (int r = 0; r <= R; ++r) {
    a.wj[r] = ldexpf(a.wj[r], S);
    a.wk[r] = ldexpf(a.wk[r], S);
    lo = lo || !exact16(storage, a.wj[r]) || !exact16(storage, a.wk[r]);
  }
  a.need_lo = lo ? 1 : 0;
  a.c1m2s = cf.c1 * st.m2s;
  a.ntk = pl.ntk;
  a.ntjk = pl.ntj * pl.ntk;
  a.ichunk = pl.ichunk;
  a.units = pl.units;
  a.src = src;
  a.timeout_ns = pl.timeout_ns;
  a.status = dev_status;
  // loads: u^n (halo box), d, s, the lo words of u^n; stores: u^{n+1} into
  // the other buffer (interior box), d, the lo words of u^{n+1}
  const CUtensorMap maps[6] = {pl.uhi[st.ubuf], pl.dmap, pl.vhi[2], pl.lo[st.ubuf], pl.vhi[1 - st.ubuf],
                               pl.lo[1 - st.ubuf]};
  const int threads = 128;
  const float4 w4 = make_float4(wi[1], wi[2], wi[3], wi[4]);
  if (storage == ST3D_BF16)
    k_mma_records<1><<<(g.xs + threads - 1) / threads, threads, 0, stream>>>(
        g.xs, R, st.Eu, st.Ed, st.Es, st.Mu, st.Md, st.Ms, st.Eu_out, st.Ed_out, st.Mu_out, st.Md_out, st.k4,
        cf.c1, cf.c2, w4, S, src.i, fabsf(src.amp), pl.mma_rec);
  else
    k_mma_records<0><<<(g.xs + threads - 1) / threads, threads, 0, stream>>>(
        g.xs, R, st.Eu, st.Ed, st.Es, st.Mu, st.Md, st.Ms, st.Eu_out, st.Ed_out, st.Mu_out, st.Md_out, st.k4,
        cf.c1, cf.c2, w4, S, src.i, fabsf(src.amp), pl.mma_rec);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return dispatch(storage, points, pl, a, maps, stream, nullptr);
}

}  // namespace st3d
