// st3d_tma.cuh -- TMA and mbarrier primitives (inline PTX, sm_90+ forms that
// sm_103a runs) and the TMA-kernel plan shared by the launcher and the
// context code.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace st3d {

// CTA tile of the TMA kernel: TK = 128 points along k (32 lanes x float4),
// TJ rows along j (one consumer warp per row), plus a producer warp.
constexpr int kTmaTK = 128;
constexpr int kTmaKHalo = 4;                    // floats loaded either side along k (16 bytes)
constexpr int kTmaUKW = kTmaTK + 2 * kTmaKHalo; // smem row width of a u tile
// Columns per tile of the tensor-core 16-bit kernel (nineteen 8-column
// blocks, one consumer warp each).
constexpr int kMmaTK = 152;

struct TmaPlan {
  int tj = 16;      // rows per tile (consumer warps)
  int nv = 3;       // pipeline stages (v/s ring depth); u ring has nv + R slots
  int ichunk = 128; // planes per work unit
  int radius = 0;
  int ntj = 0, ntk = 0, nti = 0, units = 0;
  int grid = 0, threads = 0;
  size_t smem = 0;
  uint64_t timeout_ns = 4000000000ull;
  CUtensorMap umap[5];  // halo box (kTmaUKW x (tj+2R) x 1) over each field buffer
  CUtensorMap vmap[5];  // interior box (kTmaTK x tj x 1) over each field buffer
};

// Per-plane record of the tensor-core 16-bit kernel (st3d_kernels_mma16.cu),
// written before each step: ipw, the scales of the planes i-r (ipw[2r-2])
// and i+r (ipw[2r-1]) relative to 2^X as exact 16-bit powers of two
// (packed p | p << 16); ci[r-1] = c1 * w_r * 2^X; the weights of d (wd) and
// s (wsh, wsl) relative to 2^Y; then 2^Y, c1 * 2^(E_u - S), 2^E_u and the
// encode / decode scales of the step's outputs.  128 bytes, one bulk copy.
struct alignas(128) MmaRecord {
  uint32_t ipw[8];
  float ci[4];
  uint32_t wd, wsh, wsl;
  float ys2, c1s, uc, inv_uo, inv_do, dq;
  uint32_t pad[11];
};

// Plan of the 16-bit-storage kernels (st3d_kernels_tma16.cu for the
// compensated form, st3d_kernels_delta16.cu for the delta form): same work
// decomposition; tensor maps over the 16-bit words of the u/v buffers (halo
// box and interior box), of s (interior box, index 2), over the low bytes of
// the u/v buffers, and over d.
struct Tma16Plan {
  int tj = 16, nv = 3, ichunk = 128, radius = 0;
  int ntj = 0, ntk = 0, nti = 0, units = 0;
  int grid = 0, threads = 0;
  size_t smem = 0;
  uint64_t timeout_ns = 4000000000ull;
  bool delta = false;     // FP16 / BF16 delta form (st3d_kernels_delta16.cu)
  bool pair = false;      // F16_HL: u as an FP16 hi/lo pair; lo[] are its lo words
  bool mma = false;       // delta form on the tensor-core kernel (st3d_kernels_mma16.cu):
                          // 16 x kMmaTK tiles, u box (kMmaTK+16) x 24, d/s/lo boxes kMmaTK x 16
  int nb = 1;             // mma kernel: 8-column blocks per consumer warp
  MmaRecord* mma_rec = nullptr;  // mma kernel: one record per i-plane (device)
  CUtensorMap uhi[2];
  CUtensorMap vhi[3];
  CUtensorMap lo[2];
  CUtensorMap dmap;       // delta form: interior box over d (buffer 3)
};

// Plan of the temporally blocked kernel (st3d_kernels_tb.cu): T fused
// steps, level-1 tiles of tb_rows(points, T) rows writing rows_out =
// rows - 2(T-1)R rows and 120 columns; tensor maps over the four state
// buffers (0, 1, 3, 4) and s (2): umap the halo box (kTmaUKW x rows+2R), vmap
// the interior box (kTmaTK x rows).  The kernel's transaction byte counts
// assume these boxes, so plan and kernel take the height from this one
// function.  Taller tiles recompute fewer halo rows per written row and run
// more consumer warps, up to the register and shared-memory limits: 7 points
// T=2 runs 26 rows (27 warps, 67 registers; 629 against 544 Gpts/s with 16
// at 1024^3, the same bits), T=4 18 rows (568 against 531; 20 rows do not
// fit in shared memory), 13 points T=2 18 rows (452 against 411; 20 rows cap
// the registers at 80 and spill, 372).  13 points T=4 and 25 points T=2 keep
// 2R+1 planes of T levels in register queues (80 and 72 floats a lane): 15
// rows make a 16-warp CTA whose threads may hold 128 registers.
__host__ __device__ constexpr int tb_rows(int points, int T) {
  return (points == 7 && T == 2) ? 26 : (points == 25 || (points == 13 && T == 4)) ? 15 : 18;
}
// Columns of k margin either side of a temporally blocked tile's 128 level
// columns: level t is exact in all but (t-1)R columns at either edge, so the
// margin must be >= (T-1)R.  4 (tiles write 120 columns) while (T-1)R <= 4,
// else 8 (112 columns: 13 points T=4, (T-1)R = 6).  A multiple of 4 floats,
// so every TMA x coordinate stays 16-byte aligned.
__host__ __device__ constexpr int tb_khalo(int points, int T) {
  return (T - 1) * ((points == 25) ? 4 : (points == 13) ? 2 : 1) > 4 ? 8 : 4;
}
struct TbPlan {
  int T = 2, radius = 0, rows = 0, rows_out = 0;
  int ichunk = 0, ntj = 0, ntk = 0, nti = 0, units = 0;
  int grid = 0;
  uint64_t timeout_ns = 4000000000ull;
  CUtensorMap umap[5];
  CUtensorMap vmap[5];
};

// Planes per work unit: the chunk length that minimises the modelled time
// ceil(units / ctas) * (ichunk + R/2) (a unit's 2R warm-up steps load only u,
// about a quarter of a full step's bytes), i.e. balance across the persistent
// CTAs against the warm-up re-reads of short chunks.
inline int tma_pick_ichunk(int xs, int tiles, int ctas, int R) {
  int best = xs;
  double best_cost = 1e300;
  for (int ic = 8; ic <= xs + 7; ++ic) {
    const int nti = (xs + ic - 1) / ic;
    const int chunk = (xs + nti - 1) / nti;
    const long long units = (long long)nti * tiles;
    const long long waves = (units + ctas - 1) / ctas;
    const double cost = (double)waves * (chunk + 0.5 * R);
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best = chunk;
    }
    if (chunk >= xs) break;
  }
  return best;
}

struct Layout;
// FP32 tiled tensor map over one field buffer with a box of box_k x box_j
// points; the valid extent is the row front pad + zs + kext along k and the
// front rows + ys + jext along j (st3d_api.cu).
int encode_f32_box(CUtensorMap* m, void* base, const Layout& L, uint32_t box_k, uint32_t box_j,
                   uint32_t kext, uint32_t jext);

inline size_t tma_smem_bytes(int tj, int nv, int R) {
  const size_t uslot = ((size_t)kTmaUKW * (tj + 2 * R) + 31) / 32 * 32 * 4;
  const size_t vslot = (size_t)kTmaTK * tj * 4;
  return (size_t)(nv + R) * uslot + 2 * (size_t)nv * vslot + 2 * (size_t)nv * 8 + 128;
}

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the phase of parity `parity` to complete; gives up after
// `limit_ns` nanoseconds of wall time (or 2^30 polls) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 1; it < (1u << 30); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 31u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// 3-D tiled TMA load of the box at element coordinates (x, y, z) into
// shared memory, completing on `bar` with the box's byte count.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

#endif  // __CUDACC__

}  // namespace st3d
