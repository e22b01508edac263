// st3d_batch.cu -- the batching form: many independent grids of uneven
// sizes and stencil orders (independent source shots) advancing together.
//
// One time step of every grid is one persistent launch: CTAs (at most
// #SMs x resident) pull work items -- one (grid, 12-row x 128-point or
// 24-row x 64-point tile, i-chunk) unit each -- from a device work queue (an atomic head over an item
// table ordered largest grid first), so small and large grids, 7-, 13- and
// 25-point stencils share the GPU without a launch per grid.  The producer
// warp of each CTA takes the next item, streams that grid's planes in with
// TMA (the grid's own tensor maps, kept in global memory) and tells the
// consumer warps which item each pipeline stage belongs to; the consumers run
// the stencil of the item's order (the same code and arithmetic as the
// single-grid TMA kernel, on packed FP32 pairs: 243 -> 278 Gpts/s on the
// 64-grid batch against scalar FP32).  Steps are ordered by kernel boundaries; the whole
// time loop (a queue reset and a launch per step) can be captured in a CUDA
// graph and replayed.  The baseline schedule launches the single-grid kernel
// once per grid per step.
//
// The pipelined schedule runs every step of a call in ONE persistent launch:
// the queue runs over (step, item) in step-major order, and a per-(step,
// grid) counter of finished items orders the steps of each grid.  Before a
// CTA loads an item of step t > 0 its producer waits (bounded) until every
// item of step t - 1 of the same grid has finished: step t reads U^t, which
// step t - 1 wrote, and overwrites U^{t-1}, which step t - 1 read with its
// halo.  Grids do not wait for one another, so the tail of one step (the
// smallest grids: the item order puts the largest first) overlaps the start
// of the next instead of draining the GPU at a kernel boundary.  Finishing an
// item: each consumer warp's lane 0 fences and counts the warp in a shared-
// memory counter of the item (one per item sequence number, modulo twice the
// pipeline depth), and the last warp fences (generic and async proxy) and
// adds to the global counter with release semantics; the waiting producer
// reads it with acquire semantics and fences the async proxy before its TMA
// loads.  All waits are bounded and report through the status word: a
// consumer warp whose wait gave up returns (the call's results are then
// void), the producer's own bounded waits then give up too, and its drain
// waits (bounded) for the stages it issued last.
#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "st3d_ctx.h"
#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

// Wide tiles of 12 rows x 128 points: 12 consumer warps and a producer, so a
// thread may hold 128 registers (the loop serving three stencil orders and
// two tile shapes spilled 196 bytes at the 96 of a 17-warp CTA); measured on
// the 64-grid batch: 16 rows 290.8, 12 rows 335.9, with 6 stages 362.4,
// 10 rows 312.5, 14 rows x 5 stages 364.9 Gpts/s.
constexpr int kBTJ = 12;
// Narrow tiles (24 rows x 64 points, each consumer warp serving two rows with
// 16 lanes each) for grids whose k extent fits them better: the same 1536
// points, v/s slots and warps per tile, a u slot that fits the wide one's.
constexpr int kNTJ = 24;
constexpr int kNTK = 64;
constexpr int kBNV = 6;  // pipeline stages (4 measured 335.9, 6 362.4, 8 359.8 Gpts/s)
constexpr int kItemSlots = 2 * kBNV;  // pipelined schedule: item completion counters per CTA
constexpr int kBRmax = 4;

struct BatchGrid {
  Geom g;
  Coefs<float> cf;
  float* buf[2];
  int P, R;
  int ntk, ntjk, ichunk, units;
  int src_i, src_j, src_k;
  int cur0;      // buffer holding u at the call's first step
  int map_base;  // index of the grid's 5 tensor maps: u over buf 0/1, v over buf 0/1, s
  int narrow;    // tiles of kNTJ x kNTK instead of kBTJ x kTmaTK
};

struct BatchArgs {
  const BatchGrid* grids;
  const CUtensorMap* maps;
  const int2* items;  // (grid, unit)
  int total_items;
  int n_grids;
  int* head;
  const float* amps;  // [step][grid]
  int step;           // step within the call of the launch's first step
  int nsteps;         // steps of this launch (1, or all steps of a pipelined call)
  int* done;          // pipelined: finished items per (step, grid); nullptr otherwise
  uint64_t timeout_ns;
  uint32_t* status;
};

struct BStage {
  int grid;  // -1: no more work
  int unit;
  int step;  // step within the call
  int pad;
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_gpu_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Waits until *ctr reaches `target` (acquire); false after `limit_ns`.
__device__ bool wait_counter(const int* ctr, int target, uint64_t limit_ns) {
  if (ld_acquire_gpu(ctr) >= target) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 1; it < (1u << 26); ++it) {
    __nanosleep(it < 64 ? 32 : 256);
    if (ld_acquire_gpu(ctr) >= target) return true;
    if ((it & 15u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

constexpr int kUSlot = (kTmaUKW * (kBTJ + 2 * kBRmax) + 31) / 32 * 32;  // floats
constexpr int kVSlot = kTmaTK * kBTJ;                                   // floats
constexpr int kNU = kBNV + kBRmax;

size_t batch_smem_bytes() {
  return ((size_t)kNU * kUSlot + 2 * (size_t)kBNV * kVSlot) * 4 + 2 * kBNV * 8 + kBNV * sizeof(BStage) +
         kItemSlots * sizeof(unsigned) + 128;
}

// The consumer side of one work unit (the single-grid kernel's consumer loop
// for stencil P): nsteps pipeline stages starting at global stage h0.  Warp
// w serves tile row w (wide tiles) or rows 2w and 2w + 1 with lanes 0-15 and
// 16-31 (narrow tiles); `r` and `kl` are the lane's tile row and column.  The
// tile shape is a run-time value so that one copy of the loop per order
// serves both (two template copies spilled registers).
static_assert((kNTK + 2 * kTmaKHalo) * (kNTJ + 2 * kBRmax) <= kUSlot && kNTK * kNTJ == kVSlot,
              "narrow tile does not fit the slots");
template <int P>
__device__ __forceinline__ bool consume_unit(const BatchArgs& a, const BatchGrid& G, int gi, int unit,
                                             int step, uint32_t h0, float* ur, float* vr, float* sr,
                                             uint64_t* full, uint64_t* empty, int warp, int lane) {
  constexpr int R = (P == 25) ? 4 : (P == 13) ? 2 : 1;
  constexpr int QN = 2 * R + 1;
  constexpr int NP = npairs_of(P);
  const bool narrow = G.narrow != 0;
  const int TJ = narrow ? kNTJ : kBTJ;
  const int TK = narrow ? kNTK : kTmaTK;
  const int UKW = TK + 2 * kTmaKHalo;
  const int r = narrow ? 2 * warp + (lane >> 4) : warp;
  const int kl = narrow ? (lane & 15) : lane;
  const Geom& g = G.g;
  const int ic = unit / G.ntjk;
  const int rem = unit - ic * G.ntjk;
  const int jt = rem / G.ntk;
  const int kt = rem - jt * G.ntk;
  const int j = jt * TJ + r;
  const int k = kt * TK + 4 * kl;
  const int ia = ic * G.ichunk;
  const int ib = min(ia + G.ichunk, g.xs);
  const int nsteps = (ib - ia) + 2 * R;
  const bool row_ok = j < g.ys;
  const int ub = G.cur0 ^ (step & 1);
  float* vout = G.buf[ub ^ 1];
  float* vrow = vout + g.org + (long long)j * g.sj + k;
  const float amp = (G.src_i >= 0) ? a.amps[(size_t)step * a.n_grids + gi] : 0.0f;
  float4 q[QN];
  for (int n0 = 0; n0 < nsteps; n0 += QN) {
#pragma unroll
    for (int ph = 0; ph < QN; ++ph) {
      const int n = n0 + ph;
      if (n >= nsteps) break;
      const uint32_t hh = h0 + (uint32_t)n;
      const int stage = (int)(hh % kBNV);
      if (!mbar_wait_bounded(&full[stage], (hh / kBNV) & 1u, a.timeout_ns)) {
        atomicExch(a.status, (uint32_t)kDevTimeoutFull);
        return false;
      }
      q[ph] = *reinterpret_cast<const float4*>(ur + (hh % kNU) * kUSlot + (r + R) * UKW + kTmaKHalo + 4 * kl);
      if (n >= 2 * R) {
        const int i = ia + n - 2 * R;
        const float* uc = ur + ((hh - R) % kNU) * kUSlot + (r + R) * UKW;
        const float4 c4 = q[(ph + QN - R) % QN];
        const float4 l4 = *reinterpret_cast<const float4*>(uc + 4 * kl);
        const float4 r4 = *reinterpret_cast<const float4*>(uc + 2 * kTmaKHalo + 4 * kl);
        const float w[12] = {l4.x, l4.y, l4.z, l4.w, c4.x, c4.y, c4.z, c4.w, r4.x, r4.y, r4.z, r4.w};
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
            const float4 A = *reinterpret_cast<const float4*>(uc - rr * UKW + kTmaKHalo + 4 * kl);
            const float4 B = *reinterpret_cast<const float4*>(uc + rr * UKW + kTmaKHalo + 4 * kl);
            sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                       {make_float2(B.x, B.y), make_float2(B.z, B.w)});
          } else {
            const float4 A = q[(ph + 2 * QN - R - rr) % QN];
            const float4 B = q[(ph + QN - R + rr) % QN];
            sum = add4({make_float2(A.x, A.y), make_float2(A.z, A.w)},
                       {make_float2(B.x, B.y), make_float2(B.z, B.w)});
          }
          const P4 d = add4(sum, nu2);
          acc = p == 0 ? mul4(d, splat(G.cf.cf[0])) : fma4(splat(G.cf.cf[p]), d, acc);
        }
        const float4 v4 = *reinterpret_cast<const float4*>(vr + stage * kVSlot + r * TK + 4 * kl);
        const float4 s4 = *reinterpret_cast<const float4*>(sr + stage * kVSlot + r * TK + 4 * kl);
        P4 ss = {make_float2(s4.x, s4.y), make_float2(s4.z, s4.w)};
        if (i == G.src_i && j == G.src_j && (unsigned)(G.src_k - k) < 4u) {
          const int c = G.src_k - k;
          if (c == 0) ss.a.x = ss.a.x + amp;
          if (c == 1) ss.a.y = ss.a.y + amp;
          if (c == 2) ss.b.x = ss.b.x + amp;
          if (c == 3) ss.b.y = ss.b.y + amp;
        }
        P4 t = add4(u2, {make_float2(-v4.x, -v4.y), make_float2(-v4.z, -v4.w)});
        t = fma4(splat(G.cf.c1), acc, t);
        const P4 x = fma4(splat(G.cf.c2), ss, t);
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
  return true;
}

__global__ void __launch_bounds__((kBTJ + 1) * 32, 1) k_batch(const BatchArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* ur = reinterpret_cast<float*>(smem_raw);
  float* vr = ur + kNU * kUSlot;
  float* sr = vr + kBNV * kVSlot;
  uint64_t* full = reinterpret_cast<uint64_t*>(sr + kBNV * kVSlot);
  uint64_t* empty = full + kBNV;
  BStage* info = reinterpret_cast<BStage*>(empty + kBNV);
  unsigned* finished = reinterpret_cast<unsigned*>(info + kBNV);  // warps done, per item slot

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int q = 0; q < kItemSlots; ++q) finished[q] = 0u;
    for (int s = 0; s < kBNV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kBTJ);
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if (warp == kBTJ) {
    // ---------------- producer ----------------
    if (lane != 0) return;
    uint32_t h = 0;
    bool ok = true;
    const int last = a.total_items * a.nsteps;
    while (ok) {
      const int x = atomicAdd(a.head, 1);
      const bool stop = x >= last;
      const int stage0 = (int)(h % kBNV);
      if (stop) {
        // hand the consumers a stop record through the pipeline
        if (h >= (uint32_t)kBNV &&
            !mbar_wait_bounded(&empty[stage0], ((h / kBNV) - 1) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          break;
        }
        info[stage0].grid = -1;
        mbar_arrive(&full[stage0]);
        break;
      }
      const int tl = x / a.total_items;  // step of the launch
      const int step = a.step + tl;
      const int2 it = a.items[x - tl * a.total_items];
      const BatchGrid& G = a.grids[it.x];
      const int R = G.R;
      const int unit = it.y;
      if (a.done && tl > 0) {
        // every item of the grid's previous step has finished (acquire);
        // then order the async proxy (TMA) after it
        if (!wait_counter(a.done + (size_t)(tl - 1) * a.n_grids + it.x, G.units, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutDep);
          ok = false;
          break;
        }
        fence_proxy_async_global();
      }
      const int ic = unit / G.ntjk;
      const int rem = unit - ic * G.ntjk;
      const int jt = rem / G.ntk;
      const int kt = rem - jt * G.ntk;
      const int tk = G.narrow ? kNTK : kTmaTK, tj = G.narrow ? kNTJ : kBTJ;
      const int k0 = kt * tk, j0 = jt * tj;
      const int ia = ic * G.ichunk;
      const int ib = min(ia + G.ichunk, G.g.xs);
      const int nsteps = (ib - ia) + 2 * R;
      const int ub = G.cur0 ^ (step & 1);
      const CUtensorMap* umap = &a.maps[G.map_base + ub];
      const CUtensorMap* vmap = &a.maps[G.map_base + 2 + (ub ^ 1)];
      const CUtensorMap* smap = &a.maps[G.map_base + 4];
      const uint32_t ubytes = (uint32_t)((tk + 2 * kTmaKHalo) * (tj + 2 * R) * 4);
      const uint32_t vbytes = (uint32_t)(kVSlot * 4);
      for (int n = 0; n < nsteps; ++n, ++h) {
        const int stage = (int)(h % kBNV);
        if (h >= (uint32_t)kBNV &&
            !mbar_wait_bounded(&empty[stage], ((h / kBNV) - 1) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          ok = false;
          break;
        }
        info[stage].grid = it.x;
        info[stage].unit = unit;
        info[stage].step = step;
        const bool has_vs = n >= 2 * R;
        mbar_arrive_expect_tx(&full[stage], ubytes + (has_vs ? 2 * vbytes : 0u));
        tma_load_3d(ur + (h % kNU) * kUSlot, umap, &full[stage], G.g.pk + k0 - kTmaKHalo,
                    G.g.pj + j0 - R, G.g.pi + ia - R + n);
        if (has_vs) {
          const int i = ia + n - 2 * R;
          tma_load_3d(vr + stage * kVSlot, vmap, &full[stage], G.g.pk + k0, G.g.pj + j0, G.g.pi + i);
          tma_load_3d(sr + stage * kVSlot, smap, &full[stage], G.g.pk + k0, G.g.pj + j0, G.g.pi + i);
        }
      }
    }
    // leave no copy in flight: wait until the last real stages were consumed
    for (uint32_t m = (h > (uint32_t)kBNV ? h - kBNV : 0u); m < h; ++m)
      (void)mbar_wait_bounded(&empty[m % kBNV], (m / kBNV) & 1u, a.timeout_ns);
    return;
  }

  // ---------------- consumers ----------------
  uint32_t h = 0;
  uint32_t seq = 0;  // items this warp has taken (the same sequence in every warp)
  while (true) {
    const int stage = (int)(h % kBNV);
    if (!mbar_wait_bounded(&full[stage], (h / kBNV) & 1u, a.timeout_ns)) {
      atomicExch(a.status, (uint32_t)kDevTimeoutFull);
      return;
    }
    const BStage st = info[stage];
    if (st.grid < 0) return;
    const BatchGrid& G = a.grids[st.grid];
    bool ok;
    int nsteps;
    {
      const int ic = st.unit / G.ntjk;
      const int ia = ic * G.ichunk;
      nsteps = (min(ia + G.ichunk, G.g.xs) - ia) + 2 * G.R;
    }
    switch (G.P) {
      case 7: ok = consume_unit<7>(a, G, st.grid, st.unit, st.step, h, ur, vr, sr, full, empty, warp, lane); break;
      case 13: ok = consume_unit<13>(a, G, st.grid, st.unit, st.step, h, ur, vr, sr, full, empty, warp, lane); break;
      default: ok = consume_unit<25>(a, G, st.grid, st.unit, st.step, h, ur, vr, sr, full, empty, warp, lane); break;
    }
    if (!ok) return;
    if (a.done) {
      // This warp's stores of the item are done; the last warp of the CTA to
      // get here publishes the item.  Every warp takes the CTA's items in the
      // same order, so the item's sequence number picks its counter; a warp
      // runs at most kBNV stages (so at most kBNV items) ahead of the slowest,
      // hence kItemSlots > kBNV counters never mix two items.  No blocking
      // barrier: a warp that gave up on a wait never stalls the others.
      __syncwarp();
      if (lane == 0) {
        unsigned* slot = finished + (seq % kItemSlots);
        __threadfence();
        const unsigned old = atomicAdd(slot, 1u);
        if (old == kBTJ - 1) {
          atomicExch(slot, 0u);  // free for item seq + kItemSlots
          __threadfence();
          fence_proxy_async_global();
          red_release_gpu_add(a.done + (size_t)(st.step - a.step) * a.n_grids + st.grid, 1);
        }
      }
    }
    ++seq;
    h += (uint32_t)nsteps;
  }
}

}  // namespace
}  // namespace st3d

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using namespace st3d;

struct st3d_batch {
  std::vector<st3d_ctx*> ctx;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  BatchGrid* d_grids = nullptr;
  CUtensorMap* d_maps = nullptr;
  int2* d_items = nullptr;
  int* d_head = nullptr;  // one queue head per step of the largest call
  int heads = 0;
  int* d_done = nullptr;  // pipelined schedule: finished items per (step, grid)
  size_t done_cap = 0;
  float* d_amps = nullptr;
  size_t amps_cap = 0;
  float* h_amps = nullptr;  // pinned staging of the amplitudes
  cudaEvent_t amps_copied = nullptr;  // the last copy out of h_amps has been done
  uint32_t* d_status = nullptr;
  std::vector<BatchGrid> grids;
  int total_items = 0;
  int ctas = 0;
  size_t smem = 0;
  uint64_t launches = 0;
  uint64_t points = 0;
  std::map<uint32_t, cudaGraphExec_t> graphs;  // by step count
  int device = -1;  // CUDA device ordinal of every grid (opts.device), -1: current
};

namespace {

int bfail(int status, const char* msg) { return set_error(status, "%s", msg); }

#define B_CUDA(call)                                                                            \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(e_ == cudaErrorMemoryAllocation ? ST3D_ERR_NOMEM : ST3D_ERR_CUDA,        \
                       "%s: %s", #call, cudaGetErrorString(e_));                                \
  } while (0)

void destroy_graphs(st3d_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

int ensure_steps(st3d_batch* b, uint32_t steps) {
  const size_t need = (size_t)steps * b->ctx.size();
  if (need > b->amps_cap) {
    if (b->d_amps) cudaFree(b->d_amps);
    if (b->h_amps) cudaFreeHost(b->h_amps);
    b->d_amps = nullptr;
    b->h_amps = nullptr;
    B_CUDA(cudaMalloc(&b->d_amps, need * sizeof(float)));
    B_CUDA(cudaMallocHost(&b->h_amps, need * sizeof(float)));
    b->amps_cap = need;
    destroy_graphs(b);  // captured launches point at the old buffer
  }
  if ((int)steps > b->heads) {
    if (b->d_head) cudaFree(b->d_head);
    b->d_head = nullptr;
    B_CUDA(cudaMalloc(&b->d_head, (size_t)steps * sizeof(int)));
    b->heads = (int)steps;
    destroy_graphs(b);
  }
  if (need > b->done_cap) {
    if (b->d_done) cudaFree(b->d_done);
    b->d_done = nullptr;
    B_CUDA(cudaMalloc(&b->d_done, need * sizeof(int)));
    b->done_cap = need;
  }
  return ST3D_OK;
}

// The per-call state the kernels read: the buffer holding u in each grid and
// the source amplitudes of every step.
int stage_call(st3d_batch* b, uint32_t steps) {
  const size_t n = b->ctx.size();
  // the previous call's asynchronous copy may still be reading h_amps
  B_CUDA(cudaEventSynchronize(b->amps_copied));
  for (size_t gi = 0; gi < n; ++gi) {
    st3d_ctx* c = b->ctx[gi];
    b->grids[gi].cur0 = c->ub;
    for (uint32_t t = 0; t < steps; ++t) {
      float amp = 0.0f;
      if (c->opts.src_i >= 0)
        amp = (float)st3d_ricker((double)(c->step + t) * c->opts.dt, c->opts.src_f, c->opts.src_t0);
      b->h_amps[(size_t)t * n + gi] = amp;
    }
  }
  B_CUDA(cudaMemcpyAsync(b->d_grids, b->grids.data(), n * sizeof(BatchGrid), cudaMemcpyHostToDevice,
                         b->stream));
  B_CUDA(cudaMemcpyAsync(b->d_amps, b->h_amps, (size_t)steps * n * sizeof(float),
                         cudaMemcpyHostToDevice, b->stream));
  B_CUDA(cudaEventRecord(b->amps_copied, b->stream));
  return ST3D_OK;
}

int enqueue_persistent(st3d_batch* b, uint32_t steps) {
  B_CUDA(cudaMemsetAsync(b->d_head, 0, (size_t)steps * sizeof(int), b->stream));
  for (uint32_t t = 0; t < steps; ++t) {
    BatchArgs a;
    a.grids = b->d_grids;
    a.maps = b->d_maps;
    a.items = b->d_items;
    a.total_items = b->total_items;
    a.n_grids = (int)b->ctx.size();
    a.head = b->d_head + t;
    a.amps = b->d_amps;
    a.step = (int)t;
    a.nsteps = 1;
    a.done = nullptr;
    a.timeout_ns = 4000000000ull;
    a.status = b->d_status;
    k_batch<<<b->ctas, (kBTJ + 1) * 32, b->smem, b->stream>>>(a);
    B_CUDA(cudaGetLastError());
  }
  return ST3D_OK;
}

// All steps of the call in one persistent launch: one queue over (step,
// item) and the per-(step, grid) counters of finished items, both cleared
// first.
int enqueue_pipelined(st3d_batch* b, uint32_t steps) {
  const size_t n = b->ctx.size();
  B_CUDA(cudaMemsetAsync(b->d_head, 0, sizeof(int), b->stream));
  B_CUDA(cudaMemsetAsync(b->d_done, 0, (size_t)steps * n * sizeof(int), b->stream));
  BatchArgs a;
  a.grids = b->d_grids;
  a.maps = b->d_maps;
  a.items = b->d_items;
  a.total_items = b->total_items;
  a.n_grids = (int)n;
  a.head = b->d_head;
  a.amps = b->d_amps;
  a.step = 0;
  a.nsteps = (int)steps;
  a.done = b->d_done;
  a.timeout_ns = 4000000000ull;
  a.status = b->d_status;
  k_batch<<<b->ctas, (kBTJ + 1) * 32, b->smem, b->stream>>>(a);
  B_CUDA(cudaGetLastError());
  return ST3D_OK;
}

void advance(st3d_batch* b, uint32_t steps) {
  for (st3d_ctx* c : b->ctx) {
    c->step += steps;
    c->launches += steps;
    if (steps & 1) {
      const int t = c->ub;
      c->ub = c->vb;
      c->vb = t;
    }
  }
}

}  // namespace

extern "C" {

int st3d_batch_create(uint32_t n, const st3d_grid_desc* grids, const st3d_opts* opts,
                      st3d_batch** out) {
  if (!out || !grids || !opts || n == 0) return bfail(ST3D_ERR_INVALID, "null argument or empty batch");
  *out = nullptr;
  for (uint32_t gi = 0; gi < n; ++gi) {
    const st3d_opts& o = opts[gi];
    if (o.mode != ST3D_MODE_WAVE || o.storage != ST3D_F32 || o.points == 2)
      return set_error(ST3D_ERR_UNSUPPORTED,
                       "batch grid %u: the batching form runs the FP32 wave update of 7/13/25 points", gi);
    if (o.device != opts[0].device)
      return set_error(ST3D_ERR_INVALID, "batch grid %u: every grid of a batch runs on one device", gi);
  }
  if (opts[0].device < -1) return bfail(ST3D_ERR_INVALID, "bad device ordinal");
  if (opts[0].device >= 0) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return bfail(ST3D_ERR_NODEVICE, "no CUDA device visible");
    }
    if (opts[0].device >= ndev) return bfail(ST3D_ERR_INVALID, "device ordinal out of range");
  }
  DeviceScope scope(opts[0].device);
  st3d_batch* b = new (std::nothrow) st3d_batch();
  if (!b) return bfail(ST3D_ERR_NOMEM, "host allocation failed");
  auto cleanup = [b](int rc) {
    st3d_batch_destroy(b);
    return rc;
  };
  cudaGetDevice(&b->device);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->amps_copied, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(bfail(ST3D_ERR_CUDA, "stream/event creation failed"));
  }
  int sm = 0, ccM = 0, ccm = 0;
  size_t total = 0;
  int rc = st3d_device_info(&sm, &ccM, &ccm, &total);
  if (rc != ST3D_OK) return cleanup(rc);
  b->grids.resize(n);
  std::vector<CUtensorMap> maps(5 * (size_t)n);
  for (uint32_t gi = 0; gi < n; ++gi) {
    st3d_opts o = opts[gi];
    o.kernel = ST3D_KERNEL_TMA;
    o.tile_j = 16;  // the single-grid plan, used by the sequential schedule
    o.stages = 4;
    o.temporal_block = 1;  // the batch steps one level at a time
    // Planes per unit of the batch kernel: 256 measured best on the 64-grid
    // batch (graph 350.4 against 341.6 Gpts/s with 64; pipelined 361.1
    // against 338.0): fewer units re-read fewer warm-up planes and the shared
    // queue still balances.  The grid's own context keeps the single-grid
    // planner's choice (opts.ichunk 0), which the sequential schedule runs.
    const int batch_ichunk = o.ichunk > 0 ? o.ichunk : 256;
    st3d_ctx* c = nullptr;
    rc = create_context(&grids[gi], &o, b->stream, &c);
    if (rc != ST3D_OK) return cleanup(rc);
    b->ctx.push_back(c);
    BatchGrid& G = b->grids[gi];
    memset(&G, 0, sizeof G);
    G.g = c->G;
    G.cf = c->cf32;
    G.buf[0] = (float*)c->fld[0];
    G.buf[1] = (float*)c->fld[1];
    G.P = o.points;
    G.R = c->R;
    // tile shape: the one that pads the (j, k) plane less (wide on a tie)
    const long long ys = grids[gi].ys, zs = grids[gi].zs;
    const long long wide = (ys + kBTJ - 1) / kBTJ * kBTJ * ((zs + kTmaTK - 1) / kTmaTK * kTmaTK);
    const long long thin = (ys + kNTJ - 1) / kNTJ * kNTJ * ((zs + kNTK - 1) / kNTK * kNTK);
    G.narrow = thin < wide ? 1 : 0;
    G.ichunk = batch_ichunk;
    const int tk = G.narrow ? kNTK : kTmaTK, tj = G.narrow ? kNTJ : kBTJ;
    G.ntk = (int)((zs + tk - 1) / tk);
    G.ntjk = (int)((ys + tj - 1) / tj) * G.ntk;
    G.units = G.ntjk * (int)((grids[gi].xs + G.ichunk - 1) / G.ichunk);
    G.src_i = c->opts.src_i;
    G.src_j = c->opts.src_j;
    G.src_k = c->opts.src_k;
    G.map_base = 5 * (int)gi;
    // the grid's maps in the batch's tile shape: u (halo box) over buffers 0
    // and 1, v (interior box) over 0 and 1, s
    for (int f = 0; f < 3 && rc == ST3D_OK; ++f) {
      if (f < 2)
        rc = encode_f32_box(&maps[5 * gi + f], c->fld[f], c->L, tk + 2 * kTmaKHalo, tj + 2 * c->R,
                            kTmaKHalo, c->L.pj);
      if (rc == ST3D_OK) rc = encode_f32_box(&maps[5 * gi + 2 + f], c->fld[f], c->L, tk, tj, 0, 0);
    }
    if (rc != ST3D_OK) return cleanup(rc);
    b->points += (uint64_t)grids[gi].xs * grids[gi].ys * grids[gi].zs;
  }
  // work items, the most expensive grids first (longest processing time
  // first keeps the tail short)
  std::vector<int> order(n);
  for (uint32_t gi = 0; gi < n; ++gi) order[gi] = (int)gi;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const double wx = (double)b->ctx[x]->grid.xs * b->ctx[x]->grid.ys * b->ctx[x]->grid.zs * (1 + b->grids[x].R);
    const double wy = (double)b->ctx[y]->grid.xs * b->ctx[y]->grid.ys * b->ctx[y]->grid.zs * (1 + b->grids[y].R);
    return wx > wy;
  });
  std::vector<int2> items;
  for (int gi : order)
    for (int u = 0; u < b->grids[gi].units; ++u) items.push_back(make_int2(gi, u));
  b->total_items = (int)items.size();
  b->smem = batch_smem_bytes();
  cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, (kBTJ + 1) * 32, b->smem) !=
          cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return cleanup(bfail(ST3D_ERR_UNSUPPORTED, "the batch kernel cannot be resident"));
  }
  b->ctas = std::min(sm * per_sm, b->total_items);
  if (cudaMalloc(&b->d_grids, n * sizeof(BatchGrid)) != cudaSuccess ||
      cudaMalloc(&b->d_maps, maps.size() * sizeof(CUtensorMap)) != cudaSuccess ||
      cudaMalloc(&b->d_items, items.size() * sizeof(int2)) != cudaSuccess ||
      cudaMalloc(&b->d_status, sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(bfail(ST3D_ERR_NOMEM, "cudaMalloc of the batch tables failed"));
  }
  cudaMemcpyAsync(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice,
                  b->stream);
  cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice,
                  b->stream);
  cudaMemsetAsync(b->d_status, 0, sizeof(uint32_t), b->stream);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess)
    return cleanup(bfail(ST3D_ERR_CUDA, "batch set-up failed"));
  *out = b;
  return ST3D_OK;
}

int st3d_batch_destroy(st3d_batch* b) {
  if (!b) return ST3D_OK;
  DeviceScope scope(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  destroy_graphs(b);
  for (st3d_ctx* c : b->ctx) st3d_destroy(c);
  if (b->d_grids) cudaFree(b->d_grids);
  if (b->d_maps) cudaFree(b->d_maps);
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_head) cudaFree(b->d_head);
  if (b->d_done) cudaFree(b->d_done);
  if (b->d_amps) cudaFree(b->d_amps);
  if (b->h_amps) cudaFreeHost(b->h_amps);
  if (b->d_status) cudaFree(b->d_status);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->amps_copied) cudaEventDestroy(b->amps_copied);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return ST3D_OK;
}

int st3d_batch_context(st3d_batch* b, uint32_t idx, st3d_ctx** ctx) {
  if (!b || !ctx || idx >= b->ctx.size()) return bfail(ST3D_ERR_INVALID, "bad batch index");
  *ctx = b->ctx[idx];
  return ST3D_OK;
}

int st3d_batch_get_info(const st3d_batch* b, st3d_batch_info* info) {
  if (!b || !info) return bfail(ST3D_ERR_INVALID, "null argument");
  memset(info, 0, sizeof *info);
  info->grids = (uint32_t)b->ctx.size();
  info->interior_points = b->points;
  info->work_items = (uint32_t)b->total_items;
  info->ctas = (uint32_t)b->ctas;
  info->launches = b->launches;
  info->graphs = (uint32_t)b->graphs.size();
  return ST3D_OK;
}

int st3d_batch_iterate(st3d_batch* b, uint32_t steps, int schedule) {
  if (!b) return bfail(ST3D_ERR_INVALID, "null batch");
  DeviceScope scope(b->device);
  if (steps == 0) return ST3D_OK;
  for (st3d_ctx* c : b->ctx)
    if (!(c->has_u && c->has_v && c->has_s))
      return bfail(ST3D_ERR_STATE, "upload or fill u, v and s of every grid before iterating");
  int rc;
  if (schedule == ST3D_BATCH_SEQUENTIAL) {
    for (uint32_t t = 0; t < steps; ++t)
      for (st3d_ctx* c : b->ctx)
        if ((rc = st3d_iterate(c, 1)) != ST3D_OK) return rc;
    b->launches += (uint64_t)steps * b->ctx.size();
    return ST3D_OK;
  }
  if (schedule != ST3D_BATCH_PERSISTENT && schedule != ST3D_BATCH_GRAPH &&
      schedule != ST3D_BATCH_PIPELINED)
    return bfail(ST3D_ERR_INVALID, "unknown batch schedule");
  if (schedule == ST3D_BATCH_PIPELINED && (uint64_t)steps * b->total_items > 0x7fffffffull)
    return bfail(ST3D_ERR_UNSUPPORTED, "too many steps for one pipelined launch (steps x items < 2^31)");
  if ((rc = ensure_steps(b, steps)) != ST3D_OK) return rc;
  if ((rc = stage_call(b, steps)) != ST3D_OK) return rc;
  if (schedule == ST3D_BATCH_PIPELINED) {
    if ((rc = enqueue_pipelined(b, steps)) != ST3D_OK) return rc;
    b->launches += 1;
    advance(b, steps);
    return ST3D_OK;
  }
  if (schedule == ST3D_BATCH_PERSISTENT) {
    if ((rc = enqueue_persistent(b, steps)) != ST3D_OK) return rc;
  } else {
    auto it = b->graphs.find(steps);
    if (it == b->graphs.end()) {
      cudaGraph_t graph;
      B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      rc = enqueue_persistent(b, steps);
      cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
      if (rc != ST3D_OK) return rc;
      if (e != cudaSuccess) return set_error(ST3D_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      cudaGraphExec_t exec;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return set_error(ST3D_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
      it = b->graphs.emplace(steps, exec).first;
    }
    B_CUDA(cudaGraphLaunch(it->second, b->stream));
  }
  b->launches += steps;
  advance(b, steps);
  return ST3D_OK;
}

int st3d_batch_synchronize(st3d_batch* b) {
  if (!b) return bfail(ST3D_ERR_INVALID, "null batch");
  DeviceScope scope(b->device);
  B_CUDA(cudaStreamSynchronize(b->stream));
  uint32_t st = 0;
  B_CUDA(cudaMemcpy(&st, b->d_status, sizeof st, cudaMemcpyDeviceToHost));
  if (st != kDevOk) {
    cudaMemset(b->d_status, 0, sizeof(uint32_t));
    return set_error(ST3D_ERR_TIMEOUT, "a bounded device wait in the batch kernel gave up (status %u)", st);
  }
  for (st3d_ctx* c : b->ctx) {
    int rc = st3d_synchronize(c);
    if (rc != ST3D_OK) return rc;
  }
  return ST3D_OK;
}

int st3d_batch_timer_start(st3d_batch* b) {
  if (!b) return bfail(ST3D_ERR_INVALID, "null batch");
  DeviceScope scope(b->device);
  B_CUDA(cudaEventRecord(b->ev0, b->stream));
  return ST3D_OK;
}

int st3d_batch_timer_stop(st3d_batch* b, float* ms) {
  if (!b || !ms) return bfail(ST3D_ERR_INVALID, "null argument");
  DeviceScope scope(b->device);
  B_CUDA(cudaEventRecord(b->ev1, b->stream));
  B_CUDA(cudaEventSynchronize(b->ev1));
  B_CUDA(cudaEventElapsedTime(ms, b->ev0, b->ev1));
  return ST3D_OK;
}

}  // extern "C"
