// st3d_stream.cu -- the drop-in ITERATE call with its host transfers and its
// time steps overlapped in one cooperative persistent launch.
//
// st3d_iterate_host replaces ITERATE(v, s, u, grid, ...) (iterators.h:6-29)
// on host arrays: upload v, s and u, take `iterations` steps, download v (and
// u in mode W).  Done one phase after the other the call is bound by the host
// link (GB300: ~211 GB/s host to device and ~194 device to host, measured
// alone) with the steps in between; the link carries both directions at once
// (343 GB/s together, measured), and each step of an i-plane only needs the
// previous step's planes within R of it.  So the streamed call cuts the grid
// into chunks of C planes along i and runs, in ONE launch:
//
//   - upload CTAs (the first `n_up` CTAs, all warps copying): a queue of
//     plane copies in chunk order -- every plane of u, v and s of chunk d
//     from the pinned host array into the device layout (the host array's
//     device view; halo planes with the first and last chunk), each counted
//     in the chunk's upload counter; once their queue is drained they join
//     the stencil queue;
//   - download CTAs (the next `n_down`): a queue of the final v (and u)
//     planes in chunk order, each copied out once the last step of its chunk
//     has finished (their waits never hold up an upload);
//   - stencil CTAs (the rest; the k_tma kernel's producer/consumer structure,
//     16-row x 128-point tiles, 4 stages): a queue of (step t, chunk c, tile)
//     items in wavefront order -- step t of chunk c is queued at stage
//     c + t + 1, after everything it depends on.  Before loading an item the
//     producer waits for its inputs: the upload of chunks c-1..c+1 (t = 0),
//     else every tile of step t-1 of chunks c-1..c+1 (mode W: step t reads
//     U^t of its halo planes and overwrites U^{t-1}, which step t-1 read with
//     its halo) or of chunk c alone (mode R: u and s are fixed, v is updated
//     in place without a halo).  A producer skips the check for the next
//     tile of the (step, chunk) whose inputs it saw complete.
//
// Every dependency is on an item earlier in its own queue or in the other
// queue's order, and the cooperative launch keeps all CTAs resident, so
// every wait ends.  Counters are published with release and read with
// acquire semantics (gpu scope); stencil producers fence the async proxy
// before their TMA loads.  The waits are bounded by the absence of progress:
// a wait gives up (device status word, call fails with ST3D_ERR_TIMEOUT) only
// after no tile and no plane copy finished anywhere for the timeout, so a
// long run of steps ahead of a download does not time out.
//
// The arithmetic of a step is the k_tma kernel's (st3d_kernels_tma.cu):
// the streamed call gives bit for bit the result of the phase-by-phase call.
// It applies to FP32 contexts on the TMA kernel's default tiles (16 rows, 4
// stages) without temporal blocking, when v, s and u are pinned host arrays
// (the direct host path) and the layouts allow the scatter kernels' path.
#include <cooperative_groups.h>

#include <vector>

#include "st3d_internal.h"
#include "st3d_p4.cuh"
#include "st3d_tma.cuh"

namespace st3d {

namespace {

constexpr int kSTJ = 16;  // stencil tile rows (consumer warps)
constexpr int kSNV = 4;   // pipeline stages
constexpr int kSlots = 2 * kSNV;  // item completion counters per CTA

enum XferKind : int { kUpload = 0, kDownload = 1 };

struct StreamArgs {
  Geom g;               // device layout
  RefGeom R;            // host (reference) layout
  Coefs<float> cf;
  float* fld[3];        // u/v pair and s
  const float* hin[3];  // device views of the host inputs: u, v, s
  float* hout[2];       // device views of the host outputs: u, v
  int ub0, vb0;         // buffers of u and v at the call's first step
  int steps, chunk, nchunks;
  int ntk, ntiles;      // tiles per plane along k, tiles per plane
  const int2* pairs;    // (step, chunk) in wavefront order
  int npairs;
  const int4* xfer;     // (kind, field, plane, chunk): uploads [0, nup), downloads [nup, nxfer)
  int nup, nxfer;
  const int* up_need;   // per chunk: plane copies to upload
  int* up_cnt;          // per chunk: plane copies uploaded
  int* st_cnt;          // per (step, chunk): tiles finished
  int* progress;        // tiles + plane copies finished (liveness of the waits)
  int* heads;           // [0] stencil queue, [1] upload queue, [2] download queue
  int n_up, n_down;     // upload and download CTAs
  int hx, hy, hz;       // halo widths moved
  int vec;              // rows move as float4 (16-byte aligned on both sides)
  int src_i, src_j, src_k;
  const float* amps;    // per step
  uint64_t timeout_ns;  // no-progress limit of a wait
  uint64_t cap_ns;      // limit of any wait
  uint32_t* status;
};

struct SStage {
  int t, c, tile, stop;
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned atom_add_acq_rel_cta(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], %2;"
               : "=r"(old)
               : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(p))), "r"(v)
               : "memory");
  return old;
}

__device__ __forceinline__ void proxy_fence_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Waits until *ctr >= target (acquire).  Gives up after `limit_ns` with no
// change of *progress (no tile and no plane copy finished anywhere), and in
// any case after `cap_ns` in all (the host's generous estimate of the whole
// call).
__device__ bool wait_live(const int* ctr, int target, const int* progress, uint64_t limit_ns,
                          uint64_t cap_ns) {
  if (ld_acquire(ctr) >= target) return true;
  int seen = ld_acquire(progress);
  const uint64_t start = global_ns();
  uint64_t t0 = start;
  for (uint32_t it = 1; it < (1u << 30); ++it) {
    __nanosleep(it < 64 ? 32 : 256);
    if (ld_acquire(ctr) >= target) return true;
    if ((it & 15u) == 0) {
      const int now = ld_acquire(progress);
      const uint64_t t = global_ns();
      if (now != seen) {
        seen = now;
        t0 = t;
      } else if (t - t0 > limit_ns) {
        return false;
      }
      if (t - start > cap_ns) return false;
    }
  }
  return false;
}

// One plane of one field between the host layout and the device layout:
// rows j in [j0, j1), points k in [-hz, zs + hz).  All threads of the CTA.
__device__ void copy_plane(const StreamArgs& a, bool up, int f, int i, float* dev, const float* hsrc,
                           float* hdst) {
  const Geom& g = a.g;
  const RefGeom& R = a.R;
  const int j0 = up ? -a.hy : 0, j1 = up ? R.ys + a.hy : R.ys;
  const int klen = R.zs + 2 * a.hz;
  const long long dplane = (long long)(i + g.pi) * g.si;
  const long long hplane = R.ijk_ofs + (long long)i * R.imult;
  if (a.vec) {
    const int k4 = klen / 4;  // a multiple of 4 points when vec is set
    const long long n = (long long)(j1 - j0) * k4;
    for (long long x = threadIdx.x; x < n; x += 4 * (long long)blockDim.x) {
      float4 buf[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const long long y = x + m * (long long)blockDim.x;
        if (y < n) {
          const int j = j0 + (int)(y / k4);
          const int kq = (int)(y - (long long)(j - j0) * k4);
          const long long hrow = hplane + (long long)j * R.jmult - a.hz + 4 * kq;
          const long long drow = dplane + (long long)(j + g.pj) * g.sj + g.pk - a.hz + 4 * kq;
          buf[m] = up ? *reinterpret_cast<const float4*>(hsrc + hrow)
                      : __ldcg(reinterpret_cast<const float4*>(dev + drow));
        }
      }
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const long long y = x + m * (long long)blockDim.x;
        if (y < n) {
          const int j = j0 + (int)(y / k4);
          const int kq = (int)(y - (long long)(j - j0) * k4);
          const long long hrow = hplane + (long long)j * R.jmult - a.hz + 4 * kq;
          const long long drow = dplane + (long long)(j + g.pj) * g.sj + g.pk - a.hz + 4 * kq;
          if (up)
            *reinterpret_cast<float4*>(dev + drow) = buf[m];
          else
            *reinterpret_cast<float4*>(hdst + hrow) = buf[m];
        }
      }
    }
  } else {
    const long long n = (long long)(j1 - j0) * klen;
    for (long long x = threadIdx.x; x < n; x += 8 * (long long)blockDim.x) {
      float buf[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const long long y = x + m * (long long)blockDim.x;
        if (y < n) {
          const int j = j0 + (int)(y / klen);
          const int kk = (int)(y - (long long)(j - j0) * klen);
          const long long hrow = hplane + (long long)j * R.jmult - a.hz + kk;
          const long long drow = dplane + (long long)(j + g.pj) * g.sj + g.pk - a.hz + kk;
          buf[m] = up ? hsrc[hrow] : __ldcg(dev + drow);
        }
      }
#pragma unroll
      for (int m = 0; m < 8; ++m) {
        const long long y = x + m * (long long)blockDim.x;
        if (y < n) {
          const int j = j0 + (int)(y / klen);
          const int kk = (int)(y - (long long)(j - j0) * klen);
          const long long hrow = hplane + (long long)j * R.jmult - a.hz + kk;
          const long long drow = dplane + (long long)(j + g.pj) * g.sj + g.pk - a.hz + kk;
          if (up)
            dev[drow] = buf[m];
          else
            hdst[hrow] = buf[m];
        }
      }
    }
  }
  (void)f;
}

template <int P, int MODE>
__global__ void __launch_bounds__((kSTJ + 1) * 32, 1)
    k_stream(const __grid_constant__ CUtensorMap um0, const __grid_constant__ CUtensorMap um1,
             const __grid_constant__ CUtensorMap vm0, const __grid_constant__ CUtensorMap vm1,
             const __grid_constant__ CUtensorMap smap, const StreamArgs a) {
  constexpr int R = (P == 25) ? 4 : (P == 13) ? 2 : 1;
  constexpr int QN = 2 * R + 1;
  constexpr int NV = kSNV;
  constexpr int TJ = kSTJ;
  constexpr int NU = NV + R;
  constexpr int NP = npairs_of(P);
  constexpr int TK = kTmaTK;
  constexpr int UKW = kTmaUKW;
  constexpr int USLOT = (UKW * (TJ + 2 * R) + 31) / 32 * 32;
  constexpr int VSLOT = TK * TJ;
  constexpr uint32_t UBYTES = UKW * (TJ + 2 * R) * 4;
  constexpr uint32_t VBYTES = VSLOT * 4;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  const Geom& g = a.g;
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  float* ur = reinterpret_cast<float*>(smem_raw);
  float* vr = ur + NU * USLOT;
  float* sr = vr + NV * VSLOT;
  uint64_t* full = reinterpret_cast<uint64_t*>(sr + NV * VSLOT);
  uint64_t* empty = full + NV;
  SStage* info = reinterpret_cast<SStage*>(empty + NV);
  unsigned* finished = reinterpret_cast<unsigned*>(info + NV);
  if (threadIdx.x == 0) {
    for (int q = 0; q < kSlots; ++q) finished[q] = 0u;
    for (int s = 0; s < NV; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TJ);
    }
    fence_barrier_init();
    fence_proxy_async_smem();
  }
  __syncthreads();

  if ((int)blockIdx.x < a.n_up + a.n_down) {
    // ---------------- transfer CTA ----------------
    int* s_item = reinterpret_cast<int*>(smem_raw);  // kind, field, plane, chunk, stop
    const int last_step = a.steps - 1;
    const bool up = (int)blockIdx.x < a.n_up;
    int* head = a.heads + (up ? 1 : 2);
    const int first = up ? 0 : a.nup, end = up ? a.nup : a.nxfer;
    while (true) {
      if (threadIdx.x == 0) {
        const int x = first + atomicAdd(head, 1);
        int stop = x >= end;
        int4 it = make_int4(0, 0, 0, 0);
        if (!stop) {
          it = a.xfer[x];
          if (it.x == kDownload &&
              !wait_live(a.st_cnt + (size_t)last_step * a.nchunks + it.w, a.ntiles, a.progress,
                         a.timeout_ns, a.cap_ns)) {
            atomicExch(a.status, (uint32_t)kDevTimeoutDep);
            stop = 2;
          }
        }
        s_item[0] = it.x;
        s_item[1] = it.y;
        s_item[2] = it.z;
        s_item[3] = it.w;
        s_item[4] = stop;
      }
      __syncthreads();
      const int kind = s_item[0], f = s_item[1], plane = s_item[2], chunk = s_item[3];
      if (s_item[4]) break;
      if (kind == kUpload) {
        // u, v, s of the call's first step
        const int buf = f == 0 ? a.ub0 : f == 1 ? a.vb0 : 2;
        copy_plane(a, true, f, plane, a.fld[buf], a.hin[f], nullptr);
      } else {
        // final u (f = 0) and v (f = 1): mode W swaps the pair every step
        const int flip = (MODE == ST3D_MODE_WAVE) ? (a.steps & 1) : 0;
        const int buf = (f == 0 ? a.ub0 : a.vb0) ^ flip;
        copy_plane(a, false, f, plane, a.fld[buf], nullptr, a.hout[f]);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        proxy_fence_global();
        if (kind == kUpload) red_release_add(a.up_cnt + chunk, 1);
        red_release_add(a.progress, 1);
      }
      // s_item is rewritten only after the next loop's first barrier
      __syncthreads();
    }
    // An upload CTA whose queue is drained joins the stencil queue (the
    // steps are what is left to do); s_item, which lies in the u ring, is no
    // longer read once every thread has passed this barrier.
    __syncthreads();
    if (!up || s_item[4] == 2) return;
    __syncthreads();
  }

  // ---------------- stencil CTA ----------------
  const int total = a.npairs * a.ntiles;
  if (warp == TJ) {
    // ---------------- producer ----------------
    if (lane != 0) return;
    tma_prefetch_desc(&um0);
    tma_prefetch_desc(&um1);
    tma_prefetch_desc(&vm0);
    tma_prefetch_desc(&vm1);
    tma_prefetch_desc(&smap);
    uint32_t h = 0;
    bool ok = true;
    int dep_t = -1, dep_c = -1;  // the (step, chunk) whose inputs were seen complete
    while (ok) {
      const int x = atomicAdd(&a.heads[0], 1);
      if (x >= total) {
        const int stage0 = (int)(h % NV);
        if (h >= (uint32_t)NV &&
            !mbar_wait_bounded(&empty[stage0], ((h / NV) - 1) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          break;
        }
        info[stage0].stop = 1;
        mbar_arrive(&full[stage0]);
        break;
      }
      const int pi = x / a.ntiles;
      const int tile = x - pi * a.ntiles;
      const int2 tc = a.pairs[pi];
      const int t = tc.x, c = tc.y;
      const bool wave = MODE == ST3D_MODE_WAVE;
      if (t != dep_t || c != dep_c) {
        // inputs of step t of chunk c: one pass of loads, then waits on the
        // counters not yet complete; consecutive tiles of one (step, chunk)
        // skip it
        const int* ctr[3];
        int target[3];
        bool done[3];
        for (int q = 0; q < 3; ++q) {
          const int cc = c - 1 + q;
          ctr[q] = nullptr;
          if (cc < 0 || cc >= a.nchunks) continue;
          if (t == 0) {
            ctr[q] = a.up_cnt + cc;
            target[q] = a.up_need[cc];
          } else if (wave || cc == c) {
            ctr[q] = a.st_cnt + (size_t)(t - 1) * a.nchunks + cc;
            target[q] = a.ntiles;
          }
        }
        for (int q = 0; q < 3; ++q) done[q] = !ctr[q] || ld_acquire(ctr[q]) >= target[q];
        for (int q = 0; q < 3 && ok; ++q)
          if (!done[q]) ok = wait_live(ctr[q], target[q], a.progress, a.timeout_ns, a.cap_ns);
        if (!ok) {
          atomicExch(a.status, (uint32_t)kDevTimeoutDep);
          break;
        }
        dep_t = t;
        dep_c = c;
      }
      proxy_fence_global();
      const int ub = wave ? (a.ub0 ^ (t & 1)) : a.ub0;
      const int vb = wave ? (ub ^ 1) : a.vb0;
      const CUtensorMap* um = ub ? &um1 : &um0;
      const CUtensorMap* vm = vb ? &vm1 : &vm0;
      const int jt = tile / a.ntk;
      const int kt = tile - jt * a.ntk;
      const int k0 = kt * TK, j0 = jt * TJ;
      const int ia = c * a.chunk;
      const int ib = min(ia + a.chunk, g.xs);
      const int nsteps = (ib - ia) + 2 * R;
      // the first R planes of the unit enter the consumers' queues by direct
      // loads: no pipeline step for them
      for (int n = R; n < nsteps; ++n, ++h) {
        const int stage = (int)(h % NV);
        if (h >= (uint32_t)NV &&
            !mbar_wait_bounded(&empty[stage], ((h / NV) - 1) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutEmpty);
          ok = false;
          break;
        }
        info[stage] = {t, c, tile, 0};
        const bool has_vs = n >= 2 * R;
        mbar_arrive_expect_tx(&full[stage], UBYTES + (has_vs ? 2 * VBYTES : 0u));
        tma_load_3d(ur + (h % NU) * USLOT, um, &full[stage], g.pk + k0 - kTmaKHalo, g.pj + j0 - R,
                    g.pi + ia - R + n);
        if (has_vs) {
          const int i = ia + n - 2 * R;
          tma_load_3d(vr + stage * VSLOT, vm, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
          tma_load_3d(sr + stage * VSLOT, &smap, &full[stage], g.pk + k0, g.pj + j0, g.pi + i);
        }
      }
    }
    // leave no copy in flight: wait until the last stages were consumed
    for (uint32_t m = (h > (uint32_t)NV ? h - NV : 0u); m < h; ++m)
      (void)mbar_wait_bounded(&empty[m % NV], (m / NV) & 1u, a.timeout_ns);
    return;
  }

  // ---------------- consumers (the k_tma step, one item at a time) --------
  const int r = warp;
  uint32_t h = 0;
  uint32_t seq = 0;
  float4 q[QN];
  while (true) {
    const int stage0 = (int)(h % NV);
    if (!mbar_wait_bounded(&full[stage0], (h / NV) & 1u, a.timeout_ns)) {
      atomicExch(a.status, (uint32_t)kDevTimeoutFull);
      return;
    }
    const SStage st = info[stage0];
    if (st.stop) return;
    const int t = st.t, c = st.c;
    const int jt = st.tile / a.ntk;
    const int kt = st.tile - jt * a.ntk;
    const int j = jt * TJ + r;
    const int k = kt * TK + 4 * lane;
    const int ia = c * a.chunk;
    const int ib = min(ia + a.chunk, g.xs);
    const int nsteps = (ib - ia) + 2 * R;
    const bool row_ok = j < g.ys;
    const int ub = (MODE == ST3D_MODE_WAVE) ? (a.ub0 ^ (t & 1)) : a.ub0;
    const int vb = (MODE == ST3D_MODE_WAVE) ? (ub ^ 1) : a.vb0;
    float* vrow = a.fld[vb] + g.org + (long long)j * g.sj + k;
    const float amp = a.amps ? a.amps[t] : 0.0f;
    bool ok = true;
    for (int n0 = 0; n0 < nsteps && ok; n0 += QN) {
#pragma unroll
      for (int ph = 0; ph < QN; ++ph) {
        const int n = n0 + ph;
        if (n >= nsteps) break;
        if (n < R) {
          // a queue plane below the unit (u plane ia - R + n): read straight
          // from the field, after the item's first stage completed (its
          // inputs are then visible); where the TMA tile would be out of the
          // tensor map's extent (rows >= ys + 4, columns >= zs + 4) it is zero
          const int p = ia - R + n;
          const float* src = a.fld[ub] + g.org + (long long)p * g.si + (long long)j * g.sj + k;
          float4 x4 = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j < g.ys + 4) {
            if (k + 3 < g.zs + 4) {
              x4 = __ldcg(reinterpret_cast<const float4*>(src));
            } else {
              if (k < g.zs + 4) x4.x = __ldcg(src);
              if (k + 1 < g.zs + 4) x4.y = __ldcg(src + 1);
              if (k + 2 < g.zs + 4) x4.z = __ldcg(src + 2);
            }
          }
          q[ph] = x4;
          continue;
        }
        const uint32_t hh = h + (uint32_t)(n - R);
        const int stage = (int)(hh % NV);
        if (!mbar_wait_bounded(&full[stage], (hh / NV) & 1u, a.timeout_ns)) {
          atomicExch(a.status, (uint32_t)kDevTimeoutFull);
          ok = false;
          break;
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
              acc = fma4(splat(a.cf.cf[p]), sum, p == 0 ? mul4(cu, splat(a.cf.coef0)) : acc);
            } else {
              const P4 d = add4(sum, nu2);
              acc = p == 0 ? mul4(d, splat(a.cf.cf[0])) : fma4(splat(a.cf.cf[p]), d, acc);
            }
          }
          const float4 v4 = *reinterpret_cast<const float4*>(vr + stage * VSLOT + r * TK + 4 * lane);
          const float4 s4 = *reinterpret_cast<const float4*>(sr + stage * VSLOT + r * TK + 4 * lane);
          const P4 vv = {make_float2(v4.x, v4.y), make_float2(v4.z, v4.w)};
          P4 ss = {make_float2(s4.x, s4.y), make_float2(s4.z, s4.w)};
          P4 xo;
          if (MODE == ST3D_MODE_REF) {
            const P4 tq = fma4(splat(-a.cf.K), cu, vv);
            xo = {__ffma2_rn(ss.a, acc.a, tq.a), __ffma2_rn(ss.b, acc.b, tq.b)};
          } else {
            if (i == a.src_i && j == a.src_j && (unsigned)(a.src_k - k) < 4u) {
              const int cc = a.src_k - k;
              if (cc == 0) ss.a.x = ss.a.x + amp;
              if (cc == 1) ss.a.y = ss.a.y + amp;
              if (cc == 2) ss.b.x = ss.b.x + amp;
              if (cc == 3) ss.b.y = ss.b.y + amp;
            }
            P4 tq = add4(u2, {make_float2(-vv.a.x, -vv.a.y), make_float2(-vv.b.x, -vv.b.y)});
            tq = fma4(splat(a.cf.c1), acc, tq);
            xo = fma4(splat(a.cf.c2), ss, tq);
          }
          const float o[4] = {xo.a.x, xo.a.y, xo.b.x, xo.b.y};
          if (row_ok) {
            float* dst = vrow + (long long)i * g.si;
            if (k + 3 < g.zs) {
              *reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
            } else {
#pragma unroll
              for (int m = 0; m < 4; ++m)
                if (k + m < g.zs) dst[m] = o[m];
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[stage]);
      }
    }
    if (!ok) return;
    // the tile is stored by this warp; the CTA's last warp to finish it
    // publishes it (a warp runs at most NV stages, so at most NV items,
    // ahead of the slowest: 2 NV counters never mix two items)
    // (The warp's stores are ordered before lane 0's release on the CTA
    // counter by __syncwarp; the last warp's acquire on it orders every
    // warp's stores before its gpu-scope release, which is cumulative.)
    __syncwarp();
    if (lane == 0) {
      unsigned* slot = finished + (seq % kSlots);
      const unsigned old = atom_add_acq_rel_cta(slot, 1u);
      if (old == TJ - 1) {
        atomicExch(slot, 0u);
        proxy_fence_global();
        red_release_add(a.st_cnt + (size_t)t * a.nchunks + c, 1);
        red_release_add(a.progress, 1);
      }
    }
    ++seq;
    h += (uint32_t)(nsteps - R);
  }
}

size_t stream_smem_bytes(int R) {
  const size_t uslot = ((size_t)kTmaUKW * (kSTJ + 2 * R) + 31) / 32 * 32 * 4;
  const size_t vslot = (size_t)kTmaTK * kSTJ * 4;
  return (size_t)(kSNV + R) * uslot + 2 * (size_t)kSNV * vslot + 2 * kSNV * 8 +
         kSNV * sizeof(SStage) + kSlots * sizeof(unsigned) + 128;
}

template <int P, int MODE>
cudaError_t launch_pm(const CUtensorMap* maps, const StreamArgs& a, int grid, size_t smem,
                      cudaStream_t stream, int* occ) {
  auto kern = k_stream<P, MODE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, (kSTJ + 1) * 32, smem);
  void* args[] = {(void*)&maps[0], (void*)&maps[1], (void*)&maps[2], (void*)&maps[3], (void*)&maps[4],
                  (void*)&a};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3((kSTJ + 1) * 32), args, smem,
                                     stream);
}

cudaError_t dispatch_stream(int points, int mode, const CUtensorMap* maps, const StreamArgs& a,
                            int grid, size_t smem, cudaStream_t stream, int* occ) {
  const bool w = mode == ST3D_MODE_WAVE;
  switch (points) {
    case 7: return w ? launch_pm<7, ST3D_MODE_WAVE>(maps, a, grid, smem, stream, occ)
                     : launch_pm<7, ST3D_MODE_REF>(maps, a, grid, smem, stream, occ);
    case 13: return w ? launch_pm<13, ST3D_MODE_WAVE>(maps, a, grid, smem, stream, occ)
                      : launch_pm<13, ST3D_MODE_REF>(maps, a, grid, smem, stream, occ);
    case 25: return w ? launch_pm<25, ST3D_MODE_WAVE>(maps, a, grid, smem, stream, occ)
                      : launch_pm<25, ST3D_MODE_REF>(maps, a, grid, smem, stream, occ);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

int stream_blocks_per_sm(int points, int mode) {
  StreamArgs a;
  CUtensorMap maps[5];
  int occ = 0;
  if (dispatch_stream(points, mode, maps, a, 1, stream_smem_bytes(radius_of(points)), nullptr, &occ) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return occ;
}

cudaError_t launch_stream(int points, int mode, const StreamPlan& p, const CUtensorMap* maps,
                          const StreamLaunch& L, cudaStream_t stream) {
  StreamArgs a;
  a.g = L.g;
  a.R = L.R;
  a.cf = L.cf;
  for (int f = 0; f < 3; ++f) {
    a.fld[f] = L.fld[f];
    a.hin[f] = L.hin[f];
  }
  a.hout[0] = L.hout[0];
  a.hout[1] = L.hout[1];
  a.ub0 = L.ub0;
  a.vb0 = L.vb0;
  a.steps = L.steps;
  a.chunk = p.chunk;
  a.nchunks = p.nchunks;
  a.ntk = p.ntk;
  a.ntiles = p.ntiles;
  a.pairs = L.pairs;
  a.npairs = L.steps * p.nchunks;
  a.xfer = L.xfer;
  a.nup = L.nup;
  a.nxfer = L.nxfer;
  a.up_need = L.up_need;
  a.up_cnt = L.up_cnt;
  a.st_cnt = L.st_cnt;
  a.progress = L.progress;
  a.heads = L.heads;
  a.n_up = p.n_up;
  a.n_down = p.n_down;
  a.hx = L.hx;
  a.hy = L.hy;
  a.hz = L.hz;
  a.vec = L.vec;
  a.src_i = L.src_i;
  a.src_j = L.src_j;
  a.src_k = L.src_k;
  a.amps = L.amps;
  a.timeout_ns = L.timeout_ns;
  a.cap_ns = L.cap_ns;
  a.status = L.status;
  return dispatch_stream(points, mode, maps, a, p.grid, stream_smem_bytes(radius_of(points)), stream,
                         nullptr);
}

}  // namespace st3d
