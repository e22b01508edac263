// st3d_ctx.h -- the context behind the C ABI's opaque st3d_ctx handle,
// shared by the single-grid entry points (st3d_api.cu) and the batch
// (st3d_batch.cu).
#pragma once

#include <vector>

#include "st3d_internal.h"
#include "st3d_tma.cuh"

struct st3d_ctx {
  using Layout = st3d::Layout;
  using Geom = st3d::Geom;
  using TmaPlan = st3d::TmaPlan;
  using Tma16Plan = st3d::Tma16Plan;
  using TbPlan = st3d::TbPlan;
  template <typename C>
  using Coefs = st3d::Coefs<C>;

  st3d_grid_desc grid;
  st3d_opts opts;
  int R = 0;
  int eb = 0;
  Layout L;
  Geom G;
  // [0],[1]: the u/v pair, [2]: s, [3],[4]: the second pair of a context
  // that blocks in time (a pass writes the other pair)
  void* fld[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int ub = 0, vb = 1;                          // buffers holding u and v
  TbPlan* tb = nullptr;
  double* scratch = nullptr;                   // norms partials + result
  unsigned long long* counter = nullptr;       // check()
  uint32_t* dev_status = nullptr;
  size_t scratch_doubles = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  uint64_t timer_step0 = 0;    // steps at the last timer start
  uint64_t timed_steps = 0;    // steps inside the last timer region
  float timed_ms = 0.0f;
  uint64_t step = 0;
  uint64_t launches = 0;
  int kernel = ST3D_KERNEL_SIMPLE;
  int ichunk = 64;
  bool has_u = false, has_v = false, has_s = false;
  int device = 0;
  TmaPlan* tma = nullptr;
  // 16-bit storage.  Compensated form: low bytes of the u/v buffers, scale
  // exponents E (time levels mod 3; s at 4*xs) and plane maxima M (time
  // levels mod 4; s at 4*xs).  Delta form (FP16 / BF16): u in buffers 0/1, d
  // = u^n - u^{n-1} in buffer 3; E and M hold u per buffer (0, 1), d per
  // level parity (2, 3) and s (4).  `lvl` counts the levels stepped (the
  // rotation of E and M; `step`, the source time, restarts at each upload);
  // the staging buffer holds two host arrays for the delta form, whose u/v
  // pair is valid until a step or another use of the slots.
  bool f16 = false;
  bool delta = false;
  bool pair = false;  // F16_HL: u is an FP16 hi/lo pair, lo[b] the lo words of buffer b
  bool pair_valid = false;
  uint64_t lvl = 0;
  float m2s = 0.0f;
  void* lo[2] = {nullptr, nullptr};
  int* E = nullptr;
  uint32_t* M = nullptr;
  uint32_t* halo_max = nullptr;
  Tma16Plan* tma16 = nullptr;
  float k4 = 0.0f;
  void* stage = nullptr;      // reference-layout staging buffer for host copies
  int host_path = 0;          // st3d_host_path of the last FP32/FP64 transfer
  size_t stage_bytes = 0;
  Coefs<float> cf32;
  Coefs<double> cf64;
  size_t bytes = 0;
  // the streamed drop-in call (st3d_stream.cu): its queues, counters and
  // amplitudes on the device, and their host copies (kept until the next call)
  void* stream_buf = nullptr;
  size_t stream_buf_bytes = 0;
  std::vector<unsigned char> stream_host;
};
