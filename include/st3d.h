/*
 * st3d.h -- C ABI of the GB300 stencil3d library (libst3d.so).
 *
 * The library replaces the reference's host-CPU hot path: the time loop and
 * traversal of iterators.cpp (ITERATE, iterators.h:6-29, selected by the
 * ITERATE macro of config.h:55-65) and the per-point updates of
 * stencil_{2,7,13,25}.h, on one GB300 GPU.  Every function returns an int
 * status (ST3D_OK = 0); the reference itself returns no errors and exits on
 * bad input (aux.cpp:16-69), so each entry point names the reference call it
 * replaces and the checks it adds.
 *
 * Host arrays passed to the library use the reference layout
 * (grid.cpp:20-24, stencils.h:5):
 *     IDX(i,j,k) = ijk_ofs + k + j*jmult + i*imult,
 *     jmult = zs + 2*zh, imult = jmult*(ys + 2*yh),
 *     ijk_ofs = zh + yh*jmult + xh*imult,
 * i the slowest (x) axis and k the contiguous (z) axis.  `real` is float for
 * the F32, F16, BF16 and F16_HILO storages and double for F64
 * (config.h:96-100).  The library keeps its own device layout and converts
 * at upload and download.
 *
 * Plain pointers and sizes only: no C++ or framework types cross this ABI.
 * One context per host thread; contexts share no mutable state.
 */
#ifndef ST3D_H
#define ST3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ST3D_ABI_VERSION 2

typedef enum st3d_status {
  ST3D_OK = 0,
  ST3D_ERR_INVALID = 1,     /* bad argument: size, halo, pointer, option */
  ST3D_ERR_UNSUPPORTED = 2, /* well-formed request this library does not implement */
  ST3D_ERR_CUDA = 3,        /* a CUDA runtime or driver call failed */
  ST3D_ERR_NOMEM = 4,       /* device or pinned host allocation failed */
  ST3D_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  ST3D_ERR_STATE = 6,       /* call out of order, e.g. iterate before upload */
  ST3D_ERR_NODEVICE = 7     /* no CUDA device of compute capability 10.3 */
} st3d_status;

/* Update modes. */
typedef enum st3d_mode {
  /* The update the reference code computes (stencil_7.h:31-39,
   * stencil_13.h:50-61, stencil_25.h:75-95, stencil_2.h:20-29):
   *   v <- v - K*u + s*(coef0*u + sum c_{axis,r}*(u[-r] + u[+r]))
   * (2 points: v <- coef0*(u + u[k+1])), u and s fixed between steps. */
  ST3D_MODE_REF = 0,
  /* Leapfrog acoustic wave (README.md:11-20):
   *   v <- c0*u - v + c1*sum w_{axis,r}*(u[-r] + u[+r]) + c2*(s + a_n*delta_src)
   * then u and v swap roles.  a_n is a Ricker wavelet at step n.  With
   * c0 = 2 - 2*c1*sum(w) it is evaluated as (2u - v) + c1*sum w*((u[-r] +
   * u[+r]) - 2u) + c2*s, which keeps constant fields exact in any precision
   * (the literal form lets FP32 drift ~5e-3 from FP64 in 1000 steps). */
  ST3D_MODE_WAVE = 1
} st3d_mode;

typedef enum st3d_storage {
  ST3D_F32 = 0,      /* float fields, float arithmetic */
  ST3D_F64 = 1,      /* double fields, double arithmetic (config.h:96-97) */
  /* Mode W only, zero halos.  F16 / BF16 hold u and the time difference
   * d = u^n - u^{n-1} (not u^{n-1}) as 16-bit words with a power-of-two scale
   * per i-plane, so the leapfrog velocity keeps 11 (8) significant bits;
   * float arithmetic; 10 bytes per point per step.  Uploads and downloads
   * still exchange u and v (v = u - d on the way out). */
  ST3D_F16 = 2,
  ST3D_BF16 = 3,
  /* u and v as FP16 words with a per-plane scale plus a signed byte per point
   * holding the rounding residual (~19 significant bits); 11 bytes per point
   * per step. */
  ST3D_F16_HILO = 4,
  /* The delta form with u as an FP16 hi/lo pair: u = (hi + lo) * 2^E with
   * lo = fp16(u * 2^-E - hi) (~22 significant bits), d one FP16 word; the
   * stencil's neighbours are the hi words, the centre u the whole pair;
   * 14 bytes per point per step. */
  ST3D_F16_HL = 5
} st3d_storage;

typedef enum st3d_kernel {
  ST3D_KERNEL_AUTO = 0,   /* the fastest kernel for the request */
  ST3D_KERNEL_SIMPLE = 1, /* direct-load 2.5D streaming kernel (all storages) */
  ST3D_KERNEL_TMA = 2,    /* TMA-staged 2.5D streaming kernel (F32 and the 16-bit storages) */
  /* The 16-bit delta forms (F16, BF16, F16_HL) with the j and k neighbour
   * sums as band-matrix products on the tensor cores (FP32 accumulation):
   * the same update, within FP32 rounding of the sum per step, not bit for
   * bit the TMA kernel's result. */
  ST3D_KERNEL_MMA = 3
} st3d_kernel;

typedef enum st3d_field {
  ST3D_FIELD_U = 0,
  ST3D_FIELD_V = 1,
  ST3D_FIELD_S = 2
} st3d_field;

typedef enum st3d_fill_kind {
  ST3D_FILL_CONST = 0,   /* every point, halos included: value a */
  ST3D_FILL_UNIFORM = 1, /* every point, halos included: uniform [a, b) from the seeded counter hash */
  ST3D_FILL_BLOBS = 2    /* interior: sum of (int)a Gaussian blobs of width b (seeded), halos 0 */
} st3d_fill_kind;

/* Grid geometry: the --xs/--ys/--zs/--xh/--yh/--zh values of main.cpp:125-144
 * (s_grid xsize/ysize/zsize, xhalo/yhalo/zhalo, grid.h:39-41). */
typedef struct st3d_grid_desc {
  uint32_t xs, ys, zs; /* interior points along i (x), j (y), k (z) */
  uint32_t xh, yh, zh; /* halo widths of the caller's host arrays; each >= the stencil radius */
} st3d_grid_desc;

/* How FP32/FP64 host arrays reach the device.  STAGED: one contiguous copy
 * into a device staging buffer, then a scatter kernel (a download: a gather
 * kernel, then one 2-D copy).  DIRECT: the scatter/gather kernels read and
 * write the host array itself over the host link; it applies to pinned host
 * arrays (cudaMallocHost, cudaHostAlloc, cudaHostRegister, st3d_host_alloc)
 * that lie inside one allocation.  AUTO takes DIRECT where it applies.
 * STRIDED: a 3-D strided copy, used when the host k halo exceeds the device
 * row pad.  STREAMED (st3d_iterate_host only): the DIRECT path with the
 * transfers and the steps overlapped in one launch -- CTAs copying planes of
 * u, v and s in while the others step the planes already in, as a wavefront
 * over chunks of `ichunk` planes along i (16 when 0), and copying the final
 * planes out as they are done; the same bits as the phase-by-phase call.
 * AUTO takes it for FP32 contexts on the TMA kernel's default tiles without
 * temporal blocking when v, s and u are pinned (asking for STREAMED where it
 * does not apply runs DIRECT). */
typedef enum st3d_host_path {
  ST3D_HOST_AUTO = 0,
  ST3D_HOST_STAGED = 1,
  ST3D_HOST_DIRECT = 2,
  ST3D_HOST_STRIDED = 3,
  ST3D_HOST_STREAMED = 4
} st3d_host_path;

typedef struct st3d_opts {
  int32_t points;   /* 2, 7, 13 or 25 (config.h:35-38 STENCIL_SIZE) */
  int32_t mode;     /* st3d_mode */
  int32_t storage;  /* st3d_storage */
  int32_t kernel;   /* st3d_kernel */
  /* coef[0] = coef0 (2 points: the 0.5 factor), coef[1] = K,
   * coef[2..5] = cx1..cx4, coef[6..9] = cy1..cy4, coef[10..13] = cz1..cz4.
   * Mode W uses coef[2..13] as the neighbour weights w. */
  double coef[14];
  double c0, c1, c2;                 /* mode W constants */
  int32_t src_i, src_j, src_k;       /* mode W point source (interior coordinates); src_i < 0: none */
  int32_t pad0;
  double src_f, src_t0, dt;          /* Ricker peak frequency [Hz], delay [s], time step [s] */
  int32_t temporal_block;            /* mode W steps fused per pass: 1, 2 or 4 */
  int32_t tile_j, tile_k;            /* CTA tile; 0 = automatic */
  int32_t ichunk;                    /* planes per work unit along i; 0 = automatic */
  int32_t stages;                    /* pipeline stages of the TMA kernels; 0 = automatic */
  int32_t host_path;                 /* st3d_host_path of FP32/FP64 uploads and downloads */
  /* CUDA device ordinal the context runs on (one replica per GPU); -1, the
   * st3d_default_opts value, takes the calling thread's current device.  Every
   * entry point of the context makes it current for the call and restores the
   * caller's device afterwards. */
  int32_t device;
  int32_t reserved[5];
} st3d_opts;

typedef struct st3d_info {
  uint64_t interior_points;   /* xs*ys*zs */
  uint64_t device_bytes;      /* device memory held by the context */
  uint64_t step;              /* steps taken since the last upload (mode W source clock) */
  uint64_t launches;          /* kernel launches issued by st3d_iterate so far */
  uint32_t nk, nj, ni;        /* device row pitch (elements), rows per plane, planes */
  uint32_t pk, pj, pi;        /* device front pads (elements, rows, planes) */
  int32_t kernel;             /* st3d_kernel actually used */
  int32_t radius;             /* stencil radius */
  double bytes_per_point;     /* algorithmic HBM bytes per point per step */
  double flops_per_point;     /* reference FLOPS_PER_STENCIL (config.h:67-91) */
  int32_t tile_j, tile_k, ichunk, temporal_block;
  int32_t host_path;          /* st3d_host_path of the last upload or download */
  int32_t tb_tile_j;          /* rows of a temporally blocked pass's level-1 tile; 0 = none */
  int32_t device;             /* CUDA device ordinal of the context (st3d_plan: opts.device) */
  int32_t reserved[5];
} st3d_info;

typedef struct st3d_ctx st3d_ctx;

/* ---- library ----------------------------------------------------------- */
int st3d_abi_version(void);
const char* st3d_status_string(int status);
/* Detail of the last failure on the calling thread ("" if none). */
const char* st3d_last_error(void);
/* Current device: SM count, compute capability, total memory. */
int st3d_device_info(int* sm_count, int* cc_major, int* cc_minor, size_t* total_bytes);

/* Defaults: the reference's CONSTANTS_* for `points` (stencil_*.h; for mode R
 * with F64 storage the double products of config.h's real=double build), mode W
 * weights 1 for 7 points (README.md:11-20) and stencil_*.h cx/cy/cz for 13 and
 * 25, c = 1500 m/s, dx = 10 m, dt = 1 ms, 15 Hz Ricker with t0 = 1/f at the
 * grid centre (set at st3d_create when src_i = -2). */
int st3d_default_opts(int points, int mode, int storage, st3d_opts* opts);
/* Mode W constants from physics: c1 = (vel*dt/dx)^2, c2 = dt^2,
 * c0 = 2 - 2*c1*sum(w) (README.md:11-14 for w = 1). */
int st3d_set_wave_physics(st3d_opts* opts, double vel, double dt, double dx);

/* Validate a request and compute its device layout without touching a GPU:
 * the same checks st3d_create makes before it allocates.  info->kernel is
 * the kernel st3d_create would pick on a GB300 (the TMA kernel serves FP32
 * with 7/13/25 points). */
int st3d_plan(const st3d_grid_desc* grid, const st3d_opts* opts, st3d_info* info);

/* ---- context: replaces ITERATE's implicit state ------------------------ */
/* Replaces s_grid construction (grid.cpp:9-48, main.cpp:201) and the field
 * allocation of main.cpp:246-275: allocates the device fields of `grid`. */
int st3d_create(const st3d_grid_desc* grid, const st3d_opts* opts, st3d_ctx** ctx);
int st3d_destroy(st3d_ctx* ctx);
int st3d_get_info(const st3d_ctx* ctx, st3d_info* info);
/* The context's CUDA stream (a cudaStream_t), for callers that order work. */
int st3d_get_stream(const st3d_ctx* ctx, void** stream);
/* Set the mode W source clock (the step index the next step's Ricker
 * amplitude is taken at; st3d_upload and st3d_fill reset it to 0), e.g. to
 * continue a run in another context after moving its fields there. */
int st3d_set_step(st3d_ctx* ctx, uint64_t step);
/* Move the time state of `src` into `dst` on the device: u and v as the
 * values st3d_download returns, encoded in dst's storage, and the mode W step
 * clock.  Both contexts on one device, same grid, same mode and the same host
 * element type (FP32 for f32 and the 16-bit storages, FP64 for f64); s is not
 * moved (set it in dst first: st3d_upload and st3d_fill reset the clock).
 * dst's halo planes and rows become zero.  Allocates two device arrays of
 * the reference layout for the duration of the call; synchronizes both
 * streams.  Replaces a download into host arrays followed by an upload, e.g.
 * to continue an FP16 run in the compensated storage. */
int st3d_transfer(st3d_ctx* dst, st3d_ctx* src);

/* Copy reference-layout arrays in (NULL: leave that field): interior,
 * min(halo, 4) halo planes and rows, and the k halo (the stencil reads u's
 * halo).  One contiguous copy per field through a staging buffer the context
 * allocates on first use (the size of one host array).  The arrays may be
 * host memory or device memory of the context's device (st3d_download
 * likewise).  Resets the mode W step clock to 0. */
int st3d_upload(st3d_ctx* ctx, const void* v, const void* s, const void* u);
/* Copy interior points out: the host arrays' halo planes and rows are not
 * written, as the reference never writes halos; the k-halo points between
 * interior rows are rewritten with the device's copy of them (one 2-D copy
 * per field moves whole plane spans): in mode R the values uploaded for that
 * same array, in mode W those of the buffer that holds the field, so u and v
 * should carry the same halo (a fixed boundary).  Mode W: u = newest field
 * U^n, v = U^{n-1}.  NULL: skip. */
int st3d_download(st3d_ctx* ctx, void* v, void* u);
/* Replaces ITERATE(v,s,u,grid,prefetch,dups,iterations,cacheiter)
 * (iterators.h:6-29, iterators.cpp:130-289) on device-resident fields:
 * `iterations` steps, stream-ordered, asynchronous. */
int st3d_iterate(st3d_ctx* ctx, uint32_t iterations);
/* ITERATE drop-in on host arrays: upload v, s, u; iterate; download v (and,
 * in mode W, u as well: u is then written although ITERATE declares it
 * const); synchronize.  With pinned arrays on an FP32 TMA context (host path
 * AUTO or STREAMED) the three phases overlap in one launch (see
 * ST3D_HOST_STREAMED); the host arrays end the same either way. */
int st3d_iterate_host(st3d_ctx* ctx, void* v, const void* s, void* u, uint32_t iterations);
/* Waits for the context's stream; ST3D_ERR_TIMEOUT if a bounded device-side
 * wait of a kernel gave up since the last call (the kernel then returned
 * early and its results are void; the status word is cleared and the
 * context stays usable). */
int st3d_synchronize(st3d_ctx* ctx);
/* Diagnostics: writes `code` into the context's device status word on its
 * stream, as a kernel's bounded wait does when it gives up, so that the
 * error path of st3d_synchronize (ST3D_ERR_TIMEOUT, then a usable context)
 * can be exercised without a device wait running out.  No counterpart in
 * the reference, which has no device waits.  code 0 clears the word. */
int st3d_inject_device_status(st3d_ctx* ctx, uint32_t code);

/* Device-side initialisation of one field (st3d_fill_kind); replaces
 * init_arrays (iterators.cpp:292-301) for ST3D_FILL_CONST. */
int st3d_fill(st3d_ctx* ctx, int field, int kind, uint64_t seed, double a, double b);
/* Replaces check() (iterators.cpp:304-325): counts interior points of v
 * with |v - expected| > tol. */
int st3d_check(st3d_ctx* ctx, double expected, double tol, uint64_t* errors);
/* FP64 reductions over the interior of field fa of a against field fb of b
 * (b may equal a; b = NULL: out[0] = sum a^2, out[2] = max|a|).
 * out[0] = sum (a-b)^2, out[1] = sum b^2, out[2] = max|a-b|, out[3] = max|b|. */
int st3d_norms(st3d_ctx* a, int fa, st3d_ctx* b, int fb, double out[4]);

/* FP64 norms without any allocation.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they check drift, such
 * as a solver running inside another application's time loop on buffers that
 * application owns, where cudaMalloc/cudaFree may synchronise the device or
 * fail because the memory is reserved.  a and b (b may be NULL) are device
 * fields in the reference layout of `grid` (float for ST3D_F32, double for
 * ST3D_F64); out_dev is device memory for 4 doubles with the meaning of
 * st3d_norms' out; the work is enqueued on `stream` (a cudaStream_t, NULL for
 * the legacy default stream) and nothing is synchronised.  Partial sums live
 * in a 128 KiB array inside the library image: at most 4096 planes along i
 * (larger grids are rejected with ST3D_ERR_INVALID, as is a grid beyond the
 * limits every entry point applies: axes <= 2^24, halos <= 64/64/4096),
 * calls that overlap on the GPU race on it and must be serialised, and the
 * first call on a device looks up the array's address, so make it before any
 * stream capture.  A cudaDeviceReset (a new context on the device) makes the
 * next call look the address up again: make that call outside capture too. */
int st3d_norms_noalloc(const st3d_grid_desc* grid, const void* a, int storage_a, const void* b,
                       int storage_b, double* out_dev, void* stream);

/* CUDA-event timing on the context's stream. */
int st3d_timer_start(st3d_ctx* ctx);
int st3d_timer_stop(st3d_ctx* ctx, float* ms);

/* Summary of a context's run, the numbers the reference prints after its
 * timed ITERATE (main.cpp:304-310): the last timer region (start to stop)
 * with the steps taken inside it, its throughput, the reference's GFlop/s
 * and memory-traffic figures for those steps (config.h:67-91 counts), the
 * field energy sum(u^2) and max|u| of the current u (FP64), and, with a
 * second context of the same interior, the relative L2 difference of u from
 * that context's u (-1 without one). */
typedef struct st3d_metrics {
  uint64_t steps;          /* steps since the last upload (source clock) */
  uint64_t timed_steps;    /* steps inside the last timer region */
  double elapsed_ms;       /* the last timer region */
  double gpts;             /* points x timed_steps / elapsed */
  double gflops;           /* reference FLOPS_PER_STENCIL x points x timed_steps / elapsed */
  double mem_gbs;          /* reference MEM_BYTES x points x timed_steps / elapsed */
  double energy_u;         /* sum of u^2 over the interior */
  double max_abs_u;        /* max |u| over the interior */
  double rel_l2;           /* ||u - u_ref|| / ||u_ref||, or -1 */
  double reserved[4];
} st3d_metrics;
int st3d_metrics_get(st3d_ctx* ctx, st3d_ctx* ref, st3d_metrics* out);

/* Pinned host memory for fast upload/download. */
int st3d_host_alloc(size_t bytes, void** ptr);
int st3d_host_free(void* ptr);

/* The Ricker wavelet the mode W source uses: (1 - 2a) exp(-a),
 * a = (pi f (t - t0))^2, evaluated on the host in double. */
double st3d_ricker(double t, double f, double t0);

/* ---- batching form --------------------------------------------------------
 * No counterpart in the reference, which advances one grid per process:
 * many independent grids of uneven sizes and stencil orders (independent
 * source shots) advance together.  Every grid is a context of the FP32 wave
 * form (7, 13 or 25 points) living on the batch's stream; per-grid upload,
 * download, fill and norms go through st3d_batch_context.  Schedules of one
 * call of st3d_batch_iterate:
 *   ST3D_BATCH_SEQUENTIAL  one single-grid launch per grid per step;
 *   ST3D_BATCH_PERSISTENT  one persistent launch per step whose CTAs pull
 *                          (grid, tile, chunk) items from a device work queue;
 *   ST3D_BATCH_GRAPH       the persistent schedule with the whole time loop
 *                          captured once in a CUDA graph (cached by step
 *                          count) and replayed;
 *   ST3D_BATCH_PIPELINED   every step of the call in ONE persistent launch:
 *                          a per-(step, grid) counter of finished work items
 *                          lets a grid start its next step as soon as its own
 *                          previous step is done (bounded device waits), so
 *                          no step drains the GPU.  steps x work items must
 *                          stay below 2^31. */
typedef struct st3d_batch st3d_batch;

typedef enum st3d_batch_schedule {
  ST3D_BATCH_SEQUENTIAL = 0,
  ST3D_BATCH_PERSISTENT = 1,
  ST3D_BATCH_GRAPH = 2,
  ST3D_BATCH_PIPELINED = 3
} st3d_batch_schedule;

typedef struct st3d_batch_info {
  uint32_t grids;           /* grids in the batch */
  uint32_t work_items;      /* queue items per step: one per (grid, tile, i-chunk) */
  uint32_t ctas;            /* persistent CTAs per launch */
  uint32_t graphs;          /* captured time loops */
  uint64_t interior_points; /* sum of xs*ys*zs over the grids */
  uint64_t launches;        /* kernel launches issued by st3d_batch_iterate */
  int32_t reserved[8];
} st3d_batch_info;

int st3d_batch_create(uint32_t n, const st3d_grid_desc* grids, const st3d_opts* opts,
                      st3d_batch** batch);
int st3d_batch_destroy(st3d_batch* batch);
/* The context of grid idx (owned by the batch: do not destroy it). */
int st3d_batch_context(st3d_batch* batch, uint32_t idx, st3d_ctx** ctx);
int st3d_batch_get_info(const st3d_batch* batch, st3d_batch_info* info);
/* Advance every grid `steps` leapfrog steps with the given schedule. */
int st3d_batch_iterate(st3d_batch* batch, uint32_t steps, int schedule);
int st3d_batch_synchronize(st3d_batch* batch);
int st3d_batch_timer_start(st3d_batch* batch);
int st3d_batch_timer_stop(st3d_batch* batch, float* ms);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* ST3D_H */
