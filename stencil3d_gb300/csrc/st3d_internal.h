// st3d_internal.h -- shared declarations of the libst3d CUDA sources.
//
// Device layout of one field (all storages):
//   element (i,j,k) of the interior, 0 <= i < xs etc., lives at
//   ((i + pi)*nj + (j + pj))*nk + (k + pk)
//   pk = 128 bytes of front pad per row, so every interior row starts on a
//   128-byte boundary; nk rounds pk + zs + pk up to a multiple of pk, so each
//   row pitch is a multiple of 128 bytes (TMA strides must be multiples of
//   16 bytes, coalesced rows want 128).
//   pj = pi = 4 rows / planes: the widest stencil radius (25 points, r = 4).
// The halo points the stencil reads are the caller's halo values, copied at
// upload; the rest of the padding is zero.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "st3d.h"

namespace st3d {

constexpr int kMaxRadius = 4;

struct Layout {
  uint32_t xs, ys, zs;
  uint32_t pk, pj, pi;
  uint32_t nk, nj, ni;
  size_t elems() const { return (size_t)nk * nj * ni; }
  long long sj() const { return (long long)nk; }
  long long si() const { return (long long)nk * nj; }
  // offset of interior point (0,0,0)
  long long org() const { return (long long)pi * si() + (long long)pj * sj() + pk; }
};

Layout make_layout(uint32_t xs, uint32_t ys, uint32_t zs, int elem_bytes);

inline int radius_of(int points) {
  switch (points) {
    case 2: return 1;
    case 7: return 1;
    case 13: return 2;
    case 25: return 4;
    default: return -1;
  }
}

// Neighbour-pair evaluation order of the reference sums (axis 0 = i/x,
// 1 = j/y, 2 = k/z):
//   7 : x1 y1 z1                 stencil_7.h:20
//   13: z2 z1 y2 y1 x2 x1        stencil_13.h:40-43
//   25: z4..z1 y4..y1 x4..x1     stencil_25.h:64-67
__host__ __device__ constexpr int npairs_of(int P) { return P == 7 ? 3 : P == 13 ? 6 : P == 25 ? 12 : 0; }
__host__ __device__ constexpr int pair_axis(int P, int p) {
  return P == 7 ? p : 2 - p / (P == 13 ? 2 : 4);
}
__host__ __device__ constexpr int pair_r(int P, int p) {
  return P == 7 ? 1 : (P == 13 ? 2 - (p % 2) : 4 - (p % 4));
}

// Coefficients in the compute type C, pair coefficients already in the
// evaluation order above.
template <typename C>
struct Coefs {
  C coef0, K;      // mode R
  C c0, c1, c2;    // mode W
  C cf[12];
};

template <typename C>
Coefs<C> make_coefs(const st3d_opts& o);

// Makes `dev` the calling thread's current CUDA device for the scope of one
// entry point and restores the previous device on exit, so that a context
// created on device N runs there whatever device the caller has current.
// dev < 0: leave the current device as it is.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    if (dev < 0) return;
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
      return;
    }
    if (prev == dev) {
      prev = -1;
    } else if (cudaSetDevice(dev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
  }
  ~DeviceScope() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

// The grid limits every entry point applies (st3d_api.cu): axes 1 .. 2^24,
// at most 2^36 points, halos at most 64/64/4096; ST3D_OK or the status.
int validate_grid_limits(const st3d_grid_desc* g);

// Geometry passed to kernels by value.
struct Geom {
  int xs, ys, zs;
  int pk, pj, pi;
  long long sj, si, org;
};

inline Geom geom_of(const Layout& L) {
  Geom g;
  g.xs = (int)L.xs; g.ys = (int)L.ys; g.zs = (int)L.zs;
  g.pk = (int)L.pk; g.pj = (int)L.pj; g.pi = (int)L.pi;
  g.sj = L.sj(); g.si = L.si(); g.org = L.org();
  return g;
}

// The caller's reference layout (grid.cpp:20-24).
struct RefGeom {
  int xs, ys, zs;
  long long jmult, imult, ijk_ofs;
};

// Mode W point source for one step.
struct Source {
  int i, j, k;   // interior coordinates; i < 0: none
  float amp;     // s is replaced by s + amp at the source point
  double amp_d;  // the same amplitude for double storage
};

// The streamed drop-in call (st3d_stream.cu): host transfers and time steps
// in one cooperative launch.  chunk: planes per chunk along i; n_up, n_down:
// CTAs that copy planes from the host arrays into the device layout and back.
struct StreamPlan {
  int chunk = 16, nchunks = 0;
  int ntk = 0, ntiles = 0;  // tiles per plane along k, tiles per plane
  int n_up = 16, n_down = 12, grid = 0;
};
struct StreamLaunch {
  Geom g;
  RefGeom R;
  Coefs<float> cf;
  float* fld[3];
  const float* hin[3];  // device views of the host u, v, s
  float* hout[2];       // device views of the host u, v written back
  int ub0, vb0, steps;
  const int2* pairs;
  const int4* xfer;  // uploads [0, nup), downloads [nup, nxfer)
  int nup, nxfer;
  const int* up_need;
  int *up_cnt, *st_cnt, *progress, *heads;
  int hx, hy, hz, vec;
  int src_i, src_j, src_k;
  const float* amps;
  uint64_t timeout_ns;  // a wait gives up after this long without progress anywhere
  uint64_t cap_ns;      // and after this long in all
  uint32_t* status;
};
int stream_blocks_per_sm(int points, int mode);
cudaError_t launch_stream(int points, int mode, const StreamPlan& p, const CUtensorMap* maps,
                          const StreamLaunch& L, cudaStream_t stream);

// Device status word values set by bounded waits.
enum DeviceStatus : uint32_t {
  kDevOk = 0,
  kDevTimeoutFull = 1,
  kDevTimeoutEmpty = 2,
  kDevTimeoutDep = 3,   // a wait for another CTA's finished work (batch, pipelined)
};

// Records a formatted message for st3d_last_error() and returns `status`.
int set_error(int status, const char* fmt, ...);

// st3d_create on the caller's stream (nullptr: a stream of its own).
int create_context(const st3d_grid_desc* grid, const st3d_opts* opts, cudaStream_t external,
                   st3d_ctx** out);

// ---- kernel launchers (st3d_kernels_*.cu) --------------------------------
// All launch on `stream` and return the cudaGetLastError() of the launch.
cudaError_t launch_simple(int points, int mode, int storage, const Geom& g, const void* coefs,
                          void* v, const void* u, const void* s, const Source& src,
                          int ichunk, cudaStream_t stream);

struct TmaPlan;
// ubuf/vbuf/sbuf select the tensor maps of the field buffers holding u, v, s.
cudaError_t launch_tma(const TmaPlan& plan, int points, int mode, const Geom& g, const Coefs<float>& cf,
                       float* v, int ubuf, int vbuf, int sbuf, const Source& src, uint32_t* dev_status,
                       cudaStream_t stream);
bool tma_config_supported(int tj, int nv);
// Resident CTAs per SM of the TMA kernel for this configuration (0: cannot run).
int tma_blocks_per_sm(int points, int mode, int tj, int nv, size_t smem);

// Reference layout (staging buffer) <-> library layout, element size eb.
cudaError_t launch_ref_to_dev(int eb, const Layout& L, const RefGeom& R, const void* stage,
                              void* dst, int hx, int hy, int hz, cudaStream_t stream);
cudaError_t launch_dev_to_ref(int eb, const Layout& L, const RefGeom& R, const void* src,
                              void* stage, int hz, cudaStream_t stream);

// One step of the 16-bit-storage kernel: the output buffer (words and low
// bytes), the per-plane scale exponents of U^n, U^{n-1}, s and U^{n+1}, the
// per-plane maxima (float bits) of U^n, U^{n-1}, s, the accumulator of
// U^{n+1} and the one to clear for U^{n+2}, k4 = 4*c1*sum(w), and which field
// buffers hold u and v.
struct Tma16Step {
  uint16_t* vout;
  int8_t* vlo_out;
  const int *Eu, *Ev, *Es;
  int* Eout;
  const uint32_t *Mu, *Mv, *Ms;
  uint32_t *Mout, *Mzero;
  float k4;
  int ubuf, vbuf;
};
// The FP16 / BF16 delta form (st3d_kernels_delta16.cu): u in a pair of
// buffers, d = u^n - u^{n-1} updated in place.
struct Delta16Step {
  uint16_t* uout;                  // buffer receiving u^{n+1}
  uint16_t* d;                     // d^n in, d^{n+1} out
  const int *Eu, *Ed, *Es;         // plane scales of u^n, d^n, s
  int *Eu_out, *Ed_out;            // of u^{n+1}, d^{n+1} (set before the step)
  const uint32_t *Mu, *Md, *Ms;    // plane maxima of |u^n|, |d^n|, |s|
  uint32_t *Mu_out, *Md_out;       // maxima of the new levels
  float k4, m2s;
  int ubuf;                        // buffer holding u^n
  uint16_t* lout = nullptr;        // F16_HL: lo words of u^{n+1} (those of u^n: plan map lo[ubuf])
};
struct Tma16Plan;
size_t delta16_smem_bytes(int tj, int nv, int R, bool pair = false);
int delta16_blocks_per_sm(int storage, int points, const Tma16Plan& pl);
cudaError_t launch_delta16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                           const Coefs<float>& cf, const Delta16Step& st, const Source& src,
                           uint32_t* dev_status, cudaStream_t stream);
// The plane-scale kernel run before each delta-form step (both kernels).
cudaError_t launch_scales_delta(const Geom& g, int R, const Delta16Step& st, float c2, const Source& src,
                                cudaStream_t stream);
// The delta form with the j and k neighbour sums on the tensor cores
// (st3d_kernels_mma16.cu); plan fields mma / nb.
size_t mma16_smem_bytes(int nv, int R, bool pair);
int mma16_blocks_per_sm(int storage, int points, const Tma16Plan& pl);
cudaError_t launch_mma16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                         const Coefs<float>& cf, const Delta16Step& st, const Source& src,
                         uint32_t* dev_status, cudaStream_t stream);
size_t tma16_smem_bytes(int tj, int nv, int R, bool hilo);
int tma16_blocks_per_sm(int storage, int points, const Tma16Plan& pl);
cudaError_t launch_tma16(int storage, int points, const Tma16Plan& pl, const Geom& g,
                         const Coefs<float>& cf, const Tma16Step& st, const Source& src,
                         uint32_t* dev_status, cudaStream_t stream);

// 16-bit storage transfers (st3d_kernels_copy.cu).
// With `stage2`, the field is stage - stage2 (FP32) and the halo check
// covers both arrays.
cudaError_t launch_plane_max_ref(const RefGeom& R, const float* stage, uint32_t* M,
                                 uint32_t* halo_max, int hx, int hy, int hz, cudaStream_t stream,
                                 const float* stage2 = nullptr);
// With `lo16` (F16 words only), also the lo words of the FP16 hi/lo pair.
cudaError_t launch_ref_to_dev16(int storage, const Layout& L, const RefGeom& R, const float* stage,
                                uint16_t* hi, int8_t* lo, const uint32_t* M, int* E, int hx, int hy,
                                int hz, cudaStream_t stream, const float* stage2 = nullptr,
                                uint16_t* lo16 = nullptr);
// Delta form -> reference layout: u = dec(U) (minus_d false) or
// v = dec(U) - dec(D) (minus_d true), interior rows with their k halo.
// With `ul` (the F16_HL form) u = (U + ul) * 2^Eu.
cudaError_t launch_delta_to_ref(int storage, const Layout& L, const RefGeom& R, const uint16_t* u,
                                const int* Eu, const uint16_t* d, const int* Ed, bool minus_d,
                                float* stage, int hz, cudaStream_t stream,
                                const uint16_t* ul = nullptr);
cudaError_t launch_dev16_to_ref(int storage, const Layout& L, const RefGeom& R, const uint16_t* hi,
                                const int8_t* lo, const int* E, float* stage, int hz,
                                cudaStream_t stream);

// interior_only: points outside the interior are set to 0.
// Temporal blocking (st3d_kernels_tb.cu): T in {2, 4}, 7 or 13 points.
struct TbPlan;
size_t tb_smem_bytes(int points, int T);
int tb_blocks_per_sm(int points, int T);
// One pass of T steps: reads the state in buffers ubuf/vbuf, writes U^{n+T-1}
// to out_prev and U^{n+T} to out_new; amps = the T source amplitudes.
cudaError_t launch_tb(int points, int T, const TbPlan& pl, const Geom& g, const Coefs<float>& cf,
                      float* out_prev, float* out_new, int ubuf, int vbuf, const Source& src,
                      const float* amps, uint32_t* dev_status, cudaStream_t stream);

cudaError_t launch_fill(int storage, const Layout& L, void* dst, int kind, uint64_t seed,
                        unsigned field, double a, double b, const double* blob_params, int nblobs,
                        int interior_only, cudaStream_t stream);

// A device field as the reductions read it: values (float, double or 16-bit
// words), the low bytes of the compensated form and the per-plane scale
// exponents of 16-bit storage.
struct FieldRef {
  const void* p;
  int storage;
  const int8_t* lo;
  const int* E;
  const void* p2 = nullptr;  // delta form: the value is dec(p) - dec(p2)
  const int* E2 = nullptr;
  const uint16_t* lo16 = nullptr;  // F16_HL: dec(p) = (hi + lo16) * 2^E
};
cudaError_t launch_check(const Geom& g, const FieldRef& v, double expected, double tol,
                         unsigned long long* counter, cudaStream_t stream);
// Two-pass FP64 reduction: partials of `nblocks` blocks in scratch, then one block.
cudaError_t launch_norms(const Geom& ga, const FieldRef& a, const Geom& gb, const FieldRef& b,
                         double* scratch, int nblocks, double* out_dev, cudaStream_t stream);
int norms_blocks(const Geom& g);

}  // namespace st3d
