// st3d_noalloc.cu -- FP64 field norms that allocate nothing.
//
// st3d_norms() reduces through partial sums in scratch memory that
// st3d_create() obtained with cudaMalloc.  Some callers cannot allocate
// device memory at the point where they need a drift check: a solver plugged
// into another application's time loop receives device buffers that the
// host application owns and sized up front, and there a cudaMalloc/cudaFree
// pair may implicitly synchronise the whole device or fail outright because
// the host reserved the memory for itself.  st3d_norms_noalloc() serves them:
// the caller passes the two fields (device buffers in the reference layout)
// and a device output of four doubles; the partial sums live in the
// file-scope array below, which the library image carries on every device
// that loads it until the process exits.
//
// Limits and sharing:
//   - one partial per i-plane: at most kNoAllocMaxPlanes (4096) planes,
//     4096 x 4 doubles = 128 KiB of device memory per device;
//   - every call shares the array and leaves its partials behind; each call
//     writes every slot it reads before reading it (stream order), so nothing
//     has to start at zero, but calls that overlap on the GPU (two streams,
//     or two host threads) race on the array and must be serialised by the
//     caller;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (the array's name in host code is only a host-side
//     stand-in); make that first call before any stream capture.  The address
//     is kept per device together with the identity of the CUDA context it
//     was looked up in: after a cudaDeviceReset (or any teardown and
//     re-creation of the device's context) the next call finds a new context
//     and looks the address up again, so that first call after a reset must
//     also come before any stream capture.
#include <cuda.h>

#include <mutex>

#include "st3d_internal.h"

namespace st3d {
namespace {

constexpr int kNoAllocMaxPlanes = 4096;
constexpr int kNoAllocMaxDevices = 64;
constexpr int kNoAllocThreads = 256;

// Per-plane partials: [4*i + 0..3] = sum (a-b)^2, sum b^2, max|a-b|, max|b|.
static __device__ __align__(256) double g_plane_partials[4 * kNoAllocMaxPlanes];

// per device: the partials' address and the ID of the context it belongs to
double* g_partials_dev[kNoAllocMaxDevices] = {nullptr};
unsigned long long g_partials_ctx[kNoAllocMaxDevices] = {0};
std::mutex g_setup_mutex;

struct RefLayout {
  int xs, ys, zs;
  long long jmult, imult, ijk_ofs;
};

__device__ __forceinline__ double load_ref(const void* p, int storage, long long x) {
  if (storage == ST3D_F64) return static_cast<const double*>(p)[x];
  return (double)static_cast<const float*>(p)[x];
}

// One block per i-plane.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_plane_norms(RefLayout L, const void* __restrict__ a, int sa, const void* __restrict__ b,
                  int sb, double* __restrict__ partials) {
  const int i = blockIdx.x;
  double d2 = 0.0, b2 = 0.0, dm = 0.0, bm = 0.0;
  const long long plane = L.ijk_ofs + (long long)i * L.imult;
  const long long n = (long long)L.ys * L.zs;
  for (long long q = threadIdx.x; q < n; q += blockDim.x) {
    const long long j = q / L.zs, k = q - j * L.zs;
    const long long x = plane + j * L.jmult + k;
    const double va = load_ref(a, sa, x);
    const double vb = b ? load_ref(b, sb, x) : 0.0;
    const double d = va - vb;
    d2 += d * d;
    b2 += vb * vb;
    dm = fmax(dm, fabs(d));
    bm = fmax(bm, fabs(vb));
  }
  __shared__ double sh[4][kNoAllocThreads];
  sh[0][threadIdx.x] = d2;
  sh[1][threadIdx.x] = b2;
  sh[2][threadIdx.x] = dm;
  sh[3][threadIdx.x] = bm;
  __syncthreads();
  for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
      sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + w]);
      sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partials[4 * i + threadIdx.x] = sh[threadIdx.x][0];
}

// One block: planes in a fixed order, so the result is deterministic.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_plane_norms_final(const double* __restrict__ partials, int planes, double* __restrict__ out) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < planes; i += blockDim.x) {
    acc[0] += partials[4 * i + 0];
    acc[1] += partials[4 * i + 1];
    acc[2] = fmax(acc[2], partials[4 * i + 2]);
    acc[3] = fmax(acc[3], partials[4 * i + 3]);
  }
  __shared__ double sh[4][kNoAllocThreads];
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
      sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + w]);
      sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

// Unique ID of the calling thread's current CUDA context (0 if none is
// current yet, or if the driver does not answer).  The driver calls are taken
// through the runtime's entry-point query, so the library keeps no link-time
// dependence on the driver library.
typedef CUresult (*PFN_ctx_get_current)(CUcontext*);
typedef CUresult (*PFN_ctx_get_id)(CUcontext, unsigned long long*);

unsigned long long current_context_id() {
  static PFN_ctx_get_current get_current = nullptr;
  static PFN_ctx_get_id get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_ctx_get_current>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_ctx_get_id>(f);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id) return 0;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
  if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the partials array on the current device, looked up once
// per device and context; nullptr (with `err` set) if the lookup fails.
double* noalloc_partials(cudaError_t* err) {
  int dev = 0;
  *err = cudaGetDevice(&dev);
  if (*err != cudaSuccess) return nullptr;
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  const unsigned long long id = current_context_id();
  if (!g_partials_dev[dev] || id == 0 || id != g_partials_ctx[dev]) {
    double* p = nullptr;
    *err = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_plane_partials);
    if (*err != cudaSuccess) {
      g_partials_dev[dev] = nullptr;
      return nullptr;
    }
    g_partials_dev[dev] = p;
    // the lookup made the device's context current if it was not yet
    g_partials_ctx[dev] = id != 0 ? id : current_context_id();
  }
  return g_partials_dev[dev];
}

cudaError_t launch_norms_noalloc(const st3d_grid_desc& g, const void* a, int sa, const void* b,
                                 int sb, double* partials, double* out_dev, cudaStream_t stream) {
  RefLayout L;
  L.xs = (int)g.xs;
  L.ys = (int)g.ys;
  L.zs = (int)g.zs;
  L.jmult = (long long)g.zs + 2LL * g.zh;
  L.imult = L.jmult * ((long long)g.ys + 2LL * g.yh);
  L.ijk_ofs = (long long)g.zh + (long long)g.yh * L.jmult + (long long)g.xh * L.imult;
  k_plane_norms<<<L.xs, kNoAllocThreads, 0, stream>>>(L, a, sa, b, sb, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_plane_norms_final<<<1, kNoAllocThreads, 0, stream>>>(partials, L.xs, out_dev);
  return cudaGetLastError();
}

}  // namespace
}  // namespace st3d

extern "C" int st3d_norms_noalloc(const st3d_grid_desc* grid, const void* a, int storage_a,
                                  const void* b, int storage_b, double* out_dev, void* stream) {
  using namespace st3d;
  if (!grid || !a || !out_dev) return set_error(ST3D_ERR_INVALID, "null grid, field or output");
  if ((storage_a != ST3D_F32 && storage_a != ST3D_F64) ||
      (b && storage_b != ST3D_F32 && storage_b != ST3D_F64))
    return set_error(ST3D_ERR_INVALID, "fields must be F32 or F64");
  // the limits of every other entry point (axes, point count, halos), then
  // this entry point's own plane limit
  const int grc = validate_grid_limits(grid);
  if (grc != ST3D_OK) return grc;
  if (grid->xs > (uint32_t)kNoAllocMaxPlanes)
    return set_error(ST3D_ERR_INVALID,
                     "st3d_norms_noalloc handles at most %d planes along i (got %u); "
                     "use st3d_norms for larger grids",
                     kNoAllocMaxPlanes, grid->xs);
  cudaError_t e = cudaSuccess;
  double* partials = noalloc_partials(&e);
  if (!partials)
    return set_error(ST3D_ERR_CUDA, "cudaGetSymbolAddress of the partials array failed: %s",
                     cudaGetErrorString(e));
  e = launch_norms_noalloc(*grid, a, storage_a, b, storage_b, partials, out_dev,
                           static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess)
    return set_error(ST3D_ERR_CUDA, "norms kernel launch failed: %s", cudaGetErrorString(e));
  return ST3D_OK;
}
