// st3d_kernels_aux.cu -- initialisation, known-answer check and FP64
// reductions over device fields.
//
//  - fill: the reference's init_arrays (iterators.cpp:292-301) as a
//    constant fill, plus the seeded generators of the benchmark inputs (a
//    counter hash for uniform noise, Gaussian blobs).
//  - check: the reference's check() (iterators.cpp:304-325) as a count.
//  - norms: sum (a-b)^2, sum b^2, max|a-b|, max|b| accumulated in double,
//    the energy and L2 reductions that measure drift against an FP64 run.
//    Two passes with per-block partials in a scratch buffer and a fixed
//    reduction order, so results are deterministic run to run.
#include "st3d_f16.cuh"
#include "st3d_internal.h"

namespace st3d {

namespace {

// The counter hash of the seeded uniform generator: the value at logical
// point (i,j,k) (interior coordinates; halo points negative or >= size)
// depends only on (seed, field, i, j, k).  Same definition as the host-side
// generator used to build test inputs.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return z;
}

__device__ __forceinline__ double unit_at(uint64_t seed, unsigned field, long long i, long long j,
                                          long long k) {
  uint64_t key = seed * 0x9E3779B97F4A7C15ULL + field;
  key = key * 0xD1B54A32D192ED03ULL + (uint64_t)(i + 64);
  key = key * 0xAEF17502108EF2D9ULL + (uint64_t)(j + 64);
  key = key * 0xF58C1E3A7E1C4B55ULL + (uint64_t)(k + 64);
  return (double)(mix64(key) >> 40) * (1.0 / 16777216.0);
}

struct BlobParams {
  int n;
  double p[4 * 16];  // ci, cj, ck, amplitude
};

template <typename T>
__global__ void k_fill(Layout L, T* __restrict__ dst, int kind, uint64_t seed, unsigned field,
                       double a, double b, BlobParams bp, int interior_only) {
  // one thread per element of a row segment; grid.y over rows of all planes
  const long long row = blockIdx.y + (long long)gridDim.y * blockIdx.z;
  if (row >= (long long)L.nj * L.ni) return;
  const long long ii = row / L.nj, jj = row % L.nj;
  const long long i = ii - L.pi, j = jj - L.pj;
  for (long long kk = blockIdx.x * blockDim.x + threadIdx.x; kk < L.nk;
       kk += (long long)gridDim.x * blockDim.x) {
    const long long k = kk - L.pk;
    double val;
    const bool inner = i >= 0 && i < L.xs && j >= 0 && j < L.ys && k >= 0 && k < L.zs;
    if (interior_only && !inner) {
      val = 0.0;
    } else if (kind == ST3D_FILL_CONST) {
      val = a;
    } else if (kind == ST3D_FILL_UNIFORM) {
      val = a + (b - a) * unit_at(seed, field, i, j, k);
    } else {
      val = 0.0;
      if (inner) {
        const double inv = 1.0 / (2.0 * b * b);
        for (int q = 0; q < bp.n; ++q) {
          const double di = (double)i - bp.p[4 * q], dj = (double)j - bp.p[4 * q + 1],
                       dk = (double)k - bp.p[4 * q + 2];
          val += bp.p[4 * q + 3] * exp(-(di * di + dj * dj + dk * dk) * inv);
        }
      }
    }
    dst[row * L.nk + kk] = (T)val;
  }
}

__device__ __forceinline__ double load_field(const FieldRef& f, long long i, long long x) {
  switch (f.storage) {
    case ST3D_F64: return static_cast<const double*>(f.p)[x];
    case ST3D_F32: return (double)static_cast<const float*>(f.p)[x];
    case ST3D_F16:
    case ST3D_F16_HILO: {
      const uint16_t w = static_cast<const uint16_t*>(f.p)[x];
      float v = __half2float(__ushort_as_half(w));
      if (f.lo) v = __fmaf_rn((float)f.lo[x], ulp256_f16(w), v);
      if (f.lo16) v = v + __half2float(__ushort_as_half(f.lo16[x]));  // exact: <= 22 bits
      v = v * exp2i(f.E[i]);
      if (f.p2) v = v - __half2float(__ushort_as_half(static_cast<const uint16_t*>(f.p2)[x])) * exp2i(f.E2[i]);
      return (double)v;
    }
    case ST3D_BF16: {
      const uint16_t w = static_cast<const uint16_t*>(f.p)[x];
      float v = __uint_as_float((uint32_t)w << 16) * exp2i(f.E[i]);
      if (f.p2)
        v = v - __uint_as_float((uint32_t)static_cast<const uint16_t*>(f.p2)[x] << 16) * exp2i(f.E2[i]);
      return (double)v;
    }
    default: return 0.0;
  }
}

__global__ void k_check(Geom g, FieldRef v, double expected, double tol,
                        unsigned long long* counter) {
  unsigned long long local = 0;
  const long long nrows = (long long)g.xs * g.ys;
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const long long i = r / g.ys, j = r % g.ys;
    const long long row = g.org + i * g.si + j * g.sj;
    for (int k = threadIdx.x; k < g.zs; k += blockDim.x)
      if (fabs(load_field(v, i, row + k) - expected) > tol) ++local;
  }
  if (local) atomicAdd(counter, local);
}

constexpr int kNormThreads = 256;

__global__ void __launch_bounds__(kNormThreads)
    k_norms_partial(Geom ga, FieldRef a, Geom gb, FieldRef b, double* __restrict__ partial) {
  double d2 = 0.0, b2 = 0.0, dm = 0.0, bm = 0.0;
  const long long nrows = (long long)ga.xs * ga.ys;
  for (long long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const long long i = r / ga.ys, j = r % ga.ys;
    const long long xa = ga.org + i * ga.si + j * ga.sj;
    const long long xb = gb.org + i * gb.si + j * gb.sj;
    for (int k = threadIdx.x; k < ga.zs; k += blockDim.x) {
      const double va = load_field(a, i, xa + k);
      const double vb = b.p ? load_field(b, i, xb + k) : 0.0;
      const double d = va - vb;
      d2 += d * d;
      b2 += vb * vb;
      dm = fmax(dm, fabs(d));
      bm = fmax(bm, fabs(vb));
    }
  }
  __shared__ double sh[4][kNormThreads];
  sh[0][threadIdx.x] = d2;
  sh[1][threadIdx.x] = b2;
  sh[2][threadIdx.x] = dm;
  sh[3][threadIdx.x] = bm;
  __syncthreads();
  for (int w = kNormThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + w];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + w];
      sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + w]);
      sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 4) partial[4 * (long long)blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(kNormThreads)
    k_norms_final(const double* __restrict__ partial, int nblocks, double* __restrict__ out) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int bI = threadIdx.x; bI < nblocks; bI += blockDim.x) {
    acc[0] += partial[4 * bI + 0];
    acc[1] += partial[4 * bI + 1];
    acc[2] = fmax(acc[2], partial[4 * bI + 2]);
    acc[3] = fmax(acc[3], partial[4 * bI + 3]);
  }
  __shared__ double sh[4][kNormThreads];
  for (int q = 0; q < 4; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = kNormThreads / 2; w > 0; w >>= 1) {
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

}  // namespace

cudaError_t launch_fill(int storage, const Layout& L, void* dst, int kind, uint64_t seed,
                        unsigned field, double a, double b, const double* blob_params, int nblobs,
                        int interior_only, cudaStream_t stream) {
  BlobParams bp;
  bp.n = nblobs < 0 ? 0 : (nblobs > 16 ? 16 : nblobs);
  for (int q = 0; q < 4 * bp.n; ++q) bp.p[q] = blob_params[q];
  const long long rows = (long long)L.nj * L.ni;
  dim3 block(256);
  const unsigned gy = (unsigned)(rows < 65535 ? rows : 65535);
  const unsigned gz = (unsigned)((rows + gy - 1) / gy);
  dim3 grid((L.nk + 255) / 256, gy, gz);
  const int k = kind;
  if (storage == ST3D_F32)
    k_fill<float><<<grid, block, 0, stream>>>(L, (float*)dst, k, seed, field, a, b, bp, interior_only);
  else if (storage == ST3D_F64)
    k_fill<double><<<grid, block, 0, stream>>>(L, (double*)dst, k, seed, field, a, b, bp, interior_only);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_check(const Geom& g, const FieldRef& v, double expected, double tol,
                         unsigned long long* counter, cudaStream_t stream) {
  k_check<<<4 * 152, 256, 0, stream>>>(g, v, expected, tol, counter);
  return cudaGetLastError();
}

int norms_blocks(const Geom& g) {
  const long long rows = (long long)g.xs * g.ys;
  return (int)(rows < 8 * 152 ? rows : 8 * 152);
}

cudaError_t launch_norms(const Geom& ga, const FieldRef& a, const Geom& gb, const FieldRef& b,
                         double* scratch, int nblocks, double* out_dev, cudaStream_t stream) {
  k_norms_partial<<<nblocks, kNormThreads, 0, stream>>>(ga, a, gb, b, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_norms_final<<<1, kNormThreads, 0, stream>>>(scratch, nblocks, out_dev);
  return cudaGetLastError();
}

}  // namespace st3d
