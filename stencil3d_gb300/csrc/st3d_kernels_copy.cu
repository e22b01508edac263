// st3d_kernels_copy.cu -- host-boundary layout conversion on the device.
//
// The caller's arrays use the reference layout (IDX = ijk_ofs + k +
// j*jmult + i*imult, stencils.h:5, grid.cpp:20-24); the kernels use the
// library layout (st3d_internal.h).  A strided host<->device copy of ~1M rows
// of a few KB each runs far below the link rate, so transfers go through a
// staging buffer in the reference layout instead:
//   upload:   one contiguous host->device copy of the whole host array, then
//             k_ref_to_dev scatters the region the stencil can read (interior
//             plus up to 4 halo planes/rows and up to `pk` halo points along
//             k) into the library layout;
//   download: k_dev_to_ref gathers every interior row together with its k
//             halo into the staging buffer, then one 2-D copy moves, per
//             i-plane, the span of the interior rows (ys rows of jmult
//             points) back to the host.  The j-halo rows and i-halo planes of
//             the host array are not written; the k-halo points inside the
//             span are written with the values uploaded for them.
#include "st3d_internal.h"

namespace st3d {

namespace {

template <typename T>
__global__ void k_ref_to_dev(Layout L, RefGeom R, const T* __restrict__ stage, T* __restrict__ dst,
                             int hx, int hy, int hz) {
  const int klen = R.zs + 2 * hz;
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= klen) return;
  const int j = (int)blockIdx.y - hy;
  const int i = (int)blockIdx.z - hx;
  const int k = kk - hz;
  const long long s = R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k;
  const long long d = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (k + (int)L.pk);
  dst[d] = stage[s];
}

template <typename T>
__global__ void k_dev_to_ref(Layout L, RefGeom R, const T* __restrict__ src, T* __restrict__ stage,
                             int hz) {
  const int klen = R.zs + 2 * hz;
  const int kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= klen) return;
  const int j = (int)blockIdx.y;
  const int i = (int)blockIdx.z;
  const int k = kk - hz;
  const long long s = ((long long)(i + (int)L.pi) * L.nj + (j + (int)L.pj)) * L.nk + (k + (int)L.pk);
  stage[R.ijk_ofs + (long long)i * R.imult + (long long)j * R.jmult + k] = src[s];
}

}  // namespace

cudaError_t launch_ref_to_dev(int eb, const Layout& L, const RefGeom& R, const void* stage,
                              void* dst, int hx, int hy, int hz, cudaStream_t stream) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys + 2 * hy, R.xs + 2 * hx);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (eb == 4)
    k_ref_to_dev<float><<<grid, block, 0, stream>>>(L, R, (const float*)stage, (float*)dst, hx, hy, hz);
  else if (eb == 8)
    k_ref_to_dev<double><<<grid, block, 0, stream>>>(L, R, (const double*)stage, (double*)dst, hx, hy, hz);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_dev_to_ref(int eb, const Layout& L, const RefGeom& R, const void* src,
                              void* stage, int hz, cudaStream_t stream) {
  dim3 block(256);
  dim3 grid((R.zs + 2 * hz + 255) / 256, R.ys, R.xs);
  if (grid.y > 65535 || grid.z > 65535) return cudaErrorInvalidConfiguration;
  if (eb == 4)
    k_dev_to_ref<float><<<grid, block, 0, stream>>>(L, R, (const float*)src, (float*)stage, hz);
  else if (eb == 8)
    k_dev_to_ref<double><<<grid, block, 0, stream>>>(L, R, (const double*)src, (double*)stage, hz);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace st3d
