// st3d_api.cu -- the C ABI of libst3d (include/st3d.h): contexts, layout
// conversion at the host boundary, kernel selection and the time loop.
//
// The reference drives its hot path through ITERATE (iterators.h:6-29) on
// host arrays that main.cpp allocates (main.cpp:246-275) and initialises
// (iterators.cpp:292-301).  Here a context owns the device copies of u, v,
// s in the library's own layout (st3d_internal.h), converts from and to the
// reference layout at upload and download, and runs the time loop on its own
// CUDA stream.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "st3d_ctx.h"
#include "st3d_f16.cuh"
#include "st3d_internal.h"
#include "st3d_tma.cuh"

using namespace st3d;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? ST3D_ERR_NOMEM : ST3D_ERR_CUDA, "%s: %s (%s)", what,
              cudaGetErrorString(e), cudaGetErrorName(e));
}

#define ST3D_CUDA(call)                                 \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int elem_bytes(int storage) {
  switch (storage) {
    case ST3D_F32: return 4;
    case ST3D_F64: return 8;
    case ST3D_F16:
    case ST3D_BF16:
    case ST3D_F16_HILO:
    case ST3D_F16_HL: return 2;
    default: return 0;
  }
}

int host_elem_bytes(int storage) { return storage == ST3D_F64 ? 8 : 4; }

// Algorithmic HBM bytes per point per step: read u, v, s and write v
// (config.h:76,82,88 count these 4 streams); 2 points read u and write v
// (config.h:70).  FP16 / BF16 delta form: read u, d, s and write u, d at 2
// bytes each (10 B); the compensated form: 2-byte u, v, s and written v plus
// the low bytes of the centre u, of v and of the written v (11 B); the delta
// form with u as a hi/lo pair adds the lo words of the centre u, read and
// written (14 B).
// The word format of a 16-bit context's fields: the F16_HL form's words are
// FP16 (its u carries a second word array of lo parts).
int word_storage(int storage) { return storage == ST3D_F16_HL ? ST3D_F16 : storage; }

double f16_bytes(int storage, int points, int eb) {
  if (storage == ST3D_F16_HILO) return 11.0;
  if (storage == ST3D_F16_HL) return 14.0;
  if (storage == ST3D_F16 || storage == ST3D_BF16) return 10.0;
  return (points == 2 ? 2.0 : 4.0) * eb;
}

}  // namespace

namespace st3d {

int set_error(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

Layout make_layout(uint32_t xs, uint32_t ys, uint32_t zs, int eb) {
  Layout L;
  L.xs = xs; L.ys = ys; L.zs = zs;
  L.pk = 128u / (uint32_t)eb;
  L.pj = kMaxRadius;
  L.pi = kMaxRadius;
  const uint32_t need = L.pk + zs + L.pk;
  L.nk = (need + L.pk - 1) / L.pk * L.pk;
  L.nj = ys + 2 * L.pj;
  L.ni = xs + 2 * L.pi;
  return L;
}

template <typename C>
Coefs<C> make_coefs(const st3d_opts& o) {
  Coefs<C> c;
  memset(&c, 0, sizeof c);
  c.coef0 = (C)o.coef[0];
  c.K = (C)o.coef[1];
  c.c0 = (C)o.c0;
  c.c1 = (C)o.c1;
  c.c2 = (C)o.c2;
  const int P = o.points;
  for (int p = 0; p < npairs_of(P); ++p)
    c.cf[p] = (C)o.coef[2 + 4 * pair_axis(P, p) + pair_r(P, p) - 1];
  return c;
}
template Coefs<float> make_coefs<float>(const st3d_opts&);
template Coefs<double> make_coefs<double>(const st3d_opts&);

}  // namespace st3d

// ---------------------------------------------------------------------------
// context: struct st3d_ctx is in st3d_ctx.h
// ---------------------------------------------------------------------------

namespace {

int validate(const st3d_grid_desc* g, const st3d_opts* o) {
  if (!g || !o) return fail(ST3D_ERR_INVALID, "null grid or options");
  const int R = radius_of(o->points);
  if (R < 0) return fail(ST3D_ERR_INVALID, "points must be 2, 7, 13 or 25 (got %d)", o->points);
  if (o->mode != ST3D_MODE_REF && o->mode != ST3D_MODE_WAVE)
    return fail(ST3D_ERR_INVALID, "unknown mode %d", o->mode);
  if (elem_bytes(o->storage) == 0) return fail(ST3D_ERR_INVALID, "unknown storage %d", o->storage);
  if (o->kernel < ST3D_KERNEL_AUTO || o->kernel > ST3D_KERNEL_MMA)
    return fail(ST3D_ERR_INVALID, "unknown kernel %d", o->kernel);
  const int grc = st3d::validate_grid_limits(g);
  if (grc != ST3D_OK) return grc;
  // The stencil reads u up to R points beyond the interior on every axis
  // (stencil_*.h neighbour loads); the 2-point stencil only reads k+1.
  const uint32_t rx = o->points == 2 ? 0 : R, ry = rx, rz = R;
  if (g->xh < rx || g->yh < ry || g->zh < rz)
    return fail(ST3D_ERR_INVALID, "halo (%u,%u,%u) is narrower than the %d-point stencil needs (%u,%u,%u)",
                g->xh, g->yh, g->zh, o->points, rx, ry, rz);
  if (o->mode == ST3D_MODE_WAVE && o->points == 2)
    return fail(ST3D_ERR_UNSUPPORTED, "the 2-point stencil has no wave form (it is not a Laplacian)");
  const bool s16 = o->storage == ST3D_F16 || o->storage == ST3D_BF16 || o->storage == ST3D_F16_HILO ||
                   o->storage == ST3D_F16_HL;
  if (s16 && o->mode != ST3D_MODE_WAVE)
    return fail(ST3D_ERR_UNSUPPORTED, "16-bit storage is the precision form of the wave update only");
  if (s16 && o->kernel == ST3D_KERNEL_SIMPLE)
    return fail(ST3D_ERR_UNSUPPORTED, "16-bit storage runs on the TMA kernel only");
  if (s16 && (g->xs > 65535 - 8 || g->ys > 65535 - 8 || g->zh > 64))
    return fail(ST3D_ERR_UNSUPPORTED, "16-bit storage needs xs, ys <= 65527 and zh <= 64");
  const bool delta16 = o->storage == ST3D_F16 || o->storage == ST3D_BF16 || o->storage == ST3D_F16_HL;
  if (o->kernel == ST3D_KERNEL_MMA && !delta16)
    return fail(ST3D_ERR_UNSUPPORTED, "the tensor-core kernel serves the 16-bit delta forms (F16, BF16, F16_HL)");
  if (o->kernel == ST3D_KERNEL_MMA && o->tile_j != 0 && o->tile_j != 16)
    return fail(ST3D_ERR_UNSUPPORTED, "the tensor-core kernel runs 16-row tiles, not %d", o->tile_j);
  if (o->kernel == ST3D_KERNEL_MMA && o->stages != 0 && o->stages != (o->storage == ST3D_F16_HL ? 4 : 8))
    return fail(ST3D_ERR_UNSUPPORTED, "the tensor-core kernel runs %d stages, not %d",
                o->storage == ST3D_F16_HL ? 4 : 8, o->stages);
  if (o->kernel == ST3D_KERNEL_TMA && o->storage == ST3D_F64)
    return fail(ST3D_ERR_UNSUPPORTED, "the TMA kernel serves FP32 and 16-bit storage");
  if (o->kernel == ST3D_KERNEL_TMA && o->points == 2)
    return fail(ST3D_ERR_UNSUPPORTED, "the TMA kernel serves the 7/13/25-point stencils");
  if (s16 && o->tile_j != 0 && o->tile_j != 16 &&
      !((o->tile_j == 8 || o->tile_j == 20) && o->storage != ST3D_F16_HILO))
    return fail(ST3D_ERR_UNSUPPORTED,
                "16-bit storage runs 16-row tiles (8 or 20 also in the delta forms), not %d", o->tile_j);
  if (o->temporal_block != 0 && o->temporal_block != 1 && o->temporal_block != 2 &&
      o->temporal_block != 4)
    return fail(ST3D_ERR_INVALID, "temporal blocking depth must be 1, 2 or 4 (got %d)",
                o->temporal_block);
  if (o->temporal_block > 1 &&
      (o->mode != ST3D_MODE_WAVE || o->storage != ST3D_F32 || o->points == 2))
    return fail(ST3D_ERR_UNSUPPORTED,
                "temporal blocking fuses FP32 wave steps of the 7-, 13- and 25-point stencils");
  // a level tile loses R columns per fused step at either edge; the tile
  // keeps at most 8 columns of margin, so (T - 1) * R <= 8
  if (o->temporal_block > 1 && (o->temporal_block - 1) * radius_of(o->points) > 8)
    return fail(ST3D_ERR_UNSUPPORTED,
                "temporal blocking depth %d is too deep for the %d-point stencil (at most %d)",
                o->temporal_block, o->points, o->points == 25 ? 2 : 4);
  if (o->device < -1)
    return fail(ST3D_ERR_INVALID, "device %d: a CUDA device ordinal, or -1 for the current device",
                o->device);
  if (o->mode == ST3D_MODE_WAVE && o->src_i >= 0 &&
      ((uint32_t)o->src_i >= g->xs || o->src_j < 0 || (uint32_t)o->src_j >= g->ys ||
       o->src_k < 0 || (uint32_t)o->src_k >= g->zs))
    return fail(ST3D_ERR_INVALID, "source (%d,%d,%d) outside the interior", o->src_i, o->src_j,
                o->src_k);
  return ST3D_OK;
}

// TMA plan for an FP32 context: tile rows, stages, work units, grid.
bool plan_tma(const st3d_ctx* c, int sm_count, int max_smem, TmaPlan* p) {
  const int R = c->R;
  p->radius = R;
  p->tj = c->opts.tile_j > 0 ? c->opts.tile_j : 16;
  // 4 stages measured best at 1024^3 (385 Gpts/s against 374 with 3)
  p->nv = c->opts.stages > 0 ? c->opts.stages : 4;
  if (!tma_config_supported(p->tj, p->nv)) return false;
  p->smem = tma_smem_bytes(p->tj, p->nv, R);
  if ((int)p->smem > max_smem) return false;
  const int per_sm = tma_blocks_per_sm(c->opts.points, c->opts.mode, p->tj, p->nv, p->smem);
  if (per_sm < 1) return false;
  p->ntj = (int)((c->L.ys + p->tj - 1) / p->tj);
  p->ntk = (int)((c->L.zs + kTmaTK - 1) / kTmaTK);
  const int ctas = sm_count * per_sm;
  p->ichunk = c->opts.ichunk > 0 ? c->opts.ichunk
                                 : tma_pick_ichunk((int)c->L.xs, p->ntj * p->ntk, ctas, R);
  p->nti = (int)((c->L.xs + p->ichunk - 1) / p->ichunk);
  p->units = p->ntj * p->ntk * p->nti;
  p->grid = ctas < p->units ? ctas : p->units;
  p->threads = (p->tj + 1) * 32;
  return true;
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

typedef CUresult (*PFN_pointer_attr)(void*, CUpointer_attribute, CUdeviceptr);
PFN_pointer_attr get_pointer_attr() {
  static PFN_pointer_attr fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 4000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_pointer_attr>(f);
  });
  return fn;
}

// Tensor map over one field buffer (L2 promotion to 128-byte lines: the u
// tiles' rows start 16 bytes before a line and 256-byte promotion fetched
// more than they use; measured 384.7 -> 390.3 Gpts/s for the 25-point FP32
// step at 1024^3).  The extents stop where the stencil's
// valid data stops (dim0 = row front pad + zs + `kext` halo points, dim1 =
// front rows + ys + `jext` halo rows): box parts beyond them are out of bounds,
// which TMA fills with zeros without reading memory, so partial edge tiles
// cost no DRAM bytes.
int encode_map(CUtensorMap* m, void* base, const Layout& L, uint32_t box_k, uint32_t box_j,
               uint32_t kext, uint32_t jext) {
  auto enc = get_encode();
  if (!enc) return fail(ST3D_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[3] = {(cuuint64_t)L.pk + L.zs + kext, (cuuint64_t)L.pj + L.ys + jext, L.ni};
  cuuint64_t strides[2] = {(cuuint64_t)L.nk * 4, (cuuint64_t)L.nk * L.nj * 4};
  cuuint32_t box[3] = {box_k, box_j, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ST3D_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ST3D_OK;
}

void* u_ptr(st3d_ctx* c) { return c->fld[c->ub]; }
void* v_ptr(st3d_ctx* c) { return c->fld[c->vb]; }
int u_index(const st3d_ctx* c) { return c->ub; }
int v_index(const st3d_ctx* c) { return c->vb; }

RefGeom ref_geom(const st3d_grid_desc& g) {
  RefGeom R;
  R.xs = (int)g.xs; R.ys = (int)g.ys; R.zs = (int)g.zs;
  R.jmult = (long long)g.zs + 2LL * g.zh;
  R.imult = R.jmult * ((long long)g.ys + 2LL * g.yh);
  R.ijk_ofs = (long long)g.zh + (long long)g.yh * R.jmult + (long long)g.xh * R.imult;
  return R;
}

size_t host_array_bytes(const st3d_ctx* c) {
  const st3d_grid_desc& g = c->grid;
  return ((size_t)g.xs + 2 * g.xh) * ((size_t)g.ys + 2 * g.yh) * ((size_t)g.zs + 2 * g.zh) *
         host_elem_bytes(c->opts.storage);
}

// The staged path needs the halo along k to fit the device row pad and the
// launch grid (rows x planes) to fit 65535 x 65535.
bool staged_ok(const st3d_ctx* c) {
  const st3d_grid_desc& g = c->grid;
  return host_elem_bytes(c->opts.storage) == c->eb && g.zh <= c->L.pk &&
         g.ys + 8 <= 65535 && g.xs + 8 <= 65535;
}

int ensure_stage(st3d_ctx* c, int slots = 1) {
  const size_t need = host_array_bytes(c) * (size_t)slots;
  if (c->stage && c->stage_bytes >= need) return ST3D_OK;
  if (c->stage) {
    cudaFree(c->stage);
    c->bytes -= c->stage_bytes;
    c->stage = nullptr;
  }
  cudaError_t e = cudaMalloc(&c->stage, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->stage = nullptr;
    return fail(ST3D_ERR_NOMEM, "cudaMalloc of the %zu-byte staging buffer failed", need);
  }
  c->stage_bytes = need;
  c->bytes += need;
  return ST3D_OK;
}

// Strided host<->device copy of one field (fallback when the staged path does
// not apply): interior plus min(halo, 4) per side when `with_halo`.
int copy_field_strided(st3d_ctx* c, void* dev, void* host, bool to_device, bool with_halo) {
  const st3d_grid_desc& g = c->grid;
  const int hb = host_elem_bytes(c->opts.storage);
  const uint32_t hx = with_halo ? (g.xh < 4 ? g.xh : 4) : 0;
  const uint32_t hy = with_halo ? (g.yh < 4 ? g.yh : 4) : 0;
  const uint32_t hz = with_halo ? (g.zh < 4 ? g.zh : 4) : 0;
  const size_t jmult = (size_t)g.zs + 2 * g.zh;
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof p);
  cudaPitchedPtr hp = make_cudaPitchedPtr(host, jmult * hb, jmult, g.ys + 2 * g.yh);
  cudaPitchedPtr dp = make_cudaPitchedPtr(dev, (size_t)c->L.nk * c->eb, c->L.nk, c->L.nj);
  cudaPos hpos = make_cudaPos((g.zh - hz) * hb, g.yh - hy, g.xh - hx);
  cudaPos dpos = make_cudaPos((c->L.pk - hz) * c->eb, c->L.pj - hy, c->L.pi - hx);
  if (to_device) {
    p.srcPtr = hp; p.srcPos = hpos; p.dstPtr = dp; p.dstPos = dpos;
    p.kind = cudaMemcpyDefault;
  } else {
    p.srcPtr = dp; p.srcPos = dpos; p.dstPtr = hp; p.dstPos = hpos;
    p.kind = cudaMemcpyDefault;
  }
  p.extent = make_cudaExtent((g.zs + 2 * hz) * (size_t)hb, g.ys + 2 * hy, g.xs + 2 * hx);
  ST3D_CUDA(cudaMemcpy3DAsync(&p, c->stream));
  return ST3D_OK;
}

// The device address of a host array the kernels may read and write
// directly: pinned (cudaMallocHost, cudaHostAlloc, cudaHostRegister) and
// lying inside one allocation; nullptr otherwise (pageable memory, or a range
// the CUDA runtime does not report as one pinned range), and the transfer
// then goes through staging.
void* direct_view(const void* host, size_t bytes) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  auto attr = get_pointer_attr();
  if (!attr) return nullptr;
  CUdeviceptr start = 0;
  size_t size = 0;
  const CUdeviceptr p = (CUdeviceptr)(uintptr_t)host;
  if (attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, p) != CUDA_SUCCESS ||
      attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, p) != CUDA_SUCCESS)
    return nullptr;
  if (p < start || p + bytes > start + size) return nullptr;
  return at.devicePointer;
}

// Host (reference layout) -> device field.  Staged: one contiguous copy into
// the staging buffer, then a scatter kernel into the library layout
// (interior, min(halo, 4) planes and rows, all k-halo points up to the row
// pad).  Direct: the scatter kernel reads the pinned host array itself.  A
// context that blocks in time needs a zero halo and checks it here.
int upload_field(st3d_ctx* c, void* dev, const void* host) {
  if (!staged_ok(c)) {
    if (c->tb) return fail(ST3D_ERR_UNSUPPORTED, "temporal blocking needs the staged host path (zh <= 32)");
    c->host_path = ST3D_HOST_STRIDED;
    return copy_field_strided(c, dev, const_cast<void*>(host), true, true);
  }
  const void* src = nullptr;
  if (c->opts.host_path != ST3D_HOST_STAGED) src = direct_view(host, host_array_bytes(c));
  if (c->opts.host_path == ST3D_HOST_DIRECT && !src)
    return fail(ST3D_ERR_INVALID, "the direct host path needs a pinned host array");
  if (!src) {
    int rc = ensure_stage(c);
    if (rc != ST3D_OK) return rc;
    ST3D_CUDA(cudaMemcpyAsync(c->stage, host, host_array_bytes(c), cudaMemcpyDefault, c->stream));
    src = c->stage;
    c->host_path = ST3D_HOST_STAGED;
  } else {
    c->host_path = ST3D_HOST_DIRECT;
  }
  const st3d_grid_desc& g = c->grid;
  const int hx = g.xh < 4 ? (int)g.xh : 4, hy = g.yh < 4 ? (int)g.yh : 4;
  if (c->tb) {
    ST3D_CUDA(cudaMemsetAsync(c->halo_max, 0, sizeof(uint32_t), c->stream));
    cudaError_t e = launch_plane_max_ref(ref_geom(g), (const float*)src, c->M, c->halo_max, hx, hy,
                                         (int)g.zh, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "halo check kernel");
    uint32_t halo = 0;
    ST3D_CUDA(cudaMemcpyAsync(&halo, c->halo_max, sizeof halo, cudaMemcpyDeviceToHost, c->stream));
    ST3D_CUDA(cudaStreamSynchronize(c->stream));
    if (halo != 0)
      return fail(ST3D_ERR_UNSUPPORTED,
                  "temporal blocking needs a zero halo (a zero Dirichlet boundary)");
  }
  cudaError_t e = launch_ref_to_dev(c->eb, c->L, ref_geom(g), src, dev, hx, hy, (int)g.zh, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "upload scatter kernel");
  return ST3D_OK;
}

// Device field -> host (reference layout), interior points only: a gather
// kernel writes every interior row with its k halo, into the pinned host
// array directly or into the staging buffer followed by one 2-D copy of the
// span of the ys interior rows of each i-plane.
int download_field(st3d_ctx* c, const void* dev, void* host) {
  if (!staged_ok(c)) {
    c->host_path = ST3D_HOST_STRIDED;
    return copy_field_strided(c, const_cast<void*>(dev), host, false, false);
  }
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  void* dst = nullptr;
  if (c->opts.host_path != ST3D_HOST_STAGED) dst = direct_view(host, host_array_bytes(c));
  if (c->opts.host_path == ST3D_HOST_DIRECT && !dst)
    return fail(ST3D_ERR_INVALID, "the direct host path needs a pinned host array");
  if (dst) {
    c->host_path = ST3D_HOST_DIRECT;
    cudaError_t e = launch_dev_to_ref(c->eb, c->L, R, dev, dst, (int)g.zh, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "download gather kernel");
    return ST3D_OK;
  }
  int rc = ensure_stage(c);
  if (rc != ST3D_OK) return rc;
  c->host_path = ST3D_HOST_STAGED;
  cudaError_t e = launch_dev_to_ref(c->eb, c->L, R, dev, c->stage, (int)g.zh, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "download gather kernel");
  const size_t hb = host_elem_bytes(c->opts.storage);
  const size_t off = ((size_t)g.xh * R.imult + (size_t)g.yh * R.jmult) * hb;
  ST3D_CUDA(cudaMemcpy2DAsync(static_cast<char*>(host) + off, R.imult * hb,
                              static_cast<const char*>(c->stage) + off, R.imult * hb,
                              (size_t)g.ys * R.jmult * hb, g.xs, cudaMemcpyDefault, c->stream));
  return ST3D_OK;
}

int mod(long long a, int m) { return (int)(((a % m) + m) % m); }
// compensated form: scales and maxima of time level `level` (relative to lvl)
int* E_level(st3d_ctx* c, long long level) { return c->E + (size_t)mod(level, 3) * c->grid.xs; }
uint32_t* M_level(st3d_ctx* c, long long level) { return c->M + (size_t)mod(level, 4) * c->grid.xs; }
int* E_s(st3d_ctx* c) { return c->E + 4 * (size_t)c->grid.xs; }
uint32_t* M_s(st3d_ctx* c) { return c->M + 4 * (size_t)c->grid.xs; }
// delta form: u per buffer, d per level parity
int* Eu_buf(st3d_ctx* c, int buf) { return c->E + (size_t)buf * c->grid.xs; }
uint32_t* Mu_buf(st3d_ctx* c, int buf) { return c->M + (size_t)buf * c->grid.xs; }
int* Ed_lvl(st3d_ctx* c, uint64_t lvl) { return c->E + (size_t)(2 + (lvl & 1)) * c->grid.xs; }
uint32_t* Md_lvl(st3d_ctx* c, uint64_t lvl) { return c->M + (size_t)(2 + (lvl & 1)) * c->grid.xs; }

int encode_map_t(CUtensorMap* m, CUtensorMapDataType dt, int eb, void* base, const Layout& L,
                 uint32_t box_k, uint32_t box_j, uint32_t kext, uint32_t jext) {
  auto enc = get_encode();
  if (!enc) return fail(ST3D_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[3] = {(cuuint64_t)L.pk + L.zs + kext, (cuuint64_t)L.pj + L.ys + jext, L.ni};
  cuuint64_t strides[2] = {(cuuint64_t)L.nk * eb, (cuuint64_t)L.nk * L.nj * eb};
  cuuint32_t box[3] = {box_k, box_j, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ST3D_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ST3D_OK;
}

// 16-bit plan: the FP32 decomposition with 16-bit tiles (8-word k halo).
int plan_tma16(st3d_ctx* c, int sm_count, int max_smem) {
  Tma16Plan* p = new (std::nothrow) Tma16Plan();
  if (!p) return fail(ST3D_ERR_NOMEM, "host allocation failed");
  const int R = c->R;
  const bool hilo = c->opts.storage == ST3D_F16_HILO;
  p->radius = R;
  // The delta form runs 16-, 20- or 8-row tiles (one CTA of 17 or 21 warps
  // per SM, or two of 9).  Defaults measured at 1024^3 (FP16): 25 points 20
  // rows x 10 stages 317 Gpts/s against 299 for 16 x 12; 7 points 20 x 8 545
  // against 519; 13 points 16 x 8 459 against 357 for 20 x 8.
  const int pts = c->opts.points;
  const int tj_def = (c->delta && pts != 13) ? 20 : 16;
  const int tj_want = c->opts.tile_j > 0 ? c->opts.tile_j : tj_def;
  p->tj = (c->delta && (tj_want == 8 || tj_want == 20)) ? tj_want : 16;
  p->delta = c->delta;
  p->pair = c->pair;
  auto smem_of = [&](int nv) {
    return c->delta ? delta16_smem_bytes(p->tj, nv, R, c->pair) : tma16_smem_bytes(p->tj, nv, R, hilo);
  };
  auto per_sm_of = [&](int nv) {
    p->nv = nv;
    p->smem = smem_of(nv);
    if ((int)p->smem > max_smem) return 0;
    return c->delta ? delta16_blocks_per_sm(c->opts.storage, c->opts.points, *p)
                    : tma16_blocks_per_sm(c->opts.storage, c->opts.points, *p);
  };
  // the deepest pipeline that keeps the tile's CTAs per SM (two for 8 rows,
  // one for 16 and 20); opts.stages may ask for one depth.  The delta form
  // defaults to 12 stages for 25 points on 16 rows, 10 on 20 rows and 8
  // otherwise (measured at 1024^3: 25 points on 16 rows 253 -> 299 Gpts/s
  // from 8 to 12 stages, on 20 rows 270 / 296 / 317 at 6 / 8 / 10; 7 and 13
  // points flat or slower past 8).
  const int want = c->opts.stages;
  const int first = want ? want : !c->delta ? 12 : pts != 25 ? 8 : p->tj == 20 ? 10 : 12;
  const int need = p->tj == 8 ? 2 : 1;
  // the depths the kernels are built for: 6/8/10 on 20 rows, 4/6/8/12
  // otherwise; the F16_HL form (a third tile per stage) 6/8 on 20 rows and
  // 4/6/8 otherwise
  auto built = [&](int nv) {
    if (c->pair) return p->tj == 20 ? (nv == 6 || nv == 8) : (nv == 4 || nv == 6 || nv == 8);
    return p->tj == 20 ? (nv == 6 || nv == 8 || nv == 10) : (nv == 4 || nv == 6 || nv == 8 || nv == 12);
  };
  if (want && !built(want)) {
    const int tj = p->tj;
    delete p;
    return fail(ST3D_ERR_UNSUPPORTED, "16-bit kernels on %d-row tiles run %s stages, not %d", tj,
                c->pair ? (tj == 20 ? "6 or 8" : "4, 6 or 8") : (tj == 20 ? "6, 8 or 10" : "4, 6, 8 or 12"),
                want);
  }
  int per_sm = 0;
  for (int nv : {12, 10, 8, 6, 4}) {
    if (!built(nv) || (want ? nv != want : nv > first)) continue;
    const int b = per_sm_of(nv);
    if (b >= need || (want && b >= 1)) {
      per_sm = b;
      break;
    }
  }
  if (per_sm < 1) {
    delete p;
    return fail(ST3D_ERR_UNSUPPORTED, "16-bit kernel does not fit in shared memory");
  }
  p->ntj = (int)((c->L.ys + p->tj - 1) / p->tj);
  p->ntk = (int)((c->L.zs + 127) / 128);
  const int ctas = sm_count * per_sm;
  p->ichunk = c->opts.ichunk > 0 ? c->opts.ichunk : tma_pick_ichunk((int)c->L.xs, p->ntj * p->ntk, ctas, R);
  p->nti = (int)((c->L.xs + p->ichunk - 1) / p->ichunk);
  p->units = p->ntj * p->ntk * p->nti;
  p->grid = ctas < p->units ? ctas : p->units;
  p->threads = (p->tj + 1) * 32;
  const CUtensorMapDataType w16 =
      c->opts.storage == ST3D_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  int ok = ST3D_OK;
  for (int f = 0; f < 2 && ok == ST3D_OK; ++f) {
    ok = encode_map_t(&p->uhi[f], w16, 2, c->fld[f], c->L, 144, p->tj + 2 * R, 8, c->L.pj);
    if (ok == ST3D_OK) ok = encode_map_t(&p->vhi[f], w16, 2, c->fld[f], c->L, 128, p->tj, 0, 0);
    if (ok == ST3D_OK && hilo)
      ok = encode_map_t(&p->lo[f], CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, c->lo[f], c->L, 128, p->tj, 0, 0);
    else if (ok == ST3D_OK && c->pair)
      ok = encode_map_t(&p->lo[f], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, c->lo[f], c->L, 128, p->tj, 0, 0);
    else if (ok == ST3D_OK)
      p->lo[f] = p->vhi[f];  // unused by the uncompensated kernels
  }
  if (ok == ST3D_OK) ok = encode_map_t(&p->vhi[2], w16, 2, c->fld[2], c->L, 128, p->tj, 0, 0);
  if (ok == ST3D_OK && c->delta) ok = encode_map_t(&p->dmap, w16, 2, c->fld[3], c->L, 128, p->tj, 0, 0);
  if (ok != ST3D_OK) {
    delete p;
    return ok;
  }
  c->tma16 = p;
  return ST3D_OK;
}

// The tensor-core kernel serves a delta-form request when asked for, or under
// ST3D_KERNEL_AUTO when the request names no tile height or pipeline depth of
// the scalar kernel: measured at 1024^3 on a GB300 it is the faster kernel
// of the delta forms (25 points FP16 515 against 317 Gpts/s, BF16 498 / 312,
// F16_HL 397 / 283; 13 points (1040^3) FP16 500 / 408, F16_HL 410 / 363;
// 7 points FP16 615 / 545, BF16 603 / 531, F16_HL 418 / 357).
bool mma_chosen(const st3d_opts& o) {
  const bool delta = o.storage == ST3D_F16 || o.storage == ST3D_BF16 || o.storage == ST3D_F16_HL;
  if (!delta || o.mode != ST3D_MODE_WAVE) return false;
  if (o.kernel == ST3D_KERNEL_MMA) return true;
  return o.kernel == ST3D_KERNEL_AUTO && o.tile_j == 0 && o.stages == 0;
}

// Tensor-core delta-form plan (st3d_kernels_mma16.cu): 16-row x 152-column
// tiles; tensor maps with a u box of 168 x 24 words (columns k0-8 .., rows
// j0-R ..), d / s / lo boxes of 152 x 16 words, and interior boxes of 152 x
// 16 over the u buffers for the stores of u^{n+1}; 8 pipeline stages (4 for
// the pair form).
int plan_mma16(st3d_ctx* c, int sm_count, int max_smem) {
  Tma16Plan* p = new (std::nothrow) Tma16Plan();
  if (!p) return fail(ST3D_ERR_NOMEM, "host allocation failed");
  const int R = c->R;
  p->radius = R;
  p->tj = 16;
  p->delta = true;
  p->pair = c->pair;
  p->mma = true;
  p->nb = 1;
  p->nv = c->pair ? 4 : 8;
  p->smem = mma16_smem_bytes(p->nv, R, c->pair);
  const int per_sm =
      (int)p->smem <= max_smem ? mma16_blocks_per_sm(c->opts.storage, c->opts.points, *p) : 0;
  if (per_sm < 1) {
    delete p;
    return fail(ST3D_ERR_UNSUPPORTED, "the tensor-core kernel does not fit in shared memory");
  }
  if (cudaMalloc(&p->mma_rec, (size_t)c->L.xs * sizeof(MmaRecord)) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return fail(ST3D_ERR_NOMEM, "cudaMalloc of the plane records failed");
  }
  c->bytes += (size_t)c->L.xs * sizeof(MmaRecord);
  p->ntj = (int)((c->L.ys + 15) / 16);
  p->ntk = (int)((c->L.zs + kMmaTK - 1) / kMmaTK);
  const int ctas = sm_count * per_sm;
  p->ichunk = c->opts.ichunk > 0 ? c->opts.ichunk : tma_pick_ichunk((int)c->L.xs, p->ntj * p->ntk, ctas, R);
  p->nti = (int)((c->L.xs + p->ichunk - 1) / p->ichunk);
  p->units = p->ntj * p->ntk * p->nti;
  p->grid = ctas < p->units ? ctas : p->units;
  p->threads = (kMmaTK / 8 + 1) * 32;
  const CUtensorMapDataType w16 =
      c->opts.storage == ST3D_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  int ok = ST3D_OK;
  for (int f = 0; f < 2 && ok == ST3D_OK; ++f) {
    ok = encode_map_t(&p->uhi[f], w16, 2, c->fld[f], c->L, kMmaTK + 16, 24, 8, c->L.pj);
    // the interior box the kernel stores u^{n+1} through
    if (ok == ST3D_OK) ok = encode_map_t(&p->vhi[f], w16, 2, c->fld[f], c->L, kMmaTK, 16, 0, 0);
    if (ok == ST3D_OK && c->pair)
      ok = encode_map_t(&p->lo[f], CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, c->lo[f], c->L, kMmaTK, 16, 0, 0);
    else if (ok == ST3D_OK)
      p->lo[f] = p->uhi[f];  // unused without the pair form
  }
  if (ok == ST3D_OK) ok = encode_map_t(&p->vhi[2], w16, 2, c->fld[2], c->L, kMmaTK, 16, 0, 0);
  if (ok == ST3D_OK) ok = encode_map_t(&p->dmap, w16, 2, c->fld[3], c->L, kMmaTK, 16, 0, 0);
  if (ok != ST3D_OK) {
    cudaFree(p->mma_rec);
    delete p;
    return ok;
  }
  c->tma16 = p;
  return ST3D_OK;
}

// Upload of one field into 16-bit storage from a float host array: contiguous
// copy to the staging buffer, per-plane maxima, encode + scatter with the
// planes' scales; the halo must be zero.  which: 0 = u (time level 0),
// 1 = v (time level -1), 2 = s.
int upload_field16(st3d_ctx* c, int which, const void* host) {
  int rc = ensure_stage(c);
  if (rc != ST3D_OK) return rc;
  if (host)
    ST3D_CUDA(cudaMemcpyAsync(c->stage, host, host_array_bytes(c), cudaMemcpyDefault, c->stream));
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  const int hx = g.xh < 4 ? (int)g.xh : 4, hy = g.yh < 4 ? (int)g.yh : 4, hz = (int)g.zh;
  const long long n = (long long)c->lvl;
  uint32_t* M = which == 0 ? M_level(c, n) : which == 1 ? M_level(c, n - 1) : M_s(c);
  int* E = which == 0 ? E_level(c, n) : which == 1 ? E_level(c, n - 1) : E_s(c);
  const int buf = which == 2 ? 2 : (which == 0 ? u_index(c) : v_index(c));
  ST3D_CUDA(cudaMemsetAsync(M, 0, g.xs * sizeof(uint32_t), c->stream));
  ST3D_CUDA(cudaMemsetAsync(c->halo_max, 0, sizeof(uint32_t), c->stream));
  cudaError_t e = launch_plane_max_ref(R, (const float*)c->stage, M, c->halo_max, hx, hy, hz, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "plane maximum kernel");
  const int storage = (which == 2 && c->opts.storage == ST3D_F16_HILO) ? ST3D_F16 : c->opts.storage;
  e = launch_ref_to_dev16(storage, c->L, R, (const float*)c->stage, (uint16_t*)c->fld[buf],
                          which == 2 ? nullptr : (int8_t*)c->lo[buf], M, E, hx, hy, hz, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "16-bit encode kernel");
  uint32_t halo = 0;
  ST3D_CUDA(cudaMemcpyAsync(&halo, c->halo_max, sizeof halo, cudaMemcpyDeviceToHost, c->stream));
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  if (halo != 0)
    return fail(ST3D_ERR_UNSUPPORTED,
                "16-bit storage needs a zero halo (a zero Dirichlet boundary); field %d has nonzero halo values",
                which);
  return ST3D_OK;
}

int download_field16(st3d_ctx* c, int which, void* host) {
  int rc = ensure_stage(c);
  if (rc != ST3D_OK) return rc;
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  const long long level = which == 0 ? (long long)c->lvl : (long long)c->lvl - 1;
  const int buf = which == 0 ? u_index(c) : v_index(c);
  cudaError_t e = launch_dev16_to_ref(c->opts.storage, c->L, R, (const uint16_t*)c->fld[buf],
                                      (const int8_t*)c->lo[buf], E_level(c, level), (float*)c->stage,
                                      (int)g.zh, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "16-bit decode kernel");
  const size_t off = ((size_t)g.xh * R.imult + (size_t)g.yh * R.jmult) * 4;
  ST3D_CUDA(cudaMemcpy2DAsync(static_cast<char*>(host) + off, R.imult * 4,
                              static_cast<const char*>(c->stage) + off, R.imult * 4,
                              (size_t)g.ys * R.jmult * 4, g.xs, cudaMemcpyDefault, c->stream));
  return ST3D_OK;
}

FieldRef field_ref(st3d_ctx* c, int f) {
  FieldRef r;
  r.storage = c->opts.storage;
  r.lo = nullptr;
  r.E = nullptr;
  if (f == ST3D_FIELD_S) {
    r.p = c->fld[2];
    if (c->f16) {
      r.E = E_s(c);
      if (r.storage == ST3D_F16_HILO) r.storage = ST3D_F16;
    }
    return r;
  }
  if (c->delta) {  // u = dec(U), v = dec(U) - dec(D)
    r.storage = word_storage(c->opts.storage);
    r.p = c->fld[c->ub];
    r.E = Eu_buf(c, c->ub);
    if (c->pair) r.lo16 = (const uint16_t*)c->lo[c->ub];
    if (f == ST3D_FIELD_V) {
      r.p2 = c->fld[3];
      r.E2 = Ed_lvl(c, c->lvl);
    }
    return r;
  }
  const int buf = f == ST3D_FIELD_U ? u_index(c) : v_index(c);
  r.p = c->fld[buf];
  if (c->f16) {
    r.E = E_level(c, f == ST3D_FIELD_U ? (long long)c->lvl : (long long)c->lvl - 1);
    if (r.storage == ST3D_F16_HILO) r.lo = (const int8_t*)c->lo[buf];
  }
  return r;
}

// ---- delta form host transfers ----------------------------------------------
// The staging buffer holds two host arrays: slot 0 = u, slot 1 = v (FP32,
// reference layout, zero halos).  Setting u or v re-encodes U and/or D = u - v
// from the pair; the pair is rebuilt from the device state (the values a
// download returns) when a step or another use of the slots made it stale.

float* stage_slot(st3d_ctx* c, int slot) {
  return reinterpret_cast<float*>(static_cast<char*>(c->stage) + (size_t)slot * host_array_bytes(c));
}

// Encode a (or a - b) from the staging slots into 16-bit words with per-plane
// maxima M and scales E; the halo of a (and b) must be zero.
int encode_staged16(st3d_ctx* c, const float* a, const float* b, void* words, uint32_t* M, int* E,
                    const char* what, void* lo16 = nullptr) {
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  const int hx = g.xh < 4 ? (int)g.xh : 4, hy = g.yh < 4 ? (int)g.yh : 4, hz = (int)g.zh;
  ST3D_CUDA(cudaMemsetAsync(M, 0, g.xs * sizeof(uint32_t), c->stream));
  ST3D_CUDA(cudaMemsetAsync(c->halo_max, 0, sizeof(uint32_t), c->stream));
  cudaError_t e = launch_plane_max_ref(R, a, M, c->halo_max, hx, hy, hz, c->stream, b);
  if (e != cudaSuccess) return cuda_fail(e, "plane maximum kernel");
  e = launch_ref_to_dev16(word_storage(c->opts.storage), c->L, R, a, (uint16_t*)words, nullptr, M, E,
                          hx, hy, hz, c->stream, b, (uint16_t*)lo16);
  if (e != cudaSuccess) return cuda_fail(e, "16-bit encode kernel");
  uint32_t halo = 0;
  ST3D_CUDA(cudaMemcpyAsync(&halo, c->halo_max, sizeof halo, cudaMemcpyDeviceToHost, c->stream));
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  if (halo != 0)
    return fail(ST3D_ERR_UNSUPPORTED,
                "16-bit storage needs a zero halo (a zero Dirichlet boundary); %s has nonzero halo values",
                what);
  return ST3D_OK;
}

int delta_rebuild_pair(st3d_ctx* c) {
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  ST3D_CUDA(cudaMemsetAsync(c->stage, 0, 2 * host_array_bytes(c), c->stream));
  for (int slot = 0; slot < 2; ++slot) {
    cudaError_t e = launch_delta_to_ref(word_storage(c->opts.storage), c->L, R,
                                        (const uint16_t*)c->fld[c->ub], Eu_buf(c, c->ub),
                                        (const uint16_t*)c->fld[3], Ed_lvl(c, c->lvl), slot == 1,
                                        stage_slot(c, slot), (int)g.zh, c->stream,
                                        (const uint16_t*)c->lo[c->ub]);
    if (e != cudaSuccess) return cuda_fail(e, "16-bit decode kernel");
  }
  c->pair_valid = true;
  return ST3D_OK;
}

// U from slot 0 (when u changed) and D from slot 0 - slot 1.
int delta_encode_pair(st3d_ctx* c, bool u_changed) {
  int rc;
  c->pair_valid = false;
  if (u_changed &&
      (rc = encode_staged16(c, stage_slot(c, 0), nullptr, c->fld[c->ub], Mu_buf(c, c->ub),
                            Eu_buf(c, c->ub), "u", c->pair ? c->lo[c->ub] : nullptr)) != ST3D_OK)
    return rc;
  if ((rc = encode_staged16(c, stage_slot(c, 0), stage_slot(c, 1), c->fld[3], Md_lvl(c, c->lvl),
                            Ed_lvl(c, c->lvl), "u or v")) != ST3D_OK)
    return rc;
  c->pair_valid = true;
  return ST3D_OK;
}

int delta_download(st3d_ctx* c, void* host, bool v) {
  int rc = ensure_stage(c, 2);
  if (rc != ST3D_OK) return rc;
  c->pair_valid = false;
  const st3d_grid_desc& g = c->grid;
  const RefGeom R = ref_geom(g);
  cudaError_t e = launch_delta_to_ref(word_storage(c->opts.storage), c->L, R,
                                      (const uint16_t*)c->fld[c->ub], Eu_buf(c, c->ub),
                                      (const uint16_t*)c->fld[3], Ed_lvl(c, c->lvl), v, stage_slot(c, 0),
                                      (int)g.zh, c->stream, (const uint16_t*)c->lo[c->ub]);
  if (e != cudaSuccess) return cuda_fail(e, "16-bit decode kernel");
  const size_t off = ((size_t)g.xh * R.imult + (size_t)g.yh * R.jmult) * 4;
  ST3D_CUDA(cudaMemcpy2DAsync(static_cast<char*>(host) + off, R.imult * 4,
                              reinterpret_cast<const char*>(stage_slot(c, 0)) + off, R.imult * 4,
                              (size_t)g.ys * R.jmult * 4, g.xs, cudaMemcpyDefault, c->stream));
  return ST3D_OK;
}

// Temporally blocked plan: work units of (tb_rows - 2(T-1)R) rows x (128 -
// 2 tb_khalo) columns x ichunk planes; the warm-up of a unit is 2*T*R planes.
int plan_tb(st3d_ctx* c, int sm_count) {
  TbPlan* p = new (std::nothrow) TbPlan();
  if (!p) return fail(ST3D_ERR_NOMEM, "host allocation failed");
  const int T = c->opts.temporal_block, R = c->R;
  p->T = T;
  p->radius = R;
  p->rows = tb_rows(c->opts.points, T);
  p->rows_out = p->rows - 2 * (T - 1) * R;
  int max_smem = 0;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  if ((int)tb_smem_bytes(c->opts.points, T) > max_smem || p->rows_out < 1) {
    delete p;
    return fail(ST3D_ERR_UNSUPPORTED, "temporal blocking of depth %d does not fit", T);
  }
  const int per_sm = tb_blocks_per_sm(c->opts.points, T);
  if (per_sm < 1) {
    delete p;
    return fail(ST3D_ERR_UNSUPPORTED, "the temporally blocked kernel cannot be resident");
  }
  p->ntj = (int)((c->L.ys + p->rows_out - 1) / p->rows_out);
  const int outc = 128 - 2 * tb_khalo(c->opts.points, T);
  p->ntk = (int)((c->L.zs + outc - 1) / outc);
  const int ctas = sm_count * per_sm;
  p->ichunk = c->opts.ichunk > 0 ? c->opts.ichunk
                                 : tma_pick_ichunk((int)c->L.xs, p->ntj * p->ntk, ctas, 2 * T * R);
  p->nti = (int)((c->L.xs + p->ichunk - 1) / p->ichunk);
  p->units = p->ntj * p->ntk * p->nti;
  p->grid = ctas < p->units ? ctas : p->units;
  int ok = ST3D_OK;
  for (int f : {0, 1, 3, 4}) {
    if (ok == ST3D_OK)
      ok = encode_map(&p->umap[f], c->fld[f], c->L, kTmaUKW, p->rows + 2 * R, kTmaKHalo, c->L.pj);
    if (ok == ST3D_OK) ok = encode_map(&p->vmap[f], c->fld[f], c->L, kTmaTK, p->rows, 0, 0);
  }
  if (ok == ST3D_OK) ok = encode_map(&p->vmap[2], c->fld[2], c->L, kTmaTK, p->rows, 0, 0);
  if (ok != ST3D_OK) {
    delete p;
    return ok;
  }
  c->tb = p;
  return ST3D_OK;
}

// The streamed drop-in call (st3d_stream.cu): upload, `iterations` steps and
// download in one cooperative launch.  *done = false (and nothing enqueued)
// where it does not apply; the caller then runs the phases one by one.
int iterate_host_streamed(st3d_ctx* c, void* v, const void* s, void* u, uint32_t iterations,
                          bool* done) {
  *done = false;
  const int hp = c->opts.host_path;
  if (hp != ST3D_HOST_AUTO && hp != ST3D_HOST_STREAMED) return ST3D_OK;
  if (iterations < 1 || c->opts.storage != ST3D_F32 || c->f16 || c->tb || !c->tma ||
      c->kernel != ST3D_KERNEL_TMA || c->tma->tj != 16 || c->tma->nv != 4 || !staged_ok(c))
    return ST3D_OK;
  const int pts = c->opts.points;
  if (pts != 7 && pts != 13 && pts != 25) return ST3D_OK;
  const size_t hbytes = host_array_bytes(c);
  const float* hv = static_cast<const float*>(direct_view(v, hbytes));
  const float* hs = static_cast<const float*>(direct_view(s, hbytes));
  const float* hu = static_cast<const float*>(direct_view(u, hbytes));
  if (!hv || !hs || !hu) return ST3D_OK;
  int coop = 0, sm = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, c->device);
  const int per_sm = stream_blocks_per_sm(pts, c->opts.mode);
  if (!coop || per_sm < 1) return ST3D_OK;

  const st3d_grid_desc& gd = c->grid;
  const bool wave = c->opts.mode == ST3D_MODE_WAVE;
  const int R = c->R;
  const int T = (int)iterations;
  StreamPlan p;
  p.chunk = c->opts.ichunk > 0 ? c->opts.ichunk : 16;
  if (p.chunk < R) p.chunk = R;
  p.nchunks = (int)((gd.xs + p.chunk - 1) / p.chunk);
  p.ntk = c->tma->ntk;
  p.ntiles = c->tma->ntj * c->tma->ntk;
  p.grid = sm * per_sm;
  if (p.grid < 64) {
    p.n_up = p.n_down = p.grid / 8 > 0 ? p.grid / 8 : 1;
  }
  if (p.grid - p.n_up - p.n_down < 1) return ST3D_OK;
  const int S = p.nchunks;
  if ((uint64_t)T * S * p.ntiles > 0x7fffffffull || (uint64_t)T * S > 0x7fffffffull) return ST3D_OK;

  // host tables: the stencil queue (step, chunk) in wavefront order (step t
  // of chunk c at stage c + t + 1, steps in increasing order within a stage),
  // the upload queue (chunk by chunk) followed by the download queue (chunk
  // by chunk), the plane copies each chunk's upload counts, and the source
  // amplitude of every step
  const int hx = gd.xh < 4 ? (int)gd.xh : 4, hy = gd.yh < 4 ? (int)gd.yh : 4;
  std::vector<int2> pairs;
  pairs.reserve((size_t)T * S);
  for (long long d = 1; d <= (long long)S + T - 1; ++d)
    for (int t = 0; t < T; ++t) {
      const long long cc = d - 1 - t;
      if (cc >= 0 && cc < S) pairs.push_back(make_int2(t, (int)cc));
    }
  std::vector<int4> xfer;
  std::vector<int> up_need(S, 0);
  for (int d = 0; d < S; ++d) {
    const int i0 = d * p.chunk - (d == 0 ? hx : 0);
    const int i1 = std::min((int)gd.xs, (d + 1) * p.chunk) + (d == S - 1 ? hx : 0);
    for (int f = 0; f < 3; ++f)
      for (int i = i0; i < i1; ++i) xfer.push_back(make_int4(0, f, i, d));
    up_need[d] = 3 * (i1 - i0);
  }
  const int nup = (int)xfer.size();
  for (int ch = 0; ch < S; ++ch) {
    const int i0 = ch * p.chunk, i1 = std::min((int)gd.xs, i0 + p.chunk);
    for (int f = wave ? 0 : 1; f < 2; ++f)
      for (int i = i0; i < i1; ++i) xfer.push_back(make_int4(1, f, i, ch));
  }
  std::vector<float> amps;
  if (wave && c->opts.src_i >= 0) {
    amps.resize(T);
    for (int t = 0; t < T; ++t)
      amps[t] = (float)st3d_ricker((double)t * c->opts.dt, c->opts.src_f, c->opts.src_t0);
  }

  // one device buffer: pairs | xfer | up_need | amps | counters
  auto align16 = [](size_t x) { return (x + 15) / 16 * 16; };
  const size_t o_pairs = 0;
  const size_t o_xfer = align16(o_pairs + pairs.size() * sizeof(int2));
  const size_t o_need = align16(o_xfer + xfer.size() * sizeof(int4));
  const size_t o_amps = align16(o_need + up_need.size() * sizeof(int));
  const size_t o_cnt = align16(o_amps + amps.size() * sizeof(float));
  const size_t ncnt = (size_t)S + (size_t)T * S + 1 + 3;  // up_cnt, st_cnt, progress, heads
  const size_t need = o_cnt + ncnt * sizeof(int);
  if (need > c->stream_buf_bytes) {
    if (c->stream_buf) {
      cudaFree(c->stream_buf);
      c->bytes -= c->stream_buf_bytes;
    }
    c->stream_buf = nullptr;
    c->stream_buf_bytes = 0;
    cudaError_t e = cudaMalloc(&c->stream_buf, need);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ST3D_ERR_NOMEM, "cudaMalloc of %zu bytes for the streamed call failed", need);
    }
    c->stream_buf_bytes = need;
    c->bytes += need;
  }
  // the previous call's copies out of stream_host have finished: the call
  // synchronised its stream
  c->stream_host.assign(o_cnt, 0);
  unsigned char* hb = c->stream_host.data();
  memcpy(hb + o_pairs, pairs.data(), pairs.size() * sizeof(int2));
  memcpy(hb + o_xfer, xfer.data(), xfer.size() * sizeof(int4));
  memcpy(hb + o_need, up_need.data(), up_need.size() * sizeof(int));
  if (!amps.empty()) memcpy(hb + o_amps, amps.data(), amps.size() * sizeof(float));
  unsigned char* db = static_cast<unsigned char*>(c->stream_buf);
  ST3D_CUDA(cudaMemcpyAsync(db, hb, o_cnt, cudaMemcpyHostToDevice, c->stream));
  ST3D_CUDA(cudaMemsetAsync(db + o_cnt, 0, ncnt * sizeof(int), c->stream));

  StreamLaunch L;
  L.g = c->G;
  L.R = ref_geom(gd);
  L.cf = c->cf32;
  for (int f = 0; f < 3; ++f) L.fld[f] = static_cast<float*>(c->fld[f]);
  L.hin[0] = hu;
  L.hin[1] = hv;
  L.hin[2] = hs;
  L.hout[0] = const_cast<float*>(hu);
  L.hout[1] = const_cast<float*>(hv);
  L.ub0 = c->ub;
  L.vb0 = c->vb;
  L.steps = T;
  L.pairs = reinterpret_cast<const int2*>(db + o_pairs);
  L.xfer = reinterpret_cast<const int4*>(db + o_xfer);
  L.nup = nup;
  L.nxfer = (int)xfer.size();
  L.up_need = reinterpret_cast<const int*>(db + o_need);
  int* cnt = reinterpret_cast<int*>(db + o_cnt);
  L.up_cnt = cnt;
  L.st_cnt = cnt + S;
  L.progress = cnt + S + (size_t)T * S;
  L.heads = L.progress + 1;
  L.hx = hx;
  L.hy = hy;
  L.hz = (int)gd.zh;
  const RefGeom& Rg = L.R;
  const bool aligned = (reinterpret_cast<uintptr_t>(hu) | reinterpret_cast<uintptr_t>(hv) |
                        reinterpret_cast<uintptr_t>(hs)) % 16 == 0;
  L.vec = aligned && Rg.jmult % 4 == 0 && gd.zh % 4 == 0 && gd.zs % 4 == 0 &&
          (c->L.pk - gd.zh) % 4 == 0;
  L.src_i = wave ? c->opts.src_i : -1;
  L.src_j = c->opts.src_j;
  L.src_k = c->opts.src_k;
  L.amps = amps.empty() ? nullptr : reinterpret_cast<const float*>(db + o_amps);
  L.timeout_ns = c->tma->timeout_ns;
  // any wait's cap: the timeout plus four times the call at 100 Gpts/s and
  // the transfers at 20 GB/s, far beyond any run that makes progress
  const double pts_all = (double)gd.xs * gd.ys * gd.zs;
  L.cap_ns = L.timeout_ns + (uint64_t)(4.0 * (pts_all * T / 100.0 + 5.0 * hbytes / 20.0));
  L.status = c->dev_status;
  const CUtensorMap maps[5] = {c->tma->umap[0], c->tma->umap[1], c->tma->vmap[0], c->tma->vmap[1],
                               c->tma->vmap[2]};
  cudaError_t e = launch_stream(pts, c->opts.mode, p, maps, L, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "streamed call launch");
  // the state a phase-by-phase call leaves: the source clock restarts at the
  // upload and advances T steps; mode W swaps the pair every step
  c->has_u = c->has_v = c->has_s = true;
  c->pair_valid = false;
  c->step = (uint64_t)T;
  c->lvl += (uint64_t)T;
  c->launches += 1;
  if (wave && (T & 1)) {
    const int t = c->ub;
    c->ub = c->vb;
    c->vb = t;
  }
  c->host_path = ST3D_HOST_STREAMED;
  *done = true;
  return ST3D_OK;
}

int check_device_status(st3d_ctx* c) {
  uint32_t st = 0;
  ST3D_CUDA(cudaMemcpyAsync(&st, c->dev_status, sizeof st, cudaMemcpyDeviceToHost, c->stream));
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  if (st != kDevOk) {
    ST3D_CUDA(cudaMemsetAsync(c->dev_status, 0, sizeof(uint32_t), c->stream));
    return fail(ST3D_ERR_TIMEOUT, "a bounded device wait gave up (status %u)", st);
  }
  return ST3D_OK;
}


}  // namespace

namespace st3d {
// Limits of a grid that every entry point taking one applies: each axis
// 1 .. 2^24 points, at most 2^36 interior points, halos at most 64/64/4096.
int validate_grid_limits(const st3d_grid_desc* g) {
  if (!g) return fail(ST3D_ERR_INVALID, "null grid");
  if (g->xs < 1 || g->ys < 1 || g->zs < 1)
    return fail(ST3D_ERR_INVALID, "grid sizes must be >= 1 (got %u x %u x %u)", g->xs, g->ys, g->zs);
  if (g->zs > (1u << 24) || g->ys > (1u << 24) || g->xs > (1u << 24))
    return fail(ST3D_ERR_INVALID, "grid axis beyond 2^24 points (got %u x %u x %u)", g->xs, g->ys,
                g->zs);
  if ((uint64_t)g->xs * g->ys * g->zs > (1ull << 36))
    return fail(ST3D_ERR_INVALID, "grid of %llu points is beyond the library limit 2^36",
                (unsigned long long)g->xs * g->ys * g->zs);
  if (g->xh > 64 || g->yh > 64 || g->zh > 4096)
    return fail(ST3D_ERR_INVALID, "halo (%u,%u,%u) too wide", g->xh, g->yh, g->zh);
  return ST3D_OK;
}

// FP32 tiled tensor map over one field buffer (encode_map above), for the
// batch kernel's own tile shapes.
int encode_f32_box(CUtensorMap* m, void* base, const Layout& L, uint32_t box_k, uint32_t box_j,
                   uint32_t kext, uint32_t jext) {
  return encode_map(m, base, L, box_k, box_j, kext, jext);
}
}  // namespace st3d

// ---------------------------------------------------------------------------
// library
// ---------------------------------------------------------------------------
extern "C" {

int st3d_abi_version(void) { return ST3D_ABI_VERSION; }

const char* st3d_status_string(int s) {
  switch (s) {
    case ST3D_OK: return "ok";
    case ST3D_ERR_INVALID: return "invalid argument";
    case ST3D_ERR_UNSUPPORTED: return "unsupported";
    case ST3D_ERR_CUDA: return "CUDA error";
    case ST3D_ERR_NOMEM: return "out of memory";
    case ST3D_ERR_TIMEOUT: return "device wait timed out";
    case ST3D_ERR_STATE: return "call out of order";
    case ST3D_ERR_NODEVICE: return "no GB300 (sm_103) device";
    default: return "unknown status";
  }
}

const char* st3d_last_error(void) { return g_last_error.c_str(); }

int st3d_device_info(int* sm_count, int* cc_major, int* cc_minor, size_t* total_bytes) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(ST3D_ERR_NODEVICE, "no CUDA device visible (%s)", cudaGetErrorString(e));
  }
  int dev = 0;
  ST3D_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  ST3D_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  if (total_bytes) *total_bytes = prop.totalGlobalMem;
  return ST3D_OK;
}

int st3d_default_opts(int points, int mode, int storage, st3d_opts* o) {
  if (!o) return fail(ST3D_ERR_INVALID, "null options");
  memset(o, 0, sizeof *o);
  o->points = points;
  o->mode = mode;
  o->storage = storage;
  o->kernel = ST3D_KERNEL_AUTO;
  o->temporal_block = 1;
  o->device = -1;  // the calling thread's current device
  o->src_i = -2;  // grid centre, resolved at st3d_create
  o->src_f = 15.0;
  o->src_t0 = 1.0 / 15.0;
  // Mode W has no reference code; its weights are the float constants of
  // stencil_*.h for every storage, so an FP64 run is the same stencil as the
  // FP32 run it judges.
  const bool dbl = storage == ST3D_F64 && mode == ST3D_MODE_REF;
  // The reference's CONSTANTS_* (stencil_7.h:4-8, stencil_13.h:4-22,
  // stencil_25.h:20-34).  The y/z coefficients are products formed in the
  // type of `real` (config.h:96-100): float products widened for float
  // storage, double products of the widened literals for double storage.
  auto mul = [dbl](float a, float b) -> double {
    return dbl ? (double)a * (double)b : (double)(a * b);
  };
  double* c = o->coef;
  if (points == 2) {
    c[0] = 0.5f;
  } else if (points == 7) {
    c[0] = 1.5f; c[1] = 3.5f;
    c[2] = 0.5f; c[6] = 0.5f; c[10] = 0.5f;
  } else if (points == 13) {
    const float cx[2] = {0.3f, 0.2f};
    c[0] = 1.5f; c[1] = 3.5f;
    for (int r = 0; r < 2; ++r) {
      c[2 + r] = cx[r];
      c[6 + r] = mul(cx[r], 1.1f);
      c[10 + r] = mul(cx[r], 0.9f);
    }
  } else if (points == 25) {
    const float cx[4] = {0.4f, 0.3f, 0.2f, 0.1f};
    c[0] = 1.25f; c[1] = 6.25f;
    for (int r = 0; r < 4; ++r) {
      c[2 + r] = cx[r];
      c[6 + r] = mul(cx[r], 1.1f);
      c[10 + r] = mul(cx[r], 0.9f);
    }
  } else {
    return fail(ST3D_ERR_INVALID, "points must be 2, 7, 13 or 25 (got %d)", points);
  }
  if (mode == ST3D_MODE_WAVE && points == 7) {
    // README.md:11-20: unit neighbour weights for the 7-point wave form.
    c[2] = c[6] = c[10] = 1.0;
  }
  if (mode == ST3D_MODE_WAVE) {
    c[0] = c[1] = 0.0;
    st3d_set_wave_physics(o, 1500.0, 1e-3, 10.0);
  }
  return ST3D_OK;
}

int st3d_set_wave_physics(st3d_opts* o, double vel, double dt, double dx) {
  if (!o || !(vel > 0) || !(dt > 0) || !(dx > 0))
    return fail(ST3D_ERR_INVALID, "wave physics needs positive velocity, dt and dx");
  const double c1 = (vel * dt / dx) * (vel * dt / dx);
  double wsum = 0.0;
  for (int m = 2; m < 14; ++m) wsum += o->coef[m];
  o->c0 = 2.0 - 2.0 * c1 * wsum;
  o->c1 = c1;
  o->c2 = dt * dt;
  o->dt = dt;
  return ST3D_OK;
}

double st3d_ricker(double t, double f, double t0) {
  const double pf = 3.14159265358979323846 * f * (t - t0);
  const double a = pf * pf;
  return (1.0 - 2.0 * a) * std::exp(-a);
}

int st3d_plan(const st3d_grid_desc* grid, const st3d_opts* opts, st3d_info* info) {
  if (!info) return fail(ST3D_ERR_INVALID, "null info");
  int rc = validate(grid, opts);
  if (rc != ST3D_OK) return rc;
  memset(info, 0, sizeof *info);
  const int eb = elem_bytes(opts->storage);
  const Layout L = make_layout(grid->xs, grid->ys, grid->zs, eb);
  const int R = radius_of(opts->points);
  const int T = opts->temporal_block > 0 ? opts->temporal_block : 1;
  info->interior_points = (uint64_t)grid->xs * grid->ys * grid->zs;
  const bool delta = opts->storage == ST3D_F16 || opts->storage == ST3D_BF16 ||
                     opts->storage == ST3D_F16_HL;
  info->device_bytes = (T > 1 ? 5 : delta ? 4 : 3) * L.elems() * eb;
  if (opts->storage == ST3D_F16_HL) info->device_bytes += 2 * L.elems() * 2;
  if (opts->storage == ST3D_F16_HILO) info->device_bytes += 2 * L.elems();
  info->nk = L.nk; info->nj = L.nj; info->ni = L.ni;
  info->pk = L.pk; info->pj = L.pj; info->pi = L.pi;
  info->radius = R;
  // algorithmic bytes per point and step; a fused pass of T steps reads u,
  // v, s and writes two levels
  info->bytes_per_point = T > 1 ? 20.0 / T : f16_bytes(opts->storage, opts->points, eb);
  info->flops_per_point = opts->points == 2 ? 2 : opts->points == 7 ? 12 : opts->points == 13 ? 29 : 41;
  const int tj = opts->tile_j > 0 ? opts->tile_j : 16;
  const bool f16 = eb == 2;
  const bool tma = f16 || (opts->storage == ST3D_F32 && opts->points != 2 &&
                           opts->kernel != ST3D_KERNEL_SIMPLE && tma_config_supported(tj, 4));
  info->kernel = tma ? ST3D_KERNEL_TMA : ST3D_KERNEL_SIMPLE;
  info->tile_j = tma ? tj : 0;
  info->tile_k = tma ? kTmaTK : 0;
  if (delta && mma_chosen(*opts)) {
    info->kernel = ST3D_KERNEL_MMA;
    info->tile_j = 16;
    info->tile_k = kMmaTK;
  }
  info->ichunk = opts->ichunk > 0 ? opts->ichunk : (tma ? 128 : 64);
  info->temporal_block = opts->temporal_block > 0 ? opts->temporal_block : 1;
  info->device = opts->device;
  return ST3D_OK;
}

int st3d_create(const st3d_grid_desc* grid, const st3d_opts* opts, st3d_ctx** out) {
  return st3d::create_context(grid, opts, nullptr, out);
}

}  // extern "C"

// A context on the caller's stream (the batch runs all its grids on one
// stream); external == nullptr creates the context's own stream.
int st3d::create_context(const st3d_grid_desc* grid, const st3d_opts* opts, cudaStream_t external,
                         st3d_ctx** out) {
  if (!out) return fail(ST3D_ERR_INVALID, "null context pointer");
  *out = nullptr;
  int rc = validate(grid, opts);
  if (rc != ST3D_OK) return rc;
  if (opts->device >= 0) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return fail(ST3D_ERR_NODEVICE, "no CUDA device visible");
    }
    if (opts->device >= ndev)
      return fail(ST3D_ERR_INVALID, "device %d out of range (%d devices visible)", opts->device, ndev);
  }
  DeviceScope scope(opts->device);
  int sm = 0, ccM = 0, ccm = 0;
  size_t total = 0;
  rc = st3d_device_info(&sm, &ccM, &ccm, &total);
  if (rc != ST3D_OK) return rc;
  if (ccM != 10 || ccm != 3)
    return fail(ST3D_ERR_NODEVICE, "device has compute capability %d.%d; this library is built for sm_103a",
                ccM, ccm);
  st3d_ctx* c = new (std::nothrow) st3d_ctx();
  if (!c) return fail(ST3D_ERR_NOMEM, "host allocation failed");
  c->grid = *grid;
  c->opts = *opts;
  if (c->opts.temporal_block == 0) c->opts.temporal_block = 1;
  c->R = radius_of(opts->points);
  c->eb = elem_bytes(opts->storage);
  c->L = make_layout(grid->xs, grid->ys, grid->zs, c->eb);
  c->G = geom_of(c->L);
  cudaGetDevice(&c->device);
  if (c->opts.mode == ST3D_MODE_WAVE && c->opts.src_i == -2) {
    c->opts.src_i = (int)grid->xs / 2;
    c->opts.src_j = (int)grid->ys / 2;
    c->opts.src_k = (int)grid->zs / 2;
  }
  c->cf32 = make_coefs<float>(c->opts);
  c->cf64 = make_coefs<double>(c->opts);
  auto cleanup = [c](int status) {
    st3d_destroy(c);
    return status;
  };
  const size_t fbytes = c->L.elems() * c->eb;
  // buffers: u/v pair and s; the delta form adds d (3), a context that
  // blocks in time a second u/v pair (3, 4)
  c->delta = opts->storage == ST3D_F16 || opts->storage == ST3D_BF16 || opts->storage == ST3D_F16_HL;
  c->pair = opts->storage == ST3D_F16_HL;
  const int nbuf = c->opts.temporal_block > 1 ? 5 : c->delta ? 4 : 3;
  for (int f = 0; f < nbuf; ++f) {
    cudaError_t e = cudaMalloc(&c->fld[f], fbytes);
    if (e != cudaSuccess) {
      c->fld[f] = nullptr;
      cudaGetLastError();
      return cleanup(fail(ST3D_ERR_NOMEM, "cudaMalloc of %zu bytes for field %d failed", fbytes, f));
    }
    c->bytes += fbytes;
  }
  c->scratch_doubles = 4 * (size_t)norms_blocks(c->G) + 8;
  if (cudaMalloc(&c->scratch, c->scratch_doubles * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->counter, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&c->dev_status, sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(ST3D_ERR_NOMEM, "cudaMalloc of scratch failed"));
  }
  if (external) {
    c->stream = external;
    c->own_stream = false;
  } else if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(ST3D_ERR_CUDA, "stream creation failed"));
  }
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(ST3D_ERR_CUDA, "stream/event creation failed"));
  }
  for (int f = 0; f < nbuf; ++f)
    if (cudaMemsetAsync(c->fld[f], 0, fbytes, c->stream) != cudaSuccess)
      return cleanup(fail(ST3D_ERR_CUDA, "cudaMemsetAsync failed"));
  if (nbuf == 5) {
    if (cudaMalloc(&c->M, grid->xs * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&c->halo_max, sizeof(uint32_t)) != cudaSuccess) {
      cudaGetLastError();
      return cleanup(fail(ST3D_ERR_NOMEM, "cudaMalloc of the halo check buffers failed"));
    }
    rc = plan_tb(c, sm);
    if (rc != ST3D_OK) return cleanup(rc);
  }
  cudaMemsetAsync(c->dev_status, 0, sizeof(uint32_t), c->stream);

  c->f16 = c->eb == 2;
  if (c->f16) {
    const size_t xs = grid->xs;
    bool okm = true;
    // low parts per u/v buffer: one byte (F16_HILO) or one FP16 word (F16_HL)
    const size_t lob = c->opts.storage == ST3D_F16_HILO ? c->L.elems() : c->pair ? 2 * c->L.elems() : 0;
    if (lob)
      for (int f = 0; f < 2; ++f) {
        okm = okm && cudaMalloc(&c->lo[f], lob) == cudaSuccess;
        if (okm) {
          c->bytes += lob;
          cudaMemsetAsync(c->lo[f], 0, lob, c->stream);
        }
      }
    okm = okm && cudaMalloc(&c->E, 5 * xs * sizeof(int)) == cudaSuccess &&
          cudaMalloc(&c->M, 5 * xs * sizeof(uint32_t)) == cudaSuccess &&
          cudaMalloc(&c->halo_max, sizeof(uint32_t)) == cudaSuccess;
    if (!okm) {
      cudaGetLastError();
      return cleanup(fail(ST3D_ERR_NOMEM, "cudaMalloc of the 16-bit storage buffers failed"));
    }
    cudaMemsetAsync(c->E, 0, 5 * xs * sizeof(int), c->stream);
    cudaMemsetAsync(c->M, 0, 5 * xs * sizeof(uint32_t), c->stream);
    double wsum = 0.0;
    for (int m = 2; m < 14; ++m) wsum += c->opts.coef[m];
    c->k4 = (float)(4.0 * c->opts.c1 * wsum);
    // delta form: lap = sum_p w_p (a_p + b_p) + m2s * u
    double sw = 0.0;
    for (int p = 0; p < npairs_of(c->opts.points); ++p) sw += (double)c->cf32.cf[p];
    c->m2s = (float)(-2.0 * sw);
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    const bool mma = c->delta && mma_chosen(c->opts);
    rc = mma ? plan_mma16(c, sm, max_smem) : plan_tma16(c, sm, max_smem);
    if (rc != ST3D_OK) return cleanup(rc);
    c->kernel = mma ? ST3D_KERNEL_MMA : ST3D_KERNEL_TMA;
  }

  // kernel choice
  if (!c->f16) c->kernel = ST3D_KERNEL_SIMPLE;
  c->ichunk = c->opts.ichunk > 0 ? c->opts.ichunk : 64;
  if (c->opts.storage == ST3D_F32 && c->opts.points != 2 && c->opts.kernel != ST3D_KERNEL_SIMPLE) {
    int max_smem = 0;
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
    TmaPlan* p = new (std::nothrow) TmaPlan();
    if (p && plan_tma(c, sm, max_smem, p)) {
      int ok = ST3D_OK;
      for (int f = 0; f < 5 && ok == ST3D_OK; ++f) {
        if (!c->fld[f]) continue;
        ok = encode_map(&p->umap[f], c->fld[f], c->L, kTmaUKW, p->tj + 2 * c->R, kTmaKHalo,
                        c->L.pj);
        if (ok == ST3D_OK) ok = encode_map(&p->vmap[f], c->fld[f], c->L, kTmaTK, p->tj, 0, 0);
      }
      if (ok == ST3D_OK) {
        c->tma = p;
        c->kernel = ST3D_KERNEL_TMA;
      } else {
        delete p;
        if (c->opts.kernel == ST3D_KERNEL_TMA) return cleanup(ok);
      }
    } else {
      delete p;
      if (c->opts.kernel == ST3D_KERNEL_TMA)
        return cleanup(fail(ST3D_ERR_UNSUPPORTED,
                            "the TMA kernel cannot run with this configuration"));
    }
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    return cleanup(fail(ST3D_ERR_CUDA, "initial synchronize failed"));
  *out = c;
  return ST3D_OK;
}

extern "C" {

int st3d_destroy(st3d_ctx* c) {
  if (!c) return ST3D_OK;
  DeviceScope scope(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int f = 0; f < 5; ++f)
    if (c->fld[f]) cudaFree(c->fld[f]);
  delete c->tb;
  if (c->scratch) cudaFree(c->scratch);
  if (c->counter) cudaFree(c->counter);
  if (c->dev_status) cudaFree(c->dev_status);
  if (c->stage) cudaFree(c->stage);
  if (c->stream_buf) cudaFree(c->stream_buf);
  for (int f = 0; f < 2; ++f)
    if (c->lo[f]) cudaFree(c->lo[f]);
  if (c->E) cudaFree(c->E);
  if (c->M) cudaFree(c->M);
  if (c->halo_max) cudaFree(c->halo_max);
  if (c->tma16 && c->tma16->mma_rec) cudaFree(c->tma16->mma_rec);
  delete c->tma16;
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream && c->own_stream) cudaStreamDestroy(c->stream);
  delete c->tma;
  delete c;
  return ST3D_OK;
}

int st3d_get_info(const st3d_ctx* c, st3d_info* info) {
  if (!c || !info) return fail(ST3D_ERR_INVALID, "null argument");
  memset(info, 0, sizeof *info);
  info->interior_points = (uint64_t)c->grid.xs * c->grid.ys * c->grid.zs;
  info->device_bytes = c->bytes;
  info->step = c->step;
  info->launches = c->launches;
  info->nk = c->L.nk; info->nj = c->L.nj; info->ni = c->L.ni;
  info->pk = c->L.pk; info->pj = c->L.pj; info->pi = c->L.pi;
  info->kernel = c->kernel;
  info->radius = c->R;
  info->bytes_per_point = c->tb ? 20.0 / c->tb->T : f16_bytes(c->opts.storage, c->opts.points, c->eb);
  info->flops_per_point = c->opts.points == 2 ? 2 : c->opts.points == 7 ? 12 : c->opts.points == 13 ? 29 : 41;
  info->tile_j = c->tma ? c->tma->tj : c->tma16 ? c->tma16->tj : 0;
  info->tile_k = (c->tma16 && c->tma16->mma) ? kMmaTK : (c->tma || c->tma16) ? kTmaTK : 0;
  info->ichunk = c->tma ? c->tma->ichunk : c->tma16 ? c->tma16->ichunk : c->ichunk;
  info->temporal_block = c->opts.temporal_block;
  info->host_path = c->host_path;
  info->tb_tile_j = c->tb ? c->tb->rows : 0;
  info->device = c->device;
  return ST3D_OK;
}

int st3d_set_step(st3d_ctx* c, uint64_t step) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  c->step = step;
  return ST3D_OK;
}

int st3d_transfer(st3d_ctx* dst, st3d_ctx* src) {
  if (!dst || !src) return fail(ST3D_ERR_INVALID, "null context");
  if (dst == src) return fail(ST3D_ERR_INVALID, "transfer needs two contexts");
  const st3d_grid_desc &a = dst->grid, &b = src->grid;
  if (a.xs != b.xs || a.ys != b.ys || a.zs != b.zs || a.xh != b.xh || a.yh != b.yh || a.zh != b.zh)
    return fail(ST3D_ERR_INVALID, "transfer between different grids");
  if (dst->opts.mode != src->opts.mode) return fail(ST3D_ERR_INVALID, "transfer between different modes");
  if (host_elem_bytes(dst->opts.storage) != host_elem_bytes(src->opts.storage))
    return fail(ST3D_ERR_UNSUPPORTED, "transfer between FP64 and FP32-valued storages");
  if (dst->device != src->device) return fail(ST3D_ERR_UNSUPPORTED, "transfer across devices");
  DeviceScope scope(src->device);
  if (!(src->has_u && src->has_v)) return fail(ST3D_ERR_STATE, "the source context holds no u and v");
  const size_t bytes = host_array_bytes(src);
  void* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 2 * bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ST3D_ERR_NOMEM, "transfer buffers (%zu bytes): %s", 2 * bytes, cudaGetErrorString(e));
  }
  void* vb = buf;
  void* ub = static_cast<char*>(buf) + bytes;
  const uint64_t step = src->step;
  int rc = ST3D_OK;
  // zero halos; the download writes the interior rows with their k halo
  e = cudaMemsetAsync(buf, 0, 2 * bytes, src->stream);
  if (e != cudaSuccess) rc = cuda_fail(e, "transfer buffer clear");
  if (rc == ST3D_OK) rc = st3d_download(src, vb, ub);  // synchronizes src's stream
  if (rc == ST3D_OK) rc = st3d_upload(dst, vb, nullptr, ub);
  if (rc == ST3D_OK) {
    e = cudaStreamSynchronize(dst->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "transfer upload");
  }
  if (rc == ST3D_OK) dst->step = step;
  cudaFree(buf);
  return rc;
}

int st3d_get_stream(const st3d_ctx* c, void** s) {
  if (!c || !s) return fail(ST3D_ERR_INVALID, "null argument");
  *s = (void*)c->stream;
  return ST3D_OK;
}

int st3d_upload(st3d_ctx* c, const void* v, const void* s, const void* u) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  int rc;
  if (c->delta) {
    c->step = 0;
    if ((rc = ensure_stage(c, 2)) != ST3D_OK) return rc;
    if (u || v) {
      if (!(u && v) && !c->pair_valid && (rc = delta_rebuild_pair(c)) != ST3D_OK) return rc;
      c->pair_valid = false;
      if (u)
        ST3D_CUDA(cudaMemcpyAsync(stage_slot(c, 0), u, host_array_bytes(c), cudaMemcpyDefault,
                                  c->stream));
      if (v)
        ST3D_CUDA(cudaMemcpyAsync(stage_slot(c, 1), v, host_array_bytes(c), cudaMemcpyDefault,
                                  c->stream));
      if ((rc = delta_encode_pair(c, u != nullptr)) != ST3D_OK) return rc;
      if (u) c->has_u = true;
      if (v) c->has_v = true;
    }
    if (s) {
      c->pair_valid = false;  // s passes through slot 0
      ST3D_CUDA(cudaMemcpyAsync(stage_slot(c, 0), s, host_array_bytes(c), cudaMemcpyDefault,
                                c->stream));
      if ((rc = encode_staged16(c, stage_slot(c, 0), nullptr, c->fld[2], M_s(c), E_s(c), "s")) !=
          ST3D_OK)
        return rc;
      c->has_s = true;
    }
    return ST3D_OK;
  }
  if (c->f16) {
    c->step = 0;
    if (u) {
      if ((rc = upload_field16(c, 0, u)) != ST3D_OK) return rc;
      c->has_u = true;
    }
    if (v) {
      if ((rc = upload_field16(c, 1, v)) != ST3D_OK) return rc;
      c->has_v = true;
    }
    if (s) {
      if ((rc = upload_field16(c, 2, s)) != ST3D_OK) return rc;
      c->has_s = true;
    }
    ST3D_CUDA(cudaMemsetAsync(M_level(c, (long long)c->lvl + 1), 0, c->grid.xs * sizeof(uint32_t), c->stream));
    ST3D_CUDA(cudaMemsetAsync(M_level(c, (long long)c->lvl + 2), 0, c->grid.xs * sizeof(uint32_t), c->stream));
    return ST3D_OK;
  }
  if (u) {
    if ((rc = upload_field(c, u_ptr(c), u)) != ST3D_OK) return rc;
    c->has_u = true;
  }
  if (v) {
    if ((rc = upload_field(c, v_ptr(c), v)) != ST3D_OK) return rc;
    c->has_v = true;
  }
  if (s) {
    if ((rc = upload_field(c, c->fld[2], s)) != ST3D_OK) return rc;
    c->has_s = true;
  }
  c->step = 0;
  return ST3D_OK;
}

int st3d_download(st3d_ctx* c, void* v, void* u) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  int rc;
  if (c->delta) {
    if (v && (rc = delta_download(c, v, true)) != ST3D_OK) return rc;
    if (u && (rc = delta_download(c, u, false)) != ST3D_OK) return rc;
    ST3D_CUDA(cudaStreamSynchronize(c->stream));
    return ST3D_OK;
  }
  if (c->f16) {
    if (v && (rc = download_field16(c, 1, v)) != ST3D_OK) return rc;
    if (u && (rc = download_field16(c, 0, u)) != ST3D_OK) return rc;
    ST3D_CUDA(cudaStreamSynchronize(c->stream));
    return ST3D_OK;
  }
  if (v && (rc = download_field(c, v_ptr(c), v)) != ST3D_OK) return rc;
  if (u && (rc = download_field(c, u_ptr(c), u)) != ST3D_OK) return rc;
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  return ST3D_OK;
}

int st3d_iterate(st3d_ctx* c, uint32_t iterations) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  if (!(c->has_u && c->has_v && c->has_s))
    return fail(ST3D_ERR_STATE, "upload or fill u, v and s before iterating");
  const bool wave = c->opts.mode == ST3D_MODE_WAVE;
  // fused passes of T steps while at least T remain, then single steps
  while (c->tb && iterations >= (uint32_t)c->tb->T) {
    const int T = c->tb->T;
    Source src;
    src.i = c->opts.src_i; src.j = c->opts.src_j; src.k = c->opts.src_k;
    src.amp = 0.0f; src.amp_d = 0.0;
    float amps[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int t = 0; t < T; ++t)
      if (src.i >= 0)
        amps[t] = (float)st3d_ricker((double)(c->step + t) * c->opts.dt, c->opts.src_f, c->opts.src_t0);
    int o1 = -1, o2 = -1;  // the pair not holding the state
    for (int b : {0, 1, 3, 4})
      if (b != c->ub && b != c->vb) (o1 < 0 ? o1 : o2) = b;
    cudaError_t e = launch_tb(c->opts.points, T, *c->tb, c->G, c->cf32, (float*)c->fld[o1],
                              (float*)c->fld[o2], c->ub, c->vb, src, amps, c->dev_status, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "temporally blocked kernel launch");
    c->vb = o1;
    c->ub = o2;
    c->step += T;
    c->lvl += T;
    ++c->launches;
    iterations -= T;
  }
  for (uint32_t n = 0; n < iterations; ++n) {
    Source src;
    src.i = -1; src.j = -1; src.k = -1; src.amp = 0.0f; src.amp_d = 0.0;
    if (wave && c->opts.src_i >= 0) {
      src.i = c->opts.src_i; src.j = c->opts.src_j; src.k = c->opts.src_k;
      src.amp_d = st3d_ricker((double)c->step * c->opts.dt, c->opts.src_f, c->opts.src_t0);
      src.amp = (float)src.amp_d;
    }
    cudaError_t e;
    if (c->delta) {
      Delta16Step st;
      const int ub = c->ub, un = 1 - c->ub;
      st.uout = (uint16_t*)c->fld[un];
      st.d = (uint16_t*)c->fld[3];
      st.Eu = Eu_buf(c, ub);
      st.Ed = Ed_lvl(c, c->lvl);
      st.Es = E_s(c);
      st.Eu_out = Eu_buf(c, un);
      st.Ed_out = Ed_lvl(c, c->lvl + 1);
      st.Mu = Mu_buf(c, ub);
      st.Md = Md_lvl(c, c->lvl);
      st.Ms = M_s(c);
      st.Mu_out = Mu_buf(c, un);
      st.Md_out = Md_lvl(c, c->lvl + 1);
      st.k4 = c->k4;
      st.m2s = c->m2s;
      st.ubuf = ub;
      st.lout = c->pair ? (uint16_t*)c->lo[un] : nullptr;
      e = c->tma16->mma ? launch_mma16(c->opts.storage, c->opts.points, *c->tma16, c->G, c->cf32, st,
                                       src, c->dev_status, c->stream)
                        : launch_delta16(c->opts.storage, c->opts.points, *c->tma16, c->G, c->cf32, st,
                                         src, c->dev_status, c->stream);
      c->pair_valid = false;
    } else if (c->f16) {
      const long long n = (long long)c->lvl;
      Tma16Step st;
      st.vout = (uint16_t*)v_ptr(c);
      st.vlo_out = (int8_t*)c->lo[v_index(c)];
      st.Eu = E_level(c, n);
      st.Ev = E_level(c, n - 1);
      st.Es = E_s(c);
      st.Eout = E_level(c, n + 1);
      st.Mu = M_level(c, n);
      st.Mv = M_level(c, n - 1);
      st.Ms = M_s(c);
      st.Mout = M_level(c, n + 1);
      st.Mzero = M_level(c, n + 2);
      st.k4 = c->k4;
      st.ubuf = u_index(c);
      st.vbuf = v_index(c);
      e = launch_tma16(c->opts.storage, c->opts.points, *c->tma16, c->G, c->cf32, st, src,
                       c->dev_status, c->stream);
    } else if (c->kernel == ST3D_KERNEL_TMA) {
      e = launch_tma(*c->tma, c->opts.points, c->opts.mode, c->G, c->cf32, (float*)v_ptr(c),
                     u_index(c), v_index(c), 2, src, c->dev_status, c->stream);
    } else {
      const void* cf = c->opts.storage == ST3D_F64 ? (const void*)&c->cf64 : (const void*)&c->cf32;
      e = launch_simple(c->opts.points, c->opts.mode, c->opts.storage, c->G, cf, v_ptr(c),
                        u_ptr(c), c->fld[2], src, c->ichunk, c->stream);
    }
    if (e != cudaSuccess) return cuda_fail(e, "stencil kernel launch");
    ++c->launches;
    ++c->step;
    ++c->lvl;
    if (wave) {
      const int t = c->ub;
      c->ub = c->vb;
      c->vb = t;
    }
  }
  return ST3D_OK;
}

int st3d_synchronize(st3d_ctx* c) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  return check_device_status(c);
}

int st3d_inject_device_status(st3d_ctx* c, uint32_t code) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  ST3D_CUDA(cudaMemsetAsync(c->dev_status, 0, sizeof(uint32_t), c->stream));
  if (code != 0)
    ST3D_CUDA(cudaMemcpyAsync(c->dev_status, &code, sizeof code, cudaMemcpyHostToDevice, c->stream));
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  return ST3D_OK;
}

int st3d_iterate_host(st3d_ctx* c, void* v, const void* s, void* u, uint32_t iterations) {
  if (!c || !v || !s || !u) return fail(ST3D_ERR_INVALID, "null argument");
  DeviceScope scope(c->device);
  bool streamed = false;
  int rc = iterate_host_streamed(c, v, s, u, iterations, &streamed);
  if (rc != ST3D_OK) return rc;
  if (streamed) return st3d_synchronize(c);
  rc = st3d_upload(c, v, s, u);
  if (rc == ST3D_OK) rc = st3d_iterate(c, iterations);
  if (rc == ST3D_OK)
    rc = st3d_download(c, v, c->opts.mode == ST3D_MODE_WAVE ? u : nullptr);
  if (rc == ST3D_OK) rc = st3d_synchronize(c);
  return rc;
}

int st3d_fill(st3d_ctx* c, int field, int kind, uint64_t seed, double a, double b) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  if (field < ST3D_FIELD_U || field > ST3D_FIELD_S) return fail(ST3D_ERR_INVALID, "bad field %d", field);
  if (kind < ST3D_FILL_CONST || kind > ST3D_FILL_BLOBS) return fail(ST3D_ERR_INVALID, "bad fill kind %d", kind);
  void* dst = field == ST3D_FIELD_U ? u_ptr(c) : field == ST3D_FIELD_V ? v_ptr(c) : c->fld[2];
  double bp[4 * 16];
  int nb = 0;
  if (kind == ST3D_FILL_BLOBS) {
    nb = (int)a;
    if (nb < 0 || nb > 16) return fail(ST3D_ERR_INVALID, "1..16 blobs (got %d)", nb);
    if (!(b > 0)) return fail(ST3D_ERR_INVALID, "blob width must be positive");
    // Same parameter stream as the seeded host generator: draw n of
    // splitmix64(seed + (n+1)*golden), top 24 bits.
    auto mix64 = [](uint64_t z) {
      z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ULL;
      z ^= z >> 27; z *= 0x94D049BB133111EBULL;
      z ^= z >> 31;
      return z;
    };
    auto unit = [&](unsigned n) {
      return (double)(mix64(seed + (uint64_t)(n + 1) * 0x9E3779B97F4A7C15ULL) >> 40) *
             (1.0 / 16777216.0);
    };
    for (int q = 0; q < nb; ++q) {
      bp[4 * q + 0] = unit(4 * q + 0) * c->grid.xs;
      bp[4 * q + 1] = unit(4 * q + 1) * c->grid.ys;
      bp[4 * q + 2] = unit(4 * q + 2) * c->grid.zs;
      bp[4 * q + 3] = 2.0 * unit(4 * q + 3) - 1.0;
    }
  }
  if (c->delta) {
    // fill the field's staging slot (FP32, reference layout, interior only:
    // the 16-bit forms keep a zero halo), then encode like an upload
    int rc = ensure_stage(c, 2);
    if (rc != ST3D_OK) return rc;
    if (field != ST3D_FIELD_S && !c->pair_valid && (rc = delta_rebuild_pair(c)) != ST3D_OK) return rc;
    const st3d_grid_desc& g = c->grid;
    Layout Lr;
    Lr.xs = g.xs; Lr.ys = g.ys; Lr.zs = g.zs;
    Lr.pk = g.zh; Lr.pj = g.yh; Lr.pi = g.xh;
    Lr.nk = g.zs + 2 * g.zh; Lr.nj = g.ys + 2 * g.yh; Lr.ni = g.xs + 2 * g.xh;
    c->step = 0;
    const int slot = field == ST3D_FIELD_V ? 1 : 0;
    if (field == ST3D_FIELD_S) c->pair_valid = false;  // s passes through slot 0
    cudaError_t e = launch_fill(ST3D_F32, Lr, stage_slot(c, slot), kind, seed, (unsigned)field, a, b,
                                bp, nb, 1, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "fill kernel launch");
    if (field == ST3D_FIELD_S)
      rc = encode_staged16(c, stage_slot(c, 0), nullptr, c->fld[2], M_s(c), E_s(c), "s");
    else
      rc = delta_encode_pair(c, field == ST3D_FIELD_U);
    if (rc != ST3D_OK) return rc;
  } else if (c->f16) {
    // fill the float staging buffer (reference layout, interior only: the
    // 16-bit forms keep a zero halo), then encode like an upload
    int rc = ensure_stage(c);
    if (rc != ST3D_OK) return rc;
    const st3d_grid_desc& g = c->grid;
    Layout Lr;
    Lr.xs = g.xs; Lr.ys = g.ys; Lr.zs = g.zs;
    Lr.pk = g.zh; Lr.pj = g.yh; Lr.pi = g.xh;
    Lr.nk = g.zs + 2 * g.zh; Lr.nj = g.ys + 2 * g.yh; Lr.ni = g.xs + 2 * g.xh;
    cudaError_t e = launch_fill(ST3D_F32, Lr, c->stage, kind, seed, (unsigned)field, a, b, bp, nb, 1,
                                c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "fill kernel launch");
    const int which = field == ST3D_FIELD_U ? 0 : field == ST3D_FIELD_V ? 1 : 2;
    c->step = 0;
    if ((rc = upload_field16(c, which, nullptr)) != ST3D_OK) return rc;
    ST3D_CUDA(cudaMemsetAsync(M_level(c, (long long)c->lvl + 1), 0, c->grid.xs * sizeof(uint32_t), c->stream));
    ST3D_CUDA(cudaMemsetAsync(M_level(c, (long long)c->lvl + 2), 0, c->grid.xs * sizeof(uint32_t), c->stream));
  } else {
    // a context that blocks in time keeps a zero halo
    cudaError_t e = launch_fill(c->opts.storage, c->L, dst, kind, seed, (unsigned)field, a, b, bp,
                                nb, c->tb ? 1 : 0, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "fill kernel launch");
  }
  if (field == ST3D_FIELD_U) c->has_u = true;
  if (field == ST3D_FIELD_V) c->has_v = true;
  if (field == ST3D_FIELD_S) c->has_s = true;
  c->step = 0;
  return ST3D_OK;
}

int st3d_check(st3d_ctx* c, double expected, double tol, uint64_t* errors) {
  if (!c || !errors) return fail(ST3D_ERR_INVALID, "null argument");
  DeviceScope scope(c->device);
  ST3D_CUDA(cudaMemsetAsync(c->counter, 0, sizeof(unsigned long long), c->stream));
  cudaError_t e = launch_check(c->G, field_ref(c, ST3D_FIELD_V), expected, tol, c->counter, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "check kernel launch");
  unsigned long long n = 0;
  ST3D_CUDA(cudaMemcpyAsync(&n, c->counter, sizeof n, cudaMemcpyDeviceToHost, c->stream));
  ST3D_CUDA(cudaStreamSynchronize(c->stream));
  *errors = n;
  return ST3D_OK;
}

int st3d_norms(st3d_ctx* a, int fa, st3d_ctx* b, int fb, double out[4]) {
  if (!a || !out) return fail(ST3D_ERR_INVALID, "null argument");
  if (b && b->device != a->device) return fail(ST3D_ERR_UNSUPPORTED, "norms across devices");
  DeviceScope scope(a->device);
  if (b && (b->grid.xs != a->grid.xs || b->grid.ys != a->grid.ys || b->grid.zs != a->grid.zs))
    return fail(ST3D_ERR_INVALID, "norms need equal interior sizes");
  if (fa < 0 || fa > 2 || (b && (fb < 0 || fb > 2))) return fail(ST3D_ERR_INVALID, "bad field");
  if (b && b->stream != a->stream) ST3D_CUDA(cudaStreamSynchronize(b->stream));
  const int nb = norms_blocks(a->G);
  FieldRef ra = field_ref(a, fa);
  FieldRef rb;
  rb.p = nullptr; rb.storage = 0; rb.lo = nullptr; rb.E = nullptr;
  if (b) rb = field_ref(b, fb);
  cudaError_t e = launch_norms(a->G, ra, b ? b->G : a->G, rb, a->scratch, nb,
                               a->scratch + 4 * (size_t)nb, a->stream);
  if (e != cudaSuccess) return cuda_fail(e, "norms kernel launch");
  double h[4];
  ST3D_CUDA(cudaMemcpyAsync(h, a->scratch + 4 * (size_t)nb, sizeof h, cudaMemcpyDeviceToHost, a->stream));
  ST3D_CUDA(cudaStreamSynchronize(a->stream));
  if (!b) {  // energy form: sum a^2 and max |a|
    out[0] = h[0]; out[1] = 0.0; out[2] = h[2]; out[3] = 0.0;
  } else {
    for (int q = 0; q < 4; ++q) out[q] = h[q];
  }
  return ST3D_OK;
}

int st3d_timer_start(st3d_ctx* c) {
  if (!c) return fail(ST3D_ERR_INVALID, "null context");
  DeviceScope scope(c->device);
  ST3D_CUDA(cudaEventRecord(c->ev0, c->stream));
  c->timer_step0 = c->lvl;
  return ST3D_OK;
}

int st3d_timer_stop(st3d_ctx* c, float* ms) {
  if (!c || !ms) return fail(ST3D_ERR_INVALID, "null argument");
  DeviceScope scope(c->device);
  ST3D_CUDA(cudaEventRecord(c->ev1, c->stream));
  ST3D_CUDA(cudaEventSynchronize(c->ev1));
  ST3D_CUDA(cudaEventElapsedTime(ms, c->ev0, c->ev1));
  c->timed_ms = *ms;
  c->timed_steps = c->lvl - c->timer_step0;
  return ST3D_OK;
}

int st3d_metrics_get(st3d_ctx* c, st3d_ctx* ref, st3d_metrics* m) {
  if (!c || !m) return fail(ST3D_ERR_INVALID, "null argument");
  DeviceScope scope(c->device);
  memset(m, 0, sizeof *m);
  m->steps = c->step;
  m->timed_steps = c->timed_steps;
  m->elapsed_ms = c->timed_ms;
  const double pts = (double)c->grid.xs * c->grid.ys * c->grid.zs;
  if (c->timed_ms > 0.0f && c->timed_steps > 0) {
    const double per_s = pts * (double)c->timed_steps / (c->timed_ms * 1e-3);
    const int P = c->opts.points;
    const double flops = P == 2 ? 2 : P == 7 ? 12 : P == 13 ? 29 : 41;  // config.h:67-91
    const double mem_reals = P == 2 ? 2 : 4;
    m->gpts = per_s * 1e-9;
    m->gflops = per_s * flops * 1e-9;
    m->mem_gbs = per_s * mem_reals * host_elem_bytes(c->opts.storage) * 1e-9;
  }
  double out[4];
  int rc = st3d_norms(c, ST3D_FIELD_U, nullptr, ST3D_FIELD_U, out);
  if (rc != ST3D_OK) return rc;
  m->energy_u = out[0];
  m->max_abs_u = out[2];
  m->rel_l2 = -1.0;
  if (ref) {
    if ((rc = st3d_norms(c, ST3D_FIELD_U, ref, ST3D_FIELD_U, out)) != ST3D_OK) return rc;
    m->rel_l2 = out[1] > 0.0 ? sqrt(out[0] / out[1]) : sqrt(out[0]);
  }
  return ST3D_OK;
}

int st3d_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return fail(ST3D_ERR_INVALID, "null pointer");
  *ptr = nullptr;
  cudaError_t e = cudaMallocHost(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(ST3D_ERR_NOMEM, "cudaMallocHost(%zu) failed: %s", bytes, cudaGetErrorString(e));
  }
  return ST3D_OK;
}

int st3d_host_free(void* ptr) {
  if (ptr) ST3D_CUDA(cudaFreeHost(ptr));
  return ST3D_OK;
}

}  // extern "C"
