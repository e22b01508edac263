// gstencil3d -- the hstencil3d command line on one GB300.
//
// Same flags, limits, phase log, known-answer checks and report line as the
// reference driver (main.cpp:94-332): the time loop runs on the GPU through
// the C ABI, every other step stays on the host.  The stencil size, CPU
// traversal (PAR2D/HILBERT/...) and `real` are compile-time choices in the
// reference (config.h:19-65, 96-100); here the stencil is a run-time flag,
// the traversal flags are accepted and ignored, and `real` follows
// USE_DOUBLE as in the reference (the double build runs the FP64 storage).
//
// Added flags: --stencil N (2, 7, 13, 25; default 7 as config.h:38),
// --wave (the leapfrog form, README.md:11-20, with --vel/--dt/--dx),
// --kernel simple|tma|mma|auto, --variant ref|vec8|vec16 (the reference's
// compile-time kernel variant whose results to reproduce), --storage
// f32|f16|bf16|f16_hilo|f16_hl (device storage of the wave form) and
// --temporal-block 1|2|4 (FP32 wave steps fused per pass).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "st3d_compat.hpp"

namespace {

constexpr unsigned kDefaultHaloXY = 4;    // config.h:4
constexpr unsigned kDefaultHaloZ = 16;    // config.h:5
constexpr unsigned kDefaultSizeXY = 945;  // config.h:6
constexpr unsigned kDefaultSizeZ = 880;   // config.h:7
constexpr unsigned kDefaultOfs = 16;      // config.h:8
constexpr unsigned kDefaultIter = 100;    // config.h:9

// Zero every halo point of a field in the reference layout.
void zero_halo(real* a, const s_grid& g) {
  const long long ni = g.xsize + 2LL * g.xhalo, nj = g.ysize + 2LL * g.yhalo, nk = g.zsize + 2LL * g.zhalo;
  for (long long i = 0; i < ni; ++i)
    for (long long j = 0; j < nj; ++j)
      for (long long k = 0; k < nk; ++k) {
        const bool inner = i >= g.xhalo && i < g.xhalo + g.xsize && j >= g.yhalo &&
                           j < g.yhalo + g.ysize && k >= g.zhalo && k < g.zhalo + g.zsize;
        if (!inner) a[(i * nj + j) * nk + k] = 0.0f;
      }
}

double flops_per_stencil(int points) {  // config.h:67-91
  return points == 2 ? 2 : points == 7 ? 12 : points == 13 ? 29 : 41;
}
double mem_reals_per_stencil(int points) { return points == 2 ? 2 : 4; }
double cache_reals_per_stencil(int points) {
  return points == 2 ? 2 : points == 7 ? 10 : points == 13 ? 16 : 28;
}

}  // namespace

int main(int argc, char** argv) {
  unsigned train = 0, wave = 0;
  unsigned offset = kDefaultOfs;
  unsigned maxiter = kDefaultIter;
  unsigned cacheiter = 1, dups = 1, prefetch = 64;
  unsigned xs = kDefaultSizeXY, ys = kDefaultSizeXY, zs = kDefaultSizeZ;
  unsigned xh = kDefaultHaloXY, yh = kDefaultHaloXY, zh = kDefaultHaloZ;
  unsigned xb = 1, yb = 1, zb = 16;
  unsigned jshuffle = 13, kshuffle = 3;
  unsigned points = 7;
  real sbm = 12;
  const char* kernel = "auto";
  const char* variant = "ref";
  const char* storage = sizeof(real) == sizeof(double) ? "f64" : "f32";
  unsigned tblock = 1;
  gb300_options gopt;

  int iarg = 1;
  while (iarg < argc) {
    int args = 0;
    args += get_int_arg(argv, iarg, argc, "--iter", maxiter, 1, 100000, 1);
    args += get_int_arg(argv, iarg, argc, "--citer", cacheiter, 1, 100000, 1);
    args += get_int_arg(argv, iarg, argc, "--dups", dups, 1, 64, 1);
    args += get_int_arg(argv, iarg, argc, "--ofs", offset, 0, 16384, 1);
    args += get_int_arg(argv, iarg, argc, "--pref", prefetch, 1, 512, 1);
    args += get_int_arg(argv, iarg, argc, "--xh", xh, 4, 16, 1);
    args += get_int_arg(argv, iarg, argc, "--yh", yh, 4, 16, 1);
    args += get_int_arg(argv, iarg, argc, "--zh", zh, 1, 16, 1);
    args += get_int_arg(argv, iarg, argc, "--xs", xs, 1, 1264, 1);
    args += get_int_arg(argv, iarg, argc, "--ys", ys, 1, 1264, 1);
    args += get_int_arg(argv, iarg, argc, "--zs", zs, 1, 1264, 1);
    args += get_int_arg(argv, iarg, argc, "--xb", xb, 1, 1264, 1);
    args += get_int_arg(argv, iarg, argc, "--yb", yb, 1, 1264, 1);
    args += get_int_arg(argv, iarg, argc, "--zb", zb, 1, 1264, 1);
    args += get_real_arg(argv, iarg, argc, "--sbm", sbm, 1.0, 10.0);
    args += get_flag(argv, iarg, argc, "--train", train);
    args += get_int_arg(argv, iarg, argc, "--stencil", points, 2, 25, 1);
    args += get_flag(argv, iarg, argc, "--wave", wave);
    args += get_double_arg(argv, iarg, argc, "--vel", gopt.vel, 1.0, 1e5);
    args += get_double_arg(argv, iarg, argc, "--dt", gopt.dt, 1e-9, 1.0);
    args += get_double_arg(argv, iarg, argc, "--dx", gopt.dx, 1e-6, 1e6);
    args += get_str_arg(argv, iarg, argc, "--kernel", kernel);
    args += get_str_arg(argv, iarg, argc, "--variant", variant);
    args += get_str_arg(argv, iarg, argc, "--storage", storage);
    args += get_int_arg(argv, iarg, argc, "--temporal-block", tblock, 1, 4, 1);
    if (args > 0) {
      iarg += args;
    } else {
      fprintf(stderr, "unsupported argument %s\n", argv[iarg]);
      return 2;
    }
  }
  if (points != 2 && points != 7 && points != 13 && points != 25) {
    fprintf(stderr, "--stencil must be 2, 7, 13 or 25\n");
    return 2;
  }
  if ((ys % yb) != 0) {  // main.cpp:171-174
    fprintf(stderr, "ERROR: --ys must by an exact multiple of --yb\n");
    exit(2);
  }
  const unsigned radius = points == 25 ? 4 : points == 13 ? 2 : 1;
  if (zh < radius) {
    fprintf(stderr, "--zh must be larger or equal to %u for the %u-point stencil\n", radius, points);
    exit(2);
  }
  // --variant names the reference's compile-time SUBTYPE/VLEN kernel whose
  // results to reproduce: all have the ref kernel's arithmetic except the
  // 13-point vec_16 kernel, whose K is 6.25 (stencil_13.h:391, 428)
  if (strcmp(variant, "ref") != 0 && strcmp(variant, "vec16") != 0 && strcmp(variant, "vec8") != 0) {
    fprintf(stderr, "--variant must be ref, vec8 or vec16\n");
    return 2;
  }
  if (points == 13 && strcmp(variant, "vec16") == 0 && !wave) gopt.K = 6.25;
  // host arrays are `real`: double in the USE_DOUBLE build (FP64 storage),
  // else float (FP32 or one of the 16-bit device storages)
  if (sizeof(real) == sizeof(double)) {
    if (strcmp(storage, "f64") != 0) {
      fprintf(stderr, "--storage %s needs the float build (this one has USE_DOUBLE)\n", storage);
      return 2;
    }
    gopt.storage = ST3D_F64;
  } else if (strcmp(storage, "f32") == 0) gopt.storage = ST3D_F32;
  else if (strcmp(storage, "f16") == 0) gopt.storage = ST3D_F16;
  else if (strcmp(storage, "bf16") == 0) gopt.storage = ST3D_BF16;
  else if (strcmp(storage, "f16_hilo") == 0) gopt.storage = ST3D_F16_HILO;
  else if (strcmp(storage, "f16_hl") == 0) gopt.storage = ST3D_F16_HL;
  else {
    fprintf(stderr, "--storage must be f32, f16, bf16, f16_hilo or f16_hl\n");
    return 2;
  }
  if (gopt.storage != ST3D_F32 && gopt.storage != ST3D_F64 && !wave) {
    fprintf(stderr, "--storage %s needs --wave\n", storage);
    return 2;
  }
  gopt.temporal_block = (int)tblock;
  gopt.points = (int)points;
  gopt.mode = wave ? ST3D_MODE_WAVE : ST3D_MODE_REF;
  gopt.kernel = strcmp(kernel, "simple") == 0 ? ST3D_KERNEL_SIMPLE
              : strcmp(kernel, "tma") == 0    ? ST3D_KERNEL_TMA
              : strcmp(kernel, "mma") == 0    ? ST3D_KERNEL_MMA
                                              : ST3D_KERNEL_AUTO;
  gb300_configure(gopt);

  s_grid grid(xs, ys, zs, xh, yh, zh, xb, yb, zb, sbm, jshuffle, kshuffle);
  const double flops = flops_per_stencil(points) * 1.0e-9 * (double)grid.gvol * maxiter * cacheiter;
  const double mem_bytes =
      mem_reals_per_stencil(points) * sizeof(real) * 1.0e-9 * (double)grid.gvol * maxiter * cacheiter;
  const double cache_bytes =
      cache_reals_per_stencil(points) * sizeof(real) * 1.0e-9 * (double)grid.gvol * maxiter * cacheiter;
  const int my_rank = 0;
  int phase = 0;

  printf("running STENCIL(%d) benchmark: \n", points);
  printf(" -- using a grid size of %dx%dx%d with a halo of %dx%dx%d elements totaling %f GB\n",
         grid.xsize, grid.ysize, grid.zsize, grid.xhalo, grid.yhalo, grid.zhalo,
         1e-9 * (double)grid.gsize * sizeof(real));
  printf(" -- using block tile size of %d x %d x %d\n", grid.xb_size, grid.yb_size, grid.zb_size);
  printf(" -- GB300: %s form, %s kernel, %s storage, %u step(s) per pass, one GPU\n",
         wave ? "leapfrog wave" : "reference", kernel, storage, tblock);

  // pinned host arrays, shifted like main.cpp:272-275
  const size_t page = 1UL << 16;
  const size_t asize = (((grid.gsize + 64 * (size_t)offset) * sizeof(real) / page) + 1) * page;
  real *ov = nullptr, *os = nullptr, *ou = nullptr;
  if (st3d_host_alloc(asize, (void**)&ov) || st3d_host_alloc(asize, (void**)&os) ||
      st3d_host_alloc(asize, (void**)&ou)) {
    fprintf(stderr, "error allocating host arrays: %s\n", st3d_last_error());
    exit(3);
  }
  real* v = ov;
  real* s = os + (size_t)offset * 13;
  real* u = ou + (size_t)offset * 42;

  printf("[rank%i] Phase #%i: array initialization\n", my_rank, ++phase);
  double t0 = seconds();
  init_arrays(ov, os, ou, asize / sizeof(real));
  // the 16-bit storages and fused steps hold a zero (Dirichlet) boundary
  if (wave && ((gopt.storage != ST3D_F32 && gopt.storage != ST3D_F64) || tblock > 1)) {
    zero_halo(v, grid);
    zero_halo(s, grid);
    zero_halo(u, grid);
  }
  double t1 = seconds();
  printf("[rank%i] Phase #%i: initialization took %f secs\n", my_rank, ++phase, t1 - t0);

  printf("[rank%i] Phase #%i: initial warmup\n", my_rank, ++phase);
  t0 = seconds();
  iterate_gb300(v, s, u, grid, prefetch, dups, 1U, cacheiter);
  t1 = seconds();
  printf("[rank%i] Phase #%i: finish warmup in %f secs\n", my_rank, ++phase, t1 - t0);
  if (!wave) check(v, grid, 1U);

  printf("[rank%i] Phase #%i: start compute\n", my_rank, ++phase);
  iterate_gb300(v, s, u, grid, prefetch, dups, maxiter, cacheiter);
  const gb300_timing& tm = gb300_last_timing();
  const double tc = tm.device_ms * 1e-3;  // compute only, as main.cpp:306-308 times ITERATE
  printf("[rank%i] Phase #%i: finish compute in %f secs (%f GFlop/s, mem: %f GB/s, cache: %f GB/s)\n",
         my_rank, ++phase, tc, flops / tc, mem_bytes / tc / cacheiter, cache_bytes / tc);
  printf("gb300: %.3f Gpts/s on the device, %.3f Gpts/s end to end (%.3f s incl. host<->device copies)\n",
         1e-9 * (double)grid.gvol * maxiter / tc, 1e-9 * (double)grid.gvol * maxiter / tm.total_s,
         tm.total_s);
  if (!wave) check(v, grid, maxiter + 1);
  printf("freeing data arrays\n");
  gb300_release();
  st3d_host_free(ov);
  st3d_host_free(os);
  st3d_host_free(ou);
  printf("[rank%i] Phase #%i: done!\n", my_rank, ++phase);
  return 0;
}
