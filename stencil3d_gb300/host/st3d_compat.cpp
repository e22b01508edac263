// st3d_compat.cpp -- implementation of the reference-compatible host
// interface (st3d_compat.hpp) on the C ABI of libst3d.
#include "st3d_compat.hpp"

#include <sys/time.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

gb300_options g_opts;
gb300_timing g_timing;
st3d_ctx* g_ctx = nullptr;
unsigned g_key[6] = {0, 0, 0, 0, 0, 0};

[[noreturn]] void die(int rc, const char* what) {
  fprintf(stderr, "error: %s: %s (%s)\n", what, st3d_status_string(rc), st3d_last_error());
  exit(3);
}

st3d_ctx* context_for(const s_grid& g) {
  const unsigned key[6] = {g.xsize, g.ysize, g.zsize, g.xhalo, g.yhalo, g.zhalo};
  if (g_ctx && memcmp(key, g_key, sizeof key) == 0) return g_ctx;
  gb300_release();
  // the host arrays hold `real`: double only for the FP64 storage
  if ((g_opts.storage == ST3D_F64) != (sizeof(real) == sizeof(double))) {
    fprintf(stderr, "error: storage %d does not match the host arrays' %zu-byte real\n",
            g_opts.storage, sizeof(real));
    exit(3);
  }
  st3d_grid_desc d = {g.xsize, g.ysize, g.zsize, g.xhalo, g.yhalo, g.zhalo};
  st3d_opts o;
  int rc = st3d_default_opts(g_opts.points, g_opts.mode, g_opts.storage, &o);
  if (rc) die(rc, "st3d_default_opts");
  o.kernel = g_opts.kernel;
  if (g_opts.K != 0.0) o.coef[1] = g_opts.K;
  o.temporal_block = g_opts.temporal_block;
  if (g_opts.mode == ST3D_MODE_WAVE) {
    rc = st3d_set_wave_physics(&o, g_opts.vel, g_opts.dt, g_opts.dx);
    if (rc) die(rc, "st3d_set_wave_physics");
  }
  rc = st3d_create(&d, &o, &g_ctx);
  if (rc) die(rc, "st3d_create");
  memcpy(g_key, key, sizeof key);
  return g_ctx;
}

}  // namespace

s_grid::s_grid(unsigned xs, unsigned ys, unsigned zs, unsigned xh, unsigned yh, unsigned zh,
               unsigned xb, unsigned yb, unsigned zb, real sm, unsigned jshuffle,
               unsigned kshuffle)
    : xsize(xs), ysize(ys), zsize(zs), xhalo(xh), yhalo(yh), zhalo(zh),
      xb_size(xb < xs ? xb : xs), yb_size(yb < ys ? yb : ys), zb_size(zb < zs ? zb : zs),
      sb_mib(sm), jshuf(jshuffle), kshuf(kshuffle) {
  jmult = zsize + 2 * zhalo;
  imult = jmult * (ysize + 2 * yhalo);
  ijk_ofs = zhalo + yhalo * jmult + xhalo * imult;
  gsize = (size_t)(zsize + 2 * zhalo) * (ysize + 2 * yhalo) * (xsize + 2 * xhalo);
  gvol = (size_t)zsize * ysize * xsize;
  printf("Initializing grid structure\n");
  printf("... grid dimensions %d x %d x %d with halo %d x %d x %d\n", xsize, ysize, zsize, xhalo,
         yhalo, zhalo);
  printf("... with %zu inner grid points and %zu total gridpoints\n", gvol, gsize);
}

void gb300_configure(const gb300_options& opts) {
  gb300_release();
  g_opts = opts;
}

const gb300_timing& gb300_last_timing() { return g_timing; }

void gb300_release() {
  if (g_ctx) st3d_destroy(g_ctx);
  g_ctx = nullptr;
  memset(g_key, 0, sizeof g_key);
}

void iterate_gb300(real* v, const real* s, const real* u, const s_grid& grid,
                   unsigned /*prefetch_dist*/, unsigned /*dups*/, unsigned iterations,
                   unsigned /*cacheiter*/) {
  st3d_ctx* c = context_for(grid);
  const double t0 = seconds();
  int rc = st3d_upload(c, v, s, u);
  if (rc) die(rc, "st3d_upload");
  rc = st3d_timer_start(c);
  if (rc) die(rc, "st3d_timer_start");
  rc = st3d_iterate(c, iterations);
  if (rc) die(rc, "st3d_iterate");
  float ms = 0.0f;
  rc = st3d_timer_stop(c, &ms);
  if (rc) die(rc, "st3d_timer_stop");
  rc = st3d_download(c, v, g_opts.mode == ST3D_MODE_WAVE ? const_cast<real*>(u) : nullptr);
  if (rc) die(rc, "st3d_download");
  rc = st3d_synchronize(c);
  if (rc) die(rc, "st3d_synchronize");
  g_timing.device_ms = ms;
  g_timing.total_s = seconds() - t0;
}

void init_arrays(real* v, real* s, real* u, size_t gsize) {
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < gsize; i++) {
    v[i] = 0.0f;
    u[i] = 1.0f;
    s[i] = 1.0f;
  }
}

unsigned check(const real* v, const s_grid& grid, unsigned maxiter) {
  unsigned error = 0;
#pragma omp parallel for collapse(2) reduction(+ : error) schedule(static)
  for (unsigned i = 0; i < grid.xsize; i++)
    for (unsigned j = 0; j < grid.ysize; j++)
      for (unsigned k = 0; k < grid.zsize; k++)
        if (std::fabs(v[grid.idx(i, j, k)] - (real)maxiter) > 0.1f) error++;
  printf("check: %d errors found\n", error);
  return error;
}

double seconds() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return (double)tv.tv_sec + 1e-6 * tv.tv_usec;
}

int get_int_arg(char* argv[], int iarg, int argc, const char* opt, unsigned& val, unsigned minval,
                unsigned maxval, unsigned modval) {
  if (strcmp(argv[iarg], opt) != 0) return 0;
  if (iarg + 1 >= argc) {
    fprintf(stderr, "%s requires a numeric argument [%d - %d]\n", opt, minval, maxval);
    exit(2);
  }
  val = (unsigned)atoi(argv[iarg + 1]);
  if (val < minval) {
    fprintf(stderr, "%s must be larger or equal to %d\n", opt, minval);
    exit(2);
  }
  if (val > maxval) {
    fprintf(stderr, "%s must be smaller or equal to %d\n", opt, maxval);
    exit(2);
  }
  if ((val % modval) != 0) {
    fprintf(stderr, "%s must be a multiple of %d\n", opt, modval);
    exit(2);
  }
  printf("%s set to %d\n", opt, val);
  return 2;
}

int get_real_arg(char* argv[], int iarg, int argc, const char* opt, real& val, real minval,
                 real maxval) {
  double d = val;
  const int r = get_double_arg(argv, iarg, argc, opt, d, minval, maxval);
  if (r) val = (real)d;
  return r;
}

int get_double_arg(char* argv[], int iarg, int argc, const char* opt, double& val, double minval,
                   double maxval) {
  if (strcmp(argv[iarg], opt) != 0) return 0;
  if (iarg + 1 >= argc) {
    fprintf(stderr, "%s requires a float argument [%f - %f]\n", opt, minval, maxval);
    exit(2);
  }
  val = atof(argv[iarg + 1]);
  if (val < minval) {
    fprintf(stderr, "%s must be larger or equal to %f\n", opt, minval);
    exit(2);
  }
  if (val > maxval) {
    fprintf(stderr, "%s must be smaller or equal to %f\n", opt, maxval);
    exit(2);
  }
  printf("%s set to %f\n", opt, val);
  return 2;
}

int get_str_arg(char* argv[], int iarg, int argc, const char* opt, const char*& val) {
  if (strcmp(argv[iarg], opt) != 0) return 0;
  if (iarg + 1 >= argc) {
    fprintf(stderr, "%s requires an argument\n", opt);
    exit(2);
  }
  val = argv[iarg + 1];
  printf("%s set to %s\n", opt, val);
  return 2;
}

int get_flag(char* argv[], int iarg, int /*argc*/, const char* opt, unsigned& flag) {
  if (strcmp(argv[iarg], opt) != 0) return 0;
  flag = 1;
  printf("%s set to ENABLED\n", opt);
  return 1;
}
