// Test infrastructure only: a C-ABI wrapper around the reference's own
// host-CPU stencil path, compiled from the unmodified reference sources
// (iterators.cpp, grid.cpp, gilbert2d.cpp) by oracle/Makefile.ref into
// oracle/_ref/.  Nothing in the product links or loads this file; tests and
// the golden-vector generator use it to pin the C restatement in
// oracle/st3d_oracle.c against the reference itself.
//
// One shared object is built per STENCIL_SIZE (the reference selects the
// stencil at compile time, config.h:35-53) and per `real` type
// (config.h:96-100, -DUSE_DOUBLE).
//
// Entry points:
//   ref_iterate()  -> s_grid (grid.cpp:9-48) + iterate_2d_jk_blocked
//                     (iterators.cpp:197-234), the traversal that is correct
//                     for xs != ys (iterate_3d bounds j by isize,
//                     iterators.cpp:146).
//   ref_iterate_3d() -> iterate_3d (iterators.cpp:130-157), the README host
//                     recipe; only valid for xs == ys.
//   ref_init_arrays(), ref_check() -> iterators.cpp:292-325.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <unistd.h>
#include <fcntl.h>

#include "iterators.h"

namespace {

// s_grid's constructor prints a grid report on stdout (grid.cpp:18-29,
// 73-131).  The wrapper silences it so that callers see clean output.
struct quiet_stdout {
  int saved = -1;
  quiet_stdout() {
    fflush(stdout);
    saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) {
      dup2(devnull, 1);
      close(devnull);
    }
  }
  ~quiet_stdout() {
    fflush(stdout);
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};

}  // namespace

extern "C" {

int ref_stencil_size(void) { return STENCIL_SIZE; }
int ref_real_bytes(void) { return (int)sizeof(real); }

// Same meaning as ITERATE(v,s,u,grid,prefetch,dups,iterations,cacheiter)
// at main.cpp:307 with a grid built as main.cpp:201 builds it from the
// --xs/--ys/--zs/--xh/--yh/--zh flags (block sizes xb=1, yb=1, zb=zs).
int ref_iterate(real* v, const real* s, const real* u, unsigned xs, unsigned ys,
                unsigned zs, unsigned xh, unsigned yh, unsigned zh,
                unsigned iterations) {
  quiet_stdout q;
  s_grid grid(xs, ys, zs, xh, yh, zh, 1, 1, zs, 12.0f, 13, 3);
  iterate_2d_jk_blocked(v, s, u, grid, 64, 1, iterations, 1);
  return 0;
}

int ref_iterate_3d(real* v, const real* s, const real* u, unsigned xs, unsigned ys,
                   unsigned zs, unsigned xh, unsigned yh, unsigned zh,
                   unsigned iterations) {
  quiet_stdout q;
  s_grid grid(xs, ys, zs, xh, yh, zh, 1, 1, 1, 12.0f, 13, 3);
  iterate_3d(v, s, u, grid, 64, 1, iterations, 1);
  return 0;
}

void ref_init_arrays(real* v, real* s, real* u, unsigned gsize) {
  init_arrays(v, s, u, gsize);
}

// Returns the number of interior points with |v - maxiter| > 0.1, the count
// that check() prints (iterators.cpp:304-325).
unsigned ref_check_count(const real* v, unsigned xs, unsigned ys, unsigned zs,
                         unsigned xh, unsigned yh, unsigned zh, unsigned maxiter) {
  const unsigned jmult = zs + 2 * zh;
  const unsigned imult = jmult * (ys + 2 * yh);
  const unsigned ijk_ofs = zh + yh * jmult + xh * imult;
  unsigned err = 0;
  for (unsigned i = 0; i < xs; i++)
    for (unsigned j = 0; j < ys; j++)
      for (unsigned k = 0; k < zs; k++)
        if (fabs(v[IDX(i, j, k)] - (real)maxiter) > 0.1f) err++;
  return err;
}

}  // extern "C"
