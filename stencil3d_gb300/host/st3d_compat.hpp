// st3d_compat.hpp -- the reference's C++ host interface over the C ABI.
//
// Keeps the names and argument meanings of the reference's grid and
// iterator interface so that host code written against grid.h and
// iterators.h compiles unchanged against this library:
//   - class s_grid            (grid.h:7-71, grid.cpp:9-48): geometry and the
//                              reference-layout strides.
//   - iterate_gb300(...)      the signature of every ITERATE variant
//                              (iterators.h:6-29), running on the GPU.
//   - init_arrays / check     (iterators.h:31-36, iterators.cpp:292-325).
//   - seconds / get_int_arg / get_real_arg / get_flag (aux.h, aux.cpp:9-81):
//                              the command-line helpers with the reference's
//                              messages and exit codes.
#pragma once

#include <cstddef>

#include "st3d.h"

// config.h:96-100: `real` is double in the reference's USE_DOUBLE build
// (then the library runs its FP64 storage) and float otherwise.
#ifdef USE_DOUBLE
typedef double real;
#else
typedef float real;
#endif

class s_grid {
 public:
  s_grid(unsigned xs, unsigned ys, unsigned zs, unsigned xh, unsigned yh, unsigned zh,
         unsigned xb, unsigned yb, unsigned zb, real sm, unsigned jshuffle, unsigned kshuffle);

  inline unsigned idx(unsigned i, unsigned j, unsigned k) const {
    return ijk_ofs + k + jmult * j + imult * i;
  }

  unsigned xsize, ysize, zsize;   // interior points
  unsigned xhalo, yhalo, zhalo;   // halo points per side
  size_t gsize;                   // points including halos (grid.cpp:24)
  size_t gvol;                    // interior points (grid.cpp:25)
  unsigned xb_size, yb_size, zb_size;  // CPU cache-tile hints: accepted, unused on the GPU
  real sb_mib;
  unsigned jshuf, kshuf;
  unsigned ijk_ofs, jmult, imult;
};

// GPU options the reference fixes at compile time (config.h:35-53,
// 96-100) and this library chooses at run time.
struct gb300_options {
  int points = 7;                 // STENCIL_SIZE
  int mode = ST3D_MODE_REF;
#ifdef USE_DOUBLE
  int storage = ST3D_F64;         // real = double: FP64 fields and arithmetic
#else
  int storage = ST3D_F32;         // real = float: FP32 or a 16-bit device storage
#endif
  int kernel = ST3D_KERNEL_AUTO;
  double vel = 1500.0, dt = 1e-3, dx = 10.0;  // mode W physics
  // Mode R diagonal coefficient K; 0 keeps the stencil's default.  The
  // reference's 13-point vec_16 kernel uses 6.25 (stencil_13.h:391, 428)
  // where every other 13-point kernel uses 3.5.
  double K = 0.0;
  int temporal_block = 1;         // mode W, FP32: steps fused per pass
};

// Per-call timing of the last iterate_gb300 call.
struct gb300_timing {
  double device_ms = 0;   // stencil kernels only (CUDA events)
  double total_s = 0;     // host wall clock incl. transfers
};

void gb300_configure(const gb300_options& opts);
const gb300_timing& gb300_last_timing();
// Releases the device context the shim keeps between calls.
void gb300_release();

// ITERATE(v, s, u, grid, prefetch_dist, dups, iterations, cacheiter) on the
// GPU: uploads v, s and u, advances `iterations` steps, downloads v (and u
// in mode W).  prefetch_dist, dups and cacheiter steer the reference's CPU
// traversal and are ignored.  Exits with status 3 on a library error, as the
// reference exits on allocation errors (main.cpp:53-66).
void iterate_gb300(real* v, const real* s, const real* u, const s_grid& grid,
                   unsigned prefetch_dist, unsigned dups, unsigned iterations, unsigned cacheiter);

void init_arrays(real* v, real* s, real* u, size_t gsize);
unsigned check(const real* v, const s_grid& grid, unsigned maxiter);

double seconds();
int get_int_arg(char* argv[], int iarg, int argc, const char* opt, unsigned& val, unsigned minval,
                unsigned maxval, unsigned modval);
int get_real_arg(char* argv[], int iarg, int argc, const char* opt, real& val, real minval,
                 real maxval);
int get_double_arg(char* argv[], int iarg, int argc, const char* opt, double& val, double minval,
                   double maxval);
int get_str_arg(char* argv[], int iarg, int argc, const char* opt, const char*& val);
int get_flag(char* argv[], int iarg, int argc, const char* opt, unsigned& flag);
