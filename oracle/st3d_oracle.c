/*
 * st3d_oracle.c -- CPU restatement of the stencil3d hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py load this library, and only as the checker
 * (or as the timed CPU baseline); the product path never calls it.
 *
 * What it restates (reference file:line):
 *  - reference layout: IDX(i,j,k) = ijk_ofs + k + j*jmult + i*imult with
 *    jmult = zs+2zh, imult = jmult*(ys+2yh), ijk_ofs = zh + yh*jmult +
 *    xh*imult (stencils.h:5, grid.cpp:20-22).
 *  - "mode R", the update the reference code actually computes, with u and s
 *    fixed between steps (iterators.cpp:137-156, 204-233):
 *      7-pt : stencil_7_ref_1   stencil_7.h:4-39
 *      13-pt: stencil_13_ref_1  stencil_13.h:4-61
 *      25-pt: stencil_25_ref_1  stencil_25.h:20-95
 *      2-pt : stencil_2_ref_1   stencil_2.h:4-29
 *    with the same coefficient arithmetic (CONSTANTS_*), the same
 *    left-to-right evaluation order and, for real=double (config.h:96-97),
 *    the same float-literal promotion.
 *  - init_arrays / check known-answer test (iterators.cpp:292-325).
 *  - "mode W", the leapfrog wave update v = c0*u - v + c1*L(u) + c2*s with
 *    u/v swapped each step (README.md:11-20), L using the neighbour sets of
 *    stencil_{7,13,25}.h; the reference has no code for it, so this file is
 *    its definition.
 *  - seeded input generators and a 15 Hz Ricker point source.
 *
 * Parity is pinned: in mode R with fma=0 this file reproduces the compiled
 * reference (oracle/_ref, built by oracle/Makefile.ref) bit for bit, which
 * tests/test_oracle.py checks, and tests/golden/ holds outputs of the
 * reference itself for the GPU machine where the reference is absent.
 *
 * Each update also has an fma=1 flavour that evaluates the same sums in the
 * same order with fused multiply-adds, the exact operation sequence of the
 * CUDA kernels, so that device results can be compared bit for bit.
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (see
 * oracle/build.py).  -ffp-contract=off keeps the compiler from fusing the
 * plain flavour.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  unsigned xs, ys, zs, xh, yh, zh;
  size_t jmult, imult, ijk_ofs, gsize;
} orc_layout;

static orc_layout mk_layout(const unsigned* g) {
  orc_layout L;
  L.xs = g[0]; L.ys = g[1]; L.zs = g[2];
  L.xh = g[3]; L.yh = g[4]; L.zh = g[5];
  L.jmult = (size_t)L.zs + 2u * L.zh;
  L.imult = L.jmult * ((size_t)L.ys + 2u * L.yh);
  L.ijk_ofs = L.zh + L.yh * L.jmult + L.xh * L.imult;
  L.gsize = L.imult * ((size_t)L.xs + 2u * L.xh);
  return L;
}

/* number of elements of a reference-layout array (grid.cpp:24) */
size_t orc_gsize(const unsigned* g) { return mk_layout(g).gsize; }

static int radius_of(int points) {
  switch (points) {
    case 2: return 1;
    case 7: return 1;
    case 13: return 2;
    case 25: return 4;
    default: return -1;
  }
}

/* ------------------------------------------------------------------ */
/* Coefficients                                                         */
/* ------------------------------------------------------------------ */
/*
 * Coefficient block layout shared with the C-ABI (st3d_coefs):
 *   c[0] = coef0, c[1] = K (the "-K*u0" factor of the ref_1 update),
 *   c[2..5] = cx1..cx4, c[6..9] = cy1..cy4, c[10..13] = cz1..cz4.
 * For 2 points, c[0] is the 0.5 averaging factor (CONSTANTS_2).
 */
void orc_default_coefs_f32(int points, int isotropic, float* c) {
  memset(c, 0, 14 * sizeof(float));
  if (points == 2) { c[0] = 0.5f; return; }
  if (points == 7) {                       /* stencil_7.h:4-8, :38 */
    c[0] = 1.5f; c[1] = 3.5f;
    c[2] = 0.5f; c[6] = 0.5f; c[10] = 0.5f;
    return;
  }
  if (points == 13) {                      /* stencil_13.h:4-22, :60 */
    const float cx1 = 0.3f, cx2 = 0.2f;
    c[0] = 1.5f; c[1] = 3.5f;
    c[2] = cx1; c[3] = cx2;
    if (isotropic) { c[6] = cx1; c[7] = cx2; c[10] = cx1; c[11] = cx2; }
    else {
      c[6] = cx1 * 1.1f; c[7] = cx2 * 1.1f;
      c[10] = cx1 * 0.9f; c[11] = cx2 * 0.9f;
    }
    return;
  }
  if (points == 25) {                      /* stencil_25.h:20-34, :94 */
    const float cx[4] = {0.4f, 0.3f, 0.2f, 0.1f};
    c[0] = 1.25f; c[1] = 6.25f;
    for (int r = 0; r < 4; r++) {
      c[2 + r] = cx[r];
      c[6 + r] = isotropic ? cx[r] : cx[r] * 1.1f;
      c[10 + r] = isotropic ? cx[r] : cx[r] * 0.9f;
    }
    return;
  }
}

/* real=double: the float literals of CONSTANTS_* are promoted first and the
 * products are formed in double (config.h:96-97 with stencil_*.h). */
void orc_default_coefs_f64(int points, int isotropic, double* c) {
  memset(c, 0, 14 * sizeof(double));
  if (points == 2) { c[0] = (double)0.5f; return; }
  if (points == 7) {
    c[0] = (double)1.5f; c[1] = (double)3.5f;
    c[2] = (double)0.5f; c[6] = (double)0.5f; c[10] = (double)0.5f;
    return;
  }
  if (points == 13) {
    const double cx1 = (double)0.3f, cx2 = (double)0.2f;
    c[0] = (double)1.5f; c[1] = (double)3.5f;
    c[2] = cx1; c[3] = cx2;
    if (isotropic) { c[6] = cx1; c[7] = cx2; c[10] = cx1; c[11] = cx2; }
    else {
      c[6] = cx1 * (double)1.1f; c[7] = cx2 * (double)1.1f;
      c[10] = cx1 * (double)0.9f; c[11] = cx2 * (double)0.9f;
    }
    return;
  }
  if (points == 25) {
    const double cx[4] = {(double)0.4f, (double)0.3f, (double)0.2f, (double)0.1f};
    c[0] = (double)1.25f; c[1] = (double)6.25f;
    for (int r = 0; r < 4; r++) {
      c[2 + r] = cx[r];
      c[6 + r] = isotropic ? cx[r] : cx[r] * (double)1.1f;
      c[10 + r] = isotropic ? cx[r] : cx[r] * (double)0.9f;
    }
    return;
  }
}

/*
 * Neighbour-pair order of the reference's stencil sums.  Each entry is
 * (axis, r) with axis 0 = i (x, slowest), 1 = j (y), 2 = k (z, contiguous),
 * the axis convention of stencil_25.h:64-67.
 *   7 : x1 y1 z1                       (stencil_7.h:20)
 *   13: z2 z1 y2 y1 x2 x1              (stencil_13.h:40-43)
 *   25: z4..z1 y4..y1 x4..x1           (stencil_25.h:64-67)
 */
static int pair_order(int points, int* axis, int* rad) {
  int n = 0;
  if (points == 7) {
    for (int a = 0; a < 3; a++) { axis[n] = a; rad[n] = 1; n++; }
    return n;
  }
  int R = radius_of(points);
  for (int a = 2; a >= 0; a--)
    for (int r = R; r >= 1; r--) { axis[n] = a; rad[n] = r; n++; }
  return n;
}

/* ------------------------------------------------------------------ */
/* Mode R (reference update)                                            */
/* ------------------------------------------------------------------ */
#define DEFINE_ITERATE_REF(SUFFIX, T, FMA)                                        \
  int orc_iterate_ref_##SUFFIX(T* v, const T* s, const T* u, const unsigned* g,   \
                               int points, const T* c, unsigned iterations,       \
                               int use_fma) {                                     \
    const orc_layout L = mk_layout(g);                                            \
    const int R = radius_of(points);                                              \
    if (R < 0) return 1;                                                          \
    int axis[12], rad[12];                                                        \
    const int np = points == 2 ? 0 : pair_order(points, axis, rad);               \
    long long off_m[12], off_p[12];                                               \
    T cf[12];                                                                     \
    for (int p = 0; p < np; p++) {                                                \
      const long long st = axis[p] == 0 ? (long long)L.imult                      \
                         : axis[p] == 1 ? (long long)L.jmult : 1;                 \
      off_m[p] = -st * rad[p];                                                    \
      off_p[p] = st * rad[p];                                                     \
      cf[p] = c[2 + 4 * axis[p] + rad[p] - 1];                                    \
    }                                                                             \
    const T coef0 = c[0], K = c[1];                                               \
    for (unsigned it = 0; it < iterations; it++) {                                \
      _Pragma("omp parallel for schedule(static) collapse(2)")                    \
      for (unsigned i = 0; i < L.xs; i++)                                         \
        for (unsigned j = 0; j < L.ys; j++) {                                     \
          const size_t row = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult; \
          for (unsigned k = 0; k < L.zs; k++) {                                   \
            const size_t x = row + k;                                             \
            const T u0 = u[x];                                                    \
            if (points == 2) { /* stencil_2.h:4-10, :27 */                        \
              v[x] = coef0 * (u0 + u[x + 1]);                                     \
              continue;                                                           \
            }                                                                     \
            T st = coef0 * u0;                                                    \
            if (use_fma) {                                                        \
              for (int p = 0; p < np; p++)                                        \
                st = FMA(cf[p], u[x + off_m[p]] + u[x + off_p[p]], st);           \
              const T t = FMA(-K, u0, v[x]);                                      \
              v[x] = FMA(s[x], st, t);                                            \
            } else {                                                              \
              for (int p = 0; p < np; p++)                                        \
                st = st + cf[p] * (u[x + off_m[p]] + u[x + off_p[p]]);            \
              v[x] = v[x] - K * u0 + s[x] * st;                                   \
            }                                                                     \
          }                                                                       \
        }                                                                         \
    }                                                                             \
    return 0;                                                                     \
  }

DEFINE_ITERATE_REF(f32, float, fmaf)
DEFINE_ITERATE_REF(f64, double, fma)

/* ------------------------------------------------------------------ */
/* Mode W (leapfrog wave update)                                        */
/* ------------------------------------------------------------------ */
/*
 * One step: v <- c0*u - v + c1*L(u) + c2*(s + a_n*delta_src), then the roles
 * of u and v swap.  L(u) = sum over the pairs of pair_order() of
 * w(axis,r)*(u[-r] + u[+r]); w uses the c[2..13] slots of the coefficient
 * block (c[0], c[1] unused).  amp[n] is the source amplitude of step n
 * (NULL: no source).  src = {i,j,k} interior coordinates, or i < 0.
 *
 * With c0 = 2 - 2*c1*sum(w) the update is evaluated in its difference form
 *     v <- (2u - v) + c1 * sum w*((u[-r] + u[+r]) - 2u) + c2*s_eff,
 * which is the same expression algebraically but keeps constant fields
 * exactly constant in any precision.  The literal form rounds c0 and the
 * weights separately, so c0 + 2*c1*sum(w) != 2 in float and the smoothest
 * modes drift: about 5e-3 relative L2 against FP64 after 1000 steps of a
 * blob field, against about 1e-5 for the difference form.  c0 is therefore
 * an input of the constants only, not of the update.
 *
 * On return u holds U^{n+iterations} and v holds U^{n+iterations-1}.
 *
 * fma=1 order (the device kernels' order), with u2 = 2*u0 (exact):
 *   lap = w_0*((a_0+b_0) - u2); lap = fma(w_p, (a_p+b_p) - u2, lap) ...
 *   t = u2 - v0; t = fma(c1, lap, t); v = fma(c2, s_eff, t)
 * fma=0 order: v = (u2 - v0) + c1*lap + c2*s_eff, lap summed left to right.
 */
#define DEFINE_ITERATE_WAVE(SUFFIX, T, FMA)                                       \
  int orc_iterate_wave_##SUFFIX(T* u_io, T* v_io, const T* s, const unsigned* g,  \
                                int points, const T* c, T c0, T c1, T c2,         \
                                const long long* src, const T* amp,               \
                                unsigned iterations, int use_fma) {               \
    const orc_layout L = mk_layout(g);                                            \
    const int R = radius_of(points);                                              \
    (void)c0;                                                                     \
    if (R < 0 || points == 2) return 1;                                           \
    int axis[12], rad[12];                                                        \
    const int np = pair_order(points, axis, rad);                                 \
    long long off_m[12], off_p[12];                                               \
    T cf[12];                                                                     \
    for (int p = 0; p < np; p++) {                                                \
      const long long st = axis[p] == 0 ? (long long)L.imult                      \
                         : axis[p] == 1 ? (long long)L.jmult : 1;                 \
      off_m[p] = -st * rad[p];                                                    \
      off_p[p] = st * rad[p];                                                     \
      cf[p] = c[2 + 4 * axis[p] + rad[p] - 1];                                    \
    }                                                                             \
    long long src_x = -1;                                                         \
    if (src && src[0] >= 0)                                                       \
      src_x = (long long)(L.ijk_ofs + (size_t)src[0] * L.imult +                  \
                          (size_t)src[1] * L.jmult + (size_t)src[2]);             \
    T* u = u_io;                                                                  \
    T* v = v_io;                                                                  \
    for (unsigned it = 0; it < iterations; it++) {                                \
      const T a = amp ? amp[it] : (T)0;                                           \
      _Pragma("omp parallel for schedule(static) collapse(2)")                    \
      for (unsigned i = 0; i < L.xs; i++)                                         \
        for (unsigned j = 0; j < L.ys; j++) {                                     \
          const size_t row = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult; \
          for (unsigned k = 0; k < L.zs; k++) {                                   \
            const size_t x = row + k;                                             \
            const T u0 = u[x];                                                    \
            const T u2 = u0 + u0;                                                 \
            T se = s[x];                                                          \
            if ((long long)x == src_x) se = se + a;                               \
            T lap = cf[0] * ((u[x + off_m[0]] + u[x + off_p[0]]) - u2);           \
            if (use_fma) {                                                        \
              for (int p = 1; p < np; p++)                                        \
                lap = FMA(cf[p], (u[x + off_m[p]] + u[x + off_p[p]]) - u2, lap);  \
              T t = u2 - v[x];                                                    \
              t = FMA(c1, lap, t);                                                \
              v[x] = FMA(c2, se, t);                                              \
            } else {                                                              \
              for (int p = 1; p < np; p++)                                        \
                lap = lap + cf[p] * ((u[x + off_m[p]] + u[x + off_p[p]]) - u2);   \
              v[x] = (u2 - v[x]) + c1 * lap + c2 * se;                            \
            }                                                                     \
          }                                                                       \
        }                                                                         \
      T* tmp = u; u = v; v = tmp;                                                 \
    }                                                                             \
    if (u != u_io) { /* odd number of steps: move the newest field into u_io */   \
      const size_t n = L.gsize;                                                   \
      T* tmp = (T*)malloc(n * sizeof(T));                                         \
      if (!tmp) return 2;                                                         \
      memcpy(tmp, u_io, n * sizeof(T));                                           \
      memcpy(u_io, v_io, n * sizeof(T));                                          \
      memcpy(v_io, tmp, n * sizeof(T));                                           \
      free(tmp);                                                                  \
    }                                                                             \
    return 0;                                                                     \
  }

DEFINE_ITERATE_WAVE(f32, float, fmaf)
DEFINE_ITERATE_WAVE(f64, double, fma)

/* Wave-mode constants from physical parameters: c1 = (c*dt/dx)^2, c2 = dt^2
 * (README.md:11-14) and c0 = 2 - 2*c1*sum(w), which makes the update exact
 * for constant fields (for 7 points with w = 1 this is README's 2 - 6*c1). */
void orc_wave_constants(const float* c, double vel, double dt, double dx,
                        double* out /* c0, c1, c2 */) {
  const double c1 = (vel * dt / dx) * (vel * dt / dx);
  double wsum = 0.0;
  for (int m = 2; m < 14; m++) wsum += (double)c[m];
  out[0] = 2.0 - 2.0 * c1 * wsum;
  out[1] = c1;
  out[2] = dt * dt;
}

/* ------------------------------------------------------------------ */
/* Known-answer test (iterators.cpp:292-325)                            */
/* ------------------------------------------------------------------ */
void orc_init_arrays_f32(float* v, float* s, float* u, size_t gsize) {
  for (size_t x = 0; x < gsize; x++) { v[x] = 0.0f; u[x] = 1.0f; s[x] = 1.0f; }
}

unsigned orc_check_f32(const float* v, const unsigned* g, unsigned maxiter) {
  const orc_layout L = mk_layout(g);
  unsigned err = 0;
  for (unsigned i = 0; i < L.xs; i++)
    for (unsigned j = 0; j < L.ys; j++)
      for (unsigned k = 0; k < L.zs; k++) {
        const size_t x = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k;
        if (fabs(v[x] - (float)maxiter) > 0.1f) err++;
      }
  return err;
}

/* ------------------------------------------------------------------ */
/* Seeded inputs                                                        */
/* ------------------------------------------------------------------ */
/*
 * A counter-based generator: the value at logical point (i,j,k) -- interior
 * coordinates, halo points negative or >= size -- depends only on
 * (seed, field, i, j, k), so every layout that holds the point gets the same
 * value.  key = ((((seed*P1 + field)*P2 + i+64)*P3 + j+64)*P4 + k+64) mod
 * 2^64, mixed by the splitmix64 finaliser; the top 24 bits give
 * x in [0,1) and the value is (float)(lo + (hi-lo)*x) in double.
 */
static inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ULL;
  z ^= z >> 27; z *= 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return z;
}

static inline double unit_at(uint64_t seed, unsigned field, long long i, long long j,
                             long long k) {
  uint64_t key = seed * 0x9E3779B97F4A7C15ULL + field;
  key = key * 0xD1B54A32D192ED03ULL + (uint64_t)(i + 64);
  key = key * 0xAEF17502108EF2D9ULL + (uint64_t)(j + 64);
  key = key * 0xF58C1E3A7E1C4B55ULL + (uint64_t)(k + 64);
  return (double)(mix64(key) >> 40) * (1.0 / 16777216.0);
}

double orc_unit_at(uint64_t seed, unsigned field, long long i, long long j, long long k) {
  return unit_at(seed, field, i, j, k);
}

#define DEFINE_FILL(SUFFIX, T)                                                    \
  void orc_fill_uniform_##SUFFIX(T* a, const unsigned* g, uint64_t seed,          \
                                 unsigned field, double lo, double hi) {          \
    const orc_layout L = mk_layout(g);                                            \
    const long long ni = L.xs + 2 * L.xh, nj = L.ys + 2 * L.yh,                   \
                    nk = L.zs + 2 * L.zh;                                         \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (long long ii = 0; ii < ni; ii++)                                         \
      for (long long jj = 0; jj < nj; jj++)                                       \
        for (long long kk = 0; kk < nk; kk++) {                                   \
          const double x = unit_at(seed, field, ii - L.xh, jj - L.yh, kk - L.zh); \
          a[(size_t)ii * L.imult + (size_t)jj * L.jmult + (size_t)kk] =           \
              (T)(lo + (hi - lo) * x);                                            \
        }                                                                         \
  }

DEFINE_FILL(f32, float)
DEFINE_FILL(f64, double)

/*
 * Blob parameters: a splitmix64 stream seeded with `seed`; per blob, the
 * centre (ci, cj, ck) uniform over the interior and the amplitude uniform in
 * [-1, 1).  Draw b*4+m of the stream is mix64(seed + (b*4+m+1)*golden).
 */
static double stream_unit(uint64_t seed, unsigned n) {
  return (double)(mix64(seed + (uint64_t)(n + 1) * 0x9E3779B97F4A7C15ULL) >> 40) *
         (1.0 / 16777216.0);
}

void orc_blob_params(uint64_t seed, int nblobs, const unsigned* g, double* out /* 4*nblobs */) {
  for (int b = 0; b < nblobs; b++) {
    out[4 * b + 0] = stream_unit(seed, 4 * b + 0) * g[0];
    out[4 * b + 1] = stream_unit(seed, 4 * b + 1) * g[1];
    out[4 * b + 2] = stream_unit(seed, 4 * b + 2) * g[2];
    out[4 * b + 3] = 2.0 * stream_unit(seed, 4 * b + 3) - 1.0;
  }
}

/* u(i,j,k) = sum_b A_b * exp(-((i-ci)^2+(j-cj)^2+(k-ck)^2) / (2 sigma^2)) over
 * the interior; halo points are set to 0 (a zero Dirichlet boundary). */
#define DEFINE_BLOBS(SUFFIX, T)                                                   \
  void orc_fill_blobs_##SUFFIX(T* a, const unsigned* g, uint64_t seed, int nblobs, \
                               double sigma) {                                    \
    const orc_layout L = mk_layout(g);                                            \
    double P[4 * 64];                                                             \
    if (nblobs > 64) nblobs = 64;                                                 \
    orc_blob_params(seed, nblobs, g, P);                                          \
    const double inv = 1.0 / (2.0 * sigma * sigma);                               \
    memset(a, 0, L.gsize * sizeof(T));                                            \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (long long i = 0; i < (long long)L.xs; i++)                               \
      for (unsigned j = 0; j < L.ys; j++)                                         \
        for (unsigned k = 0; k < L.zs; k++) {                                     \
          double acc = 0.0;                                                       \
          for (int b = 0; b < nblobs; b++) {                                      \
            const double di = (double)i - P[4 * b], dj = (double)j - P[4 * b + 1], \
                         dk = (double)k - P[4 * b + 2];                           \
            acc += P[4 * b + 3] * exp(-(di * di + dj * dj + dk * dk) * inv);      \
          }                                                                       \
          a[L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k] = (T)acc;  \
        }                                                                         \
  }

DEFINE_BLOBS(f32, float)
DEFINE_BLOBS(f64, double)

/* Ricker wavelet w(t) = (1 - 2a) exp(-a), a = (pi f (t - t0))^2. */
double orc_ricker(double t, double f, double t0) {
  const double pf = 3.14159265358979323846 * f * (t - t0);
  const double a = pf * pf;
  return (1.0 - 2.0 * a) * exp(-a);
}

/* ------------------------------------------------------------------ */
/* Norms over the interior (double accumulation)                        */
/* ------------------------------------------------------------------ */
/* out[0] = sum (a-b)^2, out[1] = sum b^2, out[2] = max |a-b|, out[3] = max |b| */
#define DEFINE_DIFF(SUFFIX, TA, TB)                                               \
  void orc_diff_##SUFFIX(const TA* a, const TB* b, const unsigned* g, double* out) { \
    const orc_layout L = mk_layout(g);                                            \
    double d2 = 0, b2 = 0, dm = 0, bm = 0;                                        \
    _Pragma("omp parallel for reduction(+:d2,b2) reduction(max:dm,bm) schedule(static)") \
    for (long long i = 0; i < (long long)L.xs; i++)                               \
      for (unsigned j = 0; j < L.ys; j++)                                         \
        for (unsigned k = 0; k < L.zs; k++) {                                     \
          const size_t x = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k; \
          const double d = (double)a[x] - (double)b[x];                           \
          d2 += d * d; b2 += (double)b[x] * (double)b[x];                         \
          if (fabs(d) > dm) dm = fabs(d);                                         \
          if (fabs((double)b[x]) > bm) bm = fabs((double)b[x]);                   \
        }                                                                         \
    out[0] = d2; out[1] = b2; out[2] = dm; out[3] = bm;                           \
  }

DEFINE_DIFF(f32_f32, float, float)
DEFINE_DIFF(f32_f64, float, double)
DEFINE_DIFF(f64_f64, double, double)

/* ------------------------------------------------------------------ */
/* 16-bit storage forms of mode W                                      */
/* ------------------------------------------------------------------ */
/*
 * Restates the precision form of the library (no reference code exists):
 * a field is a 16-bit word per point (FP16 kind 0 or BF16 kind 1, round to
 * nearest even) with a power-of-two scale 2^E per i-plane, plus, in the
 * compensated form (hilo), a signed byte q holding the residual in units of
 * ulp(h)/256:  x = (h + q*ulp(h)/256) * 2^E.  One step decodes u (neighbour
 * terms from the word alone, the centre from word + byte), v and s, applies
 * the FP32 fused difference-form update, and encodes the new field with the
 * scale E = floor(log2 B) - 13 of the bound
 *   B = 3*max(Mu[i], Mv[i]) + k4*max_{|d|<=R} Mu[i+d] + c2*(Ms[i] + |a_n|*[i == src_i]),
 * M = per-plane maxima of |U^n|, |U^{n-1}|, |s| (of the values before
 * encoding).  Arrays are in the reference layout; halos must be zero.
 */
static inline uint16_t f32_to_f16(float x) {
  _Float16 h = (_Float16)x;
  uint16_t b;
  memcpy(&b, &h, 2);
  return b;
}
static inline float f16_to_f32(uint16_t b) {
  _Float16 h;
  memcpy(&h, &b, 2);
  return (float)h;
}
static inline uint16_t f32_to_bf16(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
static inline float bf16_to_f32(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline float exp2i_f(int e) {
  uint32_t u = (uint32_t)(e + 127) << 23;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline float ulp256(uint16_t hb) {
  int e = (hb >> 10) & 0x1f;
  if (e == 0) e = 1;
  return exp2i_f(e - 33);
}
int orc16_scale_exponent(float B) {
  if (!(B > 0.0f) || !(B < 3.0e38f)) return -100;
  uint32_t u;
  memcpy(&u, &B, 4);
  const int e = (int)((u >> 23) & 0xff);
  if (e == 0) return -100;
  int E = (e - 127) - 13;
  return E < -100 ? -100 : (E > 100 ? 100 : E);
}
static inline float w2f(int kind, uint16_t b) { return kind ? bf16_to_f32(b) : f16_to_f32(b); }
static inline uint16_t f2w(int kind, float x) { return kind ? f32_to_bf16(x) : f32_to_f16(x); }

static inline float dec16(int kind, int hilo, uint16_t h, int8_t q, int E) {
  float x = w2f(kind, h);
  if (hilo) x = fmaf((float)q, ulp256(h), x);
  return x * exp2i_f(E);
}
static inline void enc16(int kind, int hilo, float x, int E, uint16_t* h, int8_t* q) {
  const float xs = x * exp2i_f(-E);
  *h = f2w(kind, xs);
  if (hilo) {
    const float r = xs - w2f(kind, *h);
    int e = (*h >> 10) & 0x1f;
    if (e == 0) e = 1;
    long qi = lrintf(r * exp2i_f(33 - e));
    if (qi > 127) qi = 127;
    if (qi < -127) qi = -127;
    *q = (int8_t)qi;
  }
}

/* Encode a float field (reference layout) into 16-bit storage: plane maxima
 * M (interior), scales E, words h and bytes q (q may be NULL). */
void orc16_encode(int kind, int hilo, const float* x, const unsigned* g, uint16_t* h, int8_t* q,
                  int* E, float* M) {
  const orc_layout L = mk_layout(g);
  for (unsigned i = 0; i < L.xs; i++) {
    float m = 0.0f;
    for (unsigned j = 0; j < L.ys; j++)
      for (unsigned k = 0; k < L.zs; k++) {
        const float a = fabsf(x[L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k]);
        if (a > m) m = a;
      }
    M[i] = m;
    E[i] = orc16_scale_exponent(m);
  }
  const long long ni = L.xs + 2 * L.xh, nj = L.ys + 2 * L.yh, nk = L.zs + 2 * L.zh;
  for (long long ii = 0; ii < ni; ii++) {
    const long long i = ii - L.xh;
    const int e = (i >= 0 && i < (long long)L.xs) ? E[i] : 0;
    for (long long jj = 0; jj < nj; jj++)
      for (long long kk = 0; kk < nk; kk++) {
        const size_t p = (size_t)ii * L.imult + (size_t)jj * L.jmult + (size_t)kk;
        int8_t qq = 0;
        enc16(kind, hilo && q, x[p], e, &h[p], &qq);
        if (q) q[p] = qq;
      }
  }
}

/* Decode the interior of a 16-bit field into float (halos left as they are). */
void orc16_decode(int kind, int hilo, const uint16_t* h, const int8_t* q, const int* E,
                  const unsigned* g, float* x) {
  const orc_layout L = mk_layout(g);
  for (unsigned i = 0; i < L.xs; i++)
    for (unsigned j = 0; j < L.ys; j++)
      for (unsigned k = 0; k < L.zs; k++) {
        const size_t p = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k;
        x[p] = dec16(kind, hilo && q, h[p], q ? q[p] : 0, E[i]);
      }
}

/* FP16 hi/lo pair of a scaled value xs: h = f16(xs), l = f16(xs - h); the
 * difference is exact in float, and h + l (exact in float: at most 22
 * significant bits) is the decoded value. */
static inline void enc_pair(float x, int E, uint16_t* h, uint16_t* l) {
  const float xs = x * exp2i_f(-E);
  *h = f32_to_f16(xs);
  *l = f32_to_f16(xs - f16_to_f32(*h));
}
static inline float dec_pair(uint16_t h, uint16_t l, int E) {
  return (f16_to_f32(h) + f16_to_f32(l)) * exp2i_f(E);
}

/* Encode a float field into the FP16 hi/lo pair storage (the u of the
 * F16_HL form): plane maxima M, scales E (as orc16_encode), words h and l. */
void orc16_encode_pair(const float* x, const unsigned* g, uint16_t* h, uint16_t* l, int* E,
                       float* M) {
  const orc_layout L = mk_layout(g);
  for (unsigned i = 0; i < L.xs; i++) {
    float m = 0.0f;
    for (unsigned j = 0; j < L.ys; j++)
      for (unsigned k = 0; k < L.zs; k++) {
        const float a = fabsf(x[L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k]);
        if (a > m) m = a;
      }
    M[i] = m;
    E[i] = orc16_scale_exponent(m);
  }
  const long long ni = L.xs + 2 * L.xh, nj = L.ys + 2 * L.yh, nk = L.zs + 2 * L.zh;
  for (long long ii = 0; ii < ni; ii++) {
    const long long i = ii - L.xh;
    const int e = (i >= 0 && i < (long long)L.xs) ? E[i] : 0;
    for (long long jj = 0; jj < nj; jj++)
      for (long long kk = 0; kk < nk; kk++) {
        const size_t p = (size_t)ii * L.imult + (size_t)jj * L.jmult + (size_t)kk;
        enc_pair(x[p], e, &h[p], &l[p]);
      }
  }
}

void orc16_decode_pair(const uint16_t* h, const uint16_t* l, const int* E, const unsigned* g,
                       float* x) {
  const orc_layout L = mk_layout(g);
  for (unsigned i = 0; i < L.xs; i++)
    for (unsigned j = 0; j < L.ys; j++)
      for (unsigned k = 0; k < L.zs; k++) {
        const size_t p = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k;
        x[p] = dec_pair(h[p], l[p], E[i]);
      }
}

/* `iterations` steps; on return the u arrays hold U^{n+it} and the v arrays
 * U^{n+it-1} (contents swapped back after an odd count). */
int orc16_iterate_wave(int kind, int hilo, uint16_t* uh, int8_t* uq, int* uE, float* uM,
                       uint16_t* vh, int8_t* vq, int* vE, float* vM, const uint16_t* sh,
                       const int* sE, const float* sM, const unsigned* g, int points,
                       const float* c, float c1, float c2, float k4, const long long* src,
                       const float* amp, unsigned iterations) {
  const orc_layout L = mk_layout(g);
  const int R = radius_of(points);
  if (R < 0 || points == 2) return 1;
  int axis[12], rad[12];
  const int np = pair_order(points, axis, rad);
  long long off_m[12], off_p[12];
  float cf[12];
  for (int p = 0; p < np; p++) {
    const long long st = axis[p] == 0 ? (long long)L.imult : axis[p] == 1 ? (long long)L.jmult : 1;
    off_m[p] = -st * rad[p];
    off_p[p] = st * rad[p];
    cf[p] = c[2 + 4 * axis[p] + rad[p] - 1];
  }
  const int si = (src && src[0] >= 0) ? (int)src[0] : -1;
  const long long src_x = si >= 0 ? (long long)(L.ijk_ofs + (size_t)src[0] * L.imult +
                                                (size_t)src[1] * L.jmult + (size_t)src[2])
                                  : -1;
  int* Eout = (int*)malloc(L.xs * sizeof(int));
  float* Mout = (float*)malloc(L.xs * sizeof(float));
  if (!Eout || !Mout) return 2;
  uint16_t *Uh = uh, *Vh = vh;
  int8_t *Uq = uq, *Vq = vq;
  int *UE = uE, *VE = vE;
  float *UM = uM, *VM = vM;
  for (unsigned it = 0; it < iterations; it++) {
    const float a = amp ? amp[it] : 0.0f;
    for (unsigned i = 0; i < L.xs; i++) {
      float nb = 0.0f;
      for (int d = -R; d <= R; d++) {
        const long long ii = (long long)i + d;
        if (ii >= 0 && ii < (long long)L.xs) nb = fmaxf(nb, UM[ii]);
      }
      float B = 3.0f * fmaxf(UM[i], VM[i]);
      B = B + k4 * nb;
      B = B + c2 * (sM[i] + ((int)i == si ? fabsf(a) : 0.0f));
      Eout[i] = orc16_scale_exponent(B);
      Mout[i] = 0.0f;
    }
#pragma omp parallel for schedule(static)
    for (unsigned i = 0; i < L.xs; i++) {
      float m = 0.0f;
      for (unsigned j = 0; j < L.ys; j++)
        for (unsigned k = 0; k < L.zs; k++) {
          const size_t x = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k;
          /* neighbour words decode with their own plane's scale; halo planes
             are zero whatever their scale */
          float nbv_m[12], nbv_p[12];
          for (int p = 0; p < np; p++) {
            long long im = i, ip = i;
            if (axis[p] == 0) { im = (long long)i - rad[p]; ip = (long long)i + rad[p]; }
            const int em = (im >= 0 && im < (long long)L.xs) ? UE[im] : 0;
            const int ep = (ip >= 0 && ip < (long long)L.xs) ? UE[ip] : 0;
            nbv_m[p] = w2f(kind, Uh[x + off_m[p]]) * exp2i_f(em);
            nbv_p[p] = w2f(kind, Uh[x + off_p[p]]) * exp2i_f(ep);
          }
          const float u0 = dec16(kind, hilo, Uh[x], hilo ? Uq[x] : 0, UE[i]);
          const float v0 = dec16(kind, hilo, Vh[x], hilo ? Vq[x] : 0, VE[i]);
          float s0 = dec16(kind, 0, sh[x], 0, sE[i]);
          if ((long long)x == src_x) s0 = s0 + a;
          const float u2 = u0 + u0;
          float lap = cf[0] * ((nbv_m[0] + nbv_p[0]) - u2);
          for (int p = 1; p < np; p++) lap = fmaf(cf[p], (nbv_m[p] + nbv_p[p]) - u2, lap);
          float t = u2 - v0;
          t = fmaf(c1, lap, t);
          const float out = fmaf(c2, s0, t);
          int8_t qq = 0;
          enc16(kind, hilo, out, Eout[i], &Vh[x], &qq);
          if (hilo) Vq[x] = qq;
          if (fabsf(out) > m) m = fabsf(out);
        }
      Mout[i] = m;
    }
    memcpy(VE, Eout, L.xs * sizeof(int));
    memcpy(VM, Mout, L.xs * sizeof(float));
    { uint16_t* t = Uh; Uh = Vh; Vh = t; }
    { int8_t* t = Uq; Uq = Vq; Vq = t; }
    { int* t = UE; UE = VE; VE = t; }
    { float* t = UM; UM = VM; VM = t; }
  }
  free(Eout);
  free(Mout);
  if (Uh != uh) {
    const size_t n = L.gsize;
    uint16_t* th = (uint16_t*)malloc(n * 2);
    int8_t* tq = (int8_t*)malloc(n);
    if (!th || !tq) return 2;
    memcpy(th, uh, n * 2); memcpy(uh, vh, n * 2); memcpy(vh, th, n * 2);
    if (hilo) { memcpy(tq, uq, n); memcpy(uq, vq, n); memcpy(vq, tq, n); }
    for (unsigned i = 0; i < L.xs; i++) {
      int te = uE[i]; uE[i] = vE[i]; vE[i] = te;
      float tm = uM[i]; uM[i] = vM[i]; vM[i] = tm;
    }
    free(th);
    free(tq);
  }
  return 0;
}

/* The FP16 / BF16 forms hold u and the time difference d = U^n - U^{n-1}
 * (the library's st3d_kernels_delta16.cu).  One step:
 *   scales:  Bd = fmaf(k4, max_{|e|<=R} Mu[i+e], Md[i]);
 *            Bd = fmaf(c2, Ms[i] + |a|[i == src_i], Bd);  Bu = Mu[i] + Bd
 *   point:   acc = w_0 (a_0 + b_0); acc = fmaf(w_p, a_p + b_p, acc) ...
 *            lap = fmaf(m2s, u, acc),  m2s = (float)(-2 sum_p (double)w_p)
 *            d'  = fmaf(c2, s (+a at the source), fmaf(c1, lap, d))
 *            D'  = enc(d', Ed'),  u' = u + dec(D'),  U' = enc(u', Eu')
 *   maxima:  of |u'| and |d'| per plane.
 * u (uh, uE, uM) and d (dh, dE, dM) are updated in place to the newest
 * level.  With ul (the F16_HL form, kind 0) u is the FP16 hi/lo pair
 * (uh, ul): the centre value is dec_pair(uh, ul), the neighbours are the hi
 * words alone, and u' is stored as a pair (enc_pair). */
int orc16_iterate_delta(int kind, uint16_t* uh, int* uE, float* uM, uint16_t* dh, int* dE,
                        float* dM, const uint16_t* sh, const int* sE, const float* sM,
                        const unsigned* g, int points, const float* c, float c1, float c2,
                        float k4, const long long* src, const float* amp, unsigned iterations,
                        uint16_t* ul) {
  const orc_layout L = mk_layout(g);
  const int R = radius_of(points);
  if (R < 0 || points == 2) return 1;
  int axis[12], rad[12];
  const int np = pair_order(points, axis, rad);
  long long off_m[12], off_p[12];
  float cf[12];
  double sw = 0.0;
  for (int p = 0; p < np; p++) {
    const long long st = axis[p] == 0 ? (long long)L.imult : axis[p] == 1 ? (long long)L.jmult : 1;
    off_m[p] = -st * rad[p];
    off_p[p] = st * rad[p];
    cf[p] = c[2 + 4 * axis[p] + rad[p] - 1];
    sw += (double)cf[p];
  }
  const float m2s = (float)(-2.0 * sw);
  const int si = (src && src[0] >= 0) ? (int)src[0] : -1;
  const long long src_x = si >= 0 ? (long long)(L.ijk_ofs + (size_t)src[0] * L.imult +
                                                (size_t)src[1] * L.jmult + (size_t)src[2])
                                  : -1;
  uint16_t* u2 = (uint16_t*)calloc(L.gsize, sizeof(uint16_t));
  uint16_t* l2 = ul ? (uint16_t*)calloc(L.gsize, sizeof(uint16_t)) : NULL;
  int* Ebuf = (int*)malloc(3 * (size_t)L.xs * sizeof(int));
  float* Mbuf = (float*)malloc(3 * (size_t)L.xs * sizeof(float));
  if (!u2 || !Ebuf || !Mbuf || (ul && !l2)) return 2;
  int *UE = uE, *UE2 = Ebuf, *DEo = Ebuf + L.xs;
  float *UM = uM, *UM2 = Mbuf, *DMo = Mbuf + L.xs;
  uint16_t *Uh = uh, *Uh2 = u2, *Ul = ul, *Ul2 = l2;
  for (unsigned it = 0; it < iterations; it++) {
    const float a = amp ? amp[it] : 0.0f;
    for (unsigned i = 0; i < L.xs; i++) {
      float nb = 0.0f;
      for (int e = -R; e <= R; e++) {
        const long long ii = (long long)i + e;
        if (ii >= 0 && ii < (long long)L.xs) nb = fmaxf(nb, UM[ii]);
      }
      float Bd = fmaf(k4, nb, dM[i]);
      Bd = fmaf(c2, sM[i] + ((int)i == si ? fabsf(a) : 0.0f), Bd);
      const float Bu = UM[i] + Bd;
      DEo[i] = orc16_scale_exponent(Bd);
      UE2[i] = orc16_scale_exponent(Bu);
    }
#pragma omp parallel for schedule(static)
    for (unsigned i = 0; i < L.xs; i++) {
      float mu = 0.0f, md = 0.0f;
      for (unsigned j = 0; j < L.ys; j++)
        for (unsigned k = 0; k < L.zs; k++) {
          const size_t x = L.ijk_ofs + (size_t)i * L.imult + (size_t)j * L.jmult + k;
          float acc = 0.0f;
          for (int p = 0; p < np; p++) {
            long long im = i, ip = i;
            if (axis[p] == 0) { im = (long long)i - rad[p]; ip = (long long)i + rad[p]; }
            const int em = (im >= 0 && im < (long long)L.xs) ? UE[im] : 0;
            const int ep = (ip >= 0 && ip < (long long)L.xs) ? UE[ip] : 0;
            const float sum = w2f(kind, Uh[x + off_m[p]]) * exp2i_f(em) +
                              w2f(kind, Uh[x + off_p[p]]) * exp2i_f(ep);
            acc = p == 0 ? cf[0] * sum : fmaf(cf[p], sum, acc);
          }
          /* the neighbours are the hi words; the centre is the whole pair */
          const float u0 = Ul ? dec_pair(Uh[x], Ul[x], UE[i]) : w2f(kind, Uh[x]) * exp2i_f(UE[i]);
          const float lap = fmaf(m2s, u0, acc);
          const float d0 = w2f(kind, dh[x]) * exp2i_f(dE[i]);
          float s0 = w2f(kind, sh[x]) * exp2i_f(sE[i]);
          if ((long long)x == src_x) s0 = s0 + a;
          const float dn = fmaf(c2, s0, fmaf(c1, lap, d0));
          dh[x] = f2w(kind, dn * exp2i_f(-DEo[i]));
          const float dq = w2f(kind, dh[x]) * exp2i_f(DEo[i]);
          const float un = u0 + dq;
          if (Ul)
            enc_pair(un, UE2[i], &Uh2[x], &Ul2[x]);
          else
            Uh2[x] = f2w(kind, un * exp2i_f(-UE2[i]));
          if (fabsf(un) > mu) mu = fabsf(un);
          if (fabsf(dn) > md) md = fabsf(dn);
        }
      UM2[i] = mu;
      DMo[i] = md;
    }
    memcpy(dE, DEo, L.xs * sizeof(int));
    memcpy(dM, DMo, L.xs * sizeof(float));
    { uint16_t* t = Uh; Uh = Uh2; Uh2 = t; }
    { uint16_t* t = Ul; Ul = Ul2; Ul2 = t; }
    { int* t = UE; UE = UE2; UE2 = t; }
    { float* t = UM; UM = UM2; UM2 = t; }
  }
  if (Uh != uh) {
    memcpy(uh, Uh, L.gsize * sizeof(uint16_t));
    if (ul) memcpy(ul, Ul, L.gsize * sizeof(uint16_t));
    memcpy(uE, UE, L.xs * sizeof(int));
    memcpy(uM, UM, L.xs * sizeof(float));
  }
  free(u2);
  free(l2);
  free(Ebuf);
  free(Mbuf);
  return 0;
}
