/* TEST INFRASTRUCTURE ONLY -- the CPU oracle for the VecJac hot path.
 *
 * A portable C restatement of the reference routines that the GPU library replaces:
 *   dbjac2_/zbjac2_/sbjac2_/cbjac2_ and their internal i-variants (src/?bjac2.c),
 *   dvjsvd_/zvjsvd_/svjsvd_/cvjsvd_ (src/?vjsvd.c) with their L1 kernels,
 *   and a placeholder for the libpvn pivot tables behind pjs() (src/pjs.c).
 * It is used only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline, always as the checker. The product (vecjac_gb300/) never links it.
 *
 * Pinning: tests/golden/ holds outputs of the reference compiled from its own sources
 * (oracle/Makefile -> oracle/_ref/libvjref.so, x86-64 with AVX-512 only); the tests
 * require this restatement to reproduce them bit for bit.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -frounding-math, any arch).
 */
#include <fenv.h>
#include <stdint.h>
#include <stdlib.h>

#include "vjo_nrm2.h"

/* product rounded toward -inf (the _MM_FROUND_TO_NEG_INF multiply of src/ddpscl.c:51):
 * the exact error of the round-to-nearest product decides the direction; products too
 * small for an exact error term take the slow path with the rounding mode switched. */
static inline double vjo_dmul_rd(const double x, const double y)
{
  const double p = x * y;
  if (!isfinite(p))
    return p;
  if (fabs(p) >= 0x1p-960) {
    const double e = fma(x, y, -p);
    return ((e < 0.0) ? nextafter(p, -HUGE_VAL) : p);
  }
  volatile double vx = x, vy = y, r;
  const int rm = fegetround();
  fesetround(FE_DOWNWARD);
  r = vx * vy;
  fesetround(rm);
  return r;
}

static inline float vjo_smul_rd(const float x, const float y)
{
  const float p = x * y;
  if (!isfinite(p))
    return p;
  if (fabsf(p) >= 0x1p-96f) {
    const float e = fmaf(x, y, -p);
    return ((e < 0.0f) ? nextafterf(p, -HUGE_VALF) : p);
  }
  volatile float vx = x, vy = y, r;
  const int rm = fegetround();
  fesetround(FE_DOWNWARD);
  r = vx * vy;
  fesetround(rm);
  return r;
}

/* Transformed pairs per sweep of the last SVD call (the reference's JTRACE "sw swt" lines,
 * src/dvjsvd.c:596), first 64 sweeps; read with vjo_last_swt. */
static unsigned long long vjo_trace_swt[64];
static unsigned vjo_trace_nsw;

unsigned vjo_last_swt(unsigned long long *out, unsigned max)
{
  const unsigned k = (vjo_trace_nsw < max) ? vjo_trace_nsw : max;
  for (unsigned i = 0u; i < k && i < 64u; ++i)
    out[i] = vjo_trace_swt[i];
  return vjo_trace_nsw;
}

/* ---------------- FP64: d / z ---------------- */
#define R double
#define LANES 8u
#define LOWMASK 0xFFu
#define BIG_EXP 1020.0
#define SQRT_HUGE 1.34078079299425956E+154
#define RMAX DBL_MAX
#define RTRUEMIN DBL_TRUE_MIN
#define REPS DBL_EPSILON
#define MAX_FIN_EXP 1023.0
#define ROT_EXP_R 1022
#define ROT_EXP_C 1021
#define FMA fma
#define SQRT sqrt
#define H(x) vjo_d##x
#define RBJAC2 vjo_dbjac2_
#define RBJAC2I vjo_dbjac2i
#define CBJAC2 vjo_zbjac2_
#define CBJAC2I vjo_zbjac2i
#define GSVD vjo_dzvjsvd
#define RSVD vjo_dvjsvd_
#define CSVD vjo_zvjsvd_
#include "vjo_prec.h"
/* the scaled compensated dot products on their own, for the tests of the device code */
double vjo_ddpscl_x(long long m, const double *x, const double *y, double ex, double ey, double fx, double fy)
{
  return vjo_ddpscl(m, x, y, ex, ey, fx, fy);
}
void vjo_zdpscl_x(long long m, const double *xr, const double *xi, const double *yr, const double *yi, double ex,
                  double ey, double fx, double fy, double *zr, double *zi)
{
  vjo_dzdpscl(m, xr, xi, yr, yi, ex, ey, fx, fy, zr, zi);
}
#undef R
#undef LANES
#undef LOWMASK
#undef BIG_EXP
#undef SQRT_HUGE
#undef RMAX
#undef RTRUEMIN
#undef REPS
#undef MAX_FIN_EXP
#undef ROT_EXP_R
#undef ROT_EXP_C
#undef FMA
#undef SQRT
#undef H
#undef RBJAC2
#undef RBJAC2I
#undef CBJAC2
#undef CBJAC2I
#undef GSVD
#undef RSVD
#undef CSVD

/* ---------------- FP32: s / c ---------------- */
#define R float
#define LANES 16u
#define LOWMASK 0xFFFFu
#define BIG_EXP 124.0f
#define SQRT_HUGE 1.844674297e+19f
#define RMAX FLT_MAX
#define RTRUEMIN FLT_TRUE_MIN
#define REPS FLT_EPSILON
#define MAX_FIN_EXP 127.0f
#define ROT_EXP_R 126
#define ROT_EXP_C 125
#define FMA fmaf
#define SQRT sqrtf
#define H(x) vjo_s##x
#define RBJAC2 vjo_sbjac2_
#define RBJAC2I vjo_sbjac2i
#define CBJAC2 vjo_cbjac2_
#define CBJAC2I vjo_cbjac2i
#define GSVD vjo_scvjsvd
#define RSVD vjo_svjsvd_
#define CSVD vjo_cvjsvd_
#include "vjo_prec.h"
float vjo_sdpscl_x(long long m, const float *x, const float *y, float ex, float ey, float fx, float fy)
{
  return vjo_sdpscl(m, x, y, ex, ey, fx, fy);
}
void vjo_cdpscl_x(long long m, const float *xr, const float *xi, const float *yr, const float *yi, float ex,
                  float ey, float fx, float fy, float *zr, float *zi)
{
  vjo_szdpscl(m, xr, xi, yr, yi, ex, ey, fx, fy, zr, zi);
}

/* exported column norms (for tests of the norm itself) */
double vjo_dnorm(const long long m, const double *x) { return vjo_dnrm2(m, x); }
float vjo_snorm(const long long m, const float *x) { return vjo_snrm2(m, x); }

/* ---------------- pivot tables ----------------
 * PLACEHOLDER for libpvn's pvn_cjs_* (called by src/pjs.c:28,37; ids PJS_ME=2 with
 * stp=n-1 and PJS_MM=4 with stp=n, src/pjs.h:9,15). libpvn is not vendored, pinned or
 * present, so the exact tables cannot be reproduced; these are published parallel
 * orderings with the same shape and contract (each row a permutation of 0..n-1 read as
 * n/2 pairs, p < q inside every pair):
 *   id 2: the round-robin ("circle") ordering of Brent & Luk (1985), n-1 steps;
 *   id 4: the modulus ordering of Luk & Park (1989), n steps: step k pairs i with
 *         (k - i) mod n, and pairs the two self-paired indices of even k with each other.
 * Returns a malloc'd stp*n table, or NULL. */
unsigned *vjo_pjs(const long id, const unsigned n, unsigned *stp)
{
  *stp = 0u;
  if ((n <= 1u) || (n & 1u))
    return NULL;
  if (id == 2l)
    *stp = n - 1u;
  else if (id == 4l)
    *stp = n;
  else
    return NULL;
  unsigned *const t = (unsigned*)malloc((size_t)n * (size_t)*stp * sizeof(unsigned));
  if (!t)
    return NULL;
  for (unsigned s = 0u; s < *stp; ++s) {
    unsigned *const r = t + (size_t)s * n;
    if (id == 2l) {
      const unsigned N = n - 1u;
      unsigned a = s, b = N;
      r[0] = ((a < b) ? a : b);
      r[1] = ((a < b) ? b : a);
      for (unsigned k = 1u; k < (n >> 1u); ++k) {
        a = (s + k) % N;
        b = (s + N - k) % N;
        r[2u * k] = ((a < b) ? a : b);
        r[2u * k + 1u] = ((a < b) ? b : a);
      }
    }
    else {
      unsigned w = 0u, f0 = n, f1 = n;
      for (unsigned i = 0u; i < n; ++i) {
        const unsigned j = (s + n - i) % n;
        if (j == i) {
          if (f0 == n)
            f0 = i;
          else
            f1 = i;
        }
        else if (i < j) {
          r[w++] = i;
          r[w++] = j;
        }
      }
      if (f0 != n) {
        r[w++] = f0;
        r[w++] = f1;
      }
    }
  }
  return t;
}

/* ---------------- interleaved <-> split complex matrices ----------------
 * zsplit_/zmerge_ (src/zsplit.c:3-56, src/zmerge.c:3-52) and csplit_/cmerge_: column by
 * column, Ar(i,j) = Re A(i,j), Ai(i,j) = Im A(i,j) and back. The reference permutes whole
 * vectors; the element values are moved unchanged. Its release build does no argument
 * checks and returns 1 (OpenMP build). A holds interleaved (re, im) pairs, ldA in complex
 * elements. */
#define VJO_SPLIT(NAME, T)                                                                          \
  long long NAME(const unsigned long long *m, const unsigned long long *n, const T *A,            \
                 const unsigned long long *ldA, T *Ar, const unsigned long long *ldAr, T *Ai,      \
                 const unsigned long long *ldAi)                                                   \
  {                                                                                                \
    for (unsigned long long j = 0u; j < *n; ++j)                                                   \
      for (unsigned long long i = 0u; i < *m; ++i) {                                               \
        Ar[j * *ldAr + i] = A[2u * (j * *ldA + i)];                                                \
        Ai[j * *ldAi + i] = A[2u * (j * *ldA + i) + 1u];                                           \
      }                                                                                            \
    return 1;                                                                                      \
  }
#define VJO_MERGE(NAME, T)                                                                          \
  long long NAME(const unsigned long long *m, const unsigned long long *n, const T *Ar,           \
                 const unsigned long long *ldAr, const T *Ai, const unsigned long long *ldAi, T *A, \
                 const unsigned long long *ldA)                                                    \
  {                                                                                                \
    for (unsigned long long j = 0u; j < *n; ++j)                                                   \
      for (unsigned long long i = 0u; i < *m; ++i) {                                               \
        A[2u * (j * *ldA + i)] = Ar[j * *ldAr + i];                                                \
        A[2u * (j * *ldA + i) + 1u] = Ai[j * *ldAi + i];                                           \
      }                                                                                            \
    return 1;                                                                                      \
  }
VJO_SPLIT(vjo_zsplit_, double)
VJO_MERGE(vjo_zmerge_, double)
VJO_SPLIT(vjo_csplit_, float)
VJO_MERGE(vjo_cmerge_, float)

void vjo_free(void *p) { free(p); }
