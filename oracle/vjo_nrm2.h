/* TEST INFRASTRUCTURE ONLY -- part of the CPU oracle.
 *
 * The Euclidean column norm that this project uses in place of BLAS xNRM2.
 * VecJac's dnorm2_/snorm2_/znorm2_/cnorm2_ (src/dnorm2.c:12, src/snorm2.c:12,
 * src/znorm2.c:12-14, src/cnorm2.c:12-14) call the BLAS xNRM2 of whatever library
 * is linked (MKL upstream); no reference test pins its bits. The GPU build computes
 * the norm with the algorithm below, and the oracle (both the C restatement and the
 * reference compiled from source, through oracle/ref_shim.c) uses the very same one,
 * so that the whole SVD can be compared bit for bit.
 *
 * Algorithm (two-pass power-of-two scaling, overflow- and underflow-safe):
 *   1. a = max_i |x_i|; a == 0 -> 0; a not finite -> a (inf) / NaN.
 *   2. k = floor(log2 a); y_i = x_i * 2^-k (one rounding, y_i in [0,2)).
 *   3. VJ_NRM2_LANES = 32 accumulators: lane l sums y_i^2 (fma) for i = l (mod 32)
 *      in increasing i.
 *   4. Halving tree: for w = 16,8,4,2,1: acc[l] += acc[l+w] (l < w).
 *   5. return sqrt(acc[0]) * 2^k (one rounding).
 * The complex modulus of (‖re‖, ‖im‖) uses the same scaled hypot as VecJac's VDHYPOT
 * (src/vecdef.h:80-92): M*sqrt(1+(m/M)^2).
 */
#ifndef VJO_NRM2_H
#define VJO_NRM2_H

#include "vjo_fp.h"

#define VJ_NRM2_LANES 32

static inline double vjo_dnrm2(const long long m, const double *const x)
{
  double a = 0.0;
  int nan = 0;
  for (long long i = 0; i < m; ++i) {
    const double t = vjo_dabs(x[i]);
    if (isnan(t))
      nan = 1;
    a = vjo_dmax(t, a);
  }
  if (nan)
    return vjo_dqnan();
  if (!(a <= DBL_MAX))
    return a;
  if (a == 0.0)
    return 0.0;
  const int k = vjo_dilogb(a);
  double acc[VJ_NRM2_LANES];
  for (int l = 0; l < VJ_NRM2_LANES; ++l)
    acc[l] = 0.0;
  for (long long i = 0; i < m; ++i) {
    const double y = vjo_dscale2(x[i], -k);
    acc[i % VJ_NRM2_LANES] = fma(y, y, acc[i % VJ_NRM2_LANES]);
  }
  for (int w = VJ_NRM2_LANES / 2; w >= 1; w >>= 1)
    for (int l = 0; l < w; ++l)
      acc[l] = acc[l] + acc[l + w];
  return vjo_dscale2(sqrt(acc[0]), k);
}

static inline float vjo_snrm2(const long long m, const float *const x)
{
  float a = 0.0f;
  int nan = 0;
  for (long long i = 0; i < m; ++i) {
    const float t = vjo_sabs(x[i]);
    if (isnan(t))
      nan = 1;
    a = vjo_smax(t, a);
  }
  if (nan)
    return vjo_sqnan();
  if (!(a <= FLT_MAX))
    return a;
  if (a == 0.0f)
    return 0.0f;
  const int k = vjo_silogb(a);
  float acc[VJ_NRM2_LANES];
  for (int l = 0; l < VJ_NRM2_LANES; ++l)
    acc[l] = 0.0f;
  for (long long i = 0; i < m; ++i) {
    const float y = vjo_sscale2(x[i], -k);
    acc[i % VJ_NRM2_LANES] = fmaf(y, y, acc[i % VJ_NRM2_LANES]);
  }
  for (int w = VJ_NRM2_LANES / 2; w >= 1; w >>= 1)
    for (int l = 0; l < w; ++l)
      acc[l] = acc[l] + acc[l + w];
  return vjo_sscale2(sqrtf(acc[0]), k);
}

/* VDHYPOT / VSHYPOT in scalar form */
static inline double vjo_dhypot(const double x, const double y)
{
  const double x_ = vjo_dabs(x), y_ = vjo_dabs(y);
  const double m_ = vjo_dmin(x_, y_), M_ = vjo_dmax(x_, y_);
  double z = m_ / M_;
  z = vjo_dmax(z, 0.0);
  z = fma(z, z, 1.0);
  z = sqrt(z);
  return z * M_;
}

static inline float vjo_shypot(const float x, const float y)
{
  const float x_ = vjo_sabs(x), y_ = vjo_sabs(y);
  const float m_ = vjo_smin(x_, y_), M_ = vjo_smax(x_, y_);
  float z = m_ / M_;
  z = vjo_smax(z, 0.0f);
  z = fmaf(z, z, 1.0f);
  z = sqrtf(z);
  return z * M_;
}

#endif /* !VJO_NRM2_H */
