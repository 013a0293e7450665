/* TEST INFRASTRUCTURE ONLY -- part of the CPU oracle, never linked into the product.
 *
 * Scalar restatement of the AVX-512 lane operations that the VecJac hot path uses
 * (src/vec.h, src/vecdef.h, src/defops.h, src/sefops.h), with the exact semantics of
 * the x86 instructions under the default MXCSR (round to nearest, no FTZ/DAZ):
 *   VMINPD/VMAXPD  : min(a,b) = (a < b) ? a : b ; max(a,b) = (a > b) ? a : b
 *                    (the second operand is returned when either is a NaN or both are zeros)
 *   VGETEXPPD      : floor(log2|x|) of the normalised value; 0 -> -inf; inf -> +inf
 *   VGETMANTPD     : |x| with its exponent set to 0 (interval [1,2), sign cleared)
 *   VSCALEFPD      : x * 2^floor(y), rounded once; the special cases follow the SDM table
 * Every helper is portable C (no intrinsics) so the oracle builds on x86 and on Arm.
 */
#ifndef VJO_FP_H
#define VJO_FP_H

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint64_t vjo_d2u(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double vjo_u2d(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static inline uint32_t vjo_f2u(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
static inline float vjo_u2f(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

/* ---------------- double ---------------- */
static inline double vjo_dmin(double a, double b) { return (a < b) ? a : b; }
static inline double vjo_dmax(double a, double b) { return (a > b) ? a : b; }
static inline double vjo_dabs(double x) { return vjo_u2d(vjo_d2u(x) & ~(UINT64_C(1) << 63)); }
static inline double vjo_dsgn(double x) { return vjo_u2d(vjo_d2u(x) & (UINT64_C(1) << 63)); }
static inline double vjo_dor(double a, double b) { return vjo_u2d(vjo_d2u(a) | vjo_d2u(b)); }
static inline double vjo_dxor(double a, double b) { return vjo_u2d(vjo_d2u(a) ^ vjo_d2u(b)); }
static inline double vjo_dneg(double x) { return vjo_dxor(x, -0.0); }
/* the x86 default NaN; read through a volatile so that the compiler cannot fold later
 * arithmetic on it into a NaN of another sign */
static inline double vjo_dqnan(void) { volatile uint64_t u = UINT64_C(0xFFF8000000000000); return vjo_u2d(u); }

/* floor(log2|x|) as an int for finite nonzero x */
static inline int vjo_dilogb(double x)
{
  const uint64_t u = vjo_d2u(x) & ~(UINT64_C(1) << 63);
  const int be = (int)(u >> 52);
  if (be)
    return be - 1023;
  /* subnormal: value = mant * 2^-1074 */
  int lz = 0;
  for (uint64_t t = u; !(t & (UINT64_C(1) << 63)); t <<= 1)
    ++lz;
  return -1011 - lz;
}

static inline double vjo_dgetexp(double x)
{
  if (isnan(x))
    return vjo_u2d(vjo_d2u(x) | (UINT64_C(1) << 51));
  if (isinf(x))
    return HUGE_VAL;
  if (x == 0.0)
    return -HUGE_VAL;
  return (double)vjo_dilogb(x);
}

/* |x| * 2^-ilogb(x) for finite nonzero x; 0 stays 0 */
static inline double vjo_dgetmant(double x)
{
  if (isnan(x))
    return x + x;
  if (x == 0.0)
    return 0.0;
  if (isinf(x))
    return 1.0;
  const int e = vjo_dilogb(x);
  double a = vjo_dabs(x);
  /* exact: the result is in [1,2) */
  if (e < -1000)
    a = (a * 0x1p1000) * vjo_u2d((uint64_t)(1023 - (e + 1000)) << 52);
  else if (e > 1000)
    a = (a * 0x1p-1000) * vjo_u2d((uint64_t)(1023 - (e - 1000)) << 52);
  else
    a = a * vjo_u2d((uint64_t)(1023 - e) << 52);
  return a;
}

/* x * 2^n with a single rounding (scaling up is exact until overflow; scaling down
 * takes a first exact step that keeps the result normal, so that only the last
 * multiplication may round -- the classic double-rounding-free scalbn scheme). */
static inline double vjo_dscale2(double x, int n)
{
  if (n > 1023) {
    x *= 0x1p1023; n -= 1023;
    if (n > 1023) { x *= 0x1p1023; n -= 1023; if (n > 1023) n = 1023; }
  }
  else if (n < -1022) {
    x *= 0x1p-969; n += 969;
    if (n < -1022) { x *= 0x1p-969; n += 969; if (n < -1022) n = -1022; }
  }
  return x * vjo_u2d((uint64_t)(n + 1023) << 52);
}

static inline double vjo_dquiet(double x) { return vjo_u2d(vjo_d2u(x) | (UINT64_C(1) << 51)); }

/* VSCALEFPD as measured on an AVX-512 core: a NaN x gives +inf for y = +inf and +0 for
 * y = -inf, otherwise the quieted x; a NaN y (x not NaN) gives the quieted y */
static inline double vjo_dscalef(double x, double y)
{
  if (isnan(x))
    return ((y == HUGE_VAL) ? HUGE_VAL : ((y == -HUGE_VAL) ? 0.0 : vjo_dquiet(x)));
  if (isnan(y))
    return vjo_dquiet(y);
  if (isinf(x))
    return (y == -HUGE_VAL) ? vjo_dqnan() : x;
  if (x == 0.0)
    return (y == HUGE_VAL) ? vjo_dqnan() : x;
  if (y == HUGE_VAL)
    return copysign(HUGE_VAL, x);
  if (y == -HUGE_VAL)
    return copysign(0.0, x);
  double f = floor(y);
  if (f > 4096.0)
    f = 4096.0;
  else if (f < -4096.0)
    f = -4096.0;
  return vjo_dscale2(x, (int)f);
}

/* ---------------- float ---------------- */
static inline float vjo_smin(float a, float b) { return (a < b) ? a : b; }
static inline float vjo_smax(float a, float b) { return (a > b) ? a : b; }
static inline float vjo_sabs(float x) { return vjo_u2f(vjo_f2u(x) & ~(UINT32_C(1) << 31)); }
static inline float vjo_ssgn(float x) { return vjo_u2f(vjo_f2u(x) & (UINT32_C(1) << 31)); }
static inline float vjo_sor(float a, float b) { return vjo_u2f(vjo_f2u(a) | vjo_f2u(b)); }
static inline float vjo_sxor(float a, float b) { return vjo_u2f(vjo_f2u(a) ^ vjo_f2u(b)); }
static inline float vjo_sneg(float x) { return vjo_sxor(x, -0.0f); }
static inline float vjo_sqnan(void) { volatile uint32_t u = UINT32_C(0xFFC00000); return vjo_u2f(u); }

static inline int vjo_silogb(float x)
{
  const uint32_t u = vjo_f2u(x) & ~(UINT32_C(1) << 31);
  const int be = (int)(u >> 23);
  if (be)
    return be - 127;
  int lz = 0;
  for (uint32_t t = u; !(t & (UINT32_C(1) << 31)); t <<= 1)
    ++lz;
  /* value = mant * 2^-149, mant < 2^23 */
  return -118 - lz;
}

static inline float vjo_sgetexp(float x)
{
  if (isnan(x))
    return vjo_u2f(vjo_f2u(x) | (UINT32_C(1) << 22));
  if (isinf(x))
    return HUGE_VALF;
  if (x == 0.0f)
    return -HUGE_VALF;
  return (float)vjo_silogb(x);
}

static inline float vjo_sgetmant(float x)
{
  if (isnan(x))
    return x + x;
  if (x == 0.0f)
    return 0.0f;
  if (isinf(x))
    return 1.0f;
  const int e = vjo_silogb(x);
  float a = vjo_sabs(x);
  if (e < -100)
    a = (a * 0x1p100f) * vjo_u2f((uint32_t)(127 - (e + 100)) << 23);
  else if (e > 100)
    a = (a * 0x1p-100f) * vjo_u2f((uint32_t)(127 - (e - 100)) << 23);
  else
    a = a * vjo_u2f((uint32_t)(127 - e) << 23);
  return a;
}

static inline float vjo_sscale2(float x, int n)
{
  if (n > 127) {
    x *= 0x1p127f; n -= 127;
    if (n > 127) { x *= 0x1p127f; n -= 127; if (n > 127) n = 127; }
  }
  else if (n < -126) {
    x *= 0x1p-102f; n += 102;
    if (n < -126) { x *= 0x1p-102f; n += 102; if (n < -126) n = -126; }
  }
  return x * vjo_u2f((uint32_t)(n + 127) << 23);
}

static inline float vjo_squiet(float x) { return vjo_u2f(vjo_f2u(x) | (UINT32_C(1) << 22)); }

static inline float vjo_sscalef(float x, float y)
{
  if (isnan(x))
    return ((y == HUGE_VALF) ? HUGE_VALF : ((y == -HUGE_VALF) ? 0.0f : vjo_squiet(x)));
  if (isnan(y))
    return vjo_squiet(y);
  if (isinf(x))
    return (y == -HUGE_VALF) ? vjo_sqnan() : x;
  if (x == 0.0f)
    return (y == HUGE_VALF) ? vjo_sqnan() : x;
  if (y == HUGE_VALF)
    return copysignf(HUGE_VALF, x);
  if (y == -HUGE_VALF)
    return copysignf(0.0f, x);
  float f = floorf(y);
  if (f > 512.0f)
    f = 512.0f;
  else if (f < -512.0f)
    f = -512.0f;
  return vjo_sscale2(x, (int)f);
}

#endif /* !VJO_FP_H */
