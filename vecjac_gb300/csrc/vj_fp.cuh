// Device arithmetic with the exact semantics of the AVX-512 lane operations that VecJac
// is written in (src/vec.h, src/vecdef.h, src/defops.h), so that every kernel of this
// library reproduces the reference bit for bit:
//   min/max     VMINPD/VMAXPD: (a < b) ? a : b, (a > b) ? a : b
//   getexp      VGETEXPPD: floor(log2|x|); 0 -> -inf, inf -> +inf
//   getmant     VGETMANTPD(NORM_1_2, SIGN_zero)
//   scalef      VSCALEFPD: x * 2^floor(y), one rounding, SDM special cases
// plus correctly rounded division, square root, FMA and the round-down product.
// All code is compiled with --fmad=false: a multiply and an add are never fused
// implicitly, every FMA is written out.
#pragma once
#include <cstdint>
#ifndef cuda_runtime_h
#include <cuda_runtime.h>
#endif

namespace vj {

template <typename T> struct fp;

template <> struct fp<double> {
  using U = unsigned long long;
  static constexpr int MB = 52, BIAS = 1023, EMAXB = 2046;
  static constexpr U SIGN = 1ull << 63, MANT = (1ull << 52) - 1ull;
  static __device__ __forceinline__ U bits(double x) { return (U)__double_as_longlong(x); }
  static __device__ __forceinline__ double val(U u) { return __longlong_as_double((long long)u); }
  static __device__ __forceinline__ int clz(U u) { return __clzll((long long)u); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
  static __device__ __forceinline__ double mul_rd(double a, double b) { return __dmul_rd(a, b); }
  static __device__ __forceinline__ double max_() { return 1.7976931348623157e308; }
  static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7ff0000000000000ll); }
  static __device__ __forceinline__ double qnan() { return __longlong_as_double((long long)0xfff8000000000000ull); }
  static __device__ __forceinline__ double true_min() { return __longlong_as_double(1ll); }
  // VecJac's constants (src/dzjac2.h:10,16)
  static __device__ __forceinline__ double big_exp() { return 1020.0; }
  static __device__ __forceinline__ double sqrt_huge() { return 1.34078079299425956E+154; }
};

template <> struct fp<float> {
  using U = unsigned;
  static constexpr int MB = 23, BIAS = 127, EMAXB = 254;
  static constexpr U SIGN = 1u << 31, MANT = (1u << 23) - 1u;
  static __device__ __forceinline__ U bits(float x) { return (U)__float_as_uint(x); }
  static __device__ __forceinline__ float val(U u) { return __uint_as_float(u); }
  static __device__ __forceinline__ int clz(U u) { return __clz((int)u); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
  static __device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ float mul_rd(float a, float b) { return __fmul_rd(a, b); }
  static __device__ __forceinline__ float max_() { return 3.40282347e+38f; }
  static __device__ __forceinline__ float inf() { return __uint_as_float(0x7f800000u); }
  static __device__ __forceinline__ float qnan() { return __uint_as_float(0xffc00000u); }
  static __device__ __forceinline__ float true_min() { return __uint_as_float(1u); }
  // src/scjac2.h:10,16
  static __device__ __forceinline__ float big_exp() { return 124.0f; }
  static __device__ __forceinline__ float sqrt_huge() { return 1.844674297e+19f; }
};

template <typename T> __device__ __forceinline__ T vmin(T a, T b) { return (a < b) ? a : b; }
template <typename T> __device__ __forceinline__ T vmax(T a, T b) { return (a > b) ? a : b; }
template <typename T> __device__ __forceinline__ T vabs(T x) { return fp<T>::val(fp<T>::bits(x) & ~fp<T>::SIGN); }
template <typename T> __device__ __forceinline__ T vsgn(T x) { return fp<T>::val(fp<T>::bits(x) & fp<T>::SIGN); }
template <typename T> __device__ __forceinline__ T vor(T a, T b) { return fp<T>::val(fp<T>::bits(a) | fp<T>::bits(b)); }
template <typename T> __device__ __forceinline__ T vxor(T a, T b) { return fp<T>::val(fp<T>::bits(a) ^ fp<T>::bits(b)); }
template <typename T> __device__ __forceinline__ T vneg(T x) { return fp<T>::val(fp<T>::bits(x) ^ fp<T>::SIGN); }
template <typename T> __device__ __forceinline__ bool visnan(T x) { return (fp<T>::bits(x) & ~fp<T>::SIGN) > (fp<T>::bits(fp<T>::inf())); }
template <typename T> __device__ __forceinline__ bool visfinite(T x) { return (fp<T>::bits(x) & ~fp<T>::SIGN) < (fp<T>::bits(fp<T>::inf())); }
// a NaN operand propagated the x86 way: quieted, sign and payload kept
template <typename T> __device__ __forceinline__ T vquiet(T x) { return fp<T>::val(fp<T>::bits(x) | (fp<T>::MANT ^ (fp<T>::MANT >> 1))); }

// Arithmetic with the x86 NaN rules (used only on the inf/NaN slow paths): a NaN operand
// is returned quieted, the first one in operand order; an invalid operation returns the
// x86 default NaN (negative, quiet). The GPU's own arithmetic returns a canonical NaN
// instead, whose sign would otherwise reach the sign of later zeros.
template <typename T> __device__ __forceinline__ T xadd(T a, T b)
{
  if (visnan(a)) return vquiet(a);
  if (visnan(b)) return vquiet(b);
  const T r = a + b;
  return visnan(r) ? fp<T>::qnan() : r;
}
template <typename T> __device__ __forceinline__ T xsub(T a, T b)
{
  if (visnan(a)) return vquiet(a);
  if (visnan(b)) return vquiet(b);
  const T r = a - b;
  return visnan(r) ? fp<T>::qnan() : r;
}
template <typename T> __device__ __forceinline__ T xmul(T a, T b)
{
  if (visnan(a)) return vquiet(a);
  if (visnan(b)) return vquiet(b);
  const T r = a * b;
  return visnan(r) ? fp<T>::qnan() : r;
}
template <typename T> __device__ __forceinline__ T xdiv(T a, T b)
{
  if (visnan(a)) return vquiet(a);
  if (visnan(b)) return vquiet(b);
  const T r = fp<T>::div(a, b);
  return visnan(r) ? fp<T>::qnan() : r;
}
template <typename T> __device__ __forceinline__ T xsqrt(T a)
{
  if (visnan(a)) return vquiet(a);
  const T r = fp<T>::sqrt_(a);
  return visnan(r) ? fp<T>::qnan() : r;
}
template <typename T> __device__ __forceinline__ T xfma(T a, T b, T c)
{
  if (visnan(a)) return vquiet(a);
  if (visnan(b)) return vquiet(b);
  if (visnan(c)) return vquiet(c);
  const T r = fp<T>::fma_(a, b, c);
  return visnan(r) ? fp<T>::qnan() : r;
}

// floor(log2|x|) of a finite nonzero x (subnormals normalised)
template <typename T> __device__ __forceinline__ int ilogb_(T x)
{
  using F = fp<T>;
  const typename F::U u = F::bits(x) & ~F::SIGN;
  const int be = (int)(u >> F::MB);
  if (be)
    return be - F::BIAS;
  // value = u * 2^(1 - BIAS - MB); floor(log2 u) = (bits-1) - clz(u)
  return (int)(sizeof(typename F::U) * 8 - 1) - F::clz(u) + (1 - F::BIAS - F::MB);
}

// VGETEXP
template <typename T> __device__ __forceinline__ T getexp(T x)
{
  using F = fp<T>;
  const typename F::U u = F::bits(x) & ~F::SIGN;
  if (u >= F::bits(F::inf()))
    return (u == F::bits(F::inf())) ? F::inf() : vquiet(x);  // inf -> +inf, NaN -> NaN
  if (!u)
    return vneg(F::inf());
  return (T)ilogb_(x);
}

// x * 2^n, n in [-(BIAS-1), BIAS], exactly as a power of two
template <typename T> __device__ __forceinline__ T pow2(int n)
{
  using F = fp<T>;
  return F::val((typename F::U)(n + F::BIAS) << F::MB);
}

// x * 2^n with a single rounding. Normal results of normal inputs are formed by an
// integer add on the exponent field; everything else goes through multiplications by
// powers of two, where a first exact step keeps the value normal so that only the
// last product can round (no double rounding in the subnormal range).
template <typename T> __device__ __forceinline__ T scale2(T x, int n)
{
  using F = fp<T>;
  const typename F::U u = F::bits(x);
  const int be = (int)((u & ~F::SIGN) >> F::MB);
  if ((be > 0) && (be <= F::EMAXB) && (be + n > 0) && (be + n <= F::EMAXB))
    return F::val(u + ((typename F::U)(long long)n << F::MB));
  constexpr int HI = F::BIAS, LO = 1 - F::BIAS, STEP = F::BIAS - 1 - F::MB - 1;  // 969 / 102
  if (n > HI) {
    x = x * pow2<T>(HI); n -= HI;
    if (n > HI) { x = x * pow2<T>(HI); n -= HI; if (n > HI) n = HI; }
  }
  else if (n < LO) {
    x = x * pow2<T>(-STEP); n += STEP;
    if (n < LO) { x = x * pow2<T>(-STEP); n += STEP; if (n < LO) n = LO; }
  }
  return x * pow2<T>(n);
}

// VSCALEF (x * 2^floor(y)) with the special cases of the instruction
template <typename T> __device__ __forceinline__ T scalef(T x, T y)
{
  using F = fp<T>;
  // measured on AVX-512: a NaN x gives +inf for y = +inf and +0 for y = -inf
  if (visnan(x))
    return (y == F::inf()) ? F::inf() : ((y == vneg(F::inf())) ? (T)0 : vquiet(x));
  if (visnan(y))
    return vquiet(y);
  const bool xinf = !visfinite(x);
  if (xinf)
    return (y == vneg(F::inf())) ? F::qnan() : x;
  if (x == (T)0)
    return (y == F::inf()) ? F::qnan() : x;
  if (y == F::inf())
    return vor(F::inf(), vsgn(x));
  if (y == vneg(F::inf()))
    return vsgn(x);
  const T lim = (sizeof(T) == 8) ? (T)4096 : (T)512;
  const T f = floor(vmax(vmin(y, lim), -lim));
  return scale2(x, (int)f);
}

// VGETMANT(NORM_1_2, SIGN_zero) for finite nonzero x
template <typename T> __device__ __forceinline__ T getmant_fin(T x)
{
  const int e = ilogb_(x);
  return scale2(vabs(x), -e);
}

template <typename T> __device__ __forceinline__ T getmant(T x)
{
  if (visnan(x))
    return vquiet(x);
  if (x == (T)0)
    return (T)0;
  if (!visfinite(x))
    return (T)1;
  return getmant_fin(x);
}

}  // namespace vj
