// Host models of the CUDA device intrinsics that the library's arithmetic headers
// (vecjac_gb300/csrc/vj_fp.cuh, idiv.cuh, jac2.cuh, pjs.cuh) use, so that host harnesses
// can compile those headers unchanged with g++ (-ffp-contract=off, as the device code is
// built with --fmad=false). Each model is exact: bit casts, IEEE operations that round to
// nearest (host division, square root and fma are correctly rounded), conversions with
// the named rounding. The FP64 division counts its calls (the integer-pipe division's
// fallbacks). The round-down products of the dot products use the host's rounding modes.
#pragma once
#include <algorithm>
#include <cfenv>
#include <cmath>
#include <cstdlib>
#include <cstring>

#define cuda_runtime_h
#define __host__
#define __device__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))

static long long g_host_ddiv_calls = 0;

static inline long long __double_as_longlong(double x) { long long u; memcpy(&u, &x, 8); return u; }
static inline double __longlong_as_double(long long u) { double x; memcpy(&x, &u, 8); return x; }
static inline unsigned __float_as_uint(float x) { unsigned u; memcpy(&u, &x, 4); return u; }
static inline float __uint_as_float(unsigned u) { float x; memcpy(&x, &u, 4); return x; }
static inline int __clzll(long long u) { return u ? __builtin_clzll((unsigned long long)u) : 64; }
static inline int __clz(int u) { return u ? __builtin_clz((unsigned)u) : 32; }
static inline double __ddiv_rn(double a, double b) { ++g_host_ddiv_calls; return a / b; }
static inline double __dsqrt_rn(double a) { return std::sqrt(a); }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
// products rounded toward -inf: the host's multiply under a temporary FE_DOWNWARD
// (the harnesses are built with -frounding-math, so the multiply is not moved or folded)
static inline double __dmul_rd(double a, double b)
{
  const int rm = fegetround();
  fesetround(FE_DOWNWARD);
  volatile double x = a, y = b;
  const double r = x * y;
  fesetround(rm);
  return r;
}
static inline float __fdiv_rn(float a, float b) { return a / b; }
static inline float __fsqrt_rn(float a) { return std::sqrt(a); }
static inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
static inline float __fmul_rd(float a, float b)
{
  const int rm = fegetround();
  fesetround(FE_DOWNWARD);
  volatile float x = a, y = b;
  const float r = x * y;
  fesetround(rm);
  return r;
}
// unsigned -> float toward zero (keep the top 24 significant bits), to nearest
static inline float __uint2float_rz(unsigned x)
{
  const int bl = 32 - (x ? __builtin_clz(x) : 32);
  if (bl > 24)
    x &= ~((1u << (bl - 24)) - 1u);
  return (float)x;
}
static inline float __uint2float_rn(unsigned x) { return (float)x; }
static inline unsigned __float2uint_rz(float f) { return (f <= 0.0f) ? 0u : (unsigned)f; }
static inline int min(int a, int b) { return std::min(a, b); }
static inline int max(int a, int b) { return std::max(a, b); }
