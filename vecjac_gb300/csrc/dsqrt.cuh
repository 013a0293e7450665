// Correctly rounded FP64 square root of a positive normal number with few operations on
// the FP64 pipe.
//
// GB300's FP64 unit executes about 1.7 operations per clock per SM, and in the FP64 2x2
// EVD the two square roots per element were two thirds of its FP64 work. Here:
//   1. an FP32 estimate y0 of 1/sqrt(x) (rsqrt.approx.f32, relative error about 2^-22) of
//      x's significand with its exponent halved, assembled into an FP64 value with integer
//      operations (no conversion instruction);
//   2. one coupled Newton step for the root (Goldschmidt's iteration as used by Markstein,
//      "Computation of elementary functions on the IBM RISC System/6000 processor", IBM J.
//      Res. Dev. 34, 1990): g0 = x y0, r = 1/2 - g0 y0 / 2, g1 = g0 + g0 r (relative error
//      about 2^-44), then g2 = g1 + (x - g1^2) y0 / 2 (error below 2^-66, so within one unit
//      in the last place of the root);
//   3. the exact residual d = x - g2^2 (one FMA: g2 is within an ulp of the root, so d is a
//      multiple of ulp(g2)^2 below 2^53 of them and fits a double exactly) and Tuckerman's
//      rounding test on it in integer arithmetic: with g2 = Y 2^k (Y the integer
//      significand) and D = d / 2^2k, the root lies above the midpoint g2 + ulp/2 exactly
//      when D >= Y + 1, and below the midpoint under g2 exactly when D <= -Y (or D <= -Y/2
//      when g2 is a power of two, whose lower neighbour is half an ulp away); the root of a
//      double is never a midpoint.
// Five FP64 operations and one FMA for the test, against about ten for the general
// correctly rounded routine. The result is correctly rounded while the estimate's relative
// error stays below about 2^-19 (tests/dsqrt_host.cpp: exact with the estimate moved by up
// to 28 FP32 ulps; beyond 40 the refined value can be two ulps off and the test, which
// corrects one, no longer suffices); rsqrt.approx.f32 is documented within 2^-22.9.
// Domain: 1 <= x < 2^1024 (then the residual's unit ulp(g2)^2 >= 2^-104 is far from the
// subnormal range, so the FMA forms it exactly).
#pragma once
#include "vj_fp.cuh"

namespace vj {

__device__ __forceinline__ float rsqrt_approx(float x)
{
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#elif defined(VJ_DSQRT_HOST_RSQRT)
  return VJ_DSQRT_HOST_RSQRT(x);  // a host test's model of the approximate reciprocal root
#else
  return 1.0f / std::sqrt(x);
#endif
}

// sqrt(x) rounded to nearest for 1 <= x < 2^1024
__device__ __forceinline__ double dsqrt_pos(double x)
{
  using U = unsigned long long;
  const U ux = fp<double>::bits(x);
  const int ex = (int)(ux >> 52) - 1023;
  const int k = ex >> 1;  // floor(ex / 2): x = m 4^k with m in [1, 4)
  // m in FP32: exponent ex - 2k (0 or 1), the top 23 fraction bits
  const float mf = __uint_as_float(((unsigned)(127 + ex - 2 * k) << 23) | (unsigned)((ux >> 29) & 0x7FFFFFu));
  const unsigned uy = __float_as_uint(rsqrt_approx(mf));  // ~ 1/sqrt(m) in (1/2, 1]
  const int ey = (int)(uy >> 23) - 127;
  const U frac = (U)(uy & 0x7FFFFFu) << 29;
  // y0 = 1/sqrt(x) estimate, and y0 / 2, as doubles (exact assembly from the FP32 fields)
  const double y0 = fp<double>::val(((U)(ey - k + 1023) << 52) | frac);
  const double h0 = fp<double>::val(((U)(ey - k + 1022) << 52) | frac);
  const double g0 = x * y0;
  const double r = fp<double>::fma_(-g0, h0, 0.5);
  const double g1 = fp<double>::fma_(g0, r, g0);
  const double d1 = fp<double>::fma_(-g1, g1, x);
  const double g2 = fp<double>::fma_(d1, h0, g1);
  // exact residual and the rounding test
  const double d = fp<double>::fma_(-g2, g2, x);
  const U ug = fp<double>::bits(g2), ud = fp<double>::bits(d);
  const int eg = (int)(ug >> 52) - 1023;
  const long long Y = (long long)((ug & fp<double>::MANT) | (1ull << 52));
  long long D = 0;
  if (ud << 1) {  // d != 0: D = d / 2^(2 (eg - 52)), an integer of magnitude below 2^54
    const int ed = (int)((ud >> 52) & 0x7FF) - 1023;
    const long long md = (long long)((ud & fp<double>::MANT) | (1ull << 52));
    const int sh = ed - 52 - 2 * (eg - 52);  // D = md 2^sh; sh <= 2 when g2 is within an ulp
    D = (sh >= 0) ? (md << sh) : (md >> (-sh));
    if (ud >> 63)
      D = -D;
  }
  if (D >= Y + 1)
    return fp<double>::val(ug + 1u);
  if (D <= ((Y == (1LL << 52)) ? -(Y >> 1) : -Y))
    return fp<double>::val(ug - 1u);
  return g2;
}

}  // namespace vj
