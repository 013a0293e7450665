// Correctly rounded FP64 division on the integer pipes.
//
// GB300 executes FP64 arithmetic on a narrow unit (1.68 FMA per clock per SM, and a
// correctly rounded division costs about 8.6 FMA slots), while the 32-bit integer and
// FP32 pipes are 40-70 times wider. For operands and quotients in the normal range the
// quotient is formed here by schoolbook long division of the 53-bit significands in three
// digits of at most 21 bits: each digit is estimated from an FP32 reciprocal, and the
// exact 64-bit remainder corrects the estimate by one step either way. The result does
// not rest on the estimate being within one step: 0 <= remainder < divisor is checked for
// every digit before rounding, and that check is sound while a digit estimate is off by
// less than 2^10 (the 64-bit remainder arithmetic then cannot wrap), i.e. for an FP32
// reciprocal with relative error below 2^-10 -- the estimate here is within about 2^-21,
// and one step suffices up to 4 ulps of it. Anything else -- zero, subnormal, infinite or
// NaN operands, a quotient outside the normal range, or an estimate that the bounded
// correction cannot repair -- is left to the FP64 division. Rounding is to nearest even:
// up when 2R > d, or 2R == d with an odd quotient.
#pragma once
#include "vj_fp.cuh"

namespace vj {

__device__ __forceinline__ float rcp_approx(float x)
{
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#elif defined(VJ_IDIV_HOST_RCP)
  return VJ_IDIV_HOST_RCP(x);  // a host test's model of the approximate reciprocal
#else
  return 1.0f / x;
#endif
}

// one long-division digit: given the remainder R (0 <= R < d), returns q = floor(R 2^S / d)
// and replaces R by R 2^S - q d. `inv` approximates 2^64 / d in FP32 (d in [2^52, 2^53),
// so inv is in (2^11, 2^12]), and (R >> 22) * inv * 2^(S - 42) estimates the digit. ok is
// cleared when the bounded correction does not reach 0 <= R < d.
template <int S>
__device__ __forceinline__ unsigned ldiv_digit(unsigned long long &R, unsigned long long d, float inv, bool &ok)
{
  // estimate from the top bits of R (R < 2^54, so R >> 22 fits in 32 bits)
  const float rf = __uint2float_rz((unsigned)(R >> 22));
  const float qf = rf * inv * __uint_as_float((unsigned)(127 + S - 42) << 23);
  unsigned q = __float2uint_rz(qf);
  long long r = (long long)((R << S) - (unsigned long long)q * d);
  // one correction either way: the estimate's relative error (FP32 reciprocal, products
  // and conversions, < 2^-21) is below one unit of a 20-bit digit; anything else is caught
  // by the range check below and left to the FP64 unit
  if (r < 0) {
    --q;
    r += (long long)d;
  }
  if (r >= (long long)d) {
    ++q;
    r -= (long long)d;
  }
  ok = ok && (r >= 0) && (r < (long long)d);
  R = (unsigned long long)r;
  return q;
}

// a / b, correctly rounded to nearest; falls back to the FP64 unit outside the normal range
__device__ __forceinline__ double ddiv_int(double a, double b)
{
  using F = fp<double>;
  const unsigned long long ua = F::bits(a), ub = F::bits(b);
  const int ba = (int)((ua >> 52) & 0x7ff), bb = (int)((ub >> 52) & 0x7ff);
  bool ok = (ba > 0) && (ba < 0x7ff) && (bb > 0) && (bb < 0x7ff);
  if (ok) {
    const unsigned long long ma = (ua & F::MANT) | (1ull << 52), mb = (ub & F::MANT) | (1ull << 52);
    int e = ba - bb;  // unbiased exponent difference
    unsigned long long X = ma;
    if (ma < mb) {
      X = ma << 1;
      --e;
    }
    // X / mb in [1, 2); Q = floor(X 2^52 / mb) = q1 2^32 + q2 2^12 + q3
    // 2^64 / mb: the reciprocal of mb / 2^21 is 2^21 / mb; times 2^43
    const float inv = rcp_approx(__uint2float_rn((unsigned)(mb >> 21))) * 8796093022208.0f;
    // first digit: floor(X 2^20 / mb); X < 2 mb, so start from R = X - mb (q1 has its top bit)
    unsigned long long R = X - mb;
    const unsigned q1 = (1u << 20) + ldiv_digit<20>(R, mb, inv, ok);
    const unsigned q2 = ldiv_digit<20>(R, mb, inv, ok);
    const unsigned q3 = ldiv_digit<12>(R, mb, inv, ok);
    unsigned long long Q = ((unsigned long long)q1 << 32) + ((unsigned long long)q2 << 12) + q3;
    const unsigned long long R2 = R << 1;
    Q += ((R2 > mb) || ((R2 == mb) && (Q & 1ull))) ? 1ull : 0ull;
    if (Q >> 53) {
      Q >>= 1;
      ++e;
    }
    const int eb = e + 1023;
    ok = ok && (eb >= 1) && (eb <= 2046) && (Q >> 52) == 1ull && q2 < (1u << 20) && q3 < (1u << 12);
    if (ok)
      return F::val(((ua ^ ub) & F::SIGN) | ((unsigned long long)eb << 52) | (Q & F::MANT));
  }
  return F::div(a, b);
}

}  // namespace vj
