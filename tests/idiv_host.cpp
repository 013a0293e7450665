// Host harness for the integer-pipe FP64 division of the 2x2 kernels
// (vecjac_gb300/csrc/idiv.cuh, ddiv_int), compiled with g++: the CUDA intrinsics it uses
// are modelled exactly on the host (bit casts, round-toward-zero conversions), the FP64
// fallback division is the host's IEEE division with a counter, and the FP32 reciprocal
// estimate is the correctly rounded 1/x moved by K ulps (K from -2 to 2; the device's
// rcp.approx.ftz.f32 is documented within 1 ulp).
//
//   idiv_host N SEED [stress]  ->  one line per K: "K mismatches fallbacks" over N random
//                          pairs with normal operands and quotients, then one line
//                          "special mismatches count" over edge and non-normal operands.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "cuda_host_shim.h"

static int g_ulps = 0;
#define g_fallbacks g_host_ddiv_calls

static inline float model_rcp(float x)
{
  float r = 1.0f / x;
  unsigned u = __float_as_uint(r);
  u = (unsigned)((int)u + g_ulps);
  return __uint_as_float(u);
}
#define VJ_IDIV_HOST_RCP model_rcp

#include "../vecjac_gb300/csrc/idiv.cuh"

static uint64_t g_s;
static uint64_t rnd()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return g_s;
}

static double make(int e, uint64_t mant, bool neg)
{
  const uint64_t u = ((uint64_t)neg << 63) | ((uint64_t)(e + 1023) << 52) | (mant & ((1ull << 52) - 1u));
  return __longlong_as_double((long long)u);
}

// mantissas that stress the digit estimates: random, near 1, near 2, equal and adjacent
static uint64_t mantissa(uint64_t r, uint64_t other)
{
  switch (r % 8) {
  case 0: return 0;
  case 1: return (1ull << 52) - 1u - (r >> 40) % 4;
  case 2: return (r >> 11) % 8;
  case 3: return other;
  case 4: return (other + 1u) & ((1ull << 52) - 1u);
  case 5: return (other - 1u) & ((1ull << 52) - 1u);
  default: return rnd();
  }
}

static bool same(double x, double y) { return __double_as_longlong(x) == __double_as_longlong(y); }

int main(int argc, char **argv)
{
  const long long N = (argc > 1) ? atoll(argv[1]) : 1000000;
  g_s = (argc > 2) ? strtoull(argv[2], nullptr, 0) : 88172645463325252ull;
  // "stress": estimates far outside the correction's reach, which the range check must
  // send to the FP64 unit
  const bool stress = (argc > 3) && !strcmp(argv[3], "stress");
  const int ks[] = {-2, -1, 0, 1, 2}, ks_stress[] = {-4096, -1024, 16, 1024, 4096};
  for (int ki = 0; ki < 5; ++ki) {
    g_ulps = stress ? ks_stress[ki] : ks[ki];
    long long bad = 0;
    g_fallbacks = 0;
    for (long long i = 0; i < N; ++i) {
      const uint64_t mb = rnd();
      const uint64_t ma = mantissa(rnd(), mb);
      const int eb = (int)(rnd() % 1600) - 800;
      const int ea = eb + (int)(rnd() % 400) - 200;
      const double a = make(ea, ma, rnd() & 1u), b = make(eb, mb, rnd() & 1u);
      bad += !same(vj::ddiv_int(a, b), a / b);
    }
    printf("%d %lld %lld\n", g_ulps, bad, g_fallbacks);
  }
  // edges: quotients at and beyond the normal range, subnormal, zero, inf, NaN operands
  g_ulps = 0;
  long long bad = 0, count = 0;
  const double specials[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 4.9406564584124654e-324, 2.2250738585072009e-308,
                             2.2250738585072014e-308, 1.7976931348623157e308, 1.0, -1.5, 3.0};
  for (double a : specials)
    for (double b : specials) {
      const double q = vj::ddiv_int(a, b), r = a / b;
      bad += !(same(q, r) || (std::isnan(q) && std::isnan(r)));
      ++count;
    }
  for (long long i = 0; i < N / 10; ++i) {
    const uint64_t mb = rnd();
    const double b = make((int)(rnd() % 8) - 4 + ((rnd() & 1u) ? 1018 : -1018), mb, false);
    const double a = make((int)(rnd() % 8) - 4 + ((rnd() & 1u) ? 1018 : -1018), mantissa(rnd(), mb), rnd() & 1u);
    const double q = vj::ddiv_int(a, b), r = a / b;
    bad += !same(q, r);
    ++count;
  }
  printf("special %lld %lld\n", bad, count);
  return 0;
}
