// Host harness for the AVX-512-semantics primitives of vecjac_gb300/csrc/vj_fp.cuh
// (compiled with g++ over tests/cuda_host_shim.h) against the oracle's scalar
// restatement of the same instructions (oracle/vjo_fp.h): min/max operand rules, getexp,
// getmant, ilogb, scale2 over the whole shift range (both directions, subnormal and
// overflowing results), scalef with fractional, infinite and NaN exponents, and the x86
// NaN rules of the slow-path arithmetic, in FP64 and FP32.
//
//   fp_host N SEED  ->  "checked mismatches"
#include <cstdint>
#include <cstdio>

#include "cuda_host_shim.h"
#include "../vecjac_gb300/csrc/vj_fp.cuh"
#include "../oracle/vjo_fp.h"

static uint64_t g_s;
static uint64_t rnd()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return g_s;
}

template <typename T> static T draw()
{
  using F = vj::fp<T>;
  const uint64_t r = rnd();
  switch (r % 24) {
  case 0: return (T)0;
  case 1: return -(T)0;
  case 2: return F::inf();
  case 3: return -F::inf();
  case 4: return F::qnan();
  case 5: return F::val((typename F::U)(r >> 11) | (F::bits(F::inf()) + 1u));  // NaN payloads
  case 6: return F::true_min();
  case 7: return -F::max_();
  default: {
    // any bit pattern of a finite value
    typename F::U u = (typename F::U)rnd();
    if (sizeof(T) == 4)
      u = (typename F::U)(u & 0xFFFFFFFFu);
    const T v = F::val(u);
    return std::isfinite(v) ? v : (T)1.5;
  }
  }
}

template <typename T> static bool same(T x, T y) { return vj::fp<T>::bits(x) == vj::fp<T>::bits(y); }

static long long bad = 0, checked = 0;
#define CHECK(a, b)              \
  do {                           \
    ++checked;                   \
    if (!same((a), (b))) {       \
      if (bad < 5)               \
        fprintf(stderr, "%s\n", #a); \
      ++bad;                     \
    }                            \
  } while (0)

static void run_d(long long n)
{
  for (long long i = 0; i < n; ++i) {
    const double x = draw<double>(), y = draw<double>();
    CHECK(vj::vmin(x, y), vjo_dmin(x, y));
    CHECK(vj::vmax(x, y), vjo_dmax(x, y));
    CHECK(vj::getexp(x), vjo_dgetexp(x));
    CHECK(vj::getmant(x), vjo_dgetmant(x));
    if (std::isfinite(x) && x != 0.0) {
      ++checked;
      bad += (vj::ilogb_(x) != vjo_dilogb(x));
      const int k = (int)(rnd() % 4400) - 2200;
      CHECK(vj::scale2(x, k), vjo_dscale2(x, k));
    }
    // scalef: integral, fractional, huge, infinite and NaN exponents
    const double ys[] = {y, std::floor(std::fmod(y, 3000.0)), (double)((int)(rnd() % 5000) - 2500) + 0.5};
    for (double e : ys)
      CHECK(vj::scalef(x, e), vjo_dscalef(x, e));
  }
}

static void run_s(long long n)
{
  for (long long i = 0; i < n; ++i) {
    const float x = draw<float>(), y = draw<float>();
    CHECK(vj::vmin(x, y), vjo_smin(x, y));
    CHECK(vj::vmax(x, y), vjo_smax(x, y));
    CHECK(vj::getexp(x), vjo_sgetexp(x));
    CHECK(vj::getmant(x), vjo_sgetmant(x));
    if (std::isfinite(x) && x != 0.0f) {
      ++checked;
      bad += (vj::ilogb_(x) != vjo_silogb(x));
      const int k = (int)(rnd() % 600) - 300;
      CHECK(vj::scale2(x, k), vjo_sscale2(x, k));
    }
    const float ys[] = {y, std::floor(std::fmod(y, 400.0f)), (float)((int)(rnd() % 700) - 350) + 0.5f};
    for (float e : ys)
      CHECK(vj::scalef(x, e), vjo_sscalef(x, e));
  }
}

int main(int argc, char **argv)
{
  const long long n = (argc > 1) ? atoll(argv[1]) : 1000000;
  g_s = (argc > 2) ? strtoull(argv[2], nullptr, 0) : 0x2545F4914F6CDD1Dull;
  run_d(n);
  run_s(n);
  printf("%lld %lld\n", checked, bad);
  return 0;
}
