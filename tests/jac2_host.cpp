// Host harness for the 2x2 lanes of the batched EVD kernels (vecjac_gb300/csrc/jac2.cuh:
// rjac2, cjac2 with the integer-pipe FP64 division of idiv.cuh), compiled with g++ over
// tests/cuda_host_shim.h: every element of a seeded batch is computed by the device
// source's lane and compared bit for bit with the oracle's ?bjac2_ (outputs and the
// permutation bit; NaN outputs compared as NaN, payloads aside), in both output forms
// (n < 0 sines, n > 0 tangents). Inputs: +-2^e * u with e over the whole exponent range
// (subnormals and overflow-prone values included), mixed with zeros, extremes,
// infinities and NaN.
//
//   jac2_host KIND N SEED  ->  "checked mismatches"      (KIND one of d z s c)
#include <cstdint>
#include <cstdio>
#include <vector>

#include "cuda_host_shim.h"
#include "../vecjac_gb300/csrc/jac2.cuh"

extern "C" {
long long vjo_dbjac2_(const long long *, const double *, const double *, const double *, double *, double *,
                      double *, double *, unsigned *);
long long vjo_sbjac2_(const long long *, const float *, const float *, const float *, float *, float *, float *,
                      float *, unsigned *);
long long vjo_zbjac2_(const long long *, const double *, const double *, const double *, const double *, double *,
                      double *, double *, double *, double *, unsigned *);
long long vjo_cbjac2_(const long long *, const float *, const float *, const float *, const float *, float *, float *,
                      float *, float *, float *, unsigned *);
}

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
  const int emax = (sizeof(T) == 8) ? 1023 : 127, emin = (sizeof(T) == 8) ? -1074 : -149;
  switch (r % 32) {
  case 0: return (T)0;
  case 1: return -(T)0;
  case 2: return F::inf();
  case 3: return -F::inf();
  case 4: return F::qnan();
  case 5: return F::max_();
  case 6: return -F::true_min();
  default: {
    // sign * u * 2^e, u in [1, 2), e uniform over the whole range (subnormals round)
    const int e = emin + (int)((r >> 8) % (uint64_t)(emax - emin + 1));
    const T u = (T)1 + (T)((r >> 20) & 0xFFFFFull) / (T)1048576;
    const T v = std::ldexp(u, e);
    return ((r >> 5) & 1) ? -v : v;
  }
  }
}

template <typename T> static bool same(T x, T y)
{
  if (std::isnan(x) && std::isnan(y))
    return true;
  return vj::fp<T>::bits(x) == vj::fp<T>::bits(y);
}

template <typename T, bool CPLX> static long long run(long long n)
{
  const unsigned L = (sizeof(T) == 8) ? 8u : 16u;
  std::vector<T> a11(n), a22(n), a21(n), a21i(n);
  for (long long i = 0; i < n; ++i) {
    a11[i] = draw<T>();
    a22[i] = draw<T>();
    a21[i] = draw<T>();
    a21i[i] = draw<T>();
  }
  long long bad = 0;
  for (int sgn = -1; sgn <= 1; sgn += 2) {
    const long long nn = sgn * n;
    std::vector<T> c(n), at(n), sat(n), l1(n), l2(n);
    std::vector<unsigned> p(n / L);
    if (sizeof(T) == 8) {
      if (CPLX)
        vjo_zbjac2_(&nn, (const double *)a11.data(), (const double *)a22.data(), (const double *)a21.data(),
                    (const double *)a21i.data(), (double *)c.data(), (double *)at.data(), (double *)sat.data(),
                    (double *)l1.data(), (double *)l2.data(), p.data());
      else
        vjo_dbjac2_(&nn, (const double *)a11.data(), (const double *)a22.data(), (const double *)a21.data(),
                    (double *)c.data(), (double *)at.data(), (double *)l1.data(), (double *)l2.data(), p.data());
    }
    else {
      if (CPLX)
        vjo_cbjac2_(&nn, (const float *)a11.data(), (const float *)a22.data(), (const float *)a21.data(),
                    (const float *)a21i.data(), (float *)c.data(), (float *)at.data(), (float *)sat.data(),
                    (float *)l1.data(), (float *)l2.data(), p.data());
      else
        vjo_sbjac2_(&nn, (const float *)a11.data(), (const float *)a22.data(), (const float *)a21.data(),
                    (float *)c.data(), (float *)at.data(), (float *)l1.data(), (float *)l2.data(), p.data());
    }
    for (long long i = 0; i < n; ++i) {
      T gc, gat, gsat = 0, gl1, gl2;
      unsigned perm;
      if (CPLX)
        perm = (sgn < 0) ? vj::cjac2<T, 1>(a11[i], a22[i], a21[i], a21i[i], gc, gat, gsat, gl1, gl2)
                         : vj::cjac2<T, 0>(a11[i], a22[i], a21[i], a21i[i], gc, gat, gsat, gl1, gl2);
      else
        perm = (sgn < 0) ? vj::rjac2<T, 1>(a11[i], a22[i], a21[i], gc, gat, gl1, gl2)
                         : vj::rjac2<T, 0>(a11[i], a22[i], a21[i], gc, gat, gl1, gl2);
      const unsigned want = (p[i / L] >> (i % L)) & 1u;
      const bool ok = same(gc, c[i]) && same(gat, at[i]) && (!CPLX || same(gsat, sat[i])) && same(gl1, l1[i]) &&
                      same(gl2, l2[i]) && perm == want;
      if (!ok && bad < 3)
        fprintf(stderr, "mismatch at %lld (n %s 0)\n", i, (sgn < 0) ? "<" : ">");
      bad += ok ? 0 : 1;
    }
  }
  return bad;
}

int main(int argc, char **argv)
{
  const char kind = (argc > 1) ? argv[1][0] : 'd';
  long long n = (argc > 2) ? atoll(argv[2]) : (1ll << 20);
  n -= n % 16;
  g_s = (argc > 3) ? strtoull(argv[3], nullptr, 0) : 0x9E3779B97F4A7C15ull;
  long long bad = 0;
  switch (kind) {
  case 'd': bad = run<double, false>(n); break;
  case 'z': bad = run<double, true>(n); break;
  case 's': bad = run<float, false>(n); break;
  case 'c': bad = run<float, true>(n); break;
  default: return 2;
  }
  printf("%lld %lld\n", 2 * n, bad);
  return 0;
}
