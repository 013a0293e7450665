// Host harness for the project's column norm on one warp (vecjac_gb300/csrc/svd_norm.cuh:
// warp_nrm2, which every SVD kernel uses for the column norms), compiled with g++ over
// tests/cuda_host_shim.h with a warp emulated by 32 threads (each lane's own code; the
// shuffles meet at a barrier), against the oracle's restatement (vjo_dnorm / vjo_snorm):
// bit for bit on seeded columns of 1 to thousands of rows, values near 1, graded values
// over the whole exponent range (subnormals included), zero columns, and columns holding
// an infinity or a NaN.
//
//   norm_host KIND CASES SEED  ->  "checked mismatches"      (KIND d or s)
#include <barrier>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <thread>
#include <vector>

#include "cuda_host_shim.h"

struct Dim3 {
  unsigned x, y, z;
};
static thread_local Dim3 threadIdx = {0, 0, 0};
static std::barrier<> *g_warp = nullptr;
static uint64_t g_slot[32];

// lane `src(lane)`'s value of v, for every lane of the warp
template <typename T, typename S> static T exchange(T v, S src)
{
  const unsigned lane = threadIdx.x & 31u;
  uint64_t u = 0;
  memcpy(&u, &v, sizeof(T));
  g_slot[lane] = u;
  g_warp->arrive_and_wait();
  T r;
  memcpy(&r, &g_slot[src(lane)], sizeof(T));
  g_warp->arrive_and_wait();
  return r;
}
template <typename T> static T __shfl_down_sync(unsigned, T v, int d)
{
  return exchange(v, [d](unsigned l) { return (l + (unsigned)d < 32u) ? l + (unsigned)d : l; });
}
template <typename T> static T __shfl_xor_sync(unsigned, T v, int m)
{
  return exchange(v, [m](unsigned l) { return l ^ (unsigned)m; });
}
template <typename T> static T __shfl_sync(unsigned, T v, int s)
{
  return exchange(v, [s](unsigned) { return (unsigned)s; });
}

#include "../vecjac_gb300/csrc/svd_norm.cuh"

extern "C" {
double vjo_dnorm(long long, const double *);
float vjo_snorm(long long, const float *);
}

static uint64_t g_s;
static uint64_t rnd()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return g_s;
}

template <typename T> static T value(int mode)
{
  const uint64_t r = rnd();
  const T u = (T)1 + (T)((r >> 11) & 0xFFFFF) / (T)1048576;
  const T sgn = (r & 1) ? (T)-1 : (T)1;
  if (mode == 0)
    return sgn * std::ldexp(u, (int)((r >> 40) % 9) - 4);
  const int lo = (sizeof(T) == 8) ? -1080 : -155, hi = (sizeof(T) == 8) ? 1023 : 127;
  return sgn * std::ldexp(u, lo + (int)((r >> 32) % (uint64_t)(hi - lo + 1)));
}

template <typename T> static bool same(T a, T b)
{
  return (std::isnan(a) && std::isnan(b)) || vj::fp<T>::bits(a) == vj::fp<T>::bits(b);
}

template <typename T> static long long run(int cases)
{
  long long bad = 0;
  for (int c = 0; c < cases; ++c) {
    const uint64_t r = rnd();
    const long long m = (c % 5 == 0) ? 1 + (long long)(r % 40) : 1 + (long long)(r % 5000);
    const int mode = c % 5;  // 0 near 1, 1-2 graded, 3 zeros with a few values, 4 inf or NaN
    std::vector<T> x(m);
    for (long long i = 0; i < m; ++i)
      x[i] = (mode == 3 && (rnd() % 7)) ? (T)0 : value<T>(mode == 0 ? 0 : 1);
    if (mode == 4)
      x[rnd() % m] = (r >> 63) ? std::numeric_limits<T>::infinity() : std::numeric_limits<T>::quiet_NaN();
    if (mode == 3 && (r & 2))
      std::fill(x.begin(), x.end(), (T)0);
    const T want = (sizeof(T) == 8) ? (T)vjo_dnorm(m, (const double *)x.data()) : (T)vjo_snorm(m, (const float *)x.data());
    T got[32];
    std::barrier<> bar(32);
    g_warp = &bar;
    std::vector<std::thread> th;
    for (unsigned l = 0; l < 32; ++l)
      th.emplace_back([&, l] {
        threadIdx.x = l;
        got[l] = vj::warp_nrm2<T>(x.data(), m);
      });
    for (auto &t : th)
      t.join();
    bool ok = true;
    for (unsigned l = 0; l < 32; ++l)  // every lane returns the norm
      ok = ok && same(got[l], want);
    if (!ok && bad < 3)
      fprintf(stderr, "case %d: m %lld mode %d: got %.17g want %.17g\n", c, m, mode, (double)got[0], (double)want);
    bad += ok ? 0 : 1;
  }
  return bad;
}

int main(int argc, char **argv)
{
  const char kind = (argc > 1) ? argv[1][0] : 'd';
  const int cases = (argc > 2) ? atoi(argv[2]) : 200;
  g_s = (argc > 3) ? strtoull(argv[3], nullptr, 0) : 0x94D049BB133111EBull;
  long long bad = 0;
  if (kind == 'd')
    bad = run<double>(cases);
  else if (kind == 's')
    bad = run<float>(cases);
  else
    return 2;
  printf("%d %lld\n", cases, bad);
  return 0;
}
