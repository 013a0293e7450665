// Host harness for the SVD's scaled compensated dot products (vecjac_gb300/csrc/svd_dot.cuh:
// pair_dot, the 8/16-lane form of the FP32 step and the batched kernel, and chain_dot, the
// FP64 form with one accumulator chain per warp), compiled with g++ over
// tests/cuda_host_shim.h. A warp is emulated by 32 threads: each runs the device function
// with its own threadIdx.x, and __shfl_down_sync exchanges values through a barrier, so
// the lanes' own code, order and arithmetic are what runs. The result is compared bit for
// bit with the oracle's restatement of src/ddpscl.c / src/zdpscl.c (vjo_?dpscl) on seeded
// columns: lengths from one lane group up to thousands of rows (whole and partial blocks),
// three kinds of values: near 1, scaling to normal numbers (the straight-line blocks);
// graded over the whole exponent range with each column scaled by its largest exponent,
// as the SVD scales by the column norm (subnormal scaled values: the general path); and
// exponents independent of the data, whose scaled values overflow (a NaN result must be
// a NaN there too; its sign is the hardware's, and the SVD returns an error for it).
//
//   dot_host KIND CASES SEED  ->  "checked mismatches"      (KIND one of d z s c)
#include <barrier>
#include <cstdint>
#include <cstdio>
#include <thread>
#include <vector>

#include "cuda_host_shim.h"

// one emulated warp: the lane index of each thread, and the shuffle exchange
struct Dim3 {
  unsigned x, y, z;
};
static thread_local Dim3 threadIdx = {0, 0, 0};
static std::barrier<> *g_warp = nullptr;
static uint64_t g_slot[32];

template <typename T> static T __shfl_down_sync(unsigned, T v, int delta)
{
  const unsigned lane = threadIdx.x & 31u;
  uint64_t u = 0;
  memcpy(&u, &v, sizeof(T));
  g_slot[lane] = u;
  g_warp->arrive_and_wait();
  const unsigned src = (lane + (unsigned)delta < 32u) ? lane + (unsigned)delta : lane;
  T r;
  memcpy(&r, &g_slot[src], sizeof(T));
  g_warp->arrive_and_wait();
  return r;
}

#include "../vecjac_gb300/csrc/svd_dot.cuh"

extern "C" {
double vjo_ddpscl_x(long long, const double *, const double *, double, double, double, double);
float vjo_sdpscl_x(long long, const float *, const float *, float, float, float, float);
void vjo_zdpscl_x(long long, const double *, const double *, const double *, const double *, double, double, double,
                  double, double *, double *);
void vjo_cdpscl_x(long long, const float *, const float *, const float *, const float *, float, float, float, float,
                  float *, float *);
}

static uint64_t g_s;
static uint64_t rnd()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return g_s;
}

// a column value: mode 0 keeps |x| near 1 (scaled values stay normal), modes 1 and 2 draw
// exponents over the whole range (zeros and subnormals included)
template <typename T> static T value(int mode)
{
  const uint64_t r = rnd();
  const T u = (T)1 + (T)((r >> 11) & 0xFFFFF) / (T)1048576;
  const T sgn = (r & 1) ? (T)-1 : (T)1;
  if (mode == 0)
    return sgn * std::ldexp(u, (int)((r >> 40) % 9) - 4);
  if ((r >> 60) == 0)
    return (T)0;
  const int lo = (sizeof(T) == 8) ? -1080 : -155, hi = (sizeof(T) == 8) ? 1023 : 127;
  return sgn * std::ldexp(u, lo + (int)((r >> 32) % (uint64_t)(hi - lo + 1)));
}

// run fn(lane) on 32 threads with threadIdx.x = lane
template <typename F> static void warp(F fn)
{
  std::barrier<> bar(32);
  g_warp = &bar;
  std::vector<std::thread> th;
  for (unsigned l = 0; l < 32; ++l)
    th.emplace_back([&, l] {
      threadIdx.x = l;
      fn(l);
    });
  for (auto &t : th)
    t.join();
}

// bit for bit, a NaN matching any NaN
template <typename T> static bool same(T a, T b)
{
  return (std::isnan(a) && std::isnan(b)) || vj::fp<T>::bits(a) == vj::fp<T>::bits(b);
}

template <typename T, bool CPLX> static long long run(int cases)
{
  constexpr long long L = vj::svdc<T>::LANES;
  long long bad = 0;
  for (int c = 0; c < cases; ++c) {
    const uint64_t r = rnd();
    // lengths: one lane group, a few blocks, partial blocks, long columns
    const long long m = L * (long long)((c % 4 == 0) ? 1 + (r % 4) : (c % 4 == 1) ? 5 + (r % 40) : 1 + (r % 600));
    const int mode = c % 3;
    std::vector<T> xr(m), xi(m), yr(m), yi(m);
    for (long long i = 0; i < m; ++i) {
      xr[i] = value<T>(mode);
      yr[i] = value<T>(mode);
      xi[i] = value<T>(mode);
      yi[i] = value<T>(mode);
    }
    // (e, f) of the two columns as the SVD keeps them: integral exponents, f in [1, 2);
    // mode 1 takes each column's largest exponent (plus one or two, as a norm would)
    const int er = (sizeof(T) == 8) ? 40 : 12;
    T ex = (T)((int)((r >> 8) % (2 * er + 1)) - er), ey = (T)((int)((r >> 20) % (2 * er + 1)) - er);
    if (mode == 1) {
      int mx = -100000, my = -100000;
      for (long long i = 0; i < m; ++i) {
        const T vx[2] = {xr[i], xi[i]}, vy[2] = {yr[i], yi[i]};
        for (int k = 0; k < (CPLX ? 2 : 1); ++k) {
          if (vx[k] != (T)0)
            mx = std::max(mx, std::ilogb(vx[k]));
          if (vy[k] != (T)0)
            my = std::max(my, std::ilogb(vy[k]));
        }
      }
      ex = (T)(mx + 1 + (int)((r >> 56) & 1));
      ey = (T)(my + 1 + (int)((r >> 57) & 1));
    }
    const T fx = (T)1 + (T)((r >> 32) & 0xFFF) / (T)4096, fy = (T)1 + (T)((r >> 44) & 0xFFF) / (T)4096;
    T wr = 0, wi = 0;
    if (sizeof(T) == 8) {
      if (CPLX)
        vjo_zdpscl_x(m, (const double *)xr.data(), (const double *)xi.data(), (const double *)yr.data(),
                     (const double *)yi.data(), (double)ex, (double)ey, (double)fx, (double)fy, (double *)&wr,
                     (double *)&wi);
      else
        wr = (T)vjo_ddpscl_x(m, (const double *)xr.data(), (const double *)yr.data(), (double)ex, (double)ey,
                             (double)fx, (double)fy);
    }
    else {
      if (CPLX)
        vjo_cdpscl_x(m, (const float *)xr.data(), (const float *)xi.data(), (const float *)yr.data(),
                     (const float *)yi.data(), (float)ex, (float)ey, (float)fx, (float)fy, (float *)&wr,
                     (float *)&wi);
      else
        wr = (T)vjo_sdpscl_x(m, (const float *)xr.data(), (const float *)yr.data(), (float)ex, (float)ey, (float)fx,
                             (float)fy);
    }
    // pair_dot: every lane group of the warp computes the same pair; lane 0 has it
    T zr = 0, zi = 0;
    warp([&](unsigned l) {
      T a = 0, b = 0;
      vj::pair_dot<T, CPLX>(m, xr.data(), CPLX ? xi.data() : nullptr, yr.data(), CPLX ? yi.data() : nullptr, ex, ey,
                            fx, fy, true, a, b);
      if (l == 0) {
        zr = a;
        zi = b;
      }
    });
    bool ok = same(zr, wr) && (!CPLX || same(zi, wi));
    if constexpr (sizeof(T) == 8) {
      // chain_dot: one warp per accumulator chain (real: pd, dn; complex: and their
      // imaginary parts), the sums combined as the FP64 step combines them:
      // nu = S_pd + (T_pd + (S_dn + T_dn)), z = nu / (fx fy)
      T S[4] = {0, 0, 0, 0}, Tt[4] = {0, 0, 0, 0};
      const int nch = CPLX ? 4 : 2;
      for (int ch = 0; ch < nch; ++ch)
        warp([&](unsigned l) {
          T s = 0, t = 0;
          const int l8 = (int)(l & 7u);
          const T *pxi = CPLX ? xi.data() : nullptr, *pyi = CPLX ? yi.data() : nullptr;
          switch (ch) {
          case 0: vj::chain_dot<T, CPLX, 0>(m, xr.data(), pxi, yr.data(), pyi, ex, ey, true, l8, s, t); break;
          case 1: vj::chain_dot<T, CPLX, 1>(m, xr.data(), pxi, yr.data(), pyi, ex, ey, true, l8, s, t); break;
          case 2: vj::chain_dot<T, CPLX, 2>(m, xr.data(), pxi, yr.data(), pyi, ex, ey, true, l8, s, t); break;
          default: vj::chain_dot<T, CPLX, 3>(m, xr.data(), pxi, yr.data(), pyi, ex, ey, true, l8, s, t); break;
          }
          if (l == 0) {
            S[ch] = s;
            Tt[ch] = t;
          }
        });
      const T de = fx * fy;
      const T cr = vj::fp<T>::div(S[0] + (Tt[0] + (S[1] + Tt[1])), de);
      const T ci = CPLX ? vj::fp<T>::div(S[2] + (Tt[2] + (S[3] + Tt[3])), de) : (T)0;
      ok = ok && same(cr, wr) && (!CPLX || same(ci, wi));
    }
    if (!ok && bad < 3)
      fprintf(stderr, "case %d: m %lld mode %d: got %.17g %.17g want %.17g %.17g\n", c, m, mode, (double)zr,
              (double)zi, (double)wr, (double)wi);
    bad += ok ? 0 : 1;
  }
  return bad;
}

int main(int argc, char **argv)
{
  const char kind = (argc > 1) ? argv[1][0] : 'd';
  const int cases = (argc > 2) ? atoi(argv[2]) : 200;
  g_s = (argc > 3) ? strtoull(argv[3], nullptr, 0) : 0xD1B54A32D192ED03ull;
  long long bad = 0;
  switch (kind) {
  case 'd': bad = run<double, false>(cases); break;
  case 'z': bad = run<double, true>(cases); break;
  case 's': bad = run<float, false>(cases); break;
  case 'c': bad = run<float, true>(cases); break;
  default: return 2;
  }
  printf("%d %lld\n", cases, bad);
  return 0;
}
