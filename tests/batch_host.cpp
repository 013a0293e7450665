// Host harness for the batched SVD's per-matrix driver (vecjac_gb300/csrc/batch_core.cuh:
// svd_one, the whole one-sided Jacobi SVD of one matrix by one CTA: norms, scaled dot
// products, classification, rotations and shears, rescaling, sweeps), compiled with g++.
// One CTA is emulated by NT threads running the device source with their own threadIdx.x:
// __syncthreads is a barrier of the block, warp shuffles meet at a barrier of their warp,
// atomics are the host's. The result of every matrix (return value, U, V, eS, fS) is
// compared bit for bit with the oracle's restatement of the reference driver
// (vjo_?vjsvd_) on the same pivot ordering, for seeded matrices of many shapes: Gaussian,
// graded singular values, graded columns (rescaling and shears), zero columns, a sweep cap.
//
//   batch_host KIND CASES SEED  ->  "checked mismatches"      (KIND d or s)
#include <cuda_runtime.h>
#undef __device__
#undef __host__
#undef __forceinline__
#undef __global__
#undef __shared__

#include <cstdint>
#include <cstdio>
#include <functional>
#include <vector>

#include <ucontext.h>

#include "cuda_host_shim.h"

#define __global__
#define __shared__ static

// ---- one emulated CTA: NT lanes as fibers on one host thread ----
// A scheduler resumes the lanes in turn; a lane runs until it reaches a barrier
// (__syncthreads, or either half of a shuffle) and yields, so all lanes advance in lock
// step from barrier to barrier, as the kernel's uniform control flow requires.
constexpr unsigned NT = 32;  // threads (one warp: the smallest CTA the kernel takes)
struct Dim3 {
  unsigned x, y, z;
};
static Dim3 threadIdx = {0, 0, 0};  // set by the scheduler before it resumes a lane
static Dim3 blockDim = {NT, 1, 1};
static ucontext_t g_sched, g_lane[NT];
static uint64_t g_slot[32];

static bool g_yielded;  // the resumed lane stopped at a barrier (not at its return)
static inline void barrier()
{
  g_yielded = true;
  swapcontext(&g_lane[threadIdx.x], &g_sched);
}
static inline void __syncthreads() { barrier(); }

template <typename T, typename S> static T exchange(T v, S src)
{
  const unsigned lane = threadIdx.x & 31u;
  uint64_t u = 0;
  memcpy(&u, &v, sizeof(T));
  g_slot[lane] = u;
  barrier();
  T r;
  memcpy(&r, &g_slot[src(lane)], sizeof(T));
  barrier();
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
template <typename T> static T atomic_update(T *p, T v, int op)  // 0 max, 1 min, 2 add
{
  T old = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  for (;;) {
    const T nw = (op == 0) ? (v > old ? v : old) : (op == 1) ? (v < old ? v : old) : (T)(old + v);
    if (__atomic_compare_exchange_n(p, &old, nw, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST))
      return old;
  }
}
static inline unsigned long long atomicMax(unsigned long long *p, unsigned long long v) { return atomic_update(p, v, 0); }
static inline long long atomicMin(long long *p, long long v) { return atomic_update(p, v, 1); }
static inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v) { return atomic_update(p, v, 2); }
static inline unsigned atomicAdd(unsigned *p, unsigned v) { return atomic_update(p, v, 2); }
// device-only helpers of the step kernels that svd_one does not use
static inline long long clock64() { return 0; }
static inline unsigned long long __cvta_generic_to_shared(const void *) { return 0; }

#include "../vecjac_gb300/csrc/batch_core.cuh"

extern "C" {
long long vjo_dvjsvd_(const unsigned long long *, const unsigned long long *, double *, const unsigned long long *,
                      double *, const unsigned long long *, double *, double *, const unsigned *, const unsigned *,
                      const unsigned *, double *, unsigned *);
long long vjo_svjsvd_(const unsigned long long *, const unsigned long long *, float *, const unsigned long long *,
                      float *, const unsigned long long *, float *, float *, const unsigned *, const unsigned *,
                      const unsigned *, float *, unsigned *);
unsigned *vjo_pjs(long, unsigned, unsigned *);
void vjo_free(void *);
}

static uint64_t g_s;
static uint64_t rnd()
{
  g_s ^= g_s << 13;
  g_s ^= g_s >> 7;
  g_s ^= g_s << 17;
  return g_s;
}
static double gauss()
{
  // Box-Muller from two uniform draws
  const double u1 = ((double)(rnd() >> 11) + 0.5) / 9007199254740992.0, u2 = (double)(rnd() >> 11) / 9007199254740992.0;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

// run fn(lane) on the NT fibers until all have returned
static std::function<void(unsigned)> *g_fn;
static void lane_main(unsigned t) { (*g_fn)(t); }
static void run_cta(std::function<void(unsigned)> fn)
{
  static std::vector<char> stacks((size_t)NT << 20);  // 1 MiB per lane
  g_fn = &fn;
  bool done[NT] = {};
  unsigned live = NT;
  for (unsigned t = 0; t < NT; ++t) {
    getcontext(&g_lane[t]);
    g_lane[t].uc_stack.ss_sp = stacks.data() + ((size_t)t << 20);
    g_lane[t].uc_stack.ss_size = (size_t)1 << 20;
    g_lane[t].uc_link = &g_sched;
    makecontext(&g_lane[t], (void (*)())lane_main, 1, t);
  }
  // a lane comes back either from a barrier (g_yielded set) or from its return (uc_link)
  while (live) {
    for (unsigned t = 0; t < NT; ++t) {
      if (done[t])
        continue;
      threadIdx.x = t;
      g_yielded = false;
      swapcontext(&g_sched, &g_lane[t]);
      if (!g_yielded) {
        done[t] = true;
        --live;
      }
    }
  }
}

template <typename T> static bool same(T a, T b)
{
  return (std::isnan(a) && std::isnan(b)) || vj::fp<T>::bits(a) == vj::fp<T>::bits(b);
}

template <typename T> static long long run(int cases)
{
  constexpr long long L = vj::svdc<T>::LANES;
  long long bad = 0;
  for (int c = 0; c < cases; ++c) {
    const uint64_t r = rnd();
    // shapes within the reference's rules: n/2 a multiple of L, m >= n a multiple of L
    const long long n = 2 * L * (long long)(1 + (r % ((sizeof(T) == 8) ? 3 : 2)));
    const long long m = n + L * (long long)((r >> 8) % 5);
    const int kind = c % 5;        // 0 Gaussian, 1 graded columns, 2 zero columns, 3 sweep cap, 4 tall graded
    const int strategy = ((r >> 16) & 1) ? 2 : 4;
    const unsigned swp = (kind == 3) ? 1u + (unsigned)((r >> 20) % 3) : 999u;
    std::vector<T> G((size_t)(m * n)), V((size_t)(n * n)), eS(n), fS(n);
    for (long long j = 0; j < n; ++j) {
      const double colscale = (kind == 1 || kind == 4) ? std::ldexp(1.0, (int)((rnd() >> 40) % 120) - 60) : 1.0;
      const bool zero = (kind == 2) && ((rnd() & 3) == 0);
      for (long long i = 0; i < m; ++i)
        G[(size_t)(j * m + i)] = zero ? (T)0 : (T)(gauss() * colscale);
    }
    // 64-byte aligned copies for the oracle (the reference checks the alignment)
    auto abuf = [](size_t count) { return (T *)aligned_alloc(64, ((count * sizeof(T) + 63) / 64) * 64); };
    T *Go = abuf(G.size()), *Vo = abuf((size_t)(n * n)), *eSo = abuf(n), *fSo = abuf(n), *work = abuf(16 * n + 64);
    memcpy(Go, G.data(), G.size() * sizeof(T));
    std::vector<unsigned> iwork((size_t)(n + 2), 0u);
    // the oracle on the same matrix and pivot ordering
    unsigned stp = 0;
    unsigned *js = vjo_pjs(strategy, (unsigned)n, &stp);
    const unsigned long long um = (unsigned long long)m, un = (unsigned long long)n;
    long long ro;
    if (sizeof(T) == 8)
      ro = vjo_dvjsvd_(&um, &un, (double *)Go, &um, (double *)Vo, &un, (double *)eSo, (double *)fSo, js, &stp, &swp,
                       (double *)work, iwork.data());
    else
      ro = vjo_svjsvd_(&um, &un, (float *)Go, &um, (float *)Vo, &un, (float *)eSo, (float *)fSo, js, &stp, &swp,
                       (float *)work, iwork.data());
    vjo_free(js);
    // the device driver on one emulated CTA
    vj::BatchArgs<T> a{};
    a.strategy = strategy;
    a.swp = swp;
    static vj::BatchShared<T> sh;
    long long rg = 0;
    run_cta([&](unsigned t) {
      const long long v = vj::svd_one<T>(a, sh, m, n, G.data(), V.data(), eS.data(), fS.data());
      if (t == 0)
        rg = v;
    });
    bool ok = (rg == ro);
    if (ok && ro >= 0) {
      for (size_t i = 0; ok && i < G.size(); ++i)
        ok = same(G[i], Go[i]);
      for (size_t i = 0; ok && i < V.size(); ++i)
        ok = same(V[i], Vo[i]);
      for (long long i = 0; ok && i < n; ++i)
        ok = same(eS[i], eSo[i]) && same(fS[i], fSo[i]);
    }
    free(Go);
    free(Vo);
    free(eSo);
    free(fSo);
    free(work);
    if (!ok && bad < 3)
      fprintf(stderr, "case %d: %lldx%lld kind %d strategy %d swp %u: ret %lld vs %lld\n", c, m, n, kind, strategy,
              swp, rg, ro);
    bad += ok ? 0 : 1;
  }
  return bad;
}

int main(int argc, char **argv)
{
  const char kind = (argc > 1) ? argv[1][0] : 'd';
  const int cases = (argc > 2) ? atoi(argv[2]) : 40;
  g_s = (argc > 3) ? strtoull(argv[3], nullptr, 0) : 0x5851F42D4C957F2Dull;
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
