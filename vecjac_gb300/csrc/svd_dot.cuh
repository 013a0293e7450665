// The SVD's scaled compensated dot products in the reference's lane order (src/ddpscl.c,
// src/zdpscl.c): the per-precision constants, 2Sum, the lanes' halving-tree sum, the
// 8/16-lane form (pair_dot: the FP32 step and the batched kernel) and the FP64 form with
// one accumulator chain per warp (chain_dot: the FP64 step). Device code that needs only
// vj_fp.cuh, threadIdx.x and __shfl_down_sync, so that a host harness can run it lane by
// lane.
#pragma once
#include <cfloat>

#include "vj_fp.cuh"

namespace vj {

template <typename T> struct svdc;
template <> struct svdc<double> {
  static constexpr int LANES = 8;
  static constexpr double EPS = DBL_EPSILON;
  static constexpr int ROT_R = 1022, ROT_C = 1021;
  static constexpr double MAX_FIN_EXP = 1023.0;
  static constexpr double RMAX = DBL_MAX;
};
template <> struct svdc<float> {
  static constexpr int LANES = 16;
  static constexpr float EPS = FLT_EPSILON;
  static constexpr int ROT_R = 126, ROT_C = 125;
  static constexpr float MAX_FIN_EXP = 127.0f;
  static constexpr float RMAX = FLT_MAX;
};

// 2Sum (src/d2sum.h)
template <typename T> __device__ __forceinline__ void two_sum(T a, T b, T &s, T &t)
{
  const T s_ = a + b;
  T a_ = s_ - b;
  T b_ = s_ - a_;
  a_ = a - a_;
  b_ = b - b_;
  s = s_;
  t = a_ + b_;
}

// halving tree over the LANES lanes of warp 0 (GCC's _mm512_reduce_add order); lane 0 has it
template <int LANES, typename T> __device__ __forceinline__ T hsum(T v)
{
#pragma unroll
  for (int w = LANES / 2; w >= 1; w >>= 1)
    v = __shfl_down_sync(0xffffffffu, v, w) + v;
  return v;
}

// scaled compensated dot products (src/ddpscl.c / src/zdpscl.c) by LANES lanes; x = G_q,
// y = G_p. Only the two (four for complex data) 2Sum accumulations carry a dependency from
// one element to the next; the loads, the power-of-two scaling and the exact product split
// (round-down product and its error by an FMA) of the elements of a block are independent
// of it, and blocks of normal values run as straight-line code so that their latency
// overlaps the accumulator chains.
template <typename T, bool CPLX> struct DotTerms {
  T pd[CPLX ? 4 : 1], dn[CPLX ? 4 : 1];
};

// The accumulation uses branch-free 2Sum: on GB300 a value moving from the FP64 unit to
// the integer pipes (as Fast2Sum's magnitude test would need) costs several hundred
// cycles, more than 2Sum's three extra FP64 additions.
template <typename T>
__device__ __forceinline__ void dot_acc(T pd, T dn, T &s, T &t, T &s_, T &t_)
{
  two_sum(s, pd + t, s, t);
  two_sum(s_, dn + t_, s_, t_);
}

template <typename T, bool CPLX>
__device__ void pair_dot(long long m, const T *xr, const T *xi, const T *yr, const T *yi, T ex, T ey, T fx, T fy,
                         bool live, T &zr, T &zi)
{
  using F = fp<T>;
  constexpr int L = svdc<T>::LANES;
  constexpr int NV = CPLX ? 4 : 2;  // values loaded per element
  constexpr int D = 4;              // elements per block (the next block's loads in flight)
  const int lane = (threadIdx.x & 31) % L;
  const int nx = -(int)ex, ny = -(int)ey;
  T sr = 0, tr = 0, sr_ = 0, tr_ = 0, si = 0, ti = 0, si_ = 0, ti_ = 0;
  auto load = [&](long long i, T (&v)[NV]) {
    if (i < m) {
      v[0] = xr[i];
      v[1] = yr[i];
      if (CPLX) {
        v[2] = xi[i];
        v[3] = yi[i];
      }
    }
  };
  // products of one element from its scaled values; (negations are written as FP
  // negations: the FMA folds them, with the same bits)
  auto products = [&](T xri, T yri, T xii, T yii, DotTerms<T, CPLX> &d) {
    if (CPLX) {
      const T xs[4] = {xri, xii, xri, -xii}, ys[4] = {yri, yii, yii, yri};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        d.pd[k] = F::mul_rd(xs[k], ys[k]);
        d.dn[k] = F::fma_(xs[k], ys[k], -d.pd[k]);
      }
    }
    else {
      d.pd[0] = F::mul_rd(xri, yri);
      d.dn[0] = F::fma_(xri, yri, -d.pd[0]);
    }
  };
  auto accumulate = [&](const DotTerms<T, CPLX> &c) {
    if (CPLX) {
      dot_acc(c.pd[0], c.dn[0], sr, tr, sr_, tr_);
      dot_acc(c.pd[1], c.dn[1], sr, tr, sr_, tr_);
      dot_acc(c.pd[2], c.dn[2], si, ti, si_, ti_);
      dot_acc(c.pd[3], c.dn[3], si, ti, si_, ti_);
    }
    else
      dot_acc(c.pd[0], c.dn[0], sr, tr, sr_, tr_);
  };
  auto normal_after = [&](T w, int n) {
    const int be = (int)((F::bits(w) & ~F::SIGN) >> F::MB);
    return (be > 0) && (be <= F::EMAXB) && (be + n > 0) && (be + n <= F::EMAXB);
  };
  auto fscale = [&](T w, int n) { return F::val(F::bits(w) + ((typename F::U)(long long)n << F::MB)); };
  if (live && lane < m) {
    T cur[D][NV], nxt[D][NV];
#pragma unroll
    for (int d = 0; d < D; ++d)
      load(lane + (long long)L * d, cur[d]);
    for (long long i0 = lane; i0 < m; i0 += (long long)L * D) {
#pragma unroll
      for (int d = 0; d < D; ++d)
        load(i0 + (long long)L * (D + d), nxt[d]);
      // a full block of values that scale to normal values: straight-line code (the
      // exponent add of scale2's fast path), so that the products of later elements can
      // fill the latency of the earlier elements' 2Sum recurrences
      bool fast = (i0 + (long long)L * (D - 1) < m);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        fast = fast && normal_after(cur[d][0], nx) && normal_after(cur[d][1], ny);
        if (CPLX)
          fast = fast && normal_after(cur[d][2], nx) && normal_after(cur[d][3], ny);
      }
      if (fast) {
        DotTerms<T, CPLX> tm[D];
#pragma unroll
        for (int d = 0; d < D; ++d)
          products(fscale(cur[d][0], nx), fscale(cur[d][1], ny), CPLX ? fscale(cur[d][2], nx) : (T)0,
                   CPLX ? fscale(cur[d][3], ny) : (T)0, tm[d]);
#pragma unroll
        for (int d = 0; d < D; ++d)
          accumulate(tm[d]);
      }
      else {
#pragma unroll
        for (int d = 0; d < D; ++d)
          if (i0 + (long long)L * d < m) {
            DotTerms<T, CPLX> tm;
            products(scale2(cur[d][0], nx), scale2(cur[d][1], ny), CPLX ? scale2(cur[d][2], nx) : (T)0,
                     CPLX ? scale2(cur[d][3], ny) : (T)0, tm);
            accumulate(tm);
          }
      }
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int k = 0; k < NV; ++k)
          cur[d][k] = nxt[d][k];
    }
  }
  const T nur = hsum<L>(sr) + (hsum<L>(tr) + (hsum<L>(sr_) + hsum<L>(tr_)));
  T nui = 0;
  if (CPLX)
    nui = hsum<L>(si) + (hsum<L>(ti) + (hsum<L>(si_) + hsum<L>(ti_)));
  const T de = fx * fy;
  zr = F::div(nur, de);
  zi = CPLX ? F::div(nui, de) : (T)0;
}

// The same scaled compensated dot products (FP64 only) with the independent accumulator
// chains of one lane in different warps. The reference keeps, per lane, two 2Sum
// recurrences (round-down products pd and their exact errors dn; src/ddpscl.c:46-60) for
// real data and four for complex data (real and imaginary parts; src/zdpscl.c:58-80).
// Chain C (bit 0: dn instead of pd, bit 1: imaginary part) of pairs 0..3 runs on one warp,
// pair j on lanes [8j, 8j+8): every lane keeps the reference's element order and
// recurrence, the chains of a lane just run side by side on different sub-partitions,
// each warp with one instruction stream (no per-thread selects: on GB300 an FP64 result
// that goes through the integer pipes costs hundreds of cycles). Elements are loaded a
// block (8 real, 4 complex) ahead of their accumulation, so that L2 latency (columns not
// staged in shared memory) overlaps the recurrence, and a block of normal values is
// accumulated by straight-line code whose products the scheduler can interleave with the
// recurrence. Returns the 8-lane halving-tree sums of s and t on lane 8j.
template <typename T, bool CPLX, int C>
__device__ void chain_dot(long long m, const T *xr, const T *xi, const T *yr, const T *yi, T ex, T ey, bool live,
                          int l8, T &S, T &Tt)
{
  static_assert(sizeof(T) == 8, "the chain-split dot product is the FP64 form");
  using F = fp<T>;
  constexpr bool DN = (C & 1) != 0, IM = (C & 2) != 0;
  constexpr int NV = CPLX ? 4 : 2;  // values loaded per element
  constexpr int NT = CPLX ? 2 : 1;  // terms accumulated per element
  constexpr int D = CPLX ? 4 : 8;   // elements per block: the next block's loads are in flight
                                    // while this block is accumulated (hides L2 latency)
  const int nx = -(int)ex, ny = -(int)ey;
  T s = 0, t = 0;
  auto load = [&](long long i, T (&v)[NV]) {
    if (i < m) {
      v[0] = xr[i];
      v[1] = yr[i];
      if (CPLX) {
        v[2] = xi[i];
        v[3] = yi[i];
      }
    }
  };
  // the term(s) of element i from its scaled values: real part xr yr, xi yi; imaginary part
  // xr yi, xi (-yr) (= (-xi) yr exactly)
  auto terms = [&](T xr_, T yr_, T xi_, T yi_, T (&v)[NT]) {
    const T a0 = xr_, b0 = (CPLX && IM) ? yi_ : yr_;
    const T q0 = F::mul_rd(a0, b0);
    v[0] = DN ? F::fma_(a0, b0, -q0) : q0;
    if (CPLX) {
      const T a1 = xi_, b1 = IM ? -yr_ : yi_;
      const T q1 = F::mul_rd(a1, b1);
      v[NT - 1] = DN ? F::fma_(a1, b1, -q1) : q1;
    }
  };
  // the general path: scale2 with its special cases, one element at a time
  auto acc = [&](const T (&w)[NV]) {
    T v[NT];
    terms(scale2(w[0], nx), scale2(w[1], ny), CPLX ? scale2(w[2], nx) : (T)0, CPLX ? scale2(w[3], ny) : (T)0, v);
#pragma unroll
    for (int k = 0; k < NT; ++k)
      two_sum(s, v[k] + t, s, t);
  };
  // the power-of-two scaling of a normal value to a normal result is an integer add on the
  // exponent field (scale2's fast path)
  auto normal_after = [&](T w, int n) {
    const int be = (int)((F::bits(w) & ~F::SIGN) >> F::MB);
    return (be > 0) && (be <= F::EMAXB) && (be + n > 0) && (be + n <= F::EMAXB);
  };
  auto fscale = [&](T w, int n) { return F::val(F::bits(w) + ((typename F::U)(long long)n << F::MB)); };
  if (live && l8 < m) {
    T cur[D][NV], nxt[D][NV];
#pragma unroll
    for (int d = 0; d < D; ++d)
      load(l8 + 8LL * d, cur[d]);
    for (long long i0 = l8; i0 < m; i0 += 8LL * D) {
#pragma unroll
      for (int d = 0; d < D; ++d)
        load(i0 + 8LL * (D + d), nxt[d]);
      // a full block of normal values: straight-line code, so that the products of later
      // elements fill the latency of the earlier elements' 2Sum recurrence
      bool fast = (i0 + 8LL * (D - 1) < m);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        fast = fast && normal_after(cur[d][0], nx) && normal_after(cur[d][1], ny);
        if (CPLX)
          fast = fast && normal_after(cur[d][2], nx) && normal_after(cur[d][3], ny);
      }
      if (fast) {
        T v[D][NT];
#pragma unroll
        for (int d = 0; d < D; ++d)
          terms(fscale(cur[d][0], nx), fscale(cur[d][1], ny), CPLX ? fscale(cur[d][2], nx) : (T)0,
                CPLX ? fscale(cur[d][3], ny) : (T)0, v[d]);
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int k = 0; k < NT; ++k)
            two_sum(s, v[d][k] + t, s, t);
      }
      else {
#pragma unroll
        for (int d = 0; d < D; ++d)
          if (i0 + 8LL * d < m)
            acc(cur[d]);
      }
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int k = 0; k < NV; ++k)
          cur[d][k] = nxt[d][k];
    }
  }
  S = hsum<8>(s);
  Tt = hsum<8>(t);
}

}  // namespace vj
