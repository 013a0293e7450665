// One 2x2 Hermitian eigenproblem per call, in VecJac's operation order, bit-exact with
// the reference's AVX-512 lanes:
//   real:    D8JAC2_LOOP / D8JACL_LOOP / D8JACI_LOOP   src/dbjac2.c:17-44, :51-78, :148-175
//            (FP32: S8JAC*_LOOP, src/sbjac2.c, constants src/scjac2.h)
//   complex: Z8JAC2_LOOP / Z8JACL_LOOP / Z8JACI_LOOP   src/zbjac2.c:18-62, :65-106, :179-219
// KIND 0: cosine + tangent(s), KIND 1: cosine + sine(s), KIND 2: secant + tangent(s).
// Nonzero normal inputs of moderate spread take a fast path whose scalings are exponent
// adds; other finite inputs take a path whose exponent logic (getexp, min, scalef by an
// integer) runs on the integer pipes; inputs with an inf or NaN take the literal
// transcription.
#pragma once
#include "dsqrt.cuh"
#include "idiv.cuh"
#include "vj_fp.cuh"

namespace vj {

// correctly rounded division: FP64 quotients are formed on the integer pipes (ddiv_int),
// FP32 ones by the FP32 unit
__device__ __forceinline__ double qdiv(double a, double b) { return ddiv_int(a, b); }
__device__ __forceinline__ float qdiv(float a, float b) { return fp<float>::div(a, b); }

template <typename T> __device__ __forceinline__ bool all_finite3(T a, T b, T c)
{
  return visfinite(a) && visfinite(b) && visfinite(c);
}

// 1020 - getexp(x) as an int for finite x; zero -> "huge" (the reference's DBL_MAX cap)
template <typename T> __device__ __forceinline__ int escale(T x)
{
  constexpr int BE = (sizeof(T) == 8) ? 1020 : 124;
  return ((fp<T>::bits(x) & ~fp<T>::SIGN) ? (BE - ilogb_(x)) : (1 << 20));
}

// max(q, 0) then min(., sqrt_huge) for q = |.|/|.| (q is +0, positive or NaN), as integers
template <typename T> __device__ __forceinline__ T clamp_t2(T q)
{
  using F = fp<T>;
  const typename F::U u = F::bits(q);
  const typename F::U lim = F::bits(F::sqrt_huge());
  // NaN (u > inf) and +0 give +0; otherwise min(q, sh)
  if (u > F::bits(F::inf()) || u == 0)
    return (T)0;
  return (u < lim) ? q : F::sqrt_huge();
}

// ---- the all-normal fast path ----
// When every input is a nonzero normal number and their exponents span less than the
// scaling headroom (BE + BIAS - 1 binades), the prescale exponent is es = BE + BIAS - (the
// largest biased exponent), every scaled value stays normal, and each scaling by a power of
// two is an add to the exponent field: the general path's getexp/min/scale2 sequences,
// whose rare branches the compiler would otherwise predicate into every lane, reduce to a
// few integer operations. The results are those of the general path bit for bit (the
// general path takes the same normal-range branch of every escale and scale2 then).
template <typename T> __device__ __forceinline__ int bexp(T x)
{
  return (int)((fp<T>::bits(x) & ~fp<T>::SIGN) >> fp<T>::MB);
}
// x * 2^n for a normal x whose product is normal: an integer add to the exponent field
template <typename T> __device__ __forceinline__ T addexp(T x, int n)
{
  return fp<T>::val(fp<T>::bits(x) + ((typename fp<T>::U)(long long)n << fp<T>::MB));
}
// the general scale2, kept out of line
template <typename T> __device__ __noinline__ T scale2_rare(T x, int n) { return scale2(x, n); }
// x * 2^n for a finite x: the exponent add when x and the product are normal
template <typename T> __device__ __forceinline__ T scale2_nr(T x, int n)
{
  const int be = bexp(x), bn = be + n;
  if (be > 0 && bn > 0 && bn <= fp<T>::EMAXB)
    return addexp(x, n);
  return scale2_rare(x, n);
}
// a < b for finite a, b on the integer pipes (two's-complement order of the bit patterns,
// with -0 == +0), max / min of non-negative finite values likewise
__device__ __forceinline__ long long okey(double x)
{
  const long long u = (long long)fp<double>::bits(x);
  return (u < 0) ? -(u & 0x7fffffffffffffffLL) : u;
}
__device__ __forceinline__ int okey(float x)
{
  const int u = (int)fp<float>::bits(x);
  return (u < 0) ? -(u & 0x7fffffff) : u;
}
// (FP32 compares on the wide FP32 pipe: the plain comparison, identical for finite values)
__device__ __forceinline__ bool lt_fin(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ bool lt_fin(float a, float b) { return a < b; }
__device__ __forceinline__ double nnmin(double a, double b) { return (fp<double>::bits(a) < fp<double>::bits(b)) ? a : b; }
__device__ __forceinline__ double nnmax(double a, double b) { return (fp<double>::bits(a) > fp<double>::bits(b)) ? a : b; }
__device__ __forceinline__ float nnmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float nnmax(float a, float b) { return fmaxf(a, b); }
// square root of 1 <= x < 2^EMAX: FP64 with the few-FP64-operation routine of dsqrt.cuh,
// FP32 with the FP32 unit's correctly rounded root
__device__ __forceinline__ double sqrt_ge1(double x) { return dsqrt_pos(x); }
__device__ __forceinline__ float sqrt_ge1(float x) { return fp<float>::sqrt_(x); }

template <typename T> struct fastc {
  static constexpr int BE = (sizeof(T) == 8) ? 1020 : 124;  // src/dzjac2.h:10, src/scjac2.h:10
  static constexpr int TOP = BE + fp<T>::BIAS;               // biased exponent of the largest scaled input
};

// shared tail of the real and complex lanes: angle from the prescaled (a1, a2, ab)
template <typename T> struct angle {
  T t1, s2, s1;
};

// (FAST: the square roots' arguments, 1 + t2^2 and 1 + t1^2, are at least 1 and finite --
// t2 is clamped to sqrt(huge) -- so the fast path takes sqrt_ge1)
template <typename T, bool FAST = false>
__device__ __forceinline__ angle<T> jac_angle(T a1, T a2, T ab, T &ad_out)
{
  using F = fp<T>;
  const T one = (T)1;
  const T ad = a1 - a2;
  ad_out = ad;
  const T t2 = vor(clamp_t2(qdiv(ab, vabs(ad))), vsgn(ad));
  const T t1 = qdiv(t2, one + (FAST ? sqrt_ge1(F::fma_(t2, t2, one)) : F::sqrt_(F::fma_(t2, t2, one))));
  const T s2 = F::fma_(t1, t1, one);
  return angle<T>{t1, s2, FAST ? sqrt_ge1(s2) : F::sqrt_(s2)};
}

template <typename T, int KIND, bool GEN>
__device__ __forceinline__ unsigned rjac2_body(T a1, T a2, T ar, T &c, T &at, T &l1, T &l2, int bmax)
{
  using F = fp<T>;
  const T one = (T)1;
  T L1, L2, t1, s1, s2, as;
  bool fin = false;  // L1, L2 finite: compared on the integer pipes
  (void)bmax;
  if constexpr (!GEN) {
    const int es = fastc<T>::TOP - bmax;
    ar = addexp(ar, es);
    a1 = addexp(a1, es);
    a2 = addexp(a2, es);
    const T aa = vabs(ar);
    as = vsgn(ar);
    const T ab = addexp(aa, 1);
    T ad;
    const angle<T> g = jac_angle<T, true>(a1, a2, ab, ad);
    t1 = g.t1; s2 = g.s2; s1 = g.s1;
    L1 = qdiv(F::fma_(t1, F::fma_(a2, t1, ab), a1), s2);
    L2 = qdiv(F::fma_(t1, F::fma_(a1, t1, -ab), a2), s2);
    l1 = scale2_nr(L1, -es);
    l2 = scale2_nr(L2, -es);
    fin = true;
  }
  else if (all_finite3(a1, a2, ar)) {
    const int es = min(min(escale(a1), escale(a2)), min(escale(ar), 1 << 20));
    ar = scale2(ar, es);
    a1 = scale2(a1, es);
    a2 = scale2(a2, es);
    const T aa = vabs(ar);
    as = vsgn(ar);
    const T ab = scale2(aa, 1);
    T ad;
    const angle<T> g = jac_angle(a1, a2, ab, ad);
    t1 = g.t1; s2 = g.s2; s1 = g.s1;
    L1 = qdiv(F::fma_(t1, F::fma_(a2, t1, ab), a1), s2);
    L2 = qdiv(F::fma_(t1, F::fma_(a1, t1, -ab), a2), s2);
    l1 = scale2(L1, -es);
    l2 = scale2(L2, -es);
  }
  else {
    const T zero = (T)0, sh = F::sqrt_huge(), huge = F::max_(), be = F::big_exp();
    const T e1 = xsub(be, getexp(a1)), e2 = xsub(be, getexp(a2)), er = xsub(be, getexp(ar));
    T es = vmin(vmin(e1, e2), vmin(er, huge));
    ar = scalef(ar, es);
    a1 = scalef(a1, es);
    a2 = scalef(a2, es);
    const T aa = vabs(ar);
    as = vsgn(ar);
    es = vneg(es);
    const T ab = scalef(aa, one);
    const T ad = xsub(a1, a2);
    const T t2 = vor(vmin(vmax(xdiv(ab, vabs(ad)), zero), sh), vsgn(ad));
    t1 = xdiv(t2, xadd(one, xsqrt(xfma(t2, t2, one))));
    s2 = xfma(t1, t1, one);
    s1 = xsqrt(s2);
    L1 = xdiv(xfma(t1, xfma(a2, t1, ab), a1), s2);
    L2 = xdiv(xfma(t1, xfma(a1, t1, vneg(ab)), a2), s2);
    l1 = scalef(L1, es);
    l2 = scalef(L2, es);
  }
  if (KIND == 2) {
    at = vxor(t1, as);
    c = s1;
  }
  else {
    c = qdiv(one, s1);
    at = ((KIND == 1) ? qdiv(vxor(t1, as), s1) : vxor(t1, as));
  }
  return (fin ? lt_fin(L1, L2) : (L1 < L2)) ? 1u : 0u;
}


// the general finite path and the inf/NaN transcription, out of line: their code is not
// laid out (or predicated) into the lanes of the fast path; results by value, so that the
// caller's outputs never have their address taken (they stay in registers)
template <typename T> struct r2out {
  T c, at, l1, l2;
  unsigned bit;
};
template <typename T, int KIND> __device__ __noinline__ r2out<T> rjac2_gen(T a1, T a2, T ar)
{
  r2out<T> r;
  r.bit = rjac2_body<T, KIND, true>(a1, a2, ar, r.c, r.at, r.l1, r.l2, 0);
  return r;
}

template <typename T, int KIND>
__device__ __forceinline__ unsigned rjac2(T a1, T a2, T ar, T &c, T &at, T &l1, T &l2)
{
  const int b1 = bexp(a1), b2 = bexp(a2), br = bexp(ar);
  const int bmax = max(max(b1, b2), br), bmin = min(min(b1, b2), br);
  if (bmin > 0 && bmax <= fp<T>::EMAXB && bmax - bmin < fastc<T>::TOP)
    return rjac2_body<T, KIND, false>(a1, a2, ar, c, at, l1, l2, bmax);
  const r2out<T> r = rjac2_gen<T, KIND>(a1, a2, ar);
  c = r.c;
  at = r.at;
  l1 = r.l1;
  l2 = r.l2;
  return r.bit;
}

template <typename T, int KIND, bool GEN>
__device__ __forceinline__ unsigned cjac2_body(T a1, T a2, T ar, T ai, T &c, T &cat, T &sat, T &l1, T &l2, int bmax)
{
  using F = fp<T>;
  const T one = (T)1, zero = (T)0;
  T L1, L2, t1, s1, s2, ar_, ai_;
  bool fin = false;
  (void)bmax;
  if constexpr (!GEN) {
    const int es = fastc<T>::TOP - bmax;
    ar = addexp(ar, es);
    ai = addexp(ai, es);
    a1 = addexp(a1, es);
    a2 = addexp(a2, es);
    ar_ = vabs(ar);
    ai_ = vabs(ai);
    const T as = vsgn(ar);
    // the min / max below compare non-negative finite values: integer comparisons; the
    // quotient am / aM is >= 0 and aa >= aM > 0, so the reference's max with 0 and with
    // the smallest subnormal return their first operand
    const T am = nnmin(ar_, ai_);
    const T aM = nnmax(ar_, ai_);
    T aa = qdiv(am, aM);
    aa = sqrt_ge1(F::fma_(aa, aa, one)) * aM;
    ar_ = vor(nnmin(qdiv(ar_, aa), one), as);
    ai_ = qdiv(ai, aa);
    const T ab = addexp(aa, 1);
    T ad;
    const angle<T> g = jac_angle<T, true>(a1, a2, ab, ad);
    t1 = g.t1; s2 = g.s2; s1 = g.s1;
    L1 = qdiv(F::fma_(t1, F::fma_(a2, t1, ab), a1), s2);
    L2 = qdiv(F::fma_(t1, F::fma_(a1, t1, -ab), a2), s2);
    l1 = scale2_nr(L1, -es);
    l2 = scale2_nr(L2, -es);
    fin = true;
  }
  else if (all_finite3(a1, a2, ar) && visfinite(ai)) {
    const int es = min(min(1 << 20, min(escale(a1), escale(a2))), min(escale(ar), escale(ai)));
    ar = scale2(ar, es);
    ai = scale2(ai, es);
    a1 = scale2(a1, es);
    a2 = scale2(a2, es);
    ar_ = vabs(ar);
    ai_ = vabs(ai);
    const T as = vsgn(ar);
    const T am = vmin(ar_, ai_);
    const T aM = vmax(ar_, ai_);
    T aa = vmax(qdiv(am, aM), zero);
    aa = F::sqrt_(F::fma_(aa, aa, one)) * aM;
    ar_ = vor(vmin(qdiv(ar_, aa), one), as);
    ai_ = qdiv(ai, vmax(aa, F::true_min()));
    const T ab = scale2(aa, 1);
    T ad;
    const angle<T> g = jac_angle(a1, a2, ab, ad);
    t1 = g.t1; s2 = g.s2; s1 = g.s1;
    L1 = qdiv(F::fma_(t1, F::fma_(a2, t1, ab), a1), s2);
    L2 = qdiv(F::fma_(t1, F::fma_(a1, t1, -ab), a2), s2);
    l1 = scale2(L1, -es);
    l2 = scale2(L2, -es);
  }
  else {
    const T sh = F::sqrt_huge(), huge = F::max_(), be = F::big_exp();
    const T e1 = xsub(be, getexp(a1)), e2 = xsub(be, getexp(a2)), er = xsub(be, getexp(ar)), ei = xsub(be, getexp(ai));
    T es = vmin(huge, vmin(vmin(e1, e2), vmin(er, ei)));
    ar = scalef(ar, es);
    ai = scalef(ai, es);
    a1 = scalef(a1, es);
    a2 = scalef(a2, es);
    ar_ = vabs(ar);
    ai_ = vabs(ai);
    const T as = vsgn(ar);
    const T am = vmin(ar_, ai_);
    const T aM = vmax(ar_, ai_);
    es = vneg(es);
    T aa = vmax(xdiv(am, aM), zero);
    aa = xmul(xsqrt(xfma(aa, aa, one)), aM);
    ar_ = vor(vmin(xdiv(ar_, aa), one), as);
    ai_ = xdiv(ai, vmax(aa, F::true_min()));
    const T ab = scalef(aa, one);
    const T ad = xsub(a1, a2);
    const T t2 = vor(vmin(vmax(xdiv(ab, vabs(ad)), zero), sh), vsgn(ad));
    t1 = xdiv(t2, xadd(one, xsqrt(xfma(t2, t2, one))));
    s2 = xfma(t1, t1, one);
    s1 = xsqrt(s2);
    L1 = xdiv(xfma(t1, xfma(a2, t1, ab), a1), s2);
    L2 = xdiv(xfma(t1, xfma(a1, t1, vneg(ab)), a2), s2);
    l1 = scalef(L1, es);
    l2 = scalef(L2, es);
  }
  // ai_ is NaN only for inputs with an inf or NaN: keep the x86 NaN rules there
  if (KIND == 2) {
    ar_ = ar_ * t1;
    c = s1;
    ai_ = xmul(ai_, t1);
  }
  else if (KIND == 1) {
    c = qdiv(one, s1);
    ar_ = qdiv(ar_ * t1, s1);
    ai_ = xdiv(xmul(ai_, t1), s1);
  }
  else {
    c = qdiv(one, s1);
    ar_ = ar_ * t1;
    ai_ = xmul(ai_, t1);
  }
  cat = ar_;
  sat = ai_;
  return (fin ? lt_fin(L1, L2) : (L1 < L2)) ? 1u : 0u;
}

template <typename T> struct c2out {
  T c, cat, sat, l1, l2;
  unsigned bit;
};
template <typename T, int KIND> __device__ __noinline__ c2out<T> cjac2_gen(T a1, T a2, T ar, T ai)
{
  c2out<T> r;
  r.bit = cjac2_body<T, KIND, true>(a1, a2, ar, ai, r.c, r.cat, r.sat, r.l1, r.l2, 0);
  return r;
}

template <typename T, int KIND>
__device__ __forceinline__ unsigned cjac2(T a1, T a2, T ar, T ai, T &c, T &cat, T &sat, T &l1, T &l2)
{
  const int b1 = bexp(a1), b2 = bexp(a2), br = bexp(ar), bi = bexp(ai);
  const int bmax = max(max(b1, b2), max(br, bi)), bmin = min(min(b1, b2), min(br, bi));
  if (bmin > 0 && bmax <= fp<T>::EMAXB && bmax - bmin < fastc<T>::TOP)
    return cjac2_body<T, KIND, false>(a1, a2, ar, ai, c, cat, sat, l1, l2, bmax);
  const c2out<T> r = cjac2_gen<T, KIND>(a1, a2, ar, ai);
  c = r.c;
  cat = r.cat;
  sat = r.sat;
  l1 = r.l1;
  l2 = r.l2;
  return r.bit;
}

}  // namespace vj
