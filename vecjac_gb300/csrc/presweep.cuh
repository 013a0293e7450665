// The pair rotation of the mixed SVD's plain-dot Jacobi sweeps (mixed.cu, k_presweep and
// k_presweep_reg): the Hestenes angle from a pair's Gram entries, the coefficients of the
// rotation as the columns are stored (with the FP64 sweeps' column scales), the element
// update, and the squared column norms tracked through an FP64 sweep. Device code that
// host harnesses also compile (tests/presweep_host.cpp, with models of the two atomics).
#pragma once
#include <cmath>

namespace vj {

// Hestenes rotation of a Hermitian 2x2 Gram block [[a, c], [conj c, b]]: with c = |c| e^{i phi},
// t = sn/cs the smaller root of t^2 + 2 zeta t - 1 = 0, zeta = (b - a) / (2|c|), the unitary
// [[cs, sn e^{i phi}], [-sn e^{-i phi}, cs]] applied to columns (p, q) makes them
// orthogonal, with squared norms a - t|c| and b + t|c|. Sets rot = {cs, sn cos phi,
// sn sin phi, go, swap}; go = 0 when |c| < tol sqrt(a b); swap = 1 when the rotated q
// column is the longer one, which then goes to position p (columns drift into descending
// order of norms, as in the reference's sweeps, which shortens convergence by ~30%).
// nrm: the squared norms of the two rotated columns, a - t|c| and b + t|c| (in p, q order
// before the swap), or a and b when nothing is rotated.
template <typename T> __device__ void hestenes(T a, T b, T cr, T ci, T tol, T *rot, unsigned *cnt, T *nrm)
{
  const T ac = hypot(cr, ci);
  T cs = 1, snr = 0, sni = 0, go = 0, sw = 0;
  nrm[0] = a;
  nrm[1] = b;
  if (ac > (T)0 && ac >= tol * sqrt(a) * sqrt(b)) {
    const T zeta = (b - a) / ((T)2 * ac);
    const T az = fabs(zeta);
    const T big = (sizeof(T) == 4) ? (T)1e18 : (T)1e150;
    const T t = (az > big) ? (T)0.5 / zeta : copysign((T)1, zeta) / (az + sqrt(fma(zeta, zeta, (T)1)));
    cs = (T)1 / sqrt(fma(t, t, (T)1));
    const T sn = t * cs;
    snr = sn * (cr / ac);
    sni = sn * (ci / ac);
    go = 1;
    sw = (b + t * ac > a - t * ac) ? (T)1 : (T)0;
    nrm[0] = a - t * ac;
    nrm[1] = b + t * ac;
    atomicAdd(cnt, 1u);
    // the largest |cos| of the rotated pairs of this sweep (non-negative floats order as
    // their bit patterns)
    atomicMax(cnt + 1, __float_as_uint((float)(ac / (sqrt(a) * sqrt(b)))));
  }
  rot[0] = cs;
  rot[1] = snr;
  rot[2] = sni;
  rot[3] = go;
  rot[4] = sw;
}

// Coefficients of one pair's rotation as the columns are stored:
//   general form  p := cp p - conj(u) q,  q := cq q + v p   (3 operations per output)
//   short form    p := p - conj(u) q,     q := q + v p      (2 FMAs per output)
// Without column scales cp = cq = cs and u = v = sn e^{i phi}: the rotation of hestenes.
// The FP64 sweeps store each column as d_j times a stored column (d_j in [2^-8, 1], one
// scale per column of G and of V). A rotation then factors as
//   p' = (cs d_p) (p~ - conj(sn e^{i phi}) (d_q / (cs d_p)) q~),
//   q' = (cs d_q) (q~ + sn e^{i phi} (d_p / (cs d_q)) p~),
// so the stored columns take the short form and the cosines go into the scales, which
// are multiplied into the columns once per sweep: 8 instead of 12 FP64 operations per
// complex element (2 instead of 4 per real one). A pair whose new scale would fall below
// 2^-8 takes the general form with cp = cs d_p, cq = cs d_q, u = sn e^{i phi} d_q,
// v = sn e^{i phi} d_p instead, and its scales return to 1, so that a stored column is
// never more than 2^8 times its true length. (Not the reference's arithmetic: these
// sweeps precondition the reference's own sweeps, which decide the result.)
template <typename T> struct Rot {
  T cp, cq, ur, ui, vr, vi;
  bool go, swap, shrt;
};
#ifdef VJ_PRESWEEP_COL_SCALE_MIN
constexpr double COL_SCALE_MIN = VJ_PRESWEEP_COL_SCALE_MIN;  // a host test's threshold (general form)
#else
constexpr double COL_SCALE_MIN = 1.0 / 256.0;
#endif
// only the FP64 sweeps carry column scales: the FP32 kernels are compiled for the
// unscaled rotation alone (cq = cp, v = u)
template <typename T> __host__ __device__ constexpr bool has_scales() { return sizeof(T) == 8; }
template <typename T> __device__ __forceinline__ void unscaled_form(Rot<T> &k)
{
  if (!has_scales<T>()) {
    k.shrt = false;
    k.cq = k.cp;
    k.vr = k.ur;
    k.vi = k.ui;
  }
}

// the coefficients from hestenes' {cs, sn cos phi, sn sin phi, go, swap} and the pair's
// column scales; with scales (dsc != nullptr) the new scales are written to dsc[p], dsc[q]
template <typename T>
__device__ Rot<T> pair_rot(const T *h, T dp, T dq, T *dsc, unsigned p, unsigned q)
{
  Rot<T> r;
  const T cs = h[0], snr = h[1], sni = h[2];
  r.go = h[3] != (T)0;
  r.swap = h[4] != (T)0;
  r.shrt = false;
  r.cp = r.cq = cs;
  r.ur = r.vr = snr;
  r.ui = r.vi = sni;
  if (!dsc || !r.go)
    return r;
  const T np = cs * dp, nq = cs * dq;
  if (np >= (T)COL_SCALE_MIN && nq >= (T)COL_SCALE_MIN) {
    const T k1 = dq / np, k2 = dp / nq;
    r.shrt = true;
    r.cp = r.cq = (T)1;
    r.ur = snr * k1;
    r.ui = sni * k1;
    r.vr = snr * k2;
    r.vi = sni * k2;
    dsc[p] = r.swap ? nq : np;
    dsc[q] = r.swap ? np : nq;
  }
  else {
    r.cp = np;
    r.cq = nq;
    r.ur = snr * dq;
    r.ui = sni * dq;
    r.vr = snr * dp;
    r.vi = sni * dp;
    dsc[p] = dsc[q] = (T)1;
  }
  return r;
}

// (p, q) <- the rotation above, element-wise, with explicit FMAs (the library is built
// without automatic contraction)
template <typename T, bool CPLX>
__device__ __forceinline__ void rot_elem(const Rot<T> &c, T &pr, T &pi, T &qr, T &qi)
{
  const T Pr = pr, Qr = qr;
  if (CPLX) {
    const T Pi = pi, Qi = qi;
    if (c.shrt) {
      pr = fma(-c.ur, Qr, fma(-c.ui, Qi, Pr));
      pi = fma(-c.ur, Qi, fma(c.ui, Qr, Pi));
      qr = fma(c.vr, Pr, fma(-c.vi, Pi, Qr));
      qi = fma(c.vr, Pi, fma(c.vi, Pr, Qi));
    }
    else {
      pr = fma(c.cp, Pr, -fma(c.ur, Qr, c.ui * Qi));
      pi = fma(c.cp, Pi, -fma(c.ur, Qi, -(c.ui * Qr)));
      qr = fma(c.cq, Qr, fma(c.vr, Pr, -(c.vi * Pi)));
      qi = fma(c.cq, Qi, fma(c.vr, Pi, c.vi * Pr));
    }
  }
  else if (c.shrt) {
    pr = fma(-c.ur, Qr, Pr);
    qr = fma(c.vr, Pr, Qr);
  }
  else {
    pr = fma(c.cp, Pr, -(c.ur * Qr));
    qr = fma(c.cq, Qr, c.vr * Pr);
  }
}

// Squared column norms tracked through an FP64 sweep (nrm[j], or -1 when unknown): after
// the rotation that makes a pair orthogonal its squared norms are a - t|c| and b + t|c|,
// so a step needs only the inner product c -- 4 FP64 FMAs per complex row of G instead of
// 8 (1 instead of 3 per real row). Each rotation adds a rounding of about one unit to a
// tracked norm (its columns' new entries are rounded once or twice), so over a sweep of
// n - 1 steps they stay within ~sqrt(n) units; every sweep starts from unknown norms
// (the first step of each column computes them). The rotation angle depends on b - a, so a
// pair whose tracked norms are within 1e-6 (relative) of each other computes them, and a
// norm that fell below half its old value (cancellation in a - t|c|) becomes unknown.
constexpr double NORM_NEAR = 1e-6;
// by every thread before the dot products (the same two words for the whole CTA, so no
// barrier is needed): the pair's tracked norms in nab, or -1 when the step must compute them
template <typename T> __device__ __forceinline__ void tracked_norms(const T *nrm, unsigned p, unsigned q, T *nab)
{
  nab[0] = nab[1] = (T)-1;
  if (!has_scales<T>() || !nrm)
    return;
  const T na = nrm[p], nb = nrm[q];
  if (na >= (T)0 && nb >= (T)0 && fabs(nb - na) >= (T)NORM_NEAR * (na + nb)) {
    nab[0] = na;
    nab[1] = nb;
  }
}

// the pair's rotation from its (stored) Gram entries, by thread 0 into *rs: with column
// scales the entries are scaled first; with tracked norms (nab[0] >= 0) a and b are those
// norms, and the new norms go back to nrm
template <typename T>
__device__ void pair_rotation(T a, T b, T cr, T ci, T tol, unsigned *cnt, T *dsc, unsigned p, unsigned q, Rot<T> *rs,
                              T *nrm, const T *nab)
{
  T dp = 1, dq = 1;
  if (!has_scales<T>()) {
    dsc = nullptr;
    nrm = nullptr;
  }
  if (dsc) {
    dp = dsc[p];
    dq = dsc[q];
    a *= dp * dp;
    b *= dq * dq;
    cr *= dp * dq;
    ci *= dp * dq;
  }
  if (nrm && nab[0] >= (T)0) {
    a = nab[0];
    b = nab[1];
  }
  T h[5], nn[2];
  hestenes(a, b, cr, ci, tol, h, cnt, nn);
  *rs = pair_rot(h, dp, dq, dsc, p, q);
  if (nrm) {
    const T np = (nn[0] >= (T)0.5 * a) ? nn[0] : (T)-1, nq = (nn[1] >= (T)0.5 * b) ? nn[1] : (T)-1;
    const bool sw = h[4] != (T)0;
    nrm[p] = sw ? nq : np;
    nrm[q] = sw ? np : nq;
  }
}

}  // namespace vj
