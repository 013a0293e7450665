// Device building blocks of the one-sided Jacobi SVD shared by the one-launch-per-step
// driver (jsvd.cu) and the batched persistent kernel (batch.cu): the AVX-512-exact column
// norm, the compensated scaled dot products in the reference's lane order, the pair
// classification (convergence test, shear test, prescale, 2x2) and the transformation of a
// column pair. Reference: src/dvjsvd.c:195-602, src/zvjsvd.c:214-652 and the L1 kernels
// they call (src/ddpscl.c, src/zdpscl.c, src/djrot.c, src/djrotf.c, src/zjrot.c,
// src/zjrotf.c, src/dgsscl.c, src/zgsscl.c).
#pragma once
#include <cfloat>
#include <cmath>

#include <cuda_runtime.h>

#include "jac2.cuh"
#include "svd_dot.cuh"
#include "svd_norm.cuh"
#include "vj_host.h"

namespace vj {

// control block of one pivot step (triple-buffered across launches)
struct Ctl {
  double MGbase, MVbase;  // max |G|, max |V| after this step's own rescaling (in T's range)
  unsigned long long nMG, nMV;  // atomicMax of max |.| of the transformed columns (T bits)
  int sT, sV;                   // accumulated power-of-two scalings of G and V
  int ovf;                      // a norm computed at the end of the previous step overflowed
  int pad;
};

struct SvdGlobal {
  long long err;                // 0 or the (negative) error code, atomicMin
  unsigned long long swt;       // transformed pairs in the current sweep
  Ctl ctl[3];
  // per-phase SM cycles of CTA 0 (the JTRACE split of src/dvjsvd.c:635), when tracing:
  // 0 control + rescaling, 1 staging, 2 dot products, 3 2x2 + classification, 4 rotations, 5 norms
  unsigned long long phase[8];
};

template <typename T> struct SvdArgs {
  int trace;                    // record per-phase cycles (VJ_TRACE=1)
  long long m, n, ldG, ldGi, ldV, ldVi;
  T *G, *Gi, *V, *Vi, *eS, *fS;
  const unsigned *js;
  SvdGlobal *g;
  T tol, gst;
  int nrm_exp, rot;
  long long e_dot, e_doti, e_appg, e_appv;
};

template <typename T> __device__ __forceinline__ unsigned long long tbits(T x)
{
  return (unsigned long long)fp<T>::bits(x);
}

// |x| bits, NaN above inf, so that an integer max flags NaNs as "not finite"


// ---- TMA (cp.async.bulk) staging of a column pair into shared memory ----
__device__ __forceinline__ unsigned smem_u32(const void *p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned phase)
{
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0u;
}
// bounded wait on phase 0 of the barrier; false after the iteration limit
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar)
{
  for (unsigned it = 0; it < (1u << 22); ++it)
    if (mbar_try_wait(bar, 0u))
      return true;
  return false;
}

// (e, f) of a norm d: d = f 2^e, f in [1,2) (src/dznrm2.h:4-23)
template <typename T> __device__ __forceinline__ void ef_split(T d, T &e, T &f)
{
  using F = fp<T>;
  if (visfinite(d)) {
    if (d == (T)0) {
      e = vneg(F::inf());
      f = vor((T)1, vsgn(d));
    }
    else {
      const int k = ilogb_(d);
      e = (T)k;
      f = scale2(d, -k);
    }
  }
  else {
    e = F::inf();
    f = vor((visnan(d) ? (T)0 : (T)1), vsgn(d));
  }
}


// VDHYPOT (src/vecdef.h:80-92) on scalars
template <typename T> __device__ __forceinline__ T vhypot(T x, T y)
{
  const T x_ = vabs(x), y_ = vabs(y);
  const T m_ = vmin(x_, y_), M_ = vmax(x_, y_);
  T z = fp<T>::div(m_, M_);
  z = vmax(z, (T)0);
  z = fp<T>::fma_(z, z, (T)1);
  z = fp<T>::sqrt_(z);
  return z * M_;
}

// norm of column c (real, or complex with planes) by one warp; writes eS/fS; returns d.
// xr/xi point to the column (in global or in shared memory).
template <typename T, bool CPLX> __device__ T col_norm_at(const SvdArgs<T> &a, long long c, const T *xr, const T *xi)
{
  T d = warp_nrm2(xr, a.m);
  if (CPLX) {
    const T di = warp_nrm2(xi, a.m);
    d = vhypot(d, di);
  }
  if ((threadIdx.x & 31) == 0) {
    T e, f;
    ef_split(d, e, f);
    a.eS[c] = e;
    a.fS[c] = f;
  }
  return d;
}

template <typename T, bool CPLX> __device__ T col_norm(const SvdArgs<T> &a, long long c)
{
  T d = warp_nrm2(a.G + c * a.ldG, a.m);
  if (CPLX) {
    const T di = warp_nrm2(a.Gi + c * a.ldGi, a.m);
    d = vhypot(d, di);
  }
  if ((threadIdx.x & 31) == 0) {
    T e, f;
    ef_split(d, e, f);
    a.eS[c] = e;
    a.fS[c] = f;
  }
  return d;
}

// Programmatic dependent launch: wait until the previous grid of the stream has completed
// and its writes are visible (a no-op for a launch without the attribute), then allow the
// next grid to be scheduled while this one runs, which hides the launch gap between the
// many short step kernels of a sweep.
__device__ __forceinline__ void pdl_enter()
{
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// efcmp (src/defops.h:46)
template <typename T> __device__ __forceinline__ int efcmp(T e0, T f0, T e1, T f1)
{
  if (e0 > e1) return 1;
  if (e0 < e1) return -1;
  if (f0 > f1) return 1;
  if (f0 < f1) return -1;
  return 0;
}
template <typename T> __device__ __forceinline__ bool eflt(T e0, T e1, T f0, T f1)
{
  return (e0 < e1) || ((e0 == e1) && (f0 < f1));
}
template <typename T> __device__ __forceinline__ bool efle(T e0, T e1, T f0, T f1)
{
  return (e0 < e1) || ((e0 == e1) && (f0 <= f1));
}

template <typename T> struct PairState {
  T ep, fp, eq, fq;      // norms (e, f) of columns p, q
  T a21r, a21i;          // scaled dot (cosine of the angle)
  T c, cat, sat;         // rotation: cosine, Re/Im of e^{i alpha} tangent
  int code;              // 3/-3 shear (+/- permute), 2/-2 rotate, -1 swap, 1 nothing
  int skip;              // an error stops this pair
};

// step-start decisions of src/dvjsvd.c:199-233 and the overflow branch :276-295
template <typename T> struct Decision {
  int gres, vres, ovf;   // rescale G (sR < 0), rescale V, retry after a norm overflow
  int sNg, sNv;          // exponents used
  T MG, MV;              // values after the step's rescaling
  int sT, sV;
};

template <typename T> __device__ __forceinline__ int ef_exp(T x)
{
  // dbl2ef exponent of a nonnegative finite MG / MV (> 0)
  return ilogb_(x);
}

template <typename T> __device__ Decision<T> decide(const SvdArgs<T> &a, const Ctl &cur)
{
  Decision<T> d;
  T MG = (T)cur.MGbase, MV = (T)cur.MVbase;
  const T nMG = bitst<T>(cur.nMG), nMV = bitst<T>(cur.nMV);
  MG = fmax(MG, nMG);
  MV = fmax(MV, nMV);
  int eM = ef_exp(MG);
  int sR = a.rot - eM;
  const int sN = a.nrm_exp - eM - 1;
  d.sT = cur.sT;
  d.gres = (sR < 0);
  d.sNg = sN;
  if (d.gres) {
    MG = scale2(MG, sN);
    d.sT += sN;
  }
  eM = ef_exp(MV);
  sR = a.rot - eM;
  d.sNv = sR;
  d.vres = (sR < 0);
  d.sV = cur.sV;
  if (d.vres) {
    MV = scale2(MV, sR);
    d.sV += sR;
  }
  d.ovf = (!d.gres && cur.ovf);
  if (d.ovf) {
    // the reference rescales G by its current sN, which the V block has just set (src/dvjsvd.c:227,281)
    MG = scale2(MG, d.sNv);
    d.sT += d.sNv;
  }
  d.MG = MG;
  d.MV = MV;
  return d;
}

template <typename T> __device__ void scale_cols(T *A, long long ld, long long rows, long long c0, long long c1,
                                                 int e)
{
  for (long long i = threadIdx.x; i < rows; i += blockDim.x) {
    A[c0 * ld + i] = scale2(A[c0 * ld + i], e);
    A[c1 * ld + i] = scale2(A[c1 * ld + i], e);
  }
}

template <typename T> __device__ __forceinline__ void amax(unsigned long long &m, T v)
{
  const unsigned long long b = absbits(v);
  m = (b > m) ? b : m;
}

// Convergence test, shear test, Gram prescale, 2x2 EVD and classification of one pair
// (src/dvjsvd.c:349-459): fills s.code (3/-3 shear, 2/-2 rotation, -1 swap, 1 nothing) and
// the rotation (c, cat, sat); returns whether the pair counts as transformed (|a21| >= tol).
// A swap (-1) must be completed by the caller by exchanging the pair's (eS, fS).
template <typename T, bool CPLX>
__device__ bool pair_classify(T ep, T fp_, T eq, T fq, T zr, T zi, T tol, T gst, PairState<T> &s)
{
  using F = fp<T>;
  const T ab = CPLX ? vhypot(zr, zi) : vabs(zr);
  const bool trans = (tol <= ab);
  if (trans) {
    const T e1 = ep, e2 = eq, f1 = fp_, f2 = fq;
    const bool ngs = eflt(e1, e2, f1, f2);
    T maf = ngs ? f1 : f2, mae = ngs ? e1 : e2;
    const T Maf = ngs ? f2 : f1, Mae = ngs ? e2 : e1;
    maf = gst * maf;
    mae = mae + getexp(maf);
    maf = getmant(maf);
    const bool cgs = eflt(mae, Mae, maf, Maf);
    T f12 = F::div(f1, f2), e12 = e1 - e2, f21 = F::div(f2, f1), e21 = e2 - e1;
    e12 = e12 + getexp(f12);
    f12 = getmant(f12);
    e21 = e21 + getexp(f21);
    f21 = getmant(f21);
    const bool c12 = efle(e12, e21, f12, f21);
    const T E = c12 ? e21 : e12;
    const T dd = vmin(svdc<T>::MAX_FIN_EXP - E, (T)0);
    e12 = e12 + dd;
    e21 = e21 + dd;
    const T w11 = scalef(f12, e12), w22 = scalef(f21, e21), w21r = scalef(zr, dd);
    unsigned perm;
    T cc, at, sat = 0, l1, l2;
    if (CPLX) {
      const T w21i = scalef(zi, dd);
      perm = cjac2<T, 0>(w11, w22, w21r, w21i, cc, at, sat, l1, l2);
    }
    else
      perm = rjac2<T, 0>(w11, w22, w21r, cc, at, l1, l2);
    s.c = cc;
    s.cat = at;
    s.sat = sat;
    if (!ngs && cgs)
      s.code = 3;
    else if (ngs && cgs)
      s.code = -3;
    else if (perm)
      s.code = -2;
    else
      s.code = 2;
  }
  else if (efcmp(ep, fp_, eq, fq) < 0)
    s.code = -1;
  else
    s.code = 1;
  return trans;
}

// The transformation of one classified pair applied by a group of TPP threads (ltid =
// this thread's index in the group): rotation (src/djrot.c, src/djrotf.c, src/zjrot.c,
// src/zjrotf.c), shear (src/dgsscl.c, src/zgsscl.c) or swap, to the columns of G (read from
// rp/rq[/rpi/rqi], which may be a staged copy, written to both) and of V. mG and mV collect
// max |.| of the updated G and (with TRACKV) V columns.
template <typename T, bool CPLX, bool TRACKV>
__device__ void pair_apply(const PairState<T> &s, long long m, long long nv, T *Gp, T *Gq, T *Gip, T *Giq, T *Vp,
                           T *Vq, T *Vip, T *Viq, T *rp, T *rq, T *rpi, T *rqi, T *eSp, T *eSq, T *fSp, T *fSq,
                           int ltid, int TPP, unsigned long long &mG, unsigned long long &mV)
{
  using F = fp<T>;
  const int code = s.code;
  if (code == 1) {
    // the pair is in order and orthogonal: nothing to apply
  }
  else if (code == -1) {
    #pragma unroll 4
    for (long long i = ltid; i < m; i += TPP) {
      const T x = rp[i], y = rq[i];
      Gp[i] = y; Gq[i] = x;
      if (CPLX) { const T xi = rpi[i], yi = rqi[i]; Gip[i] = yi; Giq[i] = xi; }
    }
    #pragma unroll 4
    for (long long i = ltid; i < nv; i += TPP) {
      T t = Vp[i]; Vp[i] = Vq[i]; Vq[i] = t;
      if (CPLX) { t = Vip[i]; Vip[i] = Viq[i]; Viq[i] = t; }
    }
  }
  else if (code == 3 || code == -3) {
    // Gram-Schmidt-like shear (src/dgsscl.c:5-85, src/zgsscl.c)
    const T ex = s.ep, ey = s.eq, fx = s.fp, fy = s.fq;
    const int nx = -(int)ex, ny = -(int)ey;
    const int px = (int)ex, py = (int)ey;
    if (code == 3) {
      const T ff = F::div(fy, fx);
      const T tfr = -s.a21r * ff;
      const T tfi = CPLX ? (s.a21i * ff) : (T)0;
      #pragma unroll 4
      for (long long i = ltid; i < m; i += TPP) {
        if (CPLX) {
          const T xri_ = scale2(rp[i], nx), xii_ = scale2(rpi[i], nx);
          const T yri_ = scale2(rq[i], ny), yii_ = scale2(rqi[i], ny);
          const T xr = F::fma_(tfr, xri_, F::fma_(-tfi, xii_, yri_));
          const T xi = F::fma_(tfr, xii_, F::fma_(tfi, xri_, yii_));
          const T ur = scale2(xr, py), ui = scale2(xi, py);
          Gq[i] = ur; Giq[i] = ui;
          rq[i] = ur; rqi[i] = ui;
          amax(mG, ur); amax(mG, ui);
        }
        else {
          const T xi = scale2(rp[i], nx);
          const T yi = scale2(rq[i], ny);
          const T u = scale2(F::fma_(tfr, xi, yi), py);
          Gq[i] = u;
          rq[i] = u;
          amax(mG, u);
        }
      }
    }
    else {
      const T ff = F::div(fx, fy);
      const T tfr = -s.a21r * ff;
      const T tfi = CPLX ? (-s.a21i * ff) : (T)0;
      #pragma unroll 4
      for (long long i = ltid; i < m; i += TPP) {
        if (CPLX) {
          const T yri = rq[i], yii = rqi[i], xri = rp[i], xii = rpi[i];
          Gp[i] = yri; Gip[i] = yii;
          rp[i] = yri; rpi[i] = yii;
          const T yri_ = scale2(yri, ny), yii_ = scale2(yii, ny);
          const T xri_ = scale2(xri, nx), xii_ = scale2(xii, nx);
          const T vr = F::fma_(tfr, yri_, F::fma_(-tfi, yii_, xri_));
          const T vi = F::fma_(tfr, yii_, F::fma_(tfi, yri_, xii_));
          const T ur = scale2(vr, px), ui = scale2(vi, px);
          Gq[i] = ur; Giq[i] = ui;
          rq[i] = ur; rqi[i] = ui;
          amax(mG, ur); amax(mG, ui);
        }
        else {
          const T xi = rp[i], yi = rq[i];
          Gp[i] = yi;
          rp[i] = yi;
          const T u = scale2(F::fma_(tfr, scale2(yi, ny), scale2(xi, nx)), px);
          Gq[i] = u;
          rq[i] = u;
          amax(mG, u);
        }
      }
      #pragma unroll 4
      for (long long i = ltid; i < nv; i += TPP) {
        T t = Vp[i]; Vp[i] = Vq[i]; Vq[i] = t;
        if (CPLX) { t = Vip[i]; Vip[i] = Viq[i]; Viq[i] = t; }
      }
      if (ltid == 0) {
        *eSp = s.eq; *eSq = s.ep;
        *fSp = s.fq; *fSq = s.fp;
      }
    }
  }
  else {
    // rotation (src/djrot.c, src/djrotf.c, src/zjrot.c, src/zjrotf.c); code -2 permutes
    const bool perm = (code == -2);
    const T c = s.c, at = s.cat, sat = s.sat;
    // the reference marks both columns as changed after any rotation (src/dvjsvd.c:573)
    const bool real_rot = (!CPLX) || (sat == (T)0);
    const bool cone = (c == (T)1);
    if (real_rot && at == (T)0) {
      // c == 1: identity (or a swap when permuting); c != 1 "never happens" (-4 / -10)
      if (cone && perm) {
        #pragma unroll 4
        for (long long i = ltid; i < m; i += TPP) {
          const T x = rp[i], y = rq[i];
          Gp[i] = y; Gq[i] = x; rp[i] = y; rq[i] = x;
          if (CPLX) { const T xi = rpi[i], yi = rqi[i]; Gip[i] = yi; Giq[i] = xi; rpi[i] = yi; rqi[i] = xi; }
        }
        #pragma unroll 4
        for (long long i = ltid; i < nv; i += TPP) {
          T t = Vp[i]; Vp[i] = Vq[i]; Vq[i] = t;
          if (CPLX) { t = Vip[i]; Vip[i] = Viq[i]; Viq[i] = t; }
        }
      }
    }
    else if (real_rot) {
      // the permuted form writes (y - t x) c to x and (x + t y) c to y: the same two
      // products with the destinations exchanged
      for (int pl = 0; pl < (CPLX ? 2 : 1); ++pl) {
        T *X = pl ? Gip : Gp, *Y = pl ? Giq : Gq, *RX = pl ? rpi : rp, *RY = pl ? rqi : rq;
        T *DX = perm ? Y : X, *DY = perm ? X : Y, *RDX = perm ? RY : RX, *RDY = perm ? RX : RY;
        #pragma unroll 4
        for (long long i = ltid; i < m; i += TPP) {
          const T x = RX[i], y = RY[i];
          T u = F::fma_(y, at, x);
          T w = F::fma_(-x, at, y);
          if (!cone) { u = u * c; w = w * c; }
          DX[i] = u; DY[i] = w;
          RDX[i] = u; RDY[i] = w;
          amax(mG, u); amax(mG, w);
        }
        T *XV = pl ? Vip : Vp, *YV = pl ? Viq : Vq;
        T *DXV = perm ? YV : XV, *DYV = perm ? XV : YV;
        #pragma unroll 4
        for (long long i = ltid; i < nv; i += TPP) {
          const T x = XV[i], y = YV[i];
          T u = F::fma_(y, at, x);
          T w = F::fma_(-x, at, y);
          if (!cone) { u = u * c; w = w * c; }
          DXV[i] = u; DYV[i] = w;
          if (TRACKV) { amax(mV, u); amax(mV, w); }
        }
      }
    }
    else {
      const T cta = at, sta = sat, cna = -at;
      for (int mat = 0; mat < 2; ++mat) {
        T *Xr = mat ? Vp : Gp, *Xi = mat ? Vip : Gip, *Yr = mat ? Vq : Gq, *Yi = mat ? Viq : Giq;
        const T *Rxr = mat ? Vp : rp, *Rxi = mat ? Vip : rpi, *Ryr = mat ? Vq : rq, *Ryi = mat ? Viq : rqi;
        const long long rows = mat ? nv : m;
        unsigned long long &mm = mat ? mV : mG;
        #pragma unroll 4
        for (long long i = ltid; i < rows; i += TPP) {
          const T x_r = Rxr[i], x_i = Rxi[i], y_r = Ryr[i], y_i = Ryi[i];
          T ar = F::fma_(y_r, cta, F::fma_(-y_i, sta, x_r));
          T ai = F::fma_(y_r, sta, F::fma_(y_i, cta, x_i));
          T br = F::fma_(x_r, cna, F::fma_(-x_i, sta, y_r));
          T bi = F::fma_(x_r, sta, F::fma_(x_i, cna, y_i));
          if (!cone) { ar = ar * c; ai = ai * c; br = br * c; bi = bi * c; }
          if (perm) { Yr[i] = ar; Yi[i] = ai; Xr[i] = br; Xi[i] = bi; }
          else { Xr[i] = ar; Xi[i] = ai; Yr[i] = br; Yi[i] = bi; }
          if (!mat) {
            if (perm) { rq[i] = ar; rqi[i] = ai; rp[i] = br; rpi[i] = bi; }
            else { rp[i] = ar; rpi[i] = ai; rq[i] = br; rqi[i] = bi; }
          }
          if (!mat || TRACKV) { amax(mm, ar); amax(mm, ai); amax(mm, br); amax(mm, bi); }
        }
      }
    }
  }
}

}  // namespace vj
