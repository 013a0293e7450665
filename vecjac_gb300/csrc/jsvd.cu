// One-sided Jacobi SVD: dvjsvd_/zvjsvd_/svjsvd_/cvjsvd_ on the GPU.
//
// The reference (src/dvjsvd.c:40-638, src/zvjsvd.c:40-694) runs every pivot step of a
// sweep as a sequence of OpenMP loops over the n/2 column pairs of that step: norms of
// the columns changed in the previous step, scaled compensated dot products, the
// convergence/shear test with the Gram prescale, the batched 2x2 EVD, classification,
// and the rotation / shear / swap of the columns of G and V. Here one kernel launch is
// one step and one CTA owns one pair for the whole step:
//   1. step-start decisions that the reference takes on the host (rescale G when its
//      largest element grew past 2^1022, rescale V likewise, the norm-overflow retry) are
//      recomputed identically by every CTA from a small control block written by the
//      previous launch; every CTA applies them to its own two columns, which together
//      cover all of G and V;
//   2. the dot product is accumulated by LANES threads (8 for FP64, 16 for FP32) in the
//      reference's lane order, with its 2Sum compensation, and summed by the same
//      halving tree as GCC's _mm512_reduce_add: the result is bit-identical;
//   3. one thread takes the convergence test, the shear test, the prescale and the 2x2
//      (vj::rjac2 / vj::cjac2) and picks the transformation;
//   4. all threads apply it to the columns of G and V, tracking max |.| for the overflow
//      control;
//   5. the norms of the columns this step changed are computed right away (the
//      reference computes them at the start of the next step, on the same data) by
//      one warp per column with the project's two-pass 32-lane norm.
// G and V stay in HBM/L2 (16 MiB for 1024x1024 FP64, far below the 129 MB L2); every
// launch touches each column of G and V once for the dot, once for the update and once
// for the norm. The arithmetic is FP64-pipe bound on GB300.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "jac2.cuh"
#include "vj_host.h"

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
template <typename T> __device__ __forceinline__ T bitst(unsigned long long u)
{
  return fp<T>::val((typename fp<T>::U)u);
}

// |x| bits, NaN above inf, so that an integer max flags NaNs as "not finite"
template <typename T> __device__ __forceinline__ unsigned long long absbits(T x)
{
  return (unsigned long long)(fp<T>::bits(x) & ~fp<T>::SIGN);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v) ? w : v;
  }
  return v;
}

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

// The project's column norm (two-pass power-of-two scaling, 32 lanes, halving tree) for
// one warp; every lane returns the same value.
template <typename T> __device__ T warp_nrm2(const T *x, long long m)
{
  const int lane = threadIdx.x & 31;
  unsigned long long mx = 0ull;
  for (long long i = lane; i < m; i += 32) {
    const unsigned long long a = absbits(x[i]);
    mx = (a > mx) ? a : mx;
  }
  mx = warp_max_u64(mx);
  const T a = bitst<T>(mx);
  if (!visfinite(a))
    return visnan(a) ? fp<T>::qnan() : a;
  if (mx == 0ull)
    return (T)0;
  const int k = ilogb_(a);
  T acc = (T)0;
  for (long long i = lane; i < m; i += 32) {
    const T y = scale2(x[i], -k);
    acc = fp<T>::fma_(y, y, acc);
  }
#pragma unroll
  for (int w = 16; w >= 1; w >>= 1)
    acc = acc + __shfl_down_sync(0xffffffffu, acc, w);
  acc = __shfl_sync(0xffffffffu, acc, 0);
  return scale2(fp<T>::sqrt_(acc), k);
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

// scaled compensated dot products (src/ddpscl.c / src/zdpscl.c) by warp 0; x = G_q, y = G_p.
// Only the two (four for complex data) 2Sum accumulations carry a dependency from one
// element to the next; the loads, the power-of-two scaling and the exact product split
// (round-down product and its error by an FMA) of element i + LANES are issued before the
// accumulation of element i, so that their FP64 latency overlaps the accumulator chain.
template <typename T, bool CPLX> struct DotTerms {
  T pd[CPLX ? 4 : 1], dn[CPLX ? 4 : 1];
};

template <typename T, bool CPLX>
__device__ __forceinline__ void dot_terms(const T *xr, const T *xi, const T *yr, const T *yi, long long i, int nx,
                                          int ny, DotTerms<T, CPLX> &d)
{
  const T xri = scale2(xr[i], nx);
  const T yri = scale2(yr[i], ny);
  if (CPLX) {
    const T yii = scale2(yi[i], ny);
    const T xii = scale2(xi[i], nx);
    // (negations are written as FP negations: the FMA folds them, with the same bits)
    const T xs[4] = {xri, xii, xri, -xii}, ys[4] = {yri, yii, yii, yri};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      d.pd[k] = fp<T>::mul_rd(xs[k], ys[k]);
      d.dn[k] = fp<T>::fma_(xs[k], ys[k], -d.pd[k]);
    }
  }
  else {
    d.pd[0] = fp<T>::mul_rd(xri, yri);
    d.dn[0] = fp<T>::fma_(xri, yri, -d.pd[0]);
  }
}

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
__device__ void pair_dot(const SvdArgs<T> &a, const T *xr, const T *xi, const T *yr, const T *yi, T ex, T ey, T fx,
                         T fy, bool live, T &zr, T &zi)
{
  constexpr int L = svdc<T>::LANES;
  const int lane = (threadIdx.x & 31) % L;
  const int nx = -(int)ex, ny = -(int)ey;
  T sr = 0, tr = 0, sr_ = 0, tr_ = 0, si = 0, ti = 0, si_ = 0, ti_ = 0;
  if (live && lane < a.m) {
    DotTerms<T, CPLX> cur, nxt;
    dot_terms<T, CPLX>(xr, xi, yr, yi, lane, nx, ny, cur);
    for (long long i = lane; i < a.m; i += L) {
      // the terms of the next element (of this one again on the last pass, unused), with
      // no branch so that they interleave with the accumulation below
      const long long inx = (i + L < a.m) ? (i + L) : i;
      dot_terms<T, CPLX>(xr, xi, yr, yi, inx, nx, ny, nxt);
      if (CPLX) {
        dot_acc(cur.pd[0], cur.dn[0], sr, tr, sr_, tr_);
        dot_acc(cur.pd[1], cur.dn[1], sr, tr, sr_, tr_);
        dot_acc(cur.pd[2], cur.dn[2], si, ti, si_, ti_);
        dot_acc(cur.pd[3], cur.dn[3], si, ti, si_, ti_);
      }
      else
        dot_acc(cur.pd[0], cur.dn[0], sr, tr, sr_, tr_);
      cur = nxt;
    }
  }
  const T nur = hsum<L>(sr) + (hsum<L>(tr) + (hsum<L>(sr_) + hsum<L>(tr_)));
  T nui = 0;
  if (CPLX)
    nui = hsum<L>(si) + (hsum<L>(ti) + (hsum<L>(si_) + hsum<L>(ti_)));
  const T de = fx * fy;
  zr = fp<T>::div(nur, de);
  zi = CPLX ? fp<T>::div(nui, de) : (T)0;
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

// Pairs handled by one CTA: the LANES-wide dot of pair j runs on lanes [j LANES,
// (j+1) LANES) of warp 0. GB300's FP64 unit accepts about one warp instruction every 19
// cycles per SM whatever the number of active lanes, so the four FP64 dot products of a
// CTA share every FP64 instruction (32 active lanes) instead of issuing four.
template <typename T> struct ppc { static constexpr int P = 32 / svdc<T>::LANES; };

template <typename T, bool CPLX, bool TRACKV, bool STAGE>
__global__ void __launch_bounds__(256) k_step(SvdArgs<T> a, int st, int g3, int last)
{
  using F = fp<T>;
  constexpr int P = ppc<T>::P;
  constexpr int L = svdc<T>::LANES;
  constexpr int NC = CPLX ? 4 : 2;   // staged columns per pair (real and imaginary planes)
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ PairState<T> ps[P];
  __shared__ unsigned long long red[8][2];
  __shared__ int s_err;
  __shared__ unsigned long long bar;
  SvdGlobal *const g = a.g;
  if (*(volatile long long *)&g->err)
    return;
  const Ctl &cur = g->ctl[g3];
  Ctl &nxt = g->ctl[(g3 + 1) % 3];
  Ctl &nn = g->ctl[(g3 + 2) % 3];
  const unsigned *r = a.js + (size_t)st * (size_t)a.n;
  const long long n_2 = a.n >> 1;
  const long long pair0 = (long long)blockIdx.x * P;
  const int np = (int)((n_2 - pair0 < P) ? (n_2 - pair0) : P);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool tr = a.trace && blockIdx.x == 0 && tid == 0;
  long long tmark = tr ? clock64() : 0;
  auto tphase = [&](int ph) {
    if (tr) {
      const long long t = clock64();
      atomicAdd(&g->phase[ph], (unsigned long long)(t - tmark));
      tmark = t;
    }
  };
  const Decision<T> d = decide(a, cur);
  if (blockIdx.x == 0 && tid == 0) {
    nxt.MGbase = (double)d.MG;
    nxt.MVbase = (double)d.MV;
    nxt.sT = d.sT;
    nxt.sV = d.sV;
    nn.nMG = 0ull;
    nn.nMV = 0ull;
    nn.ovf = 0;
  }
  if (tid == 0)
    s_err = 0;
  auto colp = [&](int j) { return (long long)r[2 * (pair0 + j)]; };
  auto colq = [&](int j) { return (long long)r[2 * (pair0 + j) + 1]; };
  // ---- 1. rescaling (rare) ----
  if (d.gres || d.ovf) {
    const int e = d.gres ? d.sNg : d.sNv;
    for (int j = 0; j < np; ++j) {
      scale_cols(a.G, a.ldG, a.m, colp(j), colq(j), e);
      if (CPLX)
        scale_cols(a.Gi, a.ldGi, a.m, colp(j), colq(j), e);
    }
    __syncthreads();
    if (warp < 2 * np) {
      const T nv = col_norm<T, CPLX>(a, (warp & 1) ? colq(warp >> 1) : colp(warp >> 1));
      if ((lane == 0) && !(nv <= svdc<T>::RMAX))
        s_err = 1;
    }
    __syncthreads();
    if (s_err) {
      // a second overflow after rescaling: the reference would rescale again
      if (tid == 0)
        atomicMin((long long *)&g->err, (long long)VJ_ERR_ARG);
      return;
    }
  }
  if (d.vres)
    for (int j = 0; j < np; ++j) {
      scale_cols(a.V, a.ldV, a.n, colp(j), colq(j), d.sNv);
      if (CPLX)
        scale_cols(a.Vi, a.ldVi, a.n, colp(j), colq(j), d.sNv);
    }
  tphase(0);
  // ---- stage the columns of G in shared memory (TMA bulk copies) ----
  // staged layout: pair j, column c (p, q, pi, qi) at sm + (j * NC + c) * m
  T *const sm = reinterpret_cast<T *>(smem_raw);
  auto rcol = [&](int j, int c) -> T * {
    if (STAGE)
      return sm + ((long long)j * NC + c) * a.m;
    const long long col = (c & 1) ? colq(j) : colp(j);
    return (c < 2) ? (a.G + col * a.ldG) : (a.Gi + col * a.ldGi);
  };
  if (STAGE) {
    if (tid == 0)
      mbar_init(&bar, 1u);
    __syncthreads();
    if (tid == 0) {
      const unsigned colb = (unsigned)(a.m * (long long)sizeof(T));
      mbar_expect_tx(&bar, colb * (unsigned)(NC * np));
      for (int j = 0; j < np; ++j)
        for (int c = 0; c < NC; ++c) {
          const long long col = (c & 1) ? colq(j) : colp(j);
          const T *src = (c < 2) ? (a.G + col * a.ldG) : (a.Gi + col * a.ldGi);
          T *dst = rcol(j, c);
          for (unsigned off = 0; off < colb; off += 32768u) {
            const unsigned b = (colb - off < 32768u) ? (colb - off) : 32768u;
            tma_load_1d(reinterpret_cast<char *>(dst) + off, reinterpret_cast<const char *>(src) + off, b, &bar);
          }
        }
    }
    if (!mbar_wait_bounded(&bar)) {
      // the copies did not land within the limit: flag it, give them another bounded
      // wait, and leave without touching the matrix
      if (tid == 0)
        atomicMin((long long *)&g->err, (long long)VJ_ERR_CUDA);
      (void)mbar_wait_bounded(&bar);
      return;
    }
  }
  __syncthreads();
  tphase(1);
  // ---- 2. scaled dot products: pair j on lanes [j L, (j+1) L) of warp 0 ----
  if (warp == 0) {
    const int j = lane / L;
    const bool act = (j < np);
    const int jj = act ? j : 0;
    const long long p = colp(jj), q = colq(jj);
    const T ep = a.eS[p], fp_ = a.fS[p], eq = a.eS[q], fq = a.fS[q];
    T zr = 0, zi = 0;
    const bool live = act && (eq >= -svdc<T>::RMAX) && (ep >= -svdc<T>::RMAX);
    pair_dot<T, CPLX>(a, rcol(jj, 1), CPLX ? rcol(jj, 3) : nullptr, rcol(jj, 0), CPLX ? rcol(jj, 2) : nullptr, eq,
                      ep, fq, fp_, live, zr, zi);
    tphase(2);
    if (act && (lane % L) == 0) {
      PairState<T> &s = ps[j];
      s.ep = ep; s.fp = fp_; s.eq = eq; s.fq = fq;
      if (!live) {
        zr = 0;
        zi = 0;
      }
      s.a21r = zr;
      s.a21i = zi;
      s.skip = 0;
      long long code = 0;
      if (CPLX) {
        if (!visfinite(zr))
          code = a.e_dot;
        if (!visfinite(zi))
          code = (a.e_doti < code) ? a.e_doti : code;
      }
      else if (!visfinite(zr))
        code = a.e_dot;
      if (code) {
        atomicMin((long long *)&g->err, code);
        s.skip = 1;
      }
      else {
        // ---- 3. convergence, shear test, prescale, 2x2, classification ----
        const T ab = CPLX ? vhypot(zr, zi) : vabs(zr);
        const bool trans = (a.tol <= ab);
        if (trans) {
          atomicAdd(&g->swt, 1ull);
          const T e1 = ep, e2 = eq, f1 = fp_, f2 = fq;
          const bool ngs = eflt(e1, e2, f1, f2);
          T maf = ngs ? f1 : f2, mae = ngs ? e1 : e2;
          const T Maf = ngs ? f2 : f1, Mae = ngs ? e2 : e1;
          maf = a.gst * maf;
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
        else if (efcmp(ep, fp_, eq, fq) < 0) {
          a.eS[p] = eq; a.eS[q] = ep;
          a.fS[p] = fq; a.fS[q] = fp_;
          s.code = -1;
        }
        else
          s.code = 1;
      }
    }
  }
  __syncthreads();
  tphase(3);
  // ---- 4. apply: the CTA's pairs concurrently, blockDim/P threads each; G is read from
  // the staged copy ----
  unsigned long long mG = 0ull, mV = 0ull;
  unsigned chmask = 0u;  // bit 2j: column p of pair j changed, bit 2j+1: column q
  for (int j = 0; j < np; ++j) {
    const int cj = ps[j].code;
    if (!ps[j].skip)
      chmask |= ((cj == 3 || cj == -3) ? 2u : ((cj == 2 || cj == -2) ? 3u : 0u)) << (2 * j);
  }
  const int TPP = (int)blockDim.x / P;
  const int j = tid / TPP;
  const int ltid = tid - j * TPP;
  if (j < np && !ps[j].skip) {
    const PairState<T> s = ps[j];
    const int code = s.code;
    const long long p = colp(j), q = colq(j);
    T *Gp = a.G + p * a.ldG, *Gq = a.G + q * a.ldG, *Vp = a.V + p * a.ldV, *Vq = a.V + q * a.ldV;
    T *Gip = CPLX ? (a.Gi + p * a.ldGi) : nullptr, *Giq = CPLX ? (a.Gi + q * a.ldGi) : nullptr;
    T *Vip = CPLX ? (a.Vi + p * a.ldVi) : nullptr, *Viq = CPLX ? (a.Vi + q * a.ldVi) : nullptr;
    T *rp = rcol(j, 0), *rq = rcol(j, 1), *rpi = CPLX ? rcol(j, 2) : nullptr, *rqi = CPLX ? rcol(j, 3) : nullptr;
    if (code == 1) {
    }
    else if (code == -1) {
      #pragma unroll 4
      for (long long i = ltid; i < a.m; i += TPP) {
        const T x = rp[i], y = rq[i];
        Gp[i] = y; Gq[i] = x;
        if (CPLX) { const T xi = rpi[i], yi = rqi[i]; Gip[i] = yi; Giq[i] = xi; }
      }
      #pragma unroll 4
      for (long long i = ltid; i < a.n; i += TPP) {
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
        for (long long i = ltid; i < a.m; i += TPP) {
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
        for (long long i = ltid; i < a.m; i += TPP) {
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
        for (long long i = ltid; i < a.n; i += TPP) {
          T t = Vp[i]; Vp[i] = Vq[i]; Vq[i] = t;
          if (CPLX) { t = Vip[i]; Vip[i] = Viq[i]; Viq[i] = t; }
        }
        if (ltid == 0) {
          a.eS[p] = s.eq; a.eS[q] = s.ep;
          a.fS[p] = s.fq; a.fS[q] = s.fp;
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
          for (long long i = ltid; i < a.m; i += TPP) {
            const T x = rp[i], y = rq[i];
            Gp[i] = y; Gq[i] = x; rp[i] = y; rq[i] = x;
            if (CPLX) { const T xi = rpi[i], yi = rqi[i]; Gip[i] = yi; Giq[i] = xi; rpi[i] = yi; rqi[i] = xi; }
          }
          #pragma unroll 4
          for (long long i = ltid; i < a.n; i += TPP) {
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
          for (long long i = ltid; i < a.m; i += TPP) {
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
          for (long long i = ltid; i < a.n; i += TPP) {
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
          const long long rows = mat ? a.n : a.m;
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
  tphase(4);
  // block max of |G| and |V| updates
  mG = warp_max_u64(mG);
  mV = warp_max_u64(mV);
  if (lane == 0) {
    red[warp][0] = mG;
    red[warp][1] = mV;
  }
  __syncthreads();
  if (tid == 0) {
    unsigned long long bg = 0ull, bv = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      bg = (red[w][0] > bg) ? red[w][0] : bg;
      bv = (red[w][1] > bv) ? red[w][1] : bv;
    }
    const T tG = bitst<T>(bg), tV = bitst<T>(bv);
    if (!visfinite(tG))
      atomicMin((long long *)&g->err, a.e_appg);
    else if (!visfinite(tV))
      atomicMin((long long *)&g->err, a.e_appv);
    else {
      if (bg)
        atomicMax(&nxt.nMG, bg);
      if (bv)
        atomicMax(&nxt.nMV, bv);
    }
  }
  // ---- 5. norms of the changed columns (warp w: pair w/2, column p or q), for the next step ----
  // (not after the last step of the last allowed sweep: the reference returns there with
  // the norms of those columns not yet recomputed)
  if (!last && warp < 2 * np && ((chmask >> warp) & 1u)) {
    const int j = warp >> 1, c = warp & 1;
    const long long col = c ? colq(j) : colp(j);
    const T nv = col_norm_at<T, CPLX>(a, col, rcol(j, c), CPLX ? rcol(j, 2 + c) : nullptr);
    if ((lane == 0) && !(nv <= svdc<T>::RMAX))
      atomicOr(&nxt.ovf, 1);
  }
  tphase(5);
}

// norms of all columns before the first step (src/dvjsvd.c:174-180 sets w1 = 1)
template <typename T, bool CPLX> __global__ void k_norms(SvdArgs<T> a)
{
  const long long c = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= a.n)
    return;
  const T nv = col_norm<T, CPLX>(a, c);
  if (((threadIdx.x & 31) == 0) && !(nv <= svdc<T>::RMAX))
    atomicOr(&a.g->ctl[0].ovf, 1);
}

// max |a_ij| with min(., inf) (src/dnormx.c); result as bits in *out (atomicMax)
template <typename T>
__global__ void k_normx(const T *A, long long ld, long long rows, long long cols, unsigned long long *out)
{
  unsigned long long m = 0ull;
  const unsigned long long inf = absbits(fp<T>::inf());
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x) {
      unsigned long long b = absbits(A[j * ld + i]);
      b = (b > inf) ? inf : b;  // VMINPD(|x|, inf) maps a NaN to inf
      m = (b > m) ? b : m;
    }
  m = warp_max_u64(m);
  if ((threadIdx.x & 31) == 0 && m)
    atomicMax(out, m);
}

template <typename T> __global__ void k_scale(T *A, long long ld, long long rows, long long cols, int e)
{
  for (long long j = blockIdx.y; j < cols; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (long long)gridDim.x * blockDim.x)
      A[j * ld + i] = scale2(A[j * ld + i], e);
}

template <typename T> __global__ void k_eye(T *V, long long ld, long long n, int diag)
{
  for (long long j = blockIdx.y; j < n; j += gridDim.y)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
      V[j * ld + i] = (diag && i == j) ? (T)1 : (T)0;
}

template <typename T> __global__ void k_initS(T *eS, T *fS, long long n)
{
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
    eS[j] = vneg(fp<T>::inf());
    fS[j] = (T)1;
  }
}

// U = G diag(1/f) 2^-e, eS -= sT (src/dvjsvd.c:604-631); V * 2^-sV
template <typename T, bool CPLX> __global__ void k_final(SvdArgs<T> a, int g3)
{
  const Ctl &c = a.g->ctl[g3];
  const long long j = blockIdx.y;
  const T f = a.fS[j];
  const T s = vneg(a.eS[j]);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += (long long)gridDim.x * blockDim.x) {
    a.G[j * a.ldG + i] = scalef(fp<T>::div(a.G[j * a.ldG + i], f), s);
    if (CPLX)
      a.Gi[j * a.ldGi + i] = scalef(fp<T>::div(a.Gi[j * a.ldGi + i], f), s);
  }
  if (c.sV) {
    const T sv = (T)(-c.sV);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (long long)gridDim.x * blockDim.x) {
      a.V[j * a.ldV + i] = scalef(a.V[j * a.ldV + i], sv);
      if (CPLX)
        a.Vi[j * a.ldVi + i] = scalef(a.Vi[j * a.ldVi + i], sv);
    }
  }
}

template <typename T> __global__ void k_final_e(T *eS, long long n, const SvdGlobal *g, int g3)
{
  const T sT = (T)g->ctl[g3].sT;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
    eS[j] = eS[j] - sT;
}

// host-side (e, f) exponent of a positive finite value
template <typename T> static int h_exp(T x)
{
  int e = 0;
  (void)std::frexp((double)x, &e);
  return e - 1;
}
template <typename T> static T h_scale2(T x, int n)
{
  return (T)std::ldexp((double)x, n);
}

static inline bool is_al(const void *p)
{
  return !((uintptr_t)p & 63u);
}

template <typename T, bool CPLX>
static vj_fint svd_dev(vj_fnat m_, vj_fnat n_, T *G, vj_fnat ldG, T *Gi, vj_fnat ldGi, T *V, vj_fnat ldV, T *Vi,
                       vj_fnat ldVi, T *eS, T *fS, const unsigned *js, unsigned stp, unsigned swp, int preset,
                       cudaStream_t s, unsigned char *scratch = nullptr)
{
  constexpr int L = svdc<T>::LANES;
  const long long m = (long long)m_, n = (long long)n_;
  const long long n_2 = n >> 1;
  if (!n)
    return 0;
  if (m_ < n_ || (m % L))
    return -1;
  if ((n & 1) || (n_2 % L))
    return -2;
  if (!is_al(G))
    return -3;
  if (ldG < m_ || (ldG % L))
    return -4;
  if (CPLX) {
    if (!is_al(Gi)) return -5;
    if (ldGi < m_ || (ldGi % L)) return -6;
    if (!is_al(V)) return -7;
    if (ldV < n_ || (ldV % L)) return -8;
    if (!is_al(Vi)) return -9;
    if (ldVi < n_ || (ldVi % L)) return -10;
  }
  else {
    if (!is_al(V)) return -5;
    if (ldV < n_ || (ldV % L)) return -6;
  }
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const long long E_MG = CPLX ? -92 : -80, E_MV = CPLX ? -104 : -92, E_MVZ = CPLX ? -17 : -13;
  unsigned char *ctlmem = scratch;
  if (!ctlmem) {
    host::Staging &stg = host::staging2();
    if (!stg.reserve(sizeof(SvdGlobal) + 256))
      return VJ_ERR_NOMEM;
    ctlmem = reinterpret_cast<unsigned char *>(stg.ptr);
  }
  SvdGlobal *dg = reinterpret_cast<SvdGlobal *>(ctlmem);
  unsigned long long *dmx = reinterpret_cast<unsigned long long *>(ctlmem + sizeof(SvdGlobal) + 64);
  const dim3 blk(256);
  auto grid2 = [](long long rows, long long cols) {
    long long gx = (rows + 255) / 256;
    if (gx > 64) gx = 64;
    long long gy = cols < 65535 ? cols : 65535;
    return dim3((unsigned)gx, (unsigned)(gy > 0 ? gy : 1));
  };
  auto normx = [&](const T *A, long long lda, long long rows, long long cols, const T *Ai, long long ldai,
                   T &out) -> bool {
    if (cudaMemsetAsync(dmx, 0, 8, s) != cudaSuccess) return false;
    k_normx<T><<<grid2(rows, cols), blk, 0, s>>>(A, lda, rows, cols, dmx);
    if (CPLX)
      k_normx<T><<<grid2(rows, cols), blk, 0, s>>>(Ai, ldai, rows, cols, dmx);
    unsigned long long b = 0;
    if (cudaMemcpyAsync(&b, dmx, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) return false;
    if (cudaStreamSynchronize(s) != cudaSuccess) return false;
    typename fp<T>::U u = (typename fp<T>::U)b;
    T v;
    memcpy(&v, &u, sizeof(T));
    out = v;
    return true;
  };
  T MG = 0, MV = 1;
  if (!normx(G, (long long)ldG, m, n, Gi, (long long)ldGi, MG))
    return VJ_ERR_CUDA;
  if (!(MG <= svdc<T>::RMAX))
    return E_MG;
  if (preset) {
    if (!normx(V, (long long)ldV, n, n, Vi, (long long)ldVi, MV))
      return VJ_ERR_CUDA;
    if (!(MV <= svdc<T>::RMAX))
      return E_MV;
    if (MV <= (T)0)
      return E_MVZ;
  }
  else {
    k_eye<T><<<grid2(n, n), blk, 0, s>>>(V, (long long)ldV, n, 1);
    if (CPLX)
      k_eye<T><<<grid2(n, n), blk, 0, s>>>(Vi, (long long)ldVi, n, 0);
  }
  k_initS<T><<<(unsigned)((n + 255) / 256), blk, 0, s>>>(eS, fS, n);
  if (MG == (T)0) {
    if (cudaStreamSynchronize(s) != cudaSuccess)
      return VJ_ERR_CUDA;
    return 0;
  }
  // setup of src/dvjsvd.c:120-156 (src/zvjsvd.c:135-171)
  const int ROT = CPLX ? (svdc<T>::ROT_C - 1) : svdc<T>::ROT_R;
  const T M_m = CPLX ? (svdc<T>::RMAX / ((T)((unsigned long long)m << 2u) * (T)M_SQRT2))
                     : (svdc<T>::RMAX / (T)((unsigned long long)m << 1u));
  const int NRM = h_exp(M_m);
  int eM = h_exp(MG);
  int sN = NRM - eM - 1;
  if (sN) {
    k_scale<T><<<grid2(m, n), blk, 0, s>>>(G, (long long)ldG, m, n, sN);
    if (CPLX)
      k_scale<T><<<grid2(m, n), blk, 0, s>>>(Gi, (long long)ldGi, m, n, sN);
    MG = h_scale2(MG, sN);
  }
  const int sT = sN;
  int sV = 0;
  if (preset) {
    eM = h_exp(MV);
    const int sR = ROT - eM;
    if (sR) {
      k_scale<T><<<grid2(n, n), blk, 0, s>>>(V, (long long)ldV, n, n, sR);
      if (CPLX)
        k_scale<T><<<grid2(n, n), blk, 0, s>>>(Vi, (long long)ldVi, n, n, sR);
      MV = h_scale2(MV, sR);
    }
    sV = sR;
  }
  SvdGlobal hg;
  memset(&hg, 0, sizeof(hg));
  hg.ctl[0].MGbase = (double)MG;
  hg.ctl[0].MVbase = (double)MV;
  hg.ctl[0].sT = sT;
  hg.ctl[0].sV = sV;
  if (cudaMemcpyAsync(dg, &hg, sizeof(hg), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  SvdArgs<T> a;
  a.trace = host::trace_enabled() ? 1 : 0;
  a.m = m; a.n = n; a.ldG = (long long)ldG; a.ldGi = (long long)ldGi; a.ldV = (long long)ldV;
  a.ldVi = (long long)ldVi;
  a.G = G; a.Gi = Gi; a.V = V; a.Vi = Vi; a.eS = eS; a.fS = fS; a.js = js; a.g = dg;
  a.tol = (T)(std::sqrt((T)m) * h_scale2(svdc<T>::EPS, -1));
  if (sizeof(T) == 4)
    a.tol = sqrtf((float)m) * h_scale2(svdc<T>::EPS, -1);
  a.gst = h_scale2(a.tol, (int)svdc<T>::MAX_FIN_EXP);
  a.nrm_exp = NRM;
  a.rot = ROT;
  a.e_dot = CPLX ? -345 : -320;
  a.e_doti = -347;
  a.e_appg = CPLX ? -630 : -580;
  a.e_appv = CPLX ? -638 : -588;
  if (swp)
    k_norms<T, CPLX><<<(unsigned)((n + 7) / 8), blk, 0, s>>>(a);
  if (cudaGetLastError() != cudaSuccess)
    return VJ_ERR_CUDA;
  // stage each pair's columns of G in shared memory when they fit (160 KiB per CTA)
  constexpr int P = ppc<T>::P;
  const size_t smem = (size_t)m * sizeof(T) * (CPLX ? 4u : 2u) * P;
  const bool stage = (smem <= (size_t)160 * 1024);
  const unsigned grid = (unsigned)((n_2 + P - 1) / P);
  if (stage && smem > 48 * 1024) {
    cudaFuncSetAttribute(k_step<T, CPLX, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_step<T, CPLX, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  unsigned sw = 0;
  long long gstep = 0;
  while (sw < swp) {
    if (cudaMemsetAsync(&dg->swt, 0, 8, s) != cudaSuccess)
      return VJ_ERR_CUDA;
    for (unsigned st = 0; st < stp; ++st, ++gstep) {
      const int last = ((sw + 1u == swp) && (st + 1u == stp)) ? 1 : 0;
      const int g3 = (int)(gstep % 3);
      if (stage) {
        if (preset)
          k_step<T, CPLX, true, true><<<grid, blk, smem, s>>>(a, (int)st, g3, last);
        else
          k_step<T, CPLX, false, true><<<grid, blk, smem, s>>>(a, (int)st, g3, last);
      }
      else {
        if (preset)
          k_step<T, CPLX, true, false><<<grid, blk, 0, s>>>(a, (int)st, g3, last);
        else
          k_step<T, CPLX, false, false><<<grid, blk, 0, s>>>(a, (int)st, g3, last);
      }
    }
    if (cudaGetLastError() != cudaSuccess)
      return VJ_ERR_CUDA;
    long long hv[2];
    if (cudaMemcpyAsync(hv, dg, 16, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return VJ_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess)
      return VJ_ERR_CUDA;
    if (hv[0])
      return hv[0];
    host::trace_sweep(sw, (unsigned long long)hv[1]);
    if (!hv[1])
      break;
    ++sw;
  }
  if (sw < swp) {
    dim3 gf((unsigned)((m + 255) / 256 < 16 ? (m + 255) / 256 : 16), (unsigned)n);
    k_final<T, CPLX><<<gf, blk, 0, s>>>(a, (int)(gstep % 3));
    k_final_e<T><<<(unsigned)((n + 255) / 256), blk, 0, s>>>(eS, n, dg, (int)(gstep % 3));
  }
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (a.trace) {
    unsigned long long ph[8];
    if (cudaMemcpy(ph, dg->phase, sizeof(ph), cudaMemcpyDeviceToHost) == cudaSuccess)
      host::trace_phases(ph, 6);
  }
  return (vj_fint)sw;
}

// host-pointer form: copy in, compute, copy out (G, V, eS, fS)
template <typename T, bool CPLX>
static vj_fint svd_host(const vj_fnat *m, const vj_fnat *n, T *G, const vj_fnat *ldG, T *Gi, const vj_fnat *ldGi,
                        T *V, const vj_fnat *ldV, T *Vi, const vj_fnat *ldVi, T *eS, T *fS, const unsigned *js,
                        const unsigned *stp, const unsigned *swp, T *work, unsigned *iwork)
{
  constexpr int L = svdc<T>::LANES;
  const long long mm = (long long)*m, nn = (long long)*n;
  // the reference's argument checks, in its order (src/dvjsvd.c:43-68, src/zvjsvd.c:43-80)
  if (!nn)
    return 0;
  if (*m < *n || (mm % L))
    return -1;
  if ((nn & 1) || ((nn >> 1) % L))
    return -2;
  if (!is_al(G))
    return -3;
  if (*ldG < *m || (*ldG % L))
    return -4;
  if (CPLX) {
    if (!is_al(Gi)) return -5;
    if (*ldGi < *m || (*ldGi % L)) return -6;
    if (!is_al(V)) return -7;
    if (*ldV < *n || (*ldV % L)) return -8;
    if (!is_al(Vi)) return -9;
    if (*ldVi < *n || (*ldVi % L)) return -10;
    if (!is_al(work)) return -16;
  }
  else {
    if (!is_al(V)) return -5;
    if (*ldV < *n || (*ldV % L)) return -6;
    if (!is_al(work)) return -12;
  }
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  const int preset = (*iwork != 0u);
  cudaStream_t st2[2];
  if (!host::streams2(st2))
    return VJ_ERR_CUDA;
  cudaStream_t s = st2[0];
  // device copies: G (m x n), Gi, V (n x n), Vi, eS, fS, js; compact leading dimensions
  const size_t gsz = (size_t)mm * nn * sizeof(T), vsz = (size_t)nn * nn * sizeof(T);
  const size_t jsz = (size_t)(*stp) * nn * sizeof(unsigned);
  const size_t al = 256;
  auto up = [&](size_t x) { return (x + al - 1) & ~(al - 1); };
  const size_t total = up(gsz) * (CPLX ? 2 : 1) + up(vsz) * (CPLX ? 2 : 1) + 2 * up(nn * sizeof(T)) + up(jsz);
  host::Staging &stg = host::staging();
  if (!stg.reserve(total))
    return VJ_ERR_NOMEM;
  char *b = stg.ptr;
  T *dG = (T *)b; b += up(gsz);
  T *dGi = CPLX ? (T *)b : nullptr; if (CPLX) b += up(gsz);
  T *dV = (T *)b; b += up(vsz);
  T *dVi = CPLX ? (T *)b : nullptr; if (CPLX) b += up(vsz);
  T *deS = (T *)b; b += up(nn * sizeof(T));
  T *dfS = (T *)b; b += up(nn * sizeof(T));
  unsigned *djs = (unsigned *)b;
  const size_t ms = (size_t)mm * sizeof(T), ns = (size_t)nn * sizeof(T);
  if (cudaMemcpy2DAsync(dG, ms, G, (size_t)*ldG * sizeof(T), ms, (size_t)nn, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (CPLX && cudaMemcpy2DAsync(dGi, ms, Gi, (size_t)*ldGi * sizeof(T), ms, (size_t)nn, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (preset) {
    if (cudaMemcpy2DAsync(dV, ns, V, (size_t)*ldV * sizeof(T), ns, (size_t)nn, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return VJ_ERR_CUDA;
    if (CPLX && cudaMemcpy2DAsync(dVi, ns, Vi, (size_t)*ldVi * sizeof(T), ns, (size_t)nn, cudaMemcpyHostToDevice, s) != cudaSuccess)
      return VJ_ERR_CUDA;
  }
  if (jsz && cudaMemcpyAsync(djs, js, jsz, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  host::trace_reset();
  const vj_fint r = svd_dev<T, CPLX>(*m, *n, dG, (vj_fnat)mm, dGi, (vj_fnat)mm, dV, (vj_fnat)nn, dVi, (vj_fnat)nn,
                                     deS, dfS, djs, *stp, *swp, preset, s);
  if (r == VJ_ERR_CUDA || r == VJ_ERR_NO_GPU || r == VJ_ERR_NOMEM)
    return r;
  // results (also on numerical errors: G and V then hold intermediate values)
  if (cudaMemcpy2DAsync(G, (size_t)*ldG * sizeof(T), dG, ms, ms, (size_t)nn, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (CPLX && cudaMemcpy2DAsync(Gi, (size_t)*ldGi * sizeof(T), dGi, ms, ms, (size_t)nn, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (cudaMemcpy2DAsync(V, (size_t)*ldV * sizeof(T), dV, ns, ns, (size_t)nn, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (CPLX && cudaMemcpy2DAsync(Vi, (size_t)*ldVi * sizeof(T), dVi, ns, ns, (size_t)nn, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (cudaMemcpyAsync(eS, deS, ns, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (cudaMemcpyAsync(fS, dfS, ns, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return VJ_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return VJ_ERR_CUDA;
  return r;
}

}  // namespace vj

using namespace vj;

extern "C" {

vj_fint dvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double G[], const vj_fnat ldG[1], double V[],
                const vj_fnat ldV[1], double eS[], double fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], double work[], unsigned iwork[])
{
  return svd_host<double, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, work,
                                 iwork);
}
vj_fint zvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double Gr[], const vj_fnat ldGr[1], double Gi[],
                const vj_fnat ldGi[1], double Vr[], const vj_fnat ldVr[1], double Vi[], const vj_fnat ldVi[1],
                double eS[], double fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                double work[], unsigned iwork[])
{
  return svd_host<double, true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, work, iwork);
}
vj_fint svjsvd_(const vj_fnat m[1], const vj_fnat n[1], float G[], const vj_fnat ldG[1], float V[],
                const vj_fnat ldV[1], float eS[], float fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], float work[], unsigned iwork[])
{
  return svd_host<float, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, work,
                                iwork);
}
vj_fint cvjsvd_(const vj_fnat m[1], const vj_fnat n[1], float Gr[], const vj_fnat ldGr[1], float Gi[],
                const vj_fnat ldGi[1], float Vr[], const vj_fnat ldVr[1], float Vi[], const vj_fnat ldVi[1],
                float eS[], float fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                float work[], unsigned iwork[])
{
  return svd_host<float, true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, work, iwork);
}

vj_fint vj_dvjsvd_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS, double *fS,
                      const unsigned *js, unsigned stp, unsigned swp, int preset, void *stream)
{
  return svd_dev<double, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, preset,
                                (cudaStream_t)stream);
}
vj_fint vj_zvjsvd_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                      vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                      unsigned stp, unsigned swp, int preset, void *stream)
{
  return svd_dev<double, true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, preset,
                               (cudaStream_t)stream);
}
vj_fint vj_svjsvd_dev(vj_fnat m, vj_fnat n, float *G, vj_fnat ldG, float *V, vj_fnat ldV, float *eS, float *fS,
                      const unsigned *js, unsigned stp, unsigned swp, int preset, void *stream)
{
  return svd_dev<float, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, stp, swp, preset,
                               (cudaStream_t)stream);
}
vj_fint vj_cvjsvd_dev(vj_fnat m, vj_fnat n, float *Gr, vj_fnat ldGr, float *Gi, vj_fnat ldGi, float *Vr,
                      vj_fnat ldVr, float *Vi, vj_fnat ldVi, float *eS, float *fS, const unsigned *js,
                      unsigned stp, unsigned swp, int preset, void *stream)
{
  return svd_dev<float, true>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, preset,
                              (cudaStream_t)stream);
}

}  // extern "C"

// ---------------- allocation-free FP64 SVD ----------------
// Callers that cannot allocate device memory at run time (code running inside a stream
// being captured into a CUDA graph, or an application that owns every byte of the GPU
// through its own pool and forbids library allocations) can still run the SVD through
// vj_dvjsvd_dev_noalloc. It needs no table and no scratch from the caller: its scratch --
// the control block of the call, the max |a_ij| cell and the pivot table it generates on
// the GPU -- lives in the file-scope device array below, 1 MiB + 512 bytes that every GPU
// loading this library holds until the process exits. The table limits it to n <= 512
// columns (stp * n <= 262144 entries); larger n is rejected with VJ_ERR_ARG.
namespace vj {

constexpr size_t NOALLOC_CTL = 512;
constexpr size_t NOALLOC_JS = 262144;  // unsigned entries of the pivot table
static_assert(sizeof(SvdGlobal) + 64 + 8 <= NOALLOC_CTL, "control block does not fit");
static __device__ __align__(256) unsigned char vj_noalloc_scratch[NOALLOC_CTL + NOALLOC_JS * sizeof(unsigned)];

// device address of the scratch array, looked up once per device with that device current
static unsigned char *noalloc_scratch()
{
  static std::mutex mu;
  static unsigned char *addr[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, vj_noalloc_scratch) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    addr[dev] = static_cast<unsigned char *>(p);
  }
  return addr[dev];
}

}  // namespace vj

extern "C" vj_fint vj_dvjsvd_dev_noalloc(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV,
                                         double *eS, double *fS, long strategy, unsigned swp, int preset,
                                         void *stream)
{
  using namespace vj;
  if (strategy != 2l && strategy != 4l)
    return VJ_ERR_ARG;
  const unsigned long long stp = (strategy == 2l) ? (n ? n - 1ull : 0ull) : n;
  if (n > 512ull || stp * n > NOALLOC_JS)
    return VJ_ERR_ARG;
  if (!host::gpu_ready())
    return VJ_ERR_NO_GPU;
  unsigned char *sc = noalloc_scratch();
  if (!sc)
    return VJ_ERR_CUDA;
  unsigned *js = reinterpret_cast<unsigned *>(sc + NOALLOC_CTL);
  // (odd or tiny n: no table; the SVD's own argument checks report it)
  if (n >= 2 && !(n & 1ull)) {
    const vj_fint r = vj_pjs_dev(strategy, (unsigned)n, js, stream);
    if (r < 0)
      return r;
  }
  return svd_dev<double, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, (unsigned)stp, swp,
                                preset, (cudaStream_t)stream, sc);
}
