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

#include "svd_core.cuh"

namespace vj {

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
  pdl_enter();
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
  // ---- 2. scaled dot products ----
  // FP32: pair j on lanes [j L, (j+1) L) of warp 0. FP64: one warp per accumulator chain
  // (warp c runs chain c of the CTA's four pairs, pair j on lanes [8j, 8j+8)), so that the
  // FP64 work of the step is spread over two (real) or four (complex) of the SM's
  // sub-partitions; the chains meet in shared memory.
  int cj = -1;  // the pair this thread classifies
  T zr = 0, zi = 0, ep = 0, fp_ = 0, eq = 0, fq = 0;
  bool live = false;
  if constexpr (sizeof(T) == 8) {
    constexpr int NCH = CPLX ? 4 : 2;
    constexpr int PPW = 4;  // pairs per chain warp
    __shared__ T dsum[ppc<T>::P][NCH][2];
    if (warp < NCH * (ppc<T>::P / PPW)) {
      const int jw = lane >> 3, l8 = lane & 7;
      const int j = (warp / NCH) * PPW + jw;
      const bool act = (jw < PPW) && (j < np);
      const int jj = act ? j : 0;
      const long long p = colp(jj), q = colq(jj);
      const T ep_ = a.eS[p], eq_ = a.eS[q];
      const bool lv = act && (eq_ >= -svdc<T>::RMAX) && (ep_ >= -svdc<T>::RMAX);
      const T *xr = rcol(jj, 1), *xi = CPLX ? rcol(jj, 3) : nullptr, *yr = rcol(jj, 0),
              *yi = CPLX ? rcol(jj, 2) : nullptr;
      T S = 0, Tt = 0;
      const int c = warp % NCH;
      switch (c) {
        case 0: chain_dot<T, CPLX, 0>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        case 1: chain_dot<T, CPLX, 1>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        case 2: chain_dot<T, CPLX, 2>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        default: chain_dot<T, CPLX, 3>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
      }
      if (act && l8 == 0) {
        dsum[j][c][0] = S;
        dsum[j][c][1] = Tt;
      }
    }
    __syncthreads();
    if (tid < np) {
      cj = tid;
      const long long p = colp(cj), q = colq(cj);
      ep = a.eS[p]; fp_ = a.fS[p]; eq = a.eS[q]; fq = a.fS[q];
      live = (eq >= -svdc<T>::RMAX) && (ep >= -svdc<T>::RMAX);
      // nu = S(s_pd) + (S(t_pd) + (S(s_dn) + S(t_dn))), divided by fx fy (x = G_q)
      const T de = fq * fp_;
      zr = F::div(dsum[cj][0][0] + (dsum[cj][0][1] + (dsum[cj][1][0] + dsum[cj][1][1])), de);
      if (CPLX)
        zi = F::div(dsum[cj][NCH - 2][0] + (dsum[cj][NCH - 2][1] + (dsum[cj][NCH - 1][0] + dsum[cj][NCH - 1][1])), de);
    }
  }
  else if (warp == 0) {
    const int j = lane / L;
    const bool act = (j < np);
    const int jj = act ? j : 0;
    const long long p = colp(jj), q = colq(jj);
    const T ep_ = a.eS[p], fp0 = a.fS[p], eq_ = a.eS[q], fq0 = a.fS[q];
    const bool lv = act && (eq_ >= -svdc<T>::RMAX) && (ep_ >= -svdc<T>::RMAX);
    T zr_ = 0, zi_ = 0;
    pair_dot<T, CPLX>(a.m, rcol(jj, 1), CPLX ? rcol(jj, 3) : nullptr, rcol(jj, 0), CPLX ? rcol(jj, 2) : nullptr, eq_,
                      ep_, fq0, fp0, lv, zr_, zi_);
    if (act && (lane % L) == 0) {
      cj = j;
      ep = ep_; fp_ = fp0; eq = eq_; fq = fq0;
      live = lv;
      zr = zr_;
      zi = zi_;
    }
  }
  tphase(2);
  if (cj >= 0) {
    const int j = cj;
    const long long p = colp(j), q = colq(j);
    {
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
        if (pair_classify<T, CPLX>(ep, fp_, eq, fq, zr, zi, a.tol, a.gst, s))
          atomicAdd(&g->swt, 1ull);
        if (s.code == -1) {
          a.eS[p] = eq; a.eS[q] = ep;
          a.fS[p] = fq; a.fS[q] = fp_;
        }
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
    const long long p = colp(j), q = colq(j);
    T *Gip = CPLX ? (a.Gi + p * a.ldGi) : nullptr, *Giq = CPLX ? (a.Gi + q * a.ldGi) : nullptr;
    T *Vip = CPLX ? (a.Vi + p * a.ldVi) : nullptr, *Viq = CPLX ? (a.Vi + q * a.ldVi) : nullptr;
    pair_apply<T, CPLX, TRACKV>(ps[j], a.m, a.n, a.G + p * a.ldG, a.G + q * a.ldG, Gip, Giq, a.V + p * a.ldV,
                                a.V + q * a.ldV, Vip, Viq, rcol(j, 0), rcol(j, 1), CPLX ? rcol(j, 2) : nullptr,
                                CPLX ? rcol(j, 3) : nullptr, a.eS + p, a.eS + q, a.fS + p, a.fS + q, ltid, TPP, mG,
                                mV);
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

// The cheap first pass of that check: one warp per pair of the sweep computes the pair's
// cosine |x^H y| / (|x| |y|) (x = column q scaled by 2^-e_q, y = column p; the norms are the
// sweep's own, f 2^e) with plain FP64 products, each lane summing chunks of 4 elements by
// FMAs and the chunk sums with 2Sum compensation, the lanes by a halving tree. Its rounding
// error is below 16 u |x| |y| (u = 2^-53; chunk sums: gamma_8, compensated sum: u + O(u^2),
// tree: gamma_5), so a pair whose computed cosine is at most (0.9 tol - 16 u) cannot reach
// the reference's test tol <= |z| (its compensated dot is within a few u of the exact
// value; its norms are within ~100 u of the true ones): such a pair is certified without
// the reference's arithmetic. A pair that the step would swap (not transformed, and its p
// column the shorter one) sets *flag; a pair not certified (or whose scaling would leave the
// normal range) goes to list (up to cap entries; *nlist counts them all), for k_confirm
// to decide exactly. The first step's rescaling decision is checked as in k_confirm. About
// 9 FP64 operations per complex element instead of the 76 of the reference's four
// compensated chains.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_certify(SvdArgs<double> a, unsigned stp, unsigned *flag, unsigned *list,
                                                 unsigned cap, unsigned *nlist)
{
  using T = double;
  const int lane = threadIdx.x & 31;
  const long long n_2 = a.n >> 1;
  const long long total = (long long)stp * n_2;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const double u = 1.1102230246251565e-16;
  const double lim = 0.9 * (double)a.tol - 16.0 * u;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const Decision<T> d = decide(a, a.g->ctl[0]);
    if (d.gres || d.vres || d.ovf)
      atomicOr(flag, 1u);
  }
  for (long long pi = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); pi < total; pi += nw) {
    const long long st = pi / n_2, j = pi - st * n_2;
    const long long p = (long long)a.js[(size_t)st * (size_t)a.n + 2 * j],
                    q = (long long)a.js[(size_t)st * (size_t)a.n + 2 * j + 1];
    const T ep = a.eS[p], fp_ = a.fS[p], eq = a.eS[q], fq = a.fS[q];
    const bool live = (eq >= -svdc<T>::RMAX) && (ep >= -svdc<T>::RMAX);
    if (!live) {
      // z = 0: not transformed; swapped when p is the shorter column
      if (lane == 0 && efcmp(ep, fp_, eq, fq) < 0)
        atomicOr(flag, 1u);
      continue;
    }
    // 2^-e_q as a normal double, and |y| = f_p 2^e_p as a finite double, or no certificate
    const bool ok = (eq >= -1021.0) && (eq <= 1021.0) && (ep >= -1021.0) && (ep <= 1021.0);
    bool cert = false;
    if (ok) {
      const double sx = ldexp(1.0, -(int)eq);
      const T *xr = a.G + q * a.ldG, *yr = a.G + p * a.ldG;
      const T *xi = CPLX ? (a.Gi + q * a.ldGi) : nullptr, *yi = CPLX ? (a.Gi + p * a.ldGi) : nullptr;
      double Sr = 0, Cr = 0, Si = 0, Ci = 0;
      for (long long c0 = lane; c0 < a.m; c0 += 32 * 4) {
        double cr = 0, ci = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const long long i = c0 + 32LL * k;
          if (i < a.m) {
            const double x = xr[i] * sx, y = yr[i];
            cr = fma(x, y, cr);
            if (CPLX) {
              const double x2 = xi[i] * sx, y2 = yi[i];
              cr = fma(x2, y2, cr);
              ci = fma(x, y2, ci);
              ci = fma(-x2, y, ci);
            }
          }
        }
        double s_, t_;
        two_sum(Sr, cr, s_, t_);
        Sr = s_;
        Cr += t_;
        if (CPLX) {
          two_sum(Si, ci, s_, t_);
          Si = s_;
          Ci += t_;
        }
      }
      double dr = Sr + Cr, di = Si + Ci;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        dr += __shfl_xor_sync(0xffffffffu, dr, o);
        if (CPLX)
          di += __shfl_xor_sync(0xffffffffu, di, o);
      }
      const double ny = ldexp(fp_, (int)ep);
      // (hypot: G is scaled up to near the overflow threshold, so |D| squared overflows)
      const double ad = CPLX ? hypot(dr, di) : fabs(dr);
      cert = (ad <= lim * fq * ny);
    }
    if (lane == 0) {
      if (efcmp(ep, fp_, eq, fq) < 0)
        atomicOr(flag, 1u);  // swapped if not transformed, transformed otherwise: not a no-op
      else if (!cert) {
        const unsigned k = atomicAdd(nlist, 1u);
        if (k < cap)
          list[k] = (unsigned)pi;
      }
    }
  }
}

// Every pair of one sweep checked at once (FP64), for a call whose columns are expected to
// be orthogonal already: when no pair of the sweep would be transformed or swapped and the
// first step takes no rescaling decision, the sweep changes nothing, every later step sees
// the data of the first, and the sweep's own launches are bit-for-bit a no-op. This kernel
// computes, for every pair (p, q) of the table in the table's orientation, the step's
// scaled compensated dot product exactly as k_step does (the same chain_dot calls, the same
// combination of the chains, the norms from the start of the sweep) and the step's
// classification, and sets *flag when any pair is not of class 1 (in order and orthogonal)
// or its dot product is not finite, or the first step would rescale. A persistent grid walks
// the sweep's pairs in groups of four per chain warp (warp c of a group: chain c), so that
// the FP64 work of the whole sweep spreads over every SM instead of one step at a time;
// CTAs stop early once the flag is set.
template <bool CPLX>
__global__ void __launch_bounds__(256, 2) k_confirm(SvdArgs<double> a, unsigned stp, const unsigned *list,
                                                    unsigned nlist, unsigned *flag)
{
  using T = double;
  using F = fp<T>;
  constexpr int NCH = CPLX ? 4 : 2;  // chains per pair: one warp each
  constexpr int PPW = 4;             // pairs per chain warp, 8 lanes each
  constexpr int NG = 8 / NCH;        // groups of PPW pairs per CTA of 8 warps
  constexpr int PPC = NG * PPW;      // pairs per CTA and iteration
  __shared__ T dsum[PPC][NCH][2];
  __shared__ int stop;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long n_2 = a.n >> 1;
  const long long total = list ? (long long)nlist : (long long)stp * n_2;
  if (blockIdx.x == 0 && tid == 0) {
    const Decision<T> d = decide(a, a.g->ctl[0]);
    if (d.gres || d.vres || d.ovf)
      atomicOr(flag, 1u);
  }
  // pair pi of the sweep (of the list, when given): the table's p (side 0) or q (side 1)
  auto col = [&](long long pi, int side) -> long long {
    if (list)
      pi = (long long)list[pi];
    const long long st = pi / n_2, j = pi - st * n_2;
    return (long long)a.js[(size_t)st * (size_t)a.n + 2 * j + side];
  };
  for (long long base = (long long)blockIdx.x * PPC; base < total; base += (long long)gridDim.x * PPC) {
    __syncthreads();  // the previous iteration's dsum and stop are consumed
    if (tid == 0)
      stop = (int)*(volatile unsigned *)flag;
    __syncthreads();
    if (stop)
      break;
    {
      const int grp = warp / NCH, c = warp % NCH, jw = lane >> 3, l8 = lane & 7;
      const int jc = grp * PPW + jw;  // pair within the CTA's iteration
      const long long pi = base + jc;
      const bool act = (pi < total);
      const long long p = act ? col(pi, 0) : 0, q = act ? col(pi, 1) : 0;
      const T ep_ = a.eS[p], eq_ = a.eS[q];
      const bool lv = act && (eq_ >= -svdc<T>::RMAX) && (ep_ >= -svdc<T>::RMAX);
      // x = column q, y = column p (k_step's operand order)
      const T *xr = a.G + q * a.ldG, *yr = a.G + p * a.ldG;
      const T *xi = CPLX ? (a.Gi + q * a.ldGi) : nullptr, *yi = CPLX ? (a.Gi + p * a.ldGi) : nullptr;
      T S = 0, Tt = 0;
      switch (c) {
        case 0: chain_dot<T, CPLX, 0>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        case 1: chain_dot<T, CPLX, 1>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        case 2: chain_dot<T, CPLX, 2>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
        default: chain_dot<T, CPLX, 3>(a.m, xr, xi, yr, yi, eq_, ep_, lv, l8, S, Tt); break;
      }
      if (act && l8 == 0) {
        dsum[jc][c][0] = S;
        dsum[jc][c][1] = Tt;
      }
    }
    __syncthreads();
    if (tid < PPC && base + tid < total) {
      const long long pi = base + tid;
      const long long p = col(pi, 0), q = col(pi, 1);
      const T ep = a.eS[p], fp_ = a.fS[p], eq = a.eS[q], fq = a.fS[q];
      const bool live = (eq >= -svdc<T>::RMAX) && (ep >= -svdc<T>::RMAX);
      const T de = fq * fp_;
      T zr = F::div(dsum[tid][0][0] + (dsum[tid][0][1] + (dsum[tid][1][0] + dsum[tid][1][1])), de), zi = 0;
      if (CPLX)
        zi = F::div(dsum[tid][NCH - 2][0] + (dsum[tid][NCH - 2][1] + (dsum[tid][NCH - 1][0] + dsum[tid][NCH - 1][1])),
                    de);
      if (!live) {
        zr = 0;
        zi = 0;
      }
      bool clear = visfinite(zr) && (!CPLX || visfinite(zi));
      if (clear) {
        PairState<T> s;
        clear = !pair_classify<T, CPLX>(ep, fp_, eq, fq, zr, zi, a.tol, a.gst, s) && s.code == 1;
      }
      if (!clear)
        atomicOr(flag, 1u);
    }
  }
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
  const host::NearestRounding rn;
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
  // preset == 2 (the mixed path's finishing call, whose columns are orthogonal already):
  // every pair of the first sweep is checked at once; when that sweep would change
  // nothing, its launches are skipped and the call ends as the reference's would after it
  // (sweep count 0, the final scaling with the untouched control block)
  bool confirmed = false;
  if constexpr (sizeof(T) == 8) {
    if (preset == 2 && swp && stp) {
      // flag and list count in dmx; the list in the caller-owned V scratch is not
      // available, so it lives in its own cached device buffer (cap entries)
      unsigned *flag = reinterpret_cast<unsigned *>(dmx), *nl = flag + 1;
      static host::Staging lsts[host::MAX_DEVICES];
      host::Staging &lst = lsts[host::device_slot()];
      const unsigned cap = 1u << 20;
      if (!lst.reserve((size_t)cap * sizeof(unsigned)))
        return VJ_ERR_NOMEM;
      unsigned *list = reinterpret_cast<unsigned *>(lst.ptr);
      if (cudaMemsetAsync(dmx, 0, 8, s) != cudaSuccess)
        return VJ_ERR_CUDA;
      k_certify<CPLX><<<(unsigned)(host::sm_count() * 4), blk, 0, s>>>(a, stp, flag, list, cap, nl);
      if (cudaGetLastError() != cudaSuccess)
        return VJ_ERR_CUDA;
      unsigned hf[2] = {1u, 0u};
      if (cudaMemcpyAsync(hf, flag, sizeof(hf), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess)
        return VJ_ERR_CUDA;
      if (hf[0] == 0u && hf[1] != 0u) {
        // the pairs without a certificate, decided with the reference's arithmetic (all of
        // the sweep's pairs when the list overflowed)
        const bool all = (hf[1] > cap);
        k_confirm<CPLX><<<(unsigned)(host::sm_count() * 2), blk, 0, s>>>(a, stp, all ? nullptr : list,
                                                                        all ? 0u : hf[1], flag);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(hf, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
          return VJ_ERR_CUDA;
      }
      if (a.trace)
        std::fprintf(stderr, "finishing sweep check: %u pairs without a certificate, %s\n", hf[1],
                     hf[0] ? "sweep needed" : "sweep skipped");
      confirmed = (hf[0] == 0u);
      if (confirmed)
        host::trace_sweep(0u, 0ull);
    }
  }
  while (!confirmed && sw < swp) {
    if (cudaMemsetAsync(&dg->swt, 0, 8, s) != cudaSuccess)
      return VJ_ERR_CUDA;
    for (unsigned st = 0; st < stp; ++st, ++gstep) {
      const int last = ((sw + 1u == swp) && (st + 1u == stp)) ? 1 : 0;
      const int g3 = (int)(gstep % 3);
      const int ist = (int)st;
      cudaError_t e;
      if (stage)
        e = preset ? host::launch_pdl(k_step<T, CPLX, true, true>, dim3(grid), blk, smem, s, a, ist, g3, last)
                   : host::launch_pdl(k_step<T, CPLX, false, true>, dim3(grid), blk, smem, s, a, ist, g3, last);
      else
        e = preset ? host::launch_pdl(k_step<T, CPLX, true, false>, dim3(grid), blk, 0, s, a, ist, g3, last)
                   : host::launch_pdl(k_step<T, CPLX, false, false>, dim3(grid), blk, 0, s, a, ist, g3, last);
      if (e != cudaSuccess)
        return VJ_ERR_CUDA;
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
  // the reference's argument checks, in its order (src/dvjsvd.c:43-68, src/zvjsvd.c:43-80);
  // first its floating-point environment check (IS_NOT_VFPENV, src/vec.h): the rounding
  // control of the caller's thread must be round-to-nearest (the MXCSR flush-to-zero and
  // denormals-are-zero bits it also checks have no portable reading and do not change
  // these results)
  if (fegetround() != FE_TONEAREST)
    return CPLX ? -18 : -14;
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
  std::lock_guard<std::recursive_mutex> lk(host::host_call_lock());  // the device's staging buffers
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

namespace vj {
// device-pointer SVD for other translation units (the mixed-precision driver)
template <typename T, bool CPLX>
vj_fint svd_dev_entry(vj_fnat m, vj_fnat n, T *G, vj_fnat ldG, T *Gi, vj_fnat ldGi, T *V, vj_fnat ldV, T *Vi,
                      vj_fnat ldVi, T *eS, T *fS, const unsigned *js, unsigned stp, unsigned swp, int preset,
                      cudaStream_t s)
{
  return svd_dev<T, CPLX>(m, n, G, ldG, Gi, ldGi, V, ldV, Vi, ldVi, eS, fS, js, stp, swp, preset, s);
}
template vj_fint svd_dev_entry<double, false>(vj_fnat, vj_fnat, double *, vj_fnat, double *, vj_fnat, double *,
                                              vj_fnat, double *, vj_fnat, double *, double *, const unsigned *,
                                              unsigned, unsigned, int, cudaStream_t);
template vj_fint svd_dev_entry<double, true>(vj_fnat, vj_fnat, double *, vj_fnat, double *, vj_fnat, double *,
                                             vj_fnat, double *, vj_fnat, double *, double *, const unsigned *,
                                             unsigned, unsigned, int, cudaStream_t);
template vj_fint svd_dev_entry<float, false>(vj_fnat, vj_fnat, float *, vj_fnat, float *, vj_fnat, float *,
                                             vj_fnat, float *, vj_fnat, float *, float *, const unsigned *,
                                             unsigned, unsigned, int, cudaStream_t);
template vj_fint svd_dev_entry<float, true>(vj_fnat, vj_fnat, float *, vj_fnat, float *, vj_fnat, float *,
                                            vj_fnat, float *, vj_fnat, float *, float *, const unsigned *,
                                            unsigned, unsigned, int, cudaStream_t);
}  // namespace vj

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
// Callers that cannot allocate device memory at run time (an application that owns every
// byte of the GPU through its own pool and forbids library allocations, or a latency-bound
// service that must not take the driver's allocator -- cudaMalloc can synchronise the device
// and fail with out-of-memory in the middle of a pipeline) can still run the SVD through
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

// device address of the scratch array, looked up once per device with that device current:
// the first call of vj_dvjsvd_dev_noalloc on a device does it, so that call belongs before
// any stream capture begins
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
  // (preset 2's all-pairs check keeps a list in a library buffer: not in the allocation-free form)
  return svd_dev<double, false>(m, n, G, ldG, nullptr, ldG, V, ldV, nullptr, ldV, eS, fS, js, (unsigned)stp, swp,
                                preset ? 1 : 0, (cudaStream_t)stream, sc);
}
