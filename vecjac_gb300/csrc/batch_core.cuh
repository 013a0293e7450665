// The batched SVD's per-matrix driver (svd_one): one CTA runs the reference's algorithm
// on one matrix (src/dvjsvd.c:78-638) with __syncthreads between the phases; and the
// batch's argument and shared-memory layouts. Kept apart from the kernel and its launcher
// (batch.cu) so that a host harness can run it with an emulated CTA.
#pragma once
#include "pjs.cuh"
#include "svd_core.cuh"

namespace vj {

constexpr int BATCH_MAXN = 512;

template <typename T> struct BatchArgs {
  long long count;
  const long long *m, *n, *offG, *offV, *offS;
  const int *order;
  T *G, *V, *eS, *fS;
  long long *info;
  unsigned *queue;
  int strategy;
  unsigned swp;
};

template <typename T> struct BatchShared {
  PairState<T> ps[BATCH_MAXN / 2];
  unsigned char w1[BATCH_MAXN];
  unsigned long long nmg, nmv, cnt;
  long long err;
  int flag;
};

// max |a_ij| (NaN counts as inf, as VMINPD(|x|, inf) maps it) of an rows x cols block
template <typename T> __device__ T cta_normx(const T *A, long long ld, long long rows, long long cols,
                                             unsigned long long *red)
{
  const unsigned long long inf = absbits(fp<T>::inf());
  unsigned long long mx = 0ull;
  for (long long j = 0; j < cols; ++j)
    for (long long i = threadIdx.x; i < rows; i += blockDim.x) {
      unsigned long long b = absbits(A[j * ld + i]);
      b = (b > inf) ? inf : b;
      mx = (b > mx) ? b : mx;
    }
  mx = warp_max_u64(mx);
  if ((threadIdx.x & 31) == 0)
    atomicMax(red, mx);
  __syncthreads();
  const T r = bitst<T>(*red);
  __syncthreads();
  return r;
}

template <typename T> __device__ void cta_scale(T *A, long long ld, long long rows, long long cols, int e)
{
  if (!e)
    return;
  for (long long j = 0; j < cols; ++j)
    for (long long i = threadIdx.x; i < rows; i += blockDim.x)
      A[j * ld + i] = scale2(A[j * ld + i], e);
  __syncthreads();
}

__device__ __forceinline__ void step_pair(int strategy, unsigned n, unsigned st, unsigned k, unsigned &p,
                                          unsigned &q)
{
  if (strategy == 2)
    pair_rr(n, st, k, p, q);
  else
    pair_mod(n, st, k, p, q);
}

// the whole SVD of one matrix by this CTA; returns the sweep count or an error code
template <typename T> __device__ long long svd_one(const BatchArgs<T> &a, BatchShared<T> &sh, long long m,
                                                   long long n, T *G, T *V, T *eS, T *fS)
{
  using F = fp<T>;
  constexpr int L = svdc<T>::LANES;
  constexpr int PW = 32 / L;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const long long n_2 = n >> 1;
  if (!n)
    return 0;
  if (m < n || (m % L))
    return -1;
  if ((n & 1) || (n_2 % L) || n > BATCH_MAXN)
    return -2;
  const long long E_MG = -80, E_DOT = -320, E_APPG = -580, E_APPV = -588;
  if (tid == 0)
    sh.nmg = 0ull;
  __syncthreads();
  T MG = cta_normx(G, m, m, n, &sh.nmg);
  if (!(MG <= svdc<T>::RMAX))
    return E_MG;
  // V := I, eS = -inf, fS = 1
  for (long long j = 0; j < n; ++j)
    for (long long i = tid; i < n; i += blockDim.x)
      V[j * n + i] = (i == j) ? (T)1 : (T)0;
  for (long long j = tid; j < n; j += blockDim.x) {
    eS[j] = vneg(F::inf());
    fS[j] = (T)1;
  }
  __syncthreads();
  if (MG == (T)0)
    return 0;
  // global prescale (src/dvjsvd.c:120-137)
  const int ROT = svdc<T>::ROT_R;
  const T M_m = F::div(svdc<T>::RMAX, (T)((unsigned long long)m << 1u));
  const int NRM = ilogb_(M_m);
  int eM = ilogb_(MG);
  int sN = NRM - eM - 1;
  if (sN) {
    cta_scale(G, m, m, n, sN);
    MG = scale2(MG, sN);
  }
  int sT = sN, sV = 0;
  T MV = (T)1;
  const T tol = F::sqrt_((T)m) * scale2(svdc<T>::EPS, -1);
  const T gst = scale2(tol, (int)svdc<T>::MAX_FIN_EXP);
  for (long long c = tid; c < n; c += blockDim.x)
    sh.w1[c] = a.swp ? 1 : 0;
  __syncthreads();
  const unsigned stp = (a.strategy == 2) ? (unsigned)(n - 1) : (unsigned)n;
  unsigned sw = 0;
  while (sw < a.swp) {
    unsigned long long swt = 0ull;
    for (unsigned st = 0; st < stp; ++st) {
      // ---- rescaling of G and V (src/dvjsvd.c:199-233) ----
      eM = ilogb_(MG);
      int sR = ROT - eM;
      sN = NRM - eM - 1;
      if (sR < 0) {
        cta_scale(G, m, m, n, sN);
        MG = scale2(MG, sN);
        sT += sN;
        for (long long c = tid; c < n; c += blockDim.x)
          sh.w1[c] = 1;
        __syncthreads();
      }
      eM = ilogb_(MV);
      sR = ROT - eM;
      sN = sR;
      if (sR < 0) {
        cta_scale(V, n, n, n, sN);
        MV = scale2(MV, sR);
        sV += sR;
      }
      // ---- norms of the changed columns, overflow-aware (src/dvjsvd.c:236-296) ----
      for (int tries = 0;; ++tries) {
        if (tid == 0)
          sh.flag = 0;
        __syncthreads();
        for (long long c = warp; c < n; c += nw)
          if (sh.w1[c]) {
            const T d = warp_nrm2(G + c * m, m);
            if (lane == 0) {
              T e, f;
              ef_split(d, e, f);
              eS[c] = e;
              fS[c] = f;
              if (!(d <= svdc<T>::RMAX))
                sh.flag = 1;
            }
          }
        __syncthreads();
        if (!sh.flag)
          break;
        if (tries >= 3)
          return (long long)VJ_ERR_ARG;
        cta_scale(G, m, m, n, sN);
        MG = scale2(MG, sN);
        sT += sN;
        for (long long c = tid; c < n; c += blockDim.x)
          sh.w1[c] = 1;
        __syncthreads();
      }
      // ---- all scaled dot products and the classification (src/dvjsvd.c:297-459) ----
      if (tid == 0) {
        sh.err = 0;
        sh.cnt = 0ull;
        sh.nmg = 0ull;
        sh.nmv = 0ull;
      }
      __syncthreads();
      for (long long base = (long long)warp * PW; base < n_2; base += (long long)nw * PW) {
        const int j = lane / L;
        const long long k = base + j;
        const bool act = (k < n_2);
        unsigned p = 0, q = 0;
        step_pair(a.strategy, (unsigned)n, st, (unsigned)(act ? k : base), p, q);
        const T ep = eS[p], fp_ = fS[p], eq = eS[q], fq = fS[q];
        T zr = 0, zi = 0;
        const bool live = act && (eq >= -svdc<T>::RMAX) && (ep >= -svdc<T>::RMAX);
        pair_dot<T, false>(m, G + (long long)q * m, nullptr, G + (long long)p * m, nullptr, eq, ep, fq, fp_, live,
                           zr, zi);
        if (act && (lane % L) == 0) {
          PairState<T> &s = sh.ps[k];
          s.ep = ep; s.fp = fp_; s.eq = eq; s.fq = fq;
          if (!live)
            zr = 0;
          s.a21r = zr;
          s.a21i = 0;
          s.skip = 0;
          if (!visfinite(zr)) {
            atomicMin(&sh.err, E_DOT);
            s.skip = 1;
            s.code = 1;
          }
          else if (pair_classify<T, false>(ep, fp_, eq, fq, zr, (T)0, tol, gst, s))
            atomicAdd(&sh.cnt, 1ull);
        }
      }
      __syncthreads();
      if (sh.err)
        return sh.err;
      swt += sh.cnt;
      // ---- all transformations (src/dvjsvd.c:460-574), one pair per warp at a time ----
      unsigned long long mG = 0ull, mV = 0ull;
      for (long long k = warp; k < n_2; k += nw) {
        unsigned p, q;
        step_pair(a.strategy, (unsigned)n, st, (unsigned)k, p, q);
        const PairState<T> &s = sh.ps[k];
        if (s.code == -1 && lane == 0) {
          eS[p] = s.eq; eS[q] = s.ep;
          fS[p] = s.fq; fS[q] = s.fp;
        }
        T *Gp = G + (long long)p * m, *Gq = G + (long long)q * m;
        pair_apply<T, false, false>(s, m, n, Gp, Gq, nullptr, nullptr, V + (long long)p * n, V + (long long)q * n,
                                    nullptr, nullptr, Gp, Gq, nullptr, nullptr, eS + p, eS + q, fS + p, fS + q,
                                    lane, 32, mG, mV);
        if (lane == 0) {
          const int c = s.code;
          sh.w1[p] = (c == 2 || c == -2) ? 1 : 0;
          sh.w1[q] = (c == 2 || c == -2 || c == 3 || c == -3) ? 1 : 0;
        }
      }
      mG = warp_max_u64(mG);
      if (lane == 0 && mG)
        atomicMax(&sh.nmg, mG);
      __syncthreads();
      const T nMG = bitst<T>(sh.nmg);
      if (!visfinite(nMG))
        return E_APPG;
      MG = fmax(MG, nMG);
      (void)mV;
      (void)E_APPV;
    }
    if (!swt)
      break;
    ++sw;
  }
  if (sw < a.swp) {
    // U = G diag(1/f) 2^-e and eS -= sT (src/dvjsvd.c:604-631); V is not rescaled (sV == 0)
    for (long long j = 0; j < n; ++j) {
      const T f = fS[j], sc = vneg(eS[j]);
      for (long long i = tid; i < m; i += blockDim.x)
        G[j * m + i] = scalef(F::div(G[j * m + i], f), sc);
    }
    __syncthreads();
    for (long long j = tid; j < n; j += blockDim.x)
      eS[j] = eS[j] - (T)sT;
    if (sV)
      cta_scale(V, n, n, n, -sV);
  }
  __syncthreads();
  return (long long)sw;
}

}  // namespace vj
