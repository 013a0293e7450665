// A stand-in for libvecjac_gb300.so that the command-line drivers are linked against in
// the CPU tests: pjs, the four ?vjsvd_ entry points and the complex split/merge with the
// library's prototypes,
// checking the arguments the drivers pass and writing known patterns, so that a test can
// check every byte the drivers read and write without a GPU. Not an SVD.
//
//   U(i, j) = 2 G(i, j) + j      (complex: re 2 Re + j, im 0.5 - Im)
//   V(i, j) = 1000 i + j         (complex: im -(1000 i + j))
//   eS_j = -inf (j = 0), 0 (j = 1), else a spread of integers; fS_j in [1, 2)
//   padding rows of G and V (i >= m in the leading dimension) are set to NaN
//   returns 7 (real) / 9 (complex), or a negative code naming the first bad argument
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <limits>

#include "vecjac_gb300.h"

namespace {

template <typename T> bool aligned(const T *p) { return ((uintptr_t)p % 64u) == 0u; }

template <typename T>
vj_fint check(vj_fnat m, vj_fnat n, const T *G, vj_fnat ldG, const T *V, vj_fnat ldV, const T *work,
              const unsigned *js, unsigned stp, unsigned swp, const unsigned *iwork, vj_fnat L)
{
  if (m % 4u)
    return -1;  // the tests use m = 36 / 40: a padded leading dimension with m % 4 == 0
  if (ldG < m || ldG % L)
    return -4;
  if (ldV < n || ldV % L)
    return -6;
  if (!aligned(G) || !aligned(V) || !aligned(work))
    return -3;
  if (!js || (stp != n - 1u && stp != n) || swp != 999u)
    return -11;
  if (iwork[0] != 0u)
    return -13;
  return 0;
}

template <typename T> void sigma(vj_fnat n, T *eS, T *fS)
{
  for (vj_fnat j = 0; j < n; ++j) {
    const int range = (sizeof(T) == 8) ? 2000 : 200;
    eS[j] = (j == 0) ? -std::numeric_limits<T>::infinity() : (j == 1) ? (T)0 : (T)((int)((j * 37u) % range) - range / 2);
    fS[j] = (T)1 + (T)((j * 2654435761u) % (1u << 20)) / (T)(1u << 20);
  }
}

template <typename T> void pattern_G(vj_fnat m, vj_fnat n, T *G, vj_fnat ld, T scale, T shift_re, bool by_col)
{
  for (vj_fnat j = 0; j < n; ++j) {
    for (vj_fnat i = 0; i < m; ++i)
      G[j * ld + i] = scale * G[j * ld + i] + (by_col ? (T)j : shift_re);
    for (vj_fnat i = m; i < ld; ++i)
      G[j * ld + i] = std::numeric_limits<T>::quiet_NaN();
  }
}

template <typename T> void pattern_V(vj_fnat n, T *V, vj_fnat ld, T sgn)
{
  for (vj_fnat j = 0; j < n; ++j) {
    for (vj_fnat i = 0; i < n; ++i)
      V[j * ld + i] = sgn * (T)(1000u * i + j);
    for (vj_fnat i = n; i < ld; ++i)
      V[j * ld + i] = std::numeric_limits<T>::quiet_NaN();
  }
}

template <typename T>
vj_fint real_svd(const vj_fnat *m, const vj_fnat *n, T *G, const vj_fnat *ldG, T *V, const vj_fnat *ldV, T *eS,
                 T *fS, const unsigned *js, const unsigned *stp, const unsigned *swp, T *work, unsigned *iwork,
                 vj_fnat L)
{
  const vj_fint r = check(*m, *n, G, *ldG, V, *ldV, work, js, *stp, *swp, iwork, L);
  if (r)
    return r;
  pattern_G(*m, *n, G, *ldG, (T)2, (T)0, true);
  pattern_V(*n, V, *ldV, (T)1);
  sigma(*n, eS, fS);
  return 7;
}

template <typename T>
vj_fint cplx_svd(const vj_fnat *m, const vj_fnat *n, T *Gr, const vj_fnat *ldGr, T *Gi, const vj_fnat *ldGi, T *Vr,
                 const vj_fnat *ldVr, T *Vi, const vj_fnat *ldVi, T *eS, T *fS, const unsigned *js,
                 const unsigned *stp, const unsigned *swp, T *work, unsigned *iwork, vj_fnat L)
{
  vj_fint r = check(*m, *n, Gr, *ldGr, Vr, *ldVr, work, js, *stp, *swp, iwork, L);
  if (!r)
    r = check(*m, *n, Gi, *ldGi, Vi, *ldVi, work, js, *stp, *swp, iwork, L);
  if (r)
    return r;
  pattern_G(*m, *n, Gr, *ldGr, (T)2, (T)0, true);
  pattern_G(*m, *n, Gi, *ldGi, (T)-1, (T)0.5, false);
  pattern_V(*n, Vr, *ldVr, (T)1);
  pattern_V(*n, Vi, *ldVi, (T)-1);
  sigma(*n, eS, fS);
  return 9;
}

// interleaved <-> planes, element by element (the library's zsplit_/zmerge_ semantics)
template <typename T> vj_fint split_host(vj_fnat m, vj_fnat n, const T *A, vj_fnat ld, T *Ar, vj_fnat ldr, T *Ai,
                                         vj_fnat ldi)
{
  for (vj_fnat j = 0; j < n; ++j)
    for (vj_fnat i = 0; i < m; ++i) {
      Ar[j * ldr + i] = A[2 * (j * ld + i)];
      Ai[j * ldi + i] = A[2 * (j * ld + i) + 1];
    }
  return 1;
}

template <typename T> vj_fint merge_host(vj_fnat m, vj_fnat n, const T *Ar, vj_fnat ldr, const T *Ai, vj_fnat ldi,
                                         T *A, vj_fnat ld)
{
  for (vj_fnat j = 0; j < n; ++j)
    for (vj_fnat i = 0; i < m; ++i) {
      A[2 * (j * ld + i)] = Ar[j * ldr + i];
      A[2 * (j * ld + i) + 1] = Ai[j * ldi + i];
    }
  return 1;
}

}  // namespace

extern "C" {

vj_fint zsplit_(const vj_fnat m[1], const vj_fnat n[1], const double A[], const vj_fnat ldA[1], double Ar[],
                const vj_fnat ldAr[1], double Ai[], const vj_fnat ldAi[1])
{
  return split_host<double>(*m, *n, A, *ldA, Ar, *ldAr, Ai, *ldAi);
}

vj_fint zmerge_(const vj_fnat m[1], const vj_fnat n[1], const double Ar[], const vj_fnat ldAr[1], const double Ai[],
                const vj_fnat ldAi[1], double A[], const vj_fnat ldA[1])
{
  return merge_host<double>(*m, *n, Ar, *ldAr, Ai, *ldAi, A, *ldA);
}

vj_fint csplit_(const vj_fnat m[1], const vj_fnat n[1], const float A[], const vj_fnat ldA[1], float Ar[],
                const vj_fnat ldAr[1], float Ai[], const vj_fnat ldAi[1])
{
  return split_host<float>(*m, *n, A, *ldA, Ar, *ldAr, Ai, *ldAi);
}

vj_fint cmerge_(const vj_fnat m[1], const vj_fnat n[1], const float Ar[], const vj_fnat ldAr[1], const float Ai[],
                const vj_fnat ldAi[1], float A[], const vj_fnat ldA[1])
{
  return merge_host<float>(*m, *n, Ar, *ldAr, Ai, *ldAi, A, *ldA);
}

unsigned *pjs(long id, unsigned n, unsigned stp[1])
{
  *stp = 0u;
  if (n <= 1u || (n & 1u) || (id != 2l && id != 4l))
    return nullptr;
  const unsigned st = (id == 2l) ? (n - 1u) : n;
  unsigned *t = (unsigned *)malloc((size_t)st * n * sizeof(unsigned));
  for (unsigned k = 0; t && k < st * n; ++k)
    t[k] = k % n;
  *stp = t ? st : 0u;
  return t;
}

vj_fint dvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double G[], const vj_fnat ldG[1], double V[],
                const vj_fnat ldV[1], double eS[], double fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], double work[], unsigned iwork[])
{
  return real_svd<double>(m, n, G, ldG, V, ldV, eS, fS, js, stp, swp, work, iwork, 8u);
}

vj_fint svjsvd_(const vj_fnat m[1], const vj_fnat n[1], float G[], const vj_fnat ldG[1], float V[],
                const vj_fnat ldV[1], float eS[], float fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], float work[], unsigned iwork[])
{
  return real_svd<float>(m, n, G, ldG, V, ldV, eS, fS, js, stp, swp, work, iwork, 16u);
}

vj_fint zvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double Gr[], const vj_fnat ldGr[1], double Gi[],
                const vj_fnat ldGi[1], double Vr[], const vj_fnat ldVr[1], double Vi[], const vj_fnat ldVi[1],
                double eS[], double fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                double work[], unsigned iwork[])
{
  return cplx_svd<double>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, work, iwork, 8u);
}

vj_fint cvjsvd_(const vj_fnat m[1], const vj_fnat n[1], float Gr[], const vj_fnat ldGr[1], float Gi[],
                const vj_fnat ldGi[1], float Vr[], const vj_fnat ldVr[1], float Vi[], const vj_fnat ldVi[1],
                float eS[], float fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                float work[], unsigned iwork[])
{
  return cplx_svd<float>(m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, work, iwork, 16u);
}

}  // extern "C"
