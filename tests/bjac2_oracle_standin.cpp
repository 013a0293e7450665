// A stand-in for libvecjac_gb300.so's 2x2 entry points in the CPU tests of the accuracy
// drivers (t?bjac2.exe): ?bjac2_ forwarded to the oracle's restatement, whose results the
// library's equal bit for bit. Test infrastructure only.
#include "vecjac_gb300.h"

extern "C" {
long long vjo_dbjac2_(const long long *, const double *, const double *, const double *, double *, double *,
                      double *, double *, unsigned *);
long long vjo_sbjac2_(const long long *, const float *, const float *, const float *, float *, float *, float *,
                      float *, unsigned *);
long long vjo_zbjac2_(const long long *, const double *, const double *, const double *, const double *, double *,
                      double *, double *, double *, double *, unsigned *);
long long vjo_cbjac2_(const long long *, const float *, const float *, const float *, const float *, float *, float *,
                      float *, float *, float *, unsigned *);

vj_fint dbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21[], double c[],
                double at[], double l1[], double l2[], unsigned p[])
{
  const long long nn = *n;
  return vjo_dbjac2_(&nn, a11, a22, a21, c, at, l1, l2, p);
}

vj_fint sbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21[], float c[], float at[],
                float l1[], float l2[], unsigned p[])
{
  const long long nn = *n;
  return vjo_sbjac2_(&nn, a11, a22, a21, c, at, l1, l2, p);
}

vj_fint zbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21r[],
                const double a21i[], double c[], double cat[], double sat[], double l1[], double l2[], unsigned p[])
{
  const long long nn = *n;
  return vjo_zbjac2_(&nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}

vj_fint cbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21r[], const float a21i[],
                float c[], float cat[], float sat[], float l1[], float l2[], unsigned p[])
{
  const long long nn = *n;
  return vjo_cbjac2_(&nn, a11, a22, a21r, a21i, c, cat, sat, l1, l2, p);
}
}
