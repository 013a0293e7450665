/* TEST INFRASTRUCTURE ONLY -- links into oracle/_ref/libvjref.so, the VecJac reference
 * compiled from its own sources.
 *
 * VecJac calls a Fortran BLAS xNRM2 (src/dnorm2.c:12, src/snorm2.c:12, src/znorm2.c:12-13,
 * src/cnorm2.c:12-13; ILP64 ABI under MKL_ILP64) and libm hypot through cr_hypot
 * (src/common.h:26-31, src/znorm2.c:14). This shim provides those symbols and selects,
 * at run time, between
 *   mode 0: the project's portable norm and scaled hypot (oracle/vjo_nrm2.h), which the
 *           GPU library and the C restatement also use -> bit-exact comparisons;
 *   mode 1: OpenBLAS xNRM2 from numpy's bundled scipy-openblas64 (dlopen'ed from the
 *           path given to vjref_set_blas) and libm hypot/hypotf -> the stock reference.
 */
#include <dlfcn.h>
#include <math.h>
#include <stddef.h>

#include "vjo_nrm2.h"

typedef double (*dnrm2_t)(const long long*, const double*, const long long*);
typedef float (*snrm2_t)(const long long*, const float*, const long long*);

static int vjref_mode = 0;
static dnrm2_t blas_dnrm2 = NULL;
static snrm2_t blas_snrm2 = NULL;

int vjref_set_blas(const char *const path)
{
  void *const h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h)
    return -1;
  blas_dnrm2 = (dnrm2_t)dlsym(h, "scipy_dnrm2_64_");
  blas_snrm2 = (snrm2_t)dlsym(h, "scipy_snrm2_64_");
  return ((blas_dnrm2 && blas_snrm2) ? 0 : -2);
}

int vjref_set_mode(const int mode)
{
  if ((mode == 1) && !(blas_dnrm2 && blas_snrm2))
    return -1;
  vjref_mode = mode;
  return 0;
}

double dnrm2_(const long long *n, const double *x, const long long *incx)
{
  if (vjref_mode == 1)
    return blas_dnrm2(n, x, incx);
  return vjo_dnrm2(*n, x);
}

float snrm2_(const long long *n, const float *x, const long long *incx)
{
  if (vjref_mode == 1)
    return blas_snrm2(n, x, incx);
  return vjo_snrm2(*n, x);
}

double vjref_hypot(const double x, const double y)
{
  return ((vjref_mode == 1) ? hypot(x, y) : vjo_dhypot(x, y));
}

float vjref_hypotf(const float x, const float y)
{
  return ((vjref_mode == 1) ? hypotf(x, y) : vjo_shypot(x, y));
}
