/* A C11 caller of libvecjac_gb300.so written against include/vecjac_gb300.h the way the
 * reference's drivers call VecJac (src/tdvjsvd.c: every scalar by pointer, caller-owned
 * 64-byte aligned buffers). Without a GPU it checks the argument codes the library returns
 * before touching the device and that a valid call reports VJ_ERR_NO_GPU; it prints
 * "ok <int bits>" or the first failed check. Built with and without -DVJ_LP64. */
#include <fenv.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vecjac_gb300.h"

#define CHECK(expr, want)                                                             \
  do {                                                                                \
    const long long got_ = (long long)(expr);                                         \
    if (got_ != (long long)(want)) {                                                  \
      printf("FAIL %s: %lld != %lld\n", #expr, got_, (long long)(want));              \
      return 1;                                                                       \
    }                                                                                 \
  } while (0)

int main(int argc, char **argv)
{
  const int gpu = (argc > 1) && !strcmp(argv[1], "gpu");
  double *G = (double *)aligned_alloc(64, 64 * 32 * sizeof(double));
  double *V = (double *)aligned_alloc(64, 32 * 32 * sizeof(double));
  double *w = (double *)aligned_alloc(64, 7 * 32 * sizeof(double));
  unsigned *iwork = (unsigned *)aligned_alloc(64, 64);
  unsigned js[32 * 32];
  if (!G || !V || !w || !iwork)
    return 2;
  memset(G, 0, 64 * 32 * sizeof(double));
  memset(js, 0, sizeof(js));
  iwork[0] = 0u;
  vj_fnat m = 64, n = 32, ldG = 64, ldV = 32, bad = 36, odd = 33;
  unsigned stp = 32, swp = 999;
  CHECK(vj_abi_int_bits(), 8 * (int)sizeof(vj_fint));
  CHECK(dvjsvd_(&bad, &n, G, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -1);
  CHECK(dvjsvd_(&m, &odd, G, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -2);
  CHECK(dvjsvd_(&m, &n, G + 1, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -3);
  CHECK(dvjsvd_(&m, &n, G, &bad, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -4);
  CHECK(dvjsvd_(&m, &n, G, &ldG, V + 1, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -5);
  CHECK(dvjsvd_(&m, &n, G, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 65, iwork), -12);
  const vj_fint n2 = -12;
  CHECK(dbjac2_(&n2, w, w, w, w, w, w, w, iwork), -1);
  /* the reference's floating-point environment check comes first: a rounding mode other
   * than to-nearest gives -14 (real) / -18 (complex), and the caller's mode is kept */
  fesetround(FE_UPWARD);
  CHECK(dvjsvd_(&m, &n, G, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -14);
  CHECK(zvjsvd_(&m, &n, G, &ldG, G, &ldG, V, &ldV, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), -18);
  /* the same check heads the 2x2 EVD (-10 real, -12 complex, src/dbjac2.c:84,
   * src/zbjac2.c:111) and the complex split/merge (-9, src/zsplit.c:8) */
  const vj_fint n8 = -8;
  CHECK(dbjac2_(&n8, w, w, w, w, w, w, w, iwork), -10);
  CHECK(zbjac2_(&n8, w, w, w, w, w, w, w, w, w, iwork), -12);
  CHECK(sbjac2i(&n8, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, iwork), -10);
  CHECK(cbjac2i(&n8, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w, (float *)w,
                (float *)w, iwork), -12);
  CHECK(zsplit_(&m, &n, G, &ldG, V, &ldV, V, &ldV), -9);
  CHECK(cmerge_(&m, &n, (float *)V, &ldV, (float *)V, &ldV, (float *)G, &ldG), -9);
  CHECK(fegetround(), FE_UPWARD);
  if (!gpu) {
    /* the device-pointer form computes its host-side values to nearest and restores the
     * caller's mode on return (here it returns at once: no GPU) */
    CHECK(vj_dvjsvd_dev(m, n, G, ldG, V, ldV, w, w + 32, js, stp, swp, 0, NULL), VJ_ERR_NO_GPU);
    CHECK(fegetround(), FE_UPWARD);
  }
  fesetround(FE_TONEAREST);
  /* split/merge argument codes in the reference's order (src/zsplit.c:8-27,
   * src/zmerge.c:8-27): rows in whole vectors, then each leading dimension */
  {
    vj_fnat m6 = 6, ld4 = 4, ld12 = 12, ld32 = 32, ld36 = 36, n1 = 1;
    CHECK(zsplit_(&m6, &n1, G, &ld32, V, &ld32, V, &ld32), -1);
    CHECK(zsplit_(&ld32, &n1, G, &ld4, V, &ld32, V, &ld32), -4);
    CHECK(zsplit_(&ld32, &n1, G, &ld32, V, &ld36, V, &ld32), -6);
    CHECK(zsplit_(&ld32, &n1, G, &ld32, V, &ld32, V, &ld12), -8);
    CHECK(zmerge_(&ld32, &n1, V, &ld36, V, &ld32, G, &ld32), -4);
    CHECK(zmerge_(&ld32, &n1, V, &ld32, V, &ld4, G, &ld32), -6);
    CHECK(zmerge_(&ld32, &n1, V, &ld32, V, &ld32, G, &ld4), -8);
    CHECK(csplit_(&ld12, &n1, (float *)G, &ld32, (float *)V, &ld32, (float *)V, &ld32), -1);
    CHECK(csplit_(&ld32, &n1, (float *)G, &ld36, (float *)V, &ld32, (float *)V, &ld32), -4);
    CHECK(cmerge_(&ld32, &n1, (float *)V, &ld32, (float *)V, &ld36, (float *)G, &ld32), -6);
    if (!gpu)
      CHECK(zsplit_(&ld32, &n1, G, &ld32, V, &ld32, V, &ld32), VJ_ERR_NO_GPU);
  }
  if (!gpu)
    CHECK(dvjsvd_(&m, &n, G, &ldG, V, &ldV, w, w + 32, js, &stp, &swp, w + 64, iwork), VJ_ERR_NO_GPU);
  printf("ok %d\n", vj_abi_int_bits());
  free(iwork);
  free(w);
  free(V);
  free(G);
  return 0;
}
