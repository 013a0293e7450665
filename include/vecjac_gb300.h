/* vecjac_gb300 -- GB300 (sm_103a) one-sided Jacobi SVD and batched 2x2 Hermitian EVD.
 *
 * C ABI of libvecjac_gb300.so. The entry points without a prefix are drop-in
 * replacements for VecJac's C entry points (same names, Fortran-style by-pointer
 * scalars, ILP64 integers as under MKL_ILP64, split real/imaginary planes for complex
 * data, caller-owned buffers, same error codes); they take HOST pointers, copy to the
 * GPU, compute there and copy back, synchronously. The vj_*_dev entry points take
 * DEVICE pointers and a CUDA stream (passed as void*) and are asynchronous.
 *
 * There is no CPU fallback: without a usable GPU every entry point returns
 * VJ_ERR_NO_GPU (or the CUDA error mapped to VJ_ERR_CUDA).
 */
#ifndef VECJAC_GB300_H
#define VECJAC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#ifdef VJ_LP64
typedef int vj_fint;                 /* fint under the reference's ABI=lp64 (src/common.h:184-186) */
typedef unsigned vj_fnat;            /* fnat under ABI=lp64 */
#else
typedef long long vj_fint;           /* fint under MKL_ILP64, the default (src/common.h:180-183) */
typedef unsigned long long vj_fnat;  /* fnat under MKL_ILP64 */
#endif

/* library-specific failures; never produced by the reference */
#define VJ_ERR_NO_GPU   (-100001LL)
#define VJ_ERR_CUDA     (-100002LL)
#define VJ_ERR_NOMEM    (-100003LL)
#define VJ_ERR_ARG      (-100004LL)

/* ---------------- batched 2x2 Hermitian EVD ----------------
 * n < 0: cosines and sines; n > 0: cosines and tangents. For each i < |n|:
 *   [c  -s'] [a11  a21'] [ c  s]  = diag(l1, l2) with s = at (real) or cat + i*sat (complex)
 * p[i/8] (FP64) or p[i/16] (FP32) bit (i%8 or i%16) = (L1 < L2) of the scaled eigenvalues.
 * |n| must be a multiple of 8 (d, z) or 16 (s, c); returns 1 on success (like the
 * reference's OpenMP build), -1 if |n| is not such a multiple, and (host forms, checked
 * first, as the reference's IS_NOT_VFPENV) -10 (d, s) / -12 (z, c) when the calling
 * thread's rounding mode is not round-to-nearest.
 *   replaces dbjac2_  src/dbjac2.h:6,  src/dbjac2.c:81
 *            zbjac2_  src/zbjac2.h:6,  src/zbjac2.c:108
 *            sbjac2_  src/sbjac2.h:6,  src/sbjac2.c:81
 *            cbjac2_  src/cbjac2.h:6,  src/cbjac2.c:108 */
vj_fint dbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21[],
                double c[], double at[], double l1[], double l2[], unsigned p[]);
vj_fint zbjac2_(const vj_fint n[1], const double a11[], const double a22[], const double a21r[], const double a21i[],
                double c[], double cat[], double sat[], double l1[], double l2[], unsigned p[]);
vj_fint sbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21[],
                float c[], float at[], float l1[], float l2[], unsigned p[]);
vj_fint cbjac2_(const vj_fint n[1], const float a11[], const float a22[], const float a21r[], const float a21i[],
                float c[], float cat[], float sat[], float l1[], float l2[], unsigned p[]);

/* The internal masked variants (src/dbjac2.c:178 dbjac2i, src/zbjac2.c:222 zbjac2i,
 * src/sbjac2.c sbjac2i, src/cbjac2.c cbjac2i): only the groups whose low 8 (d, z) or
 * 16 (s, c) bits of p are nonzero are computed; those bits are replaced by the
 * permutation bits and the high bits are kept. n < 0 stores secants in c. */
vj_fint dbjac2i(const vj_fint n[1], const double a11[], const double a22[], const double a21[],
                double c[], double at[], double l1[], double l2[], unsigned p[]);
vj_fint zbjac2i(const vj_fint n[1], const double a11[], const double a22[], const double a21r[], const double a21i[],
                double c[], double cat[], double sat[], double l1[], double l2[], unsigned p[]);
vj_fint sbjac2i(const vj_fint n[1], const float a11[], const float a22[], const float a21[],
                float c[], float at[], float l1[], float l2[], unsigned p[]);
vj_fint cbjac2i(const vj_fint n[1], const float a11[], const float a22[], const float a21r[], const float a21i[],
                float c[], float cat[], float sat[], float l1[], float l2[], unsigned p[]);

/* Device-pointer forms: the same computation on GPU-resident arrays, enqueued on
 * `stream` (a cudaStream_t; NULL = the legacy default stream). `internal` selects the
 * masked i-variant. Return 1, or a negative code. */
vj_fint vj_dbjac2_dev(vj_fint n, int internal, const double *a11, const double *a22, const double *a21,
                      double *c, double *at, double *l1, double *l2, unsigned *p, void *stream);
vj_fint vj_zbjac2_dev(vj_fint n, int internal, const double *a11, const double *a22, const double *a21r,
                      const double *a21i, double *c, double *cat, double *sat, double *l1, double *l2, unsigned *p,
                      void *stream);
vj_fint vj_sbjac2_dev(vj_fint n, int internal, const float *a11, const float *a22, const float *a21,
                      float *c, float *at, float *l1, float *l2, unsigned *p, void *stream);
vj_fint vj_cbjac2_dev(vj_fint n, int internal, const float *a11, const float *a22, const float *a21r,
                      const float *a21i, float *c, float *cat, float *sat, float *l1, float *l2, unsigned *p,
                      void *stream);

/* ---------------- one-sided Jacobi SVD ----------------
 * G (m x n, column-major, leading dimension ldG) is overwritten by U = G V diag(1/sigma)
 * on convergence; V (n x n) accumulates the rotations (V := I first when iwork[0] == 0,
 * otherwise V is a preset matrix that the rotations are applied to). sigma_j =
 * fS[j] * 2^eS[j]. js holds stp rows of n column indices (n/2 pairs per row, p < q);
 * swp caps the number of sweeps. Returns the number of sweeps (== *swp: not converged,
 * G and V left scaled) or a negative error code (the reference's: -1..-6, -12, -13
 * (zero preset V), and -__LINE__ codes of the reference's sources for numerical
 * failures: d/s -80, -92, -320, -580, -588; z/c -92, -104, -345, -347, -630, -638).
 * Preconditions as in the reference: m >= n, m % 8 == 0 (s, c: % 16), n even,
 * (n/2) % 8 == 0 (s, c: % 16), ld >= rows and % 8 (16), 64-byte aligned G, V, work.
 * work: >= 5n (real) / 7n (complex) elements, iwork >= n/8 (d, z) / n/16 (s, c).
 *   replaces dvjsvd_  src/dvjsvd.h:10, src/dvjsvd.c:40
 *            zvjsvd_  src/zvjsvd.h:10, src/zvjsvd.c:40
 *            svjsvd_  src/svjsvd.h:10, src/svjsvd.c:40
 *            cvjsvd_  src/cvjsvd.h:22, src/cvjsvd.c:40 */
vj_fint dvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double G[], const vj_fnat ldG[1], double V[],
                const vj_fnat ldV[1], double eS[], double fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], double work[], unsigned iwork[]);
vj_fint zvjsvd_(const vj_fnat m[1], const vj_fnat n[1], double Gr[], const vj_fnat ldGr[1], double Gi[],
                const vj_fnat ldGi[1], double Vr[], const vj_fnat ldVr[1], double Vi[], const vj_fnat ldVi[1],
                double eS[], double fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                double work[], unsigned iwork[]);
vj_fint svjsvd_(const vj_fnat m[1], const vj_fnat n[1], float G[], const vj_fnat ldG[1], float V[],
                const vj_fnat ldV[1], float eS[], float fS[], const unsigned js[], const unsigned stp[1],
                const unsigned swp[1], float work[], unsigned iwork[]);
vj_fint cvjsvd_(const vj_fnat m[1], const vj_fnat n[1], float Gr[], const vj_fnat ldGr[1], float Gi[],
                const vj_fnat ldGi[1], float Vr[], const vj_fnat ldVr[1], float Vi[], const vj_fnat ldVi[1],
                float eS[], float fS[], const unsigned js[], const unsigned stp[1], const unsigned swp[1],
                float work[], unsigned iwork[]);

/* Device-pointer SVD: all arrays (G, V, eS, fS, js) on the GPU; Gi/Vi NULL for real
 * data. preset != 0 means V holds a preset matrix. preset == 2 (FP64 only) also checks
 * every pair of the first sweep at once before it runs (plain FP64 cosines with a rigorous
 * error bound, and the reference's own arithmetic for the pairs without a certificate) and
 * skips that sweep when it would transform or swap nothing: the results are those of
 * preset == 1 bit for bit, sooner when the columns are orthogonal already. Synchronises
 * `stream` once per sweep (to test convergence). Returns like the host form. */
vj_fint vj_dvjsvd_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS, double *fS,
                      const unsigned *js, unsigned stp, unsigned swp, int preset, void *stream);
vj_fint vj_zvjsvd_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                      vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                      unsigned stp, unsigned swp, int preset, void *stream);
vj_fint vj_svjsvd_dev(vj_fnat m, vj_fnat n, float *G, vj_fnat ldG, float *V, vj_fnat ldV, float *eS, float *fS,
                      const unsigned *js, unsigned stp, unsigned swp, int preset, void *stream);
vj_fint vj_cvjsvd_dev(vj_fnat m, vj_fnat n, float *Gr, vj_fnat ldGr, float *Gi, vj_fnat ldGi, float *Vr,
                      vj_fnat ldVr, float *Vi, vj_fnat ldVi, float *eS, float *fS, const unsigned *js,
                      unsigned stp, unsigned swp, int preset, void *stream);

/* Mixed-precision SVD (FP64 data, result to FP64 accuracy): `stages` rounds (0: 2) of FP32
 * one-sided Jacobi sweeps on the current G rounded to FP32 (block sweeps on the tensor
 * cores where n allows, vj_block_sweep_dev), each followed by an FP64 Cholesky QR of the
 * accumulated rotation W (columns in ascending order of norm) and the FP64 products
 * G := G Q, V := V Q; FP64 sweeps with plain dot products on G and V to half the
 * reference's tolerance; then the FP64 finishing sweeps of dvjsvd_/zvjsvd_ with V preset
 * (the reference's iwork[0] != 0 mode, src/dvjsvd.c:88-96, src/zvjsvd.c:100-110), whose
 * first sweep is checked for every pair at once first and skipped when it would change
 * nothing. Shape rules and return values are dvjsvd_'s/zvjsvd_'s (the finishing phase's
 * sweep count or its error); presweeps (optional, 2 entries) receives the number of FP32
 * sweeps and of plain-dot FP64 sweeps. js/stp is the pivot table of every phase; swp caps
 * each phase (presweep phases at most 60). All arrays on the device. Links cuBLAS and
 * cuSOLVER for the FP64 GEMMs and the Cholesky factorisation. */
vj_fint vj_dvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS,
                            double *fS, const unsigned *js, unsigned stp, unsigned swp, unsigned stages,
                            unsigned *presweeps, void *stream);
vj_fint vj_zvjsvd_mixed_dev(vj_fnat m, vj_fnat n, double *Gr, vj_fnat ldGr, double *Gi, vj_fnat ldGi, double *Vr,
                            vj_fnat ldVr, double *Vi, vj_fnat ldVi, double *eS, double *fS, const unsigned *js,
                            unsigned stp, unsigned swp, unsigned stages, unsigned *presweeps, void *stream);

/* Block one-sided Jacobi in FP32 with split-BF16x3 tensor-core products (tcgen05, FP32
 * accumulation): the FP32 stages of the mixed-precision SVD, and its building blocks. No
 * counterpart in the reference (whose FP32 SVDs rotate column pairs, src/svjsvd.c,
 * src/cvjsvd.c). G (m x n) and W (n x n) are FP32, column-major, split planes for complex
 * data (cplx != 0; Gi, Wi NULL for real data). The columns are cut into blocks of 64 (real)
 * or 32 (complex) columns, so a pair of blocks is 128 real columns X = [G_I G_J] (complex:
 * [Re G_I Re G_J Im G_I Im G_J]); the pairs of block step `step` (0 .. n/b - 2) are those of
 * the round-robin ordering of the n/b blocks (pair k: blocks (step, n/b - 1) for k = 0, else
 * ((step + k) mod (n/b - 1), (step - k) mod (n/b - 1)), lower index first). Requirements:
 * n a multiple of 128 (real) / 64 (complex), m and the leading dimensions multiples of 4,
 * columns 16-byte aligned; otherwise VJ_ERR_ARG. terms: 6 (products as accurate as FP32)
 * or 3 (h h + h m + m h, about 16 bits).
 * vj_block_gram_dev: S (n/b/2 x 128 x 128, row-major per pair) = X^T X for every pair of
 *   the step. Returns the number of pairs. Synchronous.
 * vj_block_apply_dev: X := X R for the rows of G and of W, R (n/b/2 x 128 x 128, pair k's
 *   R[k][i] at R + k 16384 + k + 128 i) the real form of each pair's rotation (complex:
 *   [[Re R, Im R], [-Im R, Re R]]). Returns the number of pairs. Synchronous.
 * vj_block_sweep_dev: one block sweep (every block pair once): per pair the Gram matrix,
 *   `inner` cyclic Jacobi sweeps on its 2b x 2b Hermitian form (rotations where
 *   |h_pq| >= tol sqrt(h_pp h_qq)), columns ordered by descending norms, and the
 *   rotation applied to G and W. Returns the number of rotations (0: converged to tol) and
 *   the largest |h_pq| / sqrt(h_pp h_qq) of a rotated pair in *mu, or a VJ_ERR_* code. */
vj_fint vj_block_gram_dev(int cplx, vj_fnat m, vj_fnat n, const float *Gr, const float *Gi, vj_fnat ldG, int step,
                          int terms, float *S, void *stream);
vj_fint vj_block_apply_dev(int cplx, vj_fnat m, vj_fnat n, float *Gr, float *Gi, vj_fnat ldG, float *Wr, float *Wi,
                           vj_fnat ldW, int step, int terms, const float *R, void *stream);
vj_fint vj_block_sweep_dev(int cplx, vj_fnat m, vj_fnat n, float *Gr, float *Gi, vj_fnat ldG, float *Wr, float *Wi,
                           vj_fnat ldW, float tol, int inner, int terms, float *mu, void *stream);

/* Phase times of the calling thread's last vj_?vjsvd_mixed_dev call, in milliseconds:
 * out[0] FP32 sweeps, out[1] orthonormalisation of W and the GEMMs, out[2] plain-dot FP64 sweeps
 * and the column sort, out[3] the reference's finishing sweeps; out[4] the number of FP32
 * kernel launches; out[5] 1 when the FP32 stages ran as block sweeps on the tensor cores,
 * 0 for column-pair sweeps. */
vj_fint vj_last_mixed_phases(double out[6]);

/* Adjoint of the thin SVD A = U diag(S) V^T (m >= n, V square), batched over `count`
 * matrices of one shape: given the cotangents dS (n), dU (m x k) and dV (n x k) of S and of
 * the first k columns of U and V, writes dA (m x n) = the cotangent of A. All arrays on the
 * device, column-major and packed (matrix b at U + b*m*n, V + b*n*n, S/dS + b*n,
 * dU + b*m*k, dV + b*n*k, dA + b*m*n). gap >= 0 broadens 1/(s_j^2 - s_i^2) to
 * d/(d^2 + (gap*max(s_i,s_j)^2)^2) (0: exact; degenerate pairs contribute 0). The working
 * set of one matrix must fit in 227 KiB of shared memory, else VJ_ERR_ARG.
 * Returns 0 (asynchronous on `stream`) or a VJ_ERR_* code. */
vj_fint vj_ssvd_adjoint_batch_dev(vj_fint count, vj_fnat m, vj_fnat n, vj_fnat k, const float *U, const float *S,
                                  const float *V, const float *dS, const float *dU, const float *dV, float *dA,
                                  float gap, void *stream);
vj_fint vj_dsvd_adjoint_batch_dev(vj_fint count, vj_fnat m, vj_fnat n, vj_fnat k, const double *U, const double *S,
                                  const double *V, const double *dS, const double *dU, const double *dV, double *dA,
                                  double gap, void *stream);

/* Batched SVD of `count` independent real matrices in one persistent launch (FP64 d,
 * FP32 s), each with the result dvjsvd_/svjsvd_ give for it (V := I, pivot strategy 2 or 4
 * generated on the fly, sweep cap swp). All arrays are on the device: matrix b is
 * m[b] x n[b] (the reference's rules: m >= n, m % 8 / % 16, (n/2) % 8 / % 16, n <= 512),
 * column-major with leading dimension m[b] at G + offG[b]; V at V + offV[b] (n x n,
 * leading dimension n); eS/fS at offS[b]. order (optional, NULL = 0..count-1) is the order
 * in which CTAs take matrices (largest first balances the tail). info[b] receives the sweep
 * count or the error code of matrix b. block: 64, 128 or 256 threads per CTA (chosen by
 * the package's autotuner). Asynchronous on `stream`. No counterpart in the reference
 * (whose callers loop over dvjsvd_); the per-matrix arithmetic is dvjsvd_'s
 * (src/dvjsvd.c:40-638). */
vj_fint vj_dvjsvd_batch_dev(vj_fint count, const long long *m, const long long *n, double *G, const long long *offG,
                            double *V, const long long *offV, double *eS, double *fS, const long long *offS,
                            const int *order, long strategy, unsigned swp, long long *info, int block, void *stream);
vj_fint vj_svjsvd_batch_dev(vj_fint count, const long long *m, const long long *n, float *G, const long long *offG,
                            float *V, const long long *offV, float *eS, float *fS, const long long *offS,
                            const int *order, long strategy, unsigned swp, long long *info, int block, void *stream);
/* The same with the kernel's register bound chosen: `occupancy` resident CTAs of 256
 * threads per SM (2 to 6; fewer registers per thread, more CTAs, some spills above 4 for
 * FP32 and 3 for FP64; 0 = the default, 4 for FP32 and 2 for FP64). The package's
 * autotuner searches (block, occupancy) per batch. */
vj_fint vj_dvjsvd_batch_tuned_dev(vj_fint count, const long long *m, const long long *n, double *G,
                                  const long long *offG, double *V, const long long *offV, double *eS, double *fS,
                                  const long long *offS, const int *order, long strategy, unsigned swp,
                                  long long *info, int block, int occupancy, void *stream);
vj_fint vj_svjsvd_batch_tuned_dev(vj_fint count, const long long *m, const long long *n, float *G,
                                  const long long *offG, float *V, const long long *offV, float *eS, float *fS,
                                  const long long *offS, const int *order, long strategy, unsigned swp,
                                  long long *info, int block, int occupancy, void *stream);

/* Allocation-free FP64 SVD. No counterpart in the reference. For callers that must not
 * allocate GPU memory while they run -- for example an application whose memory pool owns
 * the whole device, or a service that must not call cudaMalloc (which can synchronise the
 * device or fail for lack of memory) in the middle of its work -- this form takes only the
 * matrices and the outputs: the pivot table (strategy 2 or 4, generated on the GPU) and
 * the control block live in a fixed 1 MiB + 512 B device array inside the library, present
 * on every GPU that loads it until the process exits. n must not exceed 512 (VJ_ERR_ARG
 * otherwise); the other arguments and the result are those of vj_dvjsvd_dev (it also
 * synchronises `stream` once per sweep; any nonzero preset acts as 1). The first call on
 * a device looks up that array's address for that device (with the device current) and
 * keeps it; make that first call before any stream capture begins. Every call shares the
 * array: calls that overlap on the GPU, on any stream or thread, race and must be
 * serialised by the caller. */
vj_fint vj_dvjsvd_dev_noalloc(vj_fnat m, vj_fnat n, double *G, vj_fnat ldG, double *V, vj_fnat ldV, double *eS,
                              double *fS, long strategy, unsigned swp, int preset, void *stream);

/* ---------------- interleaved <-> split complex matrices ----------------
 * zsplit_ copies an m x n interleaved complex matrix A (re, im pairs: a C `double complex`
 * array, leading dimension ldA in complex elements) into the planes Ar = Re A and
 * Ai = Im A (leading dimensions ldAr, ldAi); zmerge_ is its inverse. c* are the FP32 forms.
 * Checks in the reference's order: -9 a rounding mode other than to-nearest, -1 m not a
 * multiple of 4 (z) / 8 (c), then each leading dimension below m or not a multiple of 4 / 8
 * complex (interleaved) or 8 / 16 real (planes) elements: split -4 ldA, -6 ldAr, -8 ldAi;
 * merge -4 ldAr, -6 ldAi, -8 ldA. Returns 1 (the reference's OpenMP build). Host pointers,
 * synchronous; the vj_*_dev forms take device pointers and a stream (their alignment codes:
 * split -3 A, -5 Ar, -7 Ai; merge -3 Ar, -5 Ai, -7 A, natural alignment of the element).
 *   replaces zsplit_  src/zsplit.h:6, src/zsplit.c:3
 *            zmerge_  src/zmerge.h:6, src/zmerge.c:3
 *            csplit_  src/csplit.h:6, src/csplit.c:3
 *            cmerge_  src/cmerge.h:6, src/cmerge.c:3 */
vj_fint zsplit_(const vj_fnat m[1], const vj_fnat n[1], const double A[], const vj_fnat ldA[1], double Ar[],
                const vj_fnat ldAr[1], double Ai[], const vj_fnat ldAi[1]);
vj_fint zmerge_(const vj_fnat m[1], const vj_fnat n[1], const double Ar[], const vj_fnat ldAr[1], const double Ai[],
                const vj_fnat ldAi[1], double A[], const vj_fnat ldA[1]);
vj_fint csplit_(const vj_fnat m[1], const vj_fnat n[1], const float A[], const vj_fnat ldA[1], float Ar[],
                const vj_fnat ldAr[1], float Ai[], const vj_fnat ldAi[1]);
vj_fint cmerge_(const vj_fnat m[1], const vj_fnat n[1], const float Ar[], const vj_fnat ldAr[1], const float Ai[],
                const vj_fnat ldAi[1], float A[], const vj_fnat ldA[1]);
vj_fint vj_zsplit_dev(vj_fnat m, vj_fnat n, const double *A, vj_fnat ldA, double *Ar, vj_fnat ldAr, double *Ai,
                      vj_fnat ldAi, void *stream);
vj_fint vj_zmerge_dev(vj_fnat m, vj_fnat n, const double *Ar, vj_fnat ldAr, const double *Ai, vj_fnat ldAi,
                      double *A, vj_fnat ldA, void *stream);
vj_fint vj_csplit_dev(vj_fnat m, vj_fnat n, const float *A, vj_fnat ldA, float *Ar, vj_fnat ldAr, float *Ai,
                      vj_fnat ldAi, void *stream);
vj_fint vj_cmerge_dev(vj_fnat m, vj_fnat n, const float *Ar, vj_fnat ldAr, const float *Ai, vj_fnat ldAi, float *A,
                      vj_fnat ldA, void *stream);

/* ---------------- pivot strategy tables ----------------
 * replaces pjs() src/pjs.h:21, src/pjs.c:9: returns a malloc'ed table of *stp rows of n
 * unsigned (n/2 pairs per row, p < q inside a pair), generated on the GPU, or NULL.
 * id 2 (PJS_ME): *stp = n-1; id 4 (PJS_MM): *stp = n. The orderings are published
 * parallel orderings standing in for libpvn's (see the project's design notes): the
 * shape and pair contract match, the exact tables are not pinned. Free with free().
 * vj_pjs_dev writes the table to device memory (stp*n unsigned). */
unsigned *pjs(long id, unsigned n, unsigned stp[1]);
vj_fint vj_pjs_dev(long id, unsigned n, unsigned *table, void *stream);

/* ---------------- library ---------------- */
/* Statistics of the calling thread's last host-API SVD call, the counterpart of the
 * reference's JTRACE log (src/dvjsvd.c:596,635): transformed pairs per sweep (first 64
 * sweeps) and, when
 * VJ_TRACE=1 is set in the environment, SM cycles spent by one CTA in each phase of the
 * pivot steps: 0 control/rescaling, 1 staging, 2 dot products, 3 2x2 and classification,
 * 4 rotations, 5 norms. */
typedef struct vj_trace {
  unsigned sweeps;
  unsigned long long rotations[64];
  unsigned long long phase_cycles[8];
} vj_trace;
vj_fint vj_last_trace(vj_trace *out);
const char *vj_version(void);
/* Measured peak of the current GPU's FMA pipe: fp64 != 0 DFMA, else FFMA. Writes the
 * thread-level FMA operations per second of a kernel of independent FMA chains over every
 * SM (CUDA-event timed, best of 3) to *ops_per_s; the roofline denominator of the kernels
 * bound by arithmetic. Returns 0 or a VJ_ERR_* code. No counterpart in the reference. */
vj_fint vj_measure_fma_rate(int fp64, double *ops_per_s, void *stream);
/* The same probe in a given shape: warps_per_sm warps on every SM (1 to 8, or a multiple
 * of 8 up to 64), `lanes` active lanes per warp (the others exit first), `chains` FMA
 * chains per lane (8 independent, or 1: a dependent chain, whose rate gives the latency).
 * *ops_per_s: active-lane FMAs per second. No counterpart in the reference. */
vj_fint vj_measure_fma_shape(int fp64, int warps_per_sm, int lanes, int chains, double *ops_per_s, void *stream);
/* Width in bits of vj_fint / vj_fnat in this build: 64 (ILP64, the default, as the
 * reference's ABI=ilp64) or 32 (built with -DVJ_LP64, as the reference's ABI=lp64). */
int vj_abi_int_bits(void);

#ifdef __cplusplus
}
#endif

#endif /* !VECJAC_GB300_H */
