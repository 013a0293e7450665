/* TEST INFRASTRUCTURE ONLY -- part of the CPU oracle, never linked into the product.
 *
 * Precision-generic body of the C restatement of VecJac's hot path. It is included
 * twice by oracle/vjo.c: once for FP64 (d/z, 8 AVX-512 lanes) and once for FP32
 * (s/c, 16 lanes). Each function restates one reference routine lane by lane, in
 * the reference's operation order, so that the results are bit-identical to the
 * reference compiled from source (oracle/Makefile) when both use the same column
 * norm (oracle/vjo_nrm2.h).
 *
 * Expected macros: R, LANES, LOWMASK, BIG_EXP, SQRT_HUGE, RMAX, RTRUEMIN, REPS,
 * MAX_FIN_EXP, ROT_EXP_R, ROT_EXP_C, FMA, SQRT, H(x) (scalar helper names),
 * and the public names RBJAC2, RBJAC2I, CBJAC2, CBJAC2I, RSVD, CSVD, GSVD.
 */

/* ----- one lane of the batched 2x2 EVD -----
 * kind 0: tangents + cosines (src/dbjac2.c:17-44, D8JAC2_LOOP)
 * kind 1: sines + cosines    (src/dbjac2.c:51-78, D8JACL_LOOP)
 * kind 2: tangents + secants (src/dbjac2.c:148-175, D8JACI_LOOP)
 * returns the permutation bit (L1 < L2). */
static inline unsigned H(rjac2)(const int kind, R a1, R a2, R ar, R *c, R *at, R *l1, R *l2)
{
  const R zero = (R)0, one = (R)1, sh = SQRT_HUGE, huge = RMAX, be = BIG_EXP;
  const R e1 = be - H(getexp)(a1);
  const R e2 = be - H(getexp)(a2);
  const R er = be - H(getexp)(ar);
  R es = H(min)(H(min)(e1, e2), H(min)(er, huge));
  ar = H(scalef)(ar, es);
  a1 = H(scalef)(a1, es);
  a2 = H(scalef)(a2, es);
  const R aa = H(abs)(ar);
  const R as = H(sgn)(ar);
  es = H(neg)(es);
  const R ab = H(scalef)(aa, one);
  const R ad = a1 - a2;
  const R t2 = H(or)(H(min)(H(max)(ab / H(abs)(ad), zero), sh), H(sgn)(ad));
  const R t1 = t2 / (one + SQRT(FMA(t2, t2, one)));
  const R s2 = FMA(t1, t1, one);
  const R s1 = SQRT(s2);
  if (kind == 2) {
    *at = H(xor)(t1, as);
    *c = s1;
  }
  else {
    const R co = one / s1;
    *at = ((kind == 1) ? (H(xor)(t1, as) / s1) : H(xor)(t1, as));
    *c = co;
  }
  const R L1 = FMA(t1, FMA(a2, t1, ab), a1) / s2;
  const R L2 = FMA(t1, FMA(a1, t1, -ab), a2) / s2;
  *l1 = H(scalef)(L1, es);
  *l2 = H(scalef)(L2, es);
  return (L1 < L2);
}

/* one lane of the Hermitian 2x2 EVD (src/zbjac2.c:18-62, :65-106, :179-219) */
static inline unsigned H(cjac2)(const int kind, R a1, R a2, R ar, R ai, R *c, R *cat, R *sat, R *l1, R *l2)
{
  const R zero = (R)0, one = (R)1, sh = SQRT_HUGE, huge = RMAX, be = BIG_EXP, dtm = RTRUEMIN;
  const R e1 = be - H(getexp)(a1);
  const R e2 = be - H(getexp)(a2);
  const R er = be - H(getexp)(ar);
  const R ei = be - H(getexp)(ai);
  R es = H(min)(huge, H(min)(H(min)(e1, e2), H(min)(er, ei)));
  ar = H(scalef)(ar, es);
  ai = H(scalef)(ai, es);
  a1 = H(scalef)(a1, es);
  a2 = H(scalef)(a2, es);
  R ar_ = H(abs)(ar);
  R ai_ = H(abs)(ai);
  const R as = H(sgn)(ar);
  const R am = H(min)(ar_, ai_);
  const R aM = H(max)(ar_, ai_);
  es = H(neg)(es);
  R aa = H(max)(am / aM, zero);
  aa = SQRT(FMA(aa, aa, one)) * aM;
  ar_ = H(or)(H(min)(ar_ / aa, one), as);
  ai_ = ai / H(max)(aa, dtm);
  const R ab = H(scalef)(aa, one);
  const R ad = a1 - a2;
  const R t2 = H(or)(H(min)(H(max)(ab / H(abs)(ad), zero), sh), H(sgn)(ad));
  const R t1 = t2 / (one + SQRT(FMA(t2, t2, one)));
  const R s2 = FMA(t1, t1, one);
  const R s1 = SQRT(s2);
  if (kind == 2) {
    ar_ = ar_ * t1;
    *c = s1;
    ai_ = ai_ * t1;
  }
  else if (kind == 1) {
    const R co = one / s1;
    ar_ = (ar_ * t1) / s1;
    *c = co;
    ai_ = (ai_ * t1) / s1;
  }
  else {
    const R co = one / s1;
    ar_ = ar_ * t1;
    *c = co;
    ai_ = ai_ * t1;
  }
  *cat = ar_;
  *sat = ai_;
  const R L1 = FMA(t1, FMA(a2, t1, ab), a1) / s2;
  const R L2 = FMA(t1, FMA(a1, t1, -ab), a2) / s2;
  *l1 = H(scalef)(L1, es);
  *l2 = H(scalef)(L2, es);
  return (L1 < L2);
}

/* xbjac2_ (src/dbjac2.c:81-139, src/sbjac2.c, src/zbjac2.c:108-173, src/cbjac2.c):
 * n < 0 -> sines, n > 0 -> tangents; p[i/LANES] bit k = (L1 < L2) of lane k.
 * Returns 1 like the reference's OpenMP build; -1 when |n| is not a multiple of LANES
 * (the reference's debug-build check). */
long long RBJAC2(const long long *n, const R *a11, const R *a22, const R *a21, R *c, R *at, R *l1, R *l2, unsigned *p)
{
  if (*n % (long long)LANES)
    return -1;
  const int kind = ((*n < 0) ? 1 : 0);
  const long long nn = ((*n < 0) ? -*n : *n);
  for (long long i = 0; i < nn; i += LANES) {
    unsigned P = 0u;
    for (unsigned k = 0u; k < LANES; ++k)
      P |= (H(rjac2)(kind, a11[i + k], a22[i + k], a21[i + k], c + i + k, at + i + k, l1 + i + k, l2 + i + k) << k);
    p[i / LANES] = P;
  }
  return 1;
}

/* xbjac2i (src/dbjac2.c:178-248): masked by the low LANES bits of p, secants for n < 0 */
long long RBJAC2I(const long long *n, const R *a11, const R *a22, const R *a21, R *c, R *at, R *l1, R *l2, unsigned *p)
{
  if (*n % (long long)LANES)
    return -1;
  const int kind = ((*n < 0) ? 2 : 0);
  const long long nn = ((*n < 0) ? -*n : *n);
  for (long long i = 0; i < nn; i += LANES) {
    const long long j = i / LANES;
    if (p[j] & LOWMASK) {
      unsigned P = 0u;
      for (unsigned k = 0u; k < LANES; ++k)
        P |= (H(rjac2)(kind, a11[i + k], a22[i + k], a21[i + k], c + i + k, at + i + k, l1 + i + k, l2 + i + k) << k);
      p[j] = ((p[j] & ~(unsigned)LOWMASK) | P);
    }
  }
  return 1;
}

long long CBJAC2(const long long *n, const R *a11, const R *a22, const R *a21r, const R *a21i, R *c, R *cat, R *sat, R *l1, R *l2, unsigned *p)
{
  if (*n % (long long)LANES)
    return -1;
  const int kind = ((*n < 0) ? 1 : 0);
  const long long nn = ((*n < 0) ? -*n : *n);
  for (long long i = 0; i < nn; i += LANES) {
    unsigned P = 0u;
    for (unsigned k = 0u; k < LANES; ++k)
      P |= (H(cjac2)(kind, a11[i + k], a22[i + k], a21r[i + k], a21i[i + k], c + i + k, cat + i + k, sat + i + k, l1 + i + k, l2 + i + k) << k);
    p[i / LANES] = P;
  }
  return 1;
}

long long CBJAC2I(const long long *n, const R *a11, const R *a22, const R *a21r, const R *a21i, R *c, R *cat, R *sat, R *l1, R *l2, unsigned *p)
{
  if (*n % (long long)LANES)
    return -1;
  const int kind = ((*n < 0) ? 2 : 0);
  const long long nn = ((*n < 0) ? -*n : *n);
  for (long long i = 0; i < nn; i += LANES) {
    const long long j = i / LANES;
    if (p[j] & LOWMASK) {
      unsigned P = 0u;
      for (unsigned k = 0u; k < LANES; ++k)
        P |= (H(cjac2)(kind, a11[i + k], a22[i + k], a21r[i + k], a21i[i + k], c + i + k, cat + i + k, sat + i + k, l1 + i + k, l2 + i + k) << k);
      p[j] = ((p[j] & ~(unsigned)LOWMASK) | P);
    }
  }
  return 1;
}

/* ----- L1 kernels of the SVD driver ----- */

/* (e,f) split: x = f * 2^e, f in [1,2) (src/dznrm2.h:4-23) */
static inline void H(ef)(const R d, R *e, R *f)
{
  if (isfinite(d)) {
    if (d == (R)0) {
      *e = -(R)HUGE_VAL;
      *f = (R)copysign(1.0, (double)d);
    }
    else {
      const int k = H(ilogb)(d);
      *e = (R)k;
      *f = H(scale2)(d, -k);
    }
  }
  else {
    *e = (R)HUGE_VAL;
    *f = (R)copysign((isinf(d) ? 1.0 : 0.0), (double)d);
  }
}

/* max_ij min(|a_ij|, inf) (src/dnormx.c, src/dznrmx.h) */
static R H(normx)(const long long m, const long long n, const R *A, const long long ldA)
{
  R y = (R)0;
  for (long long j = 0; j < n; ++j)
    for (long long i = 0; i < m; ++i)
      y = H(max)(H(min)(H(abs)(A[j * ldA + i]), (R)HUGE_VAL), y);
  return y;
}

/* A * 2^e (src/dscale.c, src/dzscal.h) */
static void H(scale)(const long long m, const long long n, R *A, const long long ldA, const long long e)
{
  if (!e)
    return;
  const R e_ = (R)e;
  for (long long j = 0; j < n; ++j)
    for (long long i = 0; i < m; ++i)
      A[j * ldA + i] = H(scalef)(A[j * ldA + i], e_);
}

static void H(swp)(const long long n, R *x, R *y)
{
  for (long long i = 0; i < n; ++i) {
    const R t = x[i];
    x[i] = y[i];
    y[i] = t;
  }
}

/* the LANES-wide horizontal sum in the order of GCC's _mm512_reduce_add_{pd,ps} */
static inline R H(hsum)(R *v)
{
  for (unsigned w = LANES / 2u; w >= 1u; w >>= 1u)
    for (unsigned l = 0u; l < w; ++l)
      v[l] = v[l + w] + v[l];
  return v[0];
}

/* Moeller's 2Sum (src/d2sum.h) */
#define VJO_TWOSUM(a, b, s, t) do { const R s_ = (a) + (b); R a_ = s_ - (b); R b_ = s_ - a_; a_ = (a) - a_; b_ = (b) - b_; (s) = s_; (t) = a_ + b_; } while (0)

/* scaled compensated dot (src/ddpscl.c:7-75, USE_2SUM) */
static R H(dpscl)(const long long m, const R *x, const R *y, const R ex, const R ey, const R fx, const R fy)
{
  if (!(ex >= -RMAX))
    return (R)0;
  if (!(ey >= -RMAX))
    return (R)0;
  const R xe = H(neg)(ex), ye = H(neg)(ey);
  R spd[LANES], tpd[LANES], sdn[LANES], tdn[LANES];
  for (unsigned k = 0u; k < LANES; ++k)
    spd[k] = tpd[k] = sdn[k] = tdn[k] = (R)0;
  for (long long i = 0; i < m; i += LANES) {
    for (unsigned k = 0u; k < LANES; ++k) {
      const R xi = H(scalef)(x[i + k], xe);
      const R yi = H(scalef)(y[i + k], ye);
      const R pd = H(mul_rd)(xi, yi);
      const R dn = FMA(xi, yi, -pd);
      R a = spd[k];
      R b = pd + tpd[k];
      VJO_TWOSUM(a, b, spd[k], tpd[k]);
      a = sdn[k];
      b = dn + tdn[k];
      VJO_TWOSUM(a, b, sdn[k], tdn[k]);
    }
  }
  const R nu = (H(hsum)(spd) + (H(hsum)(tpd) + (H(hsum)(sdn) + H(hsum)(tdn))));
  const R de = (fx * fy);
  return (nu / de);
}

/* complex scaled compensated dot conj(x)*y (src/zdpscl.c:21-116, USE_2SUM) */
#define VJO_MUL2SUM(x, y, s, t, s_, t_) do { const R xy = H(mul_rd)((x), (y)); R a = (s); const R xy_ = FMA((x), (y), -xy); R b = xy + (t); VJO_TWOSUM(a, b, (s), (t)); a = (s_); b = xy_ + (t_); VJO_TWOSUM(a, b, (s_), (t_)); } while (0)

static void H(zdpscl)(const long long m, const R *xr, const R *xi, const R *yr, const R *yi, const R ex, const R ey, const R fx, const R fy, R *zr, R *zi)
{
  if (!(ex >= -RMAX) || !(ey >= -RMAX)) {
    *zr = (R)0;
    *zi = (R)0;
    return;
  }
  const R xe = H(neg)(ex), ye = H(neg)(ey);
  R sr[LANES], tr[LANES], sr_[LANES], tr_[LANES], si[LANES], ti[LANES], si_[LANES], ti_[LANES];
  for (unsigned k = 0u; k < LANES; ++k)
    sr[k] = tr[k] = sr_[k] = tr_[k] = si[k] = ti[k] = si_[k] = ti_[k] = (R)0;
  for (long long i = 0; i < m; i += LANES) {
    for (unsigned k = 0u; k < LANES; ++k) {
      const R xri = H(scalef)(xr[i + k], xe);
      const R yri = H(scalef)(yr[i + k], ye);
      const R yii = H(scalef)(yi[i + k], ye);
      R xii = H(scalef)(xi[i + k], xe);
      VJO_MUL2SUM(xri, yri, sr[k], tr[k], sr_[k], tr_[k]);
      VJO_MUL2SUM(xii, yii, sr[k], tr[k], sr_[k], tr_[k]);
      xii = H(neg)(xii);
      VJO_MUL2SUM(xri, yii, si[k], ti[k], si_[k], ti_[k]);
      VJO_MUL2SUM(xii, yri, si[k], ti[k], si_[k], ti_[k]);
    }
  }
  const R nur = (H(hsum)(sr) + (H(hsum)(tr) + (H(hsum)(sr_) + H(hsum)(tr_))));
  const R nui = (H(hsum)(si) + (H(hsum)(ti) + (H(hsum)(si_) + H(hsum)(ti_))));
  const R de = (fx * fy);
  *zr = nur / de;
  *zi = nui / de;
}

/* rotation (src/djrot.c:5-107); track != 0 returns max|out| like djrot_, else 0 like djrotf_.
 * n < 0 permutes. Cosines are multiplied (USE_SECANTS off). */
static R H(jrot)(const long long n, R *x, R *y, const R c, const R at, const int track)
{
  if (!n)
    return (R)0;
  R mx = (R)0;
  if (n < 0) {
    const long long n_ = -n;
    if (at == (R)0) {
      if (c == (R)1) {
        H(swp)(n_, x, y);
        return (R)0;
      }
      return (R)-4;
    }
    for (long long i = 0; i < n_; ++i) {
      const R x_ = x[i], y_ = y[i];
      R xr = FMA(-x_, at, y_);
      R yr = FMA(y_, at, x_);
      if (c != (R)1) {
        xr = xr * c;
        yr = yr * c;
      }
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(xr), H(abs)(yr)));
      x[i] = xr;
      y[i] = yr;
    }
  }
  else {
    if (at == (R)0)
      return ((c == (R)1) ? (R)0 : (R)-4);
    for (long long i = 0; i < n; ++i) {
      const R x_ = x[i], y_ = y[i];
      R xr = FMA(y_, at, x_);
      R yr = FMA(-x_, at, y_);
      if (c != (R)1) {
        xr = xr * c;
        yr = yr * c;
      }
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(xr), H(abs)(yr)));
      x[i] = xr;
      y[i] = yr;
    }
  }
  return mx;
}

/* VZFMA (src/vecdef.h:68-74): d = a*b + c */
#define VJO_ZFMA(dr, di, ar, ai, br, bi, cr, ci) do { dr = FMA((ar), (br), FMA(-(ai), (bi), (cr))); di = FMA((ar), (bi), FMA((ai), (br), (ci))); } while (0)

/* complex rotation (src/zjrot.c, src/zjrotf.c); real fallback when sat == 0 */
static R H(zjrot)(const long long n, R *xr, R *xi, R *yr, R *yi, const R c, const R cat, const R sat, const int track)
{
  if (!n)
    return (R)0;
  if (sat == (R)0) {
    const R r_r = H(jrot)(n, xr, yr, c, cat, track);
    if (track) {
      if (!(r_r >= (R)0))
        return (R)-10;
    }
    else if (r_r != (R)0)
      return (R)-10;
    const R r_i = H(jrot)(n, xi, yi, c, cat, track);
    if (track) {
      if (!(r_i >= (R)0))
        return (R)-11;
      return (R)fmax((double)r_r, (double)r_i);
    }
    else if (r_i != (R)0)
      return (R)-11;
    return (R)0;
  }
  const R cta = cat, sta = sat, cna = -cat;
  R mx = (R)0;
  const long long n_ = ((n < 0) ? -n : n);
  for (long long i = 0; i < n_; ++i) {
    const R x_r = xr[i], x_i = xi[i], y_r = yr[i], y_i = yi[i];
    R ar, ai, br, bi;
    VJO_ZFMA(ar, ai, y_r, y_i, cta, sta, x_r, x_i);
    VJO_ZFMA(br, bi, x_r, x_i, cna, sta, y_r, y_i);
    if (c != (R)1) {
      ar = ar * c; ai = ai * c;
      br = br * c; bi = bi * c;
    }
    if (n < 0) { /* permute: y <- a, x <- b */
      yr[i] = ar; yi[i] = ai;
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(ar), H(abs)(ai)));
      xr[i] = br; xi[i] = bi;
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(br), H(abs)(bi)));
    }
    else {
      xr[i] = ar; xi[i] = ai;
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(ar), H(abs)(ai)));
      yr[i] = br; yi[i] = bi;
      if (track)
        mx = H(max)(mx, H(max)(H(abs)(br), H(abs)(bi)));
    }
  }
  return mx;
}

/* Gram-Schmidt-like shear (src/dgsscl.c:5-85) */
static R H(gsscl)(const long long m, const R t, R *x, R *y, const R ex, const R ey, const R fx, const R fy)
{
  if (!m)
    return (R)0;
  if (!(ex >= -RMAX))
    return (R)0;
  if (!(ey >= -RMAX))
    return (R)0;
  const R x_e = H(neg)(ex), y_e = H(neg)(ey);
  R M = (R)0;
  if (m < 0) {
    const R tf = -t * (fx / fy);
    const long long m_ = -m;
    for (long long i = 0; i < m_; ++i) {
      R xi = x[i];
      R yi = y[i];
      xi = H(scalef)(xi, x_e);
      x[i] = yi;
      yi = H(scalef)(yi, y_e);
      xi = H(scalef)(FMA(tf, yi, xi), ex);
      y[i] = xi;
      M = H(max)(M, H(abs)(xi));
    }
  }
  else {
    const R tf = -t * (fy / fx);
    for (long long i = 0; i < m; ++i) {
      R xi = x[i];
      R yi = y[i];
      xi = H(scalef)(xi, x_e);
      yi = H(scalef)(yi, y_e);
      yi = H(scalef)(FMA(tf, xi, yi), ey);
      y[i] = yi;
      M = H(max)(M, H(abs)(yi));
    }
  }
  return M;
}

/* complex shear (src/zgsscl.c) */
static R H(zgsscl)(const long long m, const R tr, const R ti, R *xr, R *xi, R *yr, R *yi, const R ex, const R ey, const R fx, const R fy)
{
  if (!m)
    return (R)0;
  if (!(ex >= -RMAX))
    return (R)0;
  if (!(ey >= -RMAX))
    return (R)0;
  const R x_e = H(neg)(ex), y_e = H(neg)(ey);
  R M = (R)0;
  if (m < 0) {
    const R fx_y = (fx / fy);
    const R tfr = -tr * fx_y;
    const R tfi = -ti * fx_y;
    const long long m_ = -m;
    for (long long i = 0; i < m_; ++i) {
      R yri = yr[i], yii = yi[i];
      const R xri = xr[i], xii = xi[i];
      xr[i] = yri;
      xi[i] = yii;
      const R yri_ = H(scalef)(yri, y_e), yii_ = H(scalef)(yii, y_e);
      const R xri_ = H(scalef)(xri, x_e), xii_ = H(scalef)(xii, x_e);
      VJO_ZFMA(yri, yii, tfr, tfi, yri_, yii_, xri_, xii_);
      const R ur = H(scalef)(yri, ex), ui = H(scalef)(yii, ex);
      yr[i] = ur;
      yi[i] = ui;
      M = H(max)(M, H(abs)(ur));
      M = H(max)(M, H(abs)(ui));
    }
  }
  else {
    const R fy_x = (fy / fx);
    const R tfr = -tr * fy_x;
    const R tfi = ti * fy_x;
    for (long long i = 0; i < m; ++i) {
      R xri = xr[i], xii = xi[i];
      const R xri_ = H(scalef)(xri, x_e), xii_ = H(scalef)(xii, x_e);
      const R yri = yr[i], yii = yi[i];
      const R yri_ = H(scalef)(yri, y_e), yii_ = H(scalef)(yii, y_e);
      VJO_ZFMA(xri, xii, tfr, tfi, xri_, xii_, yri_, yii_);
      const R ur = H(scalef)(xri, ey), ui = H(scalef)(xii, ey);
      yr[i] = ur;
      yi[i] = ui;
      M = H(max)(M, H(abs)(ur));
      M = H(max)(M, H(abs)(ui));
    }
  }
  return M;
}

/* ‖x‖ split into (e,f) for the norm and its square (src/dnorm2.c, src/znorm2.c) */
static R H(norm2)(const long long m, const R *xr, const R *xi, R *e0, R *f0)
{
  R d;
  if (xi)
    d = H(hypot)(H(nrm2)(m, xr), H(nrm2)(m, xi));
  else
    d = H(nrm2)(m, xr);
  H(ef)(d, e0, f0);
  return d;
}

static inline int H(efcmp)(const R e0, const R f0, const R e1, const R f1)
{
  if (e0 > e1) return 1;
  if (e0 < e1) return -1;
  if (f0 > f1) return 1;
  if (f0 < f1) return -1;
  return 0;
}

/* (e0,f0) < (e1,f1) and <= as in VDEFLT / VDEFLE (src/defops.h:31-41) */
static inline int H(eflt)(const R e0, const R e1, const R f0, const R f1) { return (e0 < e1) || ((e0 == e1) && (f0 < f1)); }
static inline int H(efle)(const R e0, const R e1, const R f0, const R f1) { return (e0 < e1) || ((e0 == e1) && (f0 <= f1)); }

/* ----- the one-sided Jacobi SVD driver -----
 * Restates src/dvjsvd.c:40-638 (cx == 0) and src/zvjsvd.c:40-694 (cx != 0), step by step.
 * Gi/Vi are NULL for the real variant. Work areas are allocated locally; the public
 * work/iwork arguments are only checked like in the reference. */
long long GSVD(const int cx, const unsigned long long *pm, const unsigned long long *pn,
               R *Gr, const unsigned long long *ldGr, R *Gi, const unsigned long long *ldGi,
               R *Vr, const unsigned long long *ldVr, R *Vi, const unsigned long long *ldVi,
               R *eS, R *fS, const unsigned *js, const unsigned *stp, const unsigned *swp,
               R *work, unsigned *iwork)
{
  const long long m = (long long)*pm, n = (long long)*pn;
  const long long n_2 = (n >> 1);
  if (!n)
    return 0;
  if (*pm < *pn)
    return -1;
  if (m % LANES)
    return -1;
  if (n & 1)
    return -2;
  if (n_2 % LANES)
    return -2;
  if ((uintptr_t)Gr & 63u)
    return -3;
  if (*ldGr < *pm || (*ldGr % LANES))
    return -4;
  if (cx) {
    if ((uintptr_t)Gi & 63u)
      return -5;
    if (*ldGi < *pm || (*ldGi % LANES))
      return -6;
    if ((uintptr_t)Vr & 63u)
      return -7;
    if (*ldVr < *pn || (*ldVr % LANES))
      return -8;
    if ((uintptr_t)Vi & 63u)
      return -9;
    if (*ldVi < *pn || (*ldVi % LANES))
      return -10;
    if ((uintptr_t)work & 63u)
      return -16;
  }
  else {
    if ((uintptr_t)Vr & 63u)
      return -5;
    if (*ldVr < *pn || (*ldVr % LANES))
      return -6;
    if ((uintptr_t)work & 63u)
      return -12;
  }
  const long long ldG = (long long)*ldGr, ldV = (long long)*ldVr;
  const long long ldGI = (cx ? (long long)*ldGi : 0), ldVI = (cx ? (long long)*ldVi : 0);
  /* error codes of the reference: -__LINE__ of the failing statement */
  const long long E_MG = (cx ? -92 : -80), E_MV = (cx ? -104 : -92), E_DOT = (cx ? -345 : -320), E_DOTI = -347;
  const long long E_APPG = (cx ? -630 : -580), E_APPV = (cx ? -638 : -588), E_MVZ = (cx ? -17 : -13);
  const int ROT = (cx ? (ROT_EXP_C - 1) : ROT_EXP_R);

  R MG = H(normx)(m, n, Gr, ldG);
  if (cx)
    MG = H(max)(H(normx)(m, n, Gi, ldGI), MG);
  if (!(MG <= RMAX))
    return E_MG;
  R MV = (R)1;
  if (*iwork) {
    MV = H(normx)(n, n, Vr, ldV);
    if (cx)
      MV = H(max)(H(normx)(n, n, Vi, ldVI), MV);
    if (!(MV <= RMAX))
      return E_MV;
    if (MV <= (R)0)
      return E_MVZ;
  }
  else {
    for (long long j = 0; j < n; ++j) {
      for (long long i = 0; i < n; ++i) {
        Vr[j * ldV + i] = (R)0;
        if (cx)
          Vi[j * ldVI + i] = (R)0;
      }
      Vr[j * ldV + j] = (R)1;
    }
  }
  for (long long j = 0; j < n; ++j) {
    eS[j] = -(R)HUGE_VAL;
    fS[j] = (R)1;
  }
  if (MG == (R)0)
    return 0;

  const R M_m = (cx ? (RMAX / ((R)((unsigned long long)m << 2u) * (R)M_SQRT2)) : (RMAX / (R)((unsigned long long)m << 1u)));
  R es = (R)0, fs = (R)0;
  H(ef)(M_m, &es, &fs);
  const int MAX_NRM_EXP = (int)es;
  H(ef)(MG, &es, &fs);
  int eM = (int)es;
  int sR = ROT - eM;
  long long sN = MAX_NRM_EXP - eM - 1;
  if (sN) {
    H(scale)(m, n, Gr, ldG, sN);
    if (cx)
      H(scale)(m, n, Gi, ldGI, sN);
    MG = H(scale2)(MG, (int)sN);
  }
  int sT = (int)sN;
  if (*iwork) {
    H(ef)(MV, &es, &fs);
    eM = (int)es;
    sR = ROT - eM;
    sN = sR;
    if (sN) {
      H(scale)(n, n, Vr, ldV, sN);
      if (cx)
        H(scale)(n, n, Vi, ldVI, sN);
      MV = H(scale2)(MV, sR);
    }
  }
  else
    sR = 0;
  int sV = sR;
  const int vtrack = (*iwork != 0u);

  R *const w = (R*)malloc((size_t)(16 * (n_2 + LANES)) * sizeof(R));
  unsigned *const pb = (unsigned*)malloc((size_t)(2 * (n_2 / LANES + 1)) * sizeof(unsigned));
  R *const chg = (R*)malloc((size_t)n * sizeof(R));
  if (!w || !pb || !chg) {
    free(w); free(pb); free(chg);
    return -__LINE__;
  }
  R *const a21r = w, *const a21i = w + n_2, *const c = w + 2 * n_2, *const cat = w + 3 * n_2, *const sat = w + 4 * n_2;
  R *const e1v = w + 5 * n_2, *const e2v = w + 6 * n_2, *const f1v = w + 7 * n_2, *const f2v = w + 8 * n_2;
  R *const wa11 = w + 9 * n_2, *const wa22 = w + 10 * n_2, *const wa21r = w + 11 * n_2, *const wa21i = w + 12 * n_2;
  R *const l1 = w + 13 * n_2, *const l2 = w + 14 * n_2, *const w0 = w + 15 * n_2;
  unsigned *const p = pb, *const pc = pb + (n_2 / LANES + 1);

  if (*swp)
    for (long long i = 0; i < n; ++i)
      chg[i] = (R)1;

  const R tol = SQRT((R)m) * H(scale2)(REPS, -1);
  const R gst = H(scale2)(tol, (int)MAX_FIN_EXP);
  unsigned sw = 0u;
  long long ret = 0;
  vjo_trace_nsw = 0u;

  while (sw < *swp) {
    unsigned long long swt = 0u;
    for (unsigned st = 0u; st < *stp; ++st) {
      H(ef)(MG, &es, &fs);
      eM = (int)es;
      sR = ROT - eM;
      sN = MAX_NRM_EXP - eM - 1;
      if (sR < 0) {
        H(scale)(m, n, Gr, ldG, sN);
        if (cx)
          H(scale)(m, n, Gi, ldGI, sN);
        sR = (int)sN;
        MG = H(scale2)(MG, sR);
        sT += sR;
        for (long long i = 0; i < n; ++i)
          chg[i] = (R)1;
      }
      H(ef)(MV, &es, &fs);
      eM = (int)es;
      sR = ROT - eM;
      sN = sR;
      if (sR < 0) {
        H(scale)(n, n, Vr, ldV, sN);
        if (cx)
          H(scale)(n, n, Vi, ldVI, sN);
        MV = H(scale2)(MV, sR);
        sV += sR;
      }
      const unsigned *const r = js + st * (size_t)n;
      /* norms of the columns changed in the previous step, overflow-aware */
      int overflow = 0;
      do {
        R nMG = (R)0;
        for (long long pq = 0; pq < n; pq += 2) {
          if (!(nMG <= RMAX))
            break;
          const long long _p = r[pq], _q = r[pq + 1];
          if (chg[_p] == (R)1) {
            const R d = H(norm2)(m, Gr + _p * ldG, (cx ? (Gi + _p * ldGI) : NULL), eS + _p, fS + _p);
            nMG = (R)fmax((double)nMG, fmin((double)d, HUGE_VAL));
            if (!(nMG <= RMAX))
              continue;
          }
          if (chg[_q] == (R)1) {
            const R d = H(norm2)(m, Gr + _q * ldG, (cx ? (Gi + _q * ldGI) : NULL), eS + _q, fS + _q);
            nMG = (R)fmax((double)nMG, fmin((double)d, HUGE_VAL));
          }
        }
        if ((overflow = !(nMG <= RMAX))) {
          H(scale)(m, n, Gr, ldG, sN);
          if (cx)
            H(scale)(m, n, Gi, ldGI, sN);
          sR = (int)sN;
          MG = H(scale2)(MG, sR);
          sT += sR;
          for (long long i = 0; i < n; ++i)
            chg[i] = (R)1;
        }
      } while (overflow);
      /* scaled dot products; the error code is the minimum over all pairs */
      long long dot_err = 0;
      for (long long pq = 0; pq < n; pq += 2) {
        const long long _pq = (pq >> 1);
        const long long _p = r[pq], _q = r[pq + 1];
        if (cx) {
          H(zdpscl)(m, Gr + _q * ldG, Gi + _q * ldGI, Gr + _p * ldG, Gi + _p * ldGI, eS[_q], eS[_p], fS[_q], fS[_p], a21r + _pq, a21i + _pq);
          if (!isfinite(a21r[_pq]) && (E_DOT < dot_err)) dot_err = E_DOT;
          if (!isfinite(a21i[_pq]) && (E_DOTI < dot_err)) dot_err = E_DOTI;
        }
        else {
          a21r[_pq] = H(dpscl)(m, Gr + _q * ldG, Gr + _p * ldG, eS[_q], eS[_p], fS[_q], fS[_p]);
          if (!isfinite(a21r[_pq])) dot_err = E_DOT;
        }
        e1v[_pq] = eS[_p];
        e2v[_pq] = eS[_q];
        f1v[_pq] = fS[_p];
        f2v[_pq] = fS[_q];
      }
      if (dot_err) { ret = dot_err; goto theEnd; }
      /* convergence test, shear test and Gram prescale, LANES pairs at a time */
      unsigned long long stt = 0u;
      for (long long i = 0; i < n_2; i += LANES) {
        const long long j = i / LANES;
        unsigned pcj = 0u;
        for (unsigned k = 0u; k < LANES; ++k) {
          const R ab = (cx ? H(hypot)(a21r[i + k], a21i[i + k]) : H(abs)(a21r[i + k]));
          pcj |= ((unsigned)(tol <= ab) << k);
        }
        pc[j] = pcj;
        p[j] = (unsigned)__builtin_popcount(pcj);
        if (p[j]) {
          stt += p[j];
          for (unsigned k = 0u; k < LANES; ++k) {
            const long long l = i + k;
            const R f1 = f1v[l], f2 = f2v[l], e1 = e1v[l], e2 = e2v[l];
            const int ngs = H(eflt)(e1, e2, f1, f2);
            R maf = (ngs ? f1 : f2), mae = (ngs ? e1 : e2);
            const R Maf = (ngs ? f2 : f1), Mae = (ngs ? e2 : e1);
            maf = gst * maf;
            mae = mae + H(getexp)(maf);
            maf = H(getmant)(maf);
            const int cgs = H(eflt)(mae, Mae, maf, Maf);
            p[j] |= ((unsigned)(!ngs && cgs) << (k + LANES));
            pc[j] |= ((unsigned)(ngs && cgs) << (k + LANES));
            R f12 = f1 / f2, e12 = e1 - e2, f21 = f2 / f1, e21 = e2 - e1;
            e12 = e12 + H(getexp)(f12);
            f12 = H(getmant)(f12);
            e21 = e21 + H(getexp)(f21);
            f21 = H(getmant)(f21);
            const int c12 = H(efle)(e12, e21, f12, f21);
            const R E = (c12 ? e21 : e12);
            const R d = H(min)(MAX_FIN_EXP - E, (R)0);
            e12 = e12 + d;
            e21 = e21 + d;
            wa11[l] = H(scalef)(f12, e12);
            wa22[l] = H(scalef)(f21, e21);
            wa21r[l] = H(scalef)(a21r[l], d);
            if (cx)
              wa21i[l] = H(scalef)(a21i[l], d);
          }
        }
      }
      swt += stt;
      /* the 2x2 EVDs (tangents and cosines), masked per LANES group */
      for (long long i = 0; i < n_2; i += LANES) {
        const long long j = i / LANES;
        if (p[j] & LOWMASK) {
          unsigned P = 0u;
          for (unsigned k = 0u; k < LANES; ++k) {
            const long long l = i + k;
            R at_;
            if (cx)
              P |= (H(cjac2)(0, wa11[l], wa22[l], wa21r[l], wa21i[l], c + l, cat + l, sat + l, l1 + l, l2 + l) << k);
            else {
              P |= (H(rjac2)(0, wa11[l], wa22[l], wa21r[l], c + l, &at_, l1 + l, l2 + l) << k);
              cat[l] = at_;
              sat[l] = (R)0;
            }
          }
          p[j] = ((p[j] & ~(unsigned)LOWMASK) | P);
        }
      }
      /* classify */
      for (long long i = 0; i < n_2; i += LANES) {
        const long long j = i / LANES;
        unsigned gsp = (p[j] >> LANES), gsn = (pc[j] >> LANES), trans = (pc[j] & LOWMASK), perm = (p[j] & LOWMASK);
        for (unsigned k = 0u; k < LANES; ++k) {
          const long long l = i + k;
          const long long _p = r[2 * l], _q = r[2 * l + 1];
          if (trans & 1u) {
            if (gsp & 1u)
              w0[l] = (R)3;
            else if (gsn & 1u)
              w0[l] = (R)-3;
            else if (perm & 1u)
              w0[l] = (R)-2;
            else
              w0[l] = (R)2;
          }
          else if (H(efcmp)(eS[_p], fS[_p], eS[_q], fS[_q]) < 0) {
            R t = eS[_p]; eS[_p] = eS[_q]; eS[_q] = t;
            t = fS[_p]; fS[_p] = fS[_q]; fS[_q] = t;
            w0[l] = (R)-1;
          }
          else
            w0[l] = (R)1;
          gsp >>= 1u; gsn >>= 1u; trans >>= 1u; perm >>= 1u;
        }
      }
      /* apply */
      R nMG = (R)0, nMV = (R)-0.0;
      for (long long i = 0; i < n_2; ++i) {
        const long long _p = r[2 * i], _q = r[2 * i + 1];
        chg[_q] = chg[_p] = (R)0;
        R *const Grp = Gr + _p * ldG, *const Grq = Gr + _q * ldG;
        R *const Gip = (cx ? (Gi + _p * ldGI) : NULL), *const Giq = (cx ? (Gi + _q * ldGI) : NULL);
        R *const Vrp = Vr + _p * ldV, *const Vrq = Vr + _q * ldV;
        R *const Vip = (cx ? (Vi + _p * ldVI) : NULL), *const Viq = (cx ? (Vi + _q * ldVI) : NULL);
        const R code = w0[i];
        if ((code == (R)-3) || (code == (R)3)) {
          const long long mm = ((code < (R)0) ? -m : m);
          R tG;
          if (cx)
            tG = H(zgsscl)(mm, a21r[i], a21i[i], Grp, Gip, Grq, Giq, eS[_p], eS[_q], fS[_p], fS[_q]);
          else
            tG = H(gsscl)(mm, a21r[i], Grp, Grq, eS[_p], eS[_q], fS[_p], fS[_q]);
          if (!isfinite(tG)) { ret = E_APPG; goto theEnd; }
          nMG = (R)fmax((double)nMG, (double)tG);
          if (code < (R)0) {
            H(swp)(n, Vrp, Vrq);
            if (cx)
              H(swp)(n, Vip, Viq);
            nMV = (R)fmax((double)nMV, 0.0);
            R t = eS[_p]; eS[_p] = eS[_q]; eS[_q] = t;
            t = fS[_p]; fS[_p] = fS[_q]; fS[_q] = t;
          }
          else
            nMV = (R)fmax((double)nMV, 0.0);
          chg[_q] = (R)1;
        }
        else if ((code == (R)-2) || (code == (R)2)) {
          const long long mm = ((code < (R)0) ? -m : m), nn = ((code < (R)0) ? -n : n);
          R tG, tV;
          if (cx)
            tG = H(zjrot)(mm, Grp, Gip, Grq, Giq, c[i], cat[i], sat[i], 1);
          else
            tG = H(jrot)(mm, Grp, Grq, c[i], cat[i], 1);
          if (!isfinite(tG)) { ret = E_APPG; goto theEnd; }
          nMG = (R)fmax((double)nMG, (double)tG);
          if (cx)
            tV = H(zjrot)(nn, Vrp, Vip, Vrq, Viq, c[i], cat[i], sat[i], vtrack);
          else
            tV = H(jrot)(nn, Vrp, Vrq, c[i], cat[i], vtrack);
          if (!isfinite(tV)) { ret = E_APPV; goto theEnd; }
          nMV = (R)fmax((double)nMV, (double)tV);
          chg[_q] = chg[_p] = (R)1;
        }
        else if (code == (R)-1) {
          H(swp)(m, Grp, Grq);
          if (cx)
            H(swp)(m, Gip, Giq);
          nMG = (R)fmax((double)nMG, 0.0);
          H(swp)(n, Vrp, Vrq);
          if (cx)
            H(swp)(n, Vip, Viq);
          nMV = (R)fmax((double)nMV, 0.0);
        }
        else {
          nMG = (R)fmax((double)nMG, 0.0);
          nMV = (R)fmax((double)nMV, 0.0);
        }
      }
      MG = (R)fmax((double)MG, (double)nMG);
      MV = (R)fmax((double)MV, (double)nMV);
    }
    if (sw < 64u)
      vjo_trace_swt[sw] = swt;
    vjo_trace_nsw = sw + 1u;
    if (!swt)
      break;
    ++sw;
  }

  if (sw < *swp) {
    for (long long j = 0; j < n; ++j) {
      const R f_ = fS[j], s_ = -eS[j];
      for (long long i = 0; i < m; ++i) {
        Gr[j * ldG + i] = H(scalef)(Gr[j * ldG + i] / f_, s_);
        if (cx)
          Gi[j * ldGI + i] = H(scalef)(Gi[j * ldGI + i] / f_, s_);
      }
      eS[j] -= (R)sT;
    }
    if (sV) {
      const R s_ = (R)-sV;
      for (long long j = 0; j < n; ++j)
        for (long long i = 0; i < n; ++i) {
          Vr[j * ldV + i] = H(scalef)(Vr[j * ldV + i], s_);
          if (cx)
            Vi[j * ldVI + i] = H(scalef)(Vi[j * ldVI + i], s_);
        }
    }
  }
  ret = (long long)sw;
 theEnd:
  free(w);
  free(pb);
  free(chg);
  return ret;
}

long long RSVD(const unsigned long long *m, const unsigned long long *n, R *G, const unsigned long long *ldG, R *V, const unsigned long long *ldV, R *eS, R *fS, const unsigned *js, const unsigned *stp, const unsigned *swp, R *work, unsigned *iwork)
{
  return GSVD(0, m, n, G, ldG, NULL, NULL, V, ldV, NULL, NULL, eS, fS, js, stp, swp, work, iwork);
}

long long CSVD(const unsigned long long *m, const unsigned long long *n, R *Gr, const unsigned long long *ldGr, R *Gi, const unsigned long long *ldGi, R *Vr, const unsigned long long *ldVr, R *Vi, const unsigned long long *ldVi, R *eS, R *fS, const unsigned *js, const unsigned *stp, const unsigned *swp, R *work, unsigned *iwork)
{
  return GSVD(1, m, n, Gr, ldGr, Gi, ldGi, Vr, ldVr, Vi, ldVi, eS, fS, js, stp, swp, work, iwork);
}

#undef VJO_TWOSUM
#undef VJO_MUL2SUM
#undef VJO_ZFMA
