/*
 * wl_oracle_body.h -- precision-generic body of the CPU restatement.
 *
 * TEST INFRASTRUCTURE ONLY (see wl_oracle.h).  Included twice by wl_oracle.c:
 * once with REAL = double (the FP64 oracle) and once with REAL = float (the
 * reference formula as plain C, the timed CPU baseline).  Each function names
 * the reference lines it restates.
 */

/* Ei(x) = -E1(-x) for x < -1 by Lentz's continued fraction
 * (intEV.cu:29-61, intEVff.cu:19-49; returns 0 when it does not converge). */
static REAL SFX(expint)(REAL x) {
  const int maxit = 400;
  REAL b = -x + (REAL)1, c = (REAL)1.0e10, d = (REAL)1 / b, h = d;
  for (int i = 1; i <= maxit; i++) {
    REAL an = -(REAL)i * (REAL)i;
    b += (REAL)2;
    d = (REAL)1 / (an * d + b);
    c = b + an / c;
    REAL del = c * d;
    h *= del;
    if (FABS(del - (REAL)1) <= EXPINT_EPS) return -h * EXP(x);
  }
  return (REAL)0;
}

/* bump function (intEV.cu:151-159, intEVff.cu:134-139) */
static REAL SFX(bump)(REAL x) {
  if (x * x < (REAL)0.999) return EXP(-(REAL)1 / ((REAL)1 - x * x));
  return (REAL)0;
}

/* Phi of the fixflux profile: threshold 0.999 in intEV.cu:161-174,
 * 1.0 in intEVff.cu:147-157 */
static REAL SFX(phi)(REAL x, int ffv) {
  const REAL onemx2 = (REAL)1 - x * x;
  const REAL thr = ffv ? (REAL)1 : (REAL)0.999;
  if (x < thr)
    return (REAL)1 - ((REAL)0.5 / (REAL)WLO_Q2) *
                         (onemx2 * EXP(-(REAL)1 / onemx2) +
                          SFX(expint)(-(REAL)1 / onemx2));
  return (REAL)1;
}

/* Chi of the fixflux profile: intEV.cu:176-198 (logistic fit) or
 * intEVff.cu:159-176 (cosh-ratio fit) */
static REAL SFX(chi)(REAL x, REAL n, REAL lam, REAL a, int ffv) {
  const REAL onemx2 = (REAL)1 - x * x;
  const REAL x2 = x * x, x4 = x2 * x2;
  const REAL lo = ffv ? (REAL)-1 : (REAL)-0.999;
  const REAL hi = ffv ? (REAL)1 : (REAL)0.999;
  if (x <= lo) return (REAL)0;
  if (x2 < hi) {
    REAL ans = (REAL)0.5 * (-onemx2 * EXP(-(REAL)1 / onemx2) -
                            SFX(expint)(-(REAL)1 / onemx2));
    if (ffv)
      ans += (REAL)2 * n * a / lam *
             ((REAL)0.218 + (REAL)0.393 * x *
                                COSH((REAL)0.806 * x4 - (REAL)0.696 * x2 + (REAL)0.0902) /
                                COSH((REAL)0.825 * x2 - (REAL)0.0234 * x + (REAL)0.375));
    else
      ans += (REAL)2 * n * a / lam * (REAL)0.444 /
             ((REAL)1 + EXP(-((REAL)3.31 * x + (REAL)5.25 * x * x2 * SIN(x) *
                                                    COS(-(REAL)0.907 * x2 - (REAL)1.29 * x4 * x4)) /
                             COS(x)));
    return ans;
  }
  return (REAL)2 * n * a * (REAL)WLO_Q1 / lam;
}

/* periodic (radial shell) profile f_lambda (intEV.cu:201-232) */
static REAL SFX(flperi)(REAL rho2, REAL l2, REAL a) {
  const int N = 2;
  REAL rho = SQRT(rho2), lam = SQRT(l2);
  REAL flraf = FLOOR(rho / a), f = (REAL)0;
  if ((int)flraf - N > 0) f = (REAL)0.5 * (flraf - (REAL)N - (REAL)1) * (flraf - (REAL)N);
  for (int i = (int)flraf - N; i <= (int)flraf + N; i++) {
    if (i == 0) {
      REAL ex = EXP(-rho / lam), exp1 = (REAL)1 + ex;
      f = -rho / a * (ex / exp1) - lam / a * LOG(exp1);
    } else if (i > 0) {
      f = f + (REAL)i / ((REAL)1 + EXP(-(rho - (REAL)i * a) / lam));
    }
  }
  return a / (lam * LOG((REAL)2)) * f + (REAL)1;
}

/* periodic profile f'_lambda (intEV.cu:300-328) */
static REAL SFX(fplperi)(REAL rho2, REAL l2, REAL a) {
  const int N = 2;
  REAL rho = SQRT(rho2), lam = SQRT(l2);
  REAL flraf = FLOOR(rho / a), f = (REAL)0;
  for (int i = (int)flraf - N; i <= (int)flraf + N; i++) {
    if (i == 0) {
      REAL ex = EXP(-rho / lam), exp1 = (REAL)1 + ex;
      f = ex / (a * exp1 * exp1);
    } else if (i > 0) {
      REAL ea = EXP(-(rho - (REAL)i * a) / lam), ea1 = (REAL)1 + ea;
      f = f + ((REAL)i / rho) * ea / (ea1 * ea1);
    }
  }
  return a / ((REAL)2 * l2 * LOG((REAL)2)) * f;
}

/* fixflux profile f_lambda (intEV.cu:236-257, intEVff.cu:194-214) */
static REAL SFX(ffixflux)(REAL rho2, REAL l2, REAL a, REAL lmin, int ffv) {
  const REAL lam = SQRT(l2);
  const REAL lml = (lam - lmin) / (a - lmin);
  const REAL aml = (a - lam) / (a - lmin);
  const REAL n = FLOOR((SQRT(rho2) + a / (REAL)2) / a);
  if (rho2 <= a * a / (REAL)4)
    return ((REAL)1 - (REAL)0.75 * lml) * SFX(phi)((REAL)2 * SQRT(rho2 / l2), ffv) +
           (REAL)3 * rho2 / (a * a) * lml;
  REAL ans = (REAL)1 + (REAL)0.75 * ((REAL)4 * rho2 / (a * a) - (REAL)1) * lml +
             (REAL)3 * n * (n - (REAL)1) * aml;
  ans += (REAL)3 * lam / ((REAL)WLO_Q1 * a) * aml *
         SFX(chi)((REAL)2 * (SQRT(rho2) - n * a) / lam, n, lam, a, ffv);
  return ans;
}

/* fixflux profile f'_lambda (intEV.cu:333-357, intEVff.cu:224-250) */
static REAL SFX(fpfixflux)(REAL rho2, REAL l2, REAL a, REAL lmin) {
  const REAL lam = SQRT(l2);
  const REAL lml = (lam - lmin) / (a - lmin);
  const REAL rho = SQRT(rho2);
  const REAL n = FLOOR((rho + a / (REAL)2) / a);
  const REAL aml = (a - lam) / (a - lmin);
  const REAL bbg = (REAL)3 / (a * a) * lml;
  if (rho <= a / (REAL)2)
    return bbg + (REAL)2 / (l2 * (REAL)WLO_Q2) * ((REAL)1 - (REAL)0.75 * lml) *
                     SFX(bump)((REAL)2 * rho / lam);
  return bbg + (REAL)6 / ((REAL)WLO_Q1 * lam * a) * aml *
                   SFX(bump)((REAL)2 * (rho - n * a) / lam);
}

/* f_lambda(rho2) (intEV.cu:260-297) */
static REAL SFX(flambda)(REAL r2, const wlo_field *f) {
  const REAL l2 = (REAL)f->lambda2;
  switch (f->profile) {
    case WLO_STEP: return r2 < l2 ? r2 / l2 : (REAL)1;
    case WLO_SMOOTH: return r2 / (l2 + r2);
    case WLO_QUADRATIC: return r2 < l2 ? r2 / l2 * ((REAL)2 - r2 / l2) : (REAL)1;
    case WLO_GAUSSIAN: return GAUSS_1MEXP(r2 / l2);
    case WLO_PERIODIC: return SFX(flperi)(r2, l2, (REAL)f->tubedist);
    case WLO_SPLINE: return (REAL)spline_f((double)r2, f);
    case WLO_FIXFLUX:
      return SFX(ffixflux)(r2, l2, (REAL)f->tubedist, (REAL)f->lmin, f->ff_variant);
    default: return (REAL)0;
  }
}

/* f_lambda(rho2) / rho2, the scalar Simpson integrand.  For the closed-form
 * profiles the quotient is simplified algebraically (identical in exact
 * arithmetic and finite at rho2 = 0); the others divide. */
static REAL SFX(flrho2)(REAL r2, const wlo_field *f) {
  const REAL l2 = (REAL)f->lambda2;
  switch (f->profile) {
    case WLO_STEP: return r2 < l2 ? (REAL)1 / l2 : (REAL)1 / r2;
    case WLO_SMOOTH: return (REAL)1 / (l2 + r2);
    case WLO_QUADRATIC: return r2 < l2 ? ((REAL)2 - r2 / l2) / l2 : (REAL)1 / r2;
    case WLO_GAUSSIAN:
      return r2 > (REAL)0 ? GAUSS_1MEXP(r2 / l2) / r2 : (REAL)1 / l2;
    default: return SFX(flambda)(r2, f) / r2;
  }
}

/* f'_lambda(rho2) = d f / d rho2 (intEV.cu:360-406) */
static REAL SFX(fplambda)(REAL r2, const wlo_field *f) {
  const REAL l2 = (REAL)f->lambda2;
  switch (f->profile) {
    case WLO_STEP: return r2 < l2 ? (REAL)1 / l2 : (REAL)0;
    case WLO_SMOOTH: return l2 / ((l2 + r2) * (l2 + r2));
    case WLO_QUADRATIC: return r2 < l2 ? (REAL)2 / l2 * ((REAL)1 - r2 / l2) : (REAL)0;
    case WLO_GAUSSIAN: return (REAL)1 / l2 * EXP(-r2 / l2);
    case WLO_PERIODIC: return SFX(fplperi)(r2, l2, (REAL)f->tubedist);
    case WLO_SPLINE: return (REAL)spline_fp((double)r2, f);
    case WLO_FIXFLUX:
      return SFX(fpfixflux)(r2, l2, (REAL)f->tubedist, (REAL)f->lmin);
    default: return (REAL)0;
  }
}

/* composite Simpson over t in [0,1] of rho^2(t) = a + 2bt + ct^2
 * (intEV.cu:408-459).  The reference clamps a, b, c and the end value to
 * >= 1e-8 and interior values to >= 1e-10 (intEV.cu:418-422, 439); the exact
 * mode only keeps a 1e-30 floor for the profiles that divide by rho^2.      */
static void SFX(idt)(REAL a, REAL b, REAL c, const wlo_field *f, REAL *scalI,
                     REAL *fermI) {
  const int n = f->nint;
  const REAL h = (REAL)1 / (REAL)n;
  const int refc = (f->mode == WLO_REFCOMPAT);
  const int divides = !(f->profile == WLO_STEP || f->profile == WLO_SMOOTH ||
                        f->profile == WLO_QUADRATIC || f->profile == WLO_GAUSSIAN);
  const REAL floor_exact = divides ? (REAL)1e-30 : (REAL)0;
  if (refc) {
    if (a < (REAL)1.0e-8) a = (REAL)1.0e-8;
    if (b < (REAL)1.0e-8) b = (REAL)1.0e-8;
    if (c < (REAL)1.0e-8) c = (REAL)1.0e-8;
  }
  REAL ae = a + (REAL)2 * b + c;
  if (refc) {
    if (ae < (REAL)1.0e-8) ae = (REAL)1.0e-8;
  } else {
    if (a < floor_exact) a = floor_exact;
    if (ae < floor_exact) ae = floor_exact;
  }
  REAL sx = SFX(flrho2)(a, f) + SFX(flrho2)(ae, f), sy = 0, sz = 0;
  REAL fx = 0, fy = 0, fz = 0;
  if (f->fermion) fx = SFX(fplambda)(a, f) + SFX(fplambda)(ae, f);
  for (int i = 1; i < n; i++) {
    REAL t = (REAL)i * h;
    REAL r2 = a + (REAL)2 * b * t + c * t * t;
    if (refc) {
      if (r2 < (REAL)1.0e-10) r2 = (REAL)1.0e-10;
    } else if (r2 < floor_exact) {
      r2 = floor_exact;
    }
    if (i % 2 == 0) {
      sz += SFX(flrho2)(r2, f);
      if (f->fermion) fz += SFX(fplambda)(r2, f);
    } else {
      sy += SFX(flrho2)(r2, f);
      if (f->fermion) fy += SFX(fplambda)(r2, f);
    }
  }
  *scalI = (sx + (REAL)2 * sz + (REAL)4 * sy) * h / (REAL)3;
  *fermI = f->fermion ? (fx + (REAL)2 * fz + (REAL)4 * fy) * h / (REAL)3 : (REAL)0;
}

/* sub-loop successor of point i (intEV.cu:461-506): odd points form the N/2
 * loop, i = 0 mod 4 the first N/4 loop, i = 2 mod 4 the second.          */
static int SFX(succ)(int i, int ppl) {
  if (i % 2 == 1) return i == ppl - 1 ? 1 : i + 2;
  if (i % 4 == 0) return i == ppl - 4 ? 0 : i + 4;
  return i == ppl - 2 ? 2 : i + 4;
}

/* per-loop geometric sums (WilsonLoop, intEV.cu:508-552) with F = 1 */
static void SFX(loop_sums_impl)(const float *w, int ppl, REAL cx, REAL cy, REAL rtT,
                                const wlo_field *f, REAL gs[3], REAL gf[3]) {
  gs[0] = gs[1] = gs[2] = 0;
  gf[0] = gf[1] = gf[2] = 0;
  for (int i = 0; i < ppl; i++) {
    int j = SFX(succ)(i, ppl);
    REAL zix = cx + rtT * (REAL)w[4 * i], ziy = cy + rtT * (REAL)w[4 * i + 1];
    REAL zjx = cx + rtT * (REAL)w[4 * j], zjy = cy + rtT * (REAL)w[4 * j + 1];
    REAL a = zix * zix + ziy * ziy;
    REAL b = zix * (zjx - zix) + ziy * (zjy - ziy);
    REAL c = (zjx - zix) * (zjx - zix) + (zjy - ziy) * (zjy - ziy);
    REAL sI, fI;
    SFX(idt)(a, b, c, f, &sI, &fI);
    REAL xyyx = zix * zjy - ziy * zjx;
    int k = (i % 2 == 1) ? 0 : ((i % 4 == 0) ? 2 : 1);
    gs[k] += xyyx * sI;
    gf[k] += fI;
  }
}
