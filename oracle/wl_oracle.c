/*
 * wl_oracle.c -- CPU restatement of the reference's Wilson-loop path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU library (tests, smoke
 * check, CPU-baseline leg of the benchmark).  Never linked by the product.
 * Function-level citations are in wl_oracle.h and wl_oracle_body.h.
 *
 * Build: gcc -O2 -fPIC -shared -fopenmp -ffp-contract=off wl_oracle.c -lm
 * (contraction off so that x86 and Arm builds round identically).
 */
#include "wl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define WLO_Q1 0.443991  /* fixflux constants (analysis-scripts/EAscffvsconst.sage:6-7) */
#define WLO_Q2 0.0742478

/* ------------------------------------------------------ spline profile -- */
/* periodic.c:17-164: f(rho) = int_0^rho (2/lambda^2) s exp(-sin^2(pi s/a)/
 * lambda^2) ds at the knots rho_i = i h, i = 1..n, h = 20/n (the reference
 * steps an 8th-order Runge-Kutta; here: composite Simpson with 256
 * sub-intervals per step), then the clamped cubic spline with zero end slopes
 * in x = rho^2 at the knots rounded to float (periodic.c:46-110; here in the
 * second-derivative form, solved by the Thomas algorithm).  interp
 * (intEV.cu:64-107) gives 0 outside (x_0, x_{n-1}).  One table is kept, for
 * the last (lambda^2, a).                                                      */
static struct {
  double l2, a;
  int n;
  double *x, *f, *M;
} g_sp = {0, 0, 0, NULL, NULL, NULL};

static void spline_build(double l2, double a, int n) {
  if (g_sp.n == n && g_sp.l2 == l2 && g_sp.a == a) return;
  free(g_sp.x);
  free(g_sp.f);
  free(g_sp.M);
  g_sp.x = (double *)malloc(sizeof(double) * n);
  g_sp.f = (double *)malloc(sizeof(double) * n);
  g_sp.M = (double *)malloc(sizeof(double) * n);
  const double h = 20.0 / n;
  const int sub = 256;
  double acc = 0.0;
  for (int i = 0; i < n; i++) {
    const double lo = i * h, dh = h / sub;
    double s = 0.0;
    for (int k = 0; k <= sub; k++) {
      const double t = lo + k * dh, sn = sin(M_PI * t / a);
      const double v = 2.0 / l2 * t * exp(-sn * sn / l2);
      s += (k == 0 || k == sub) ? v : (k % 2 ? 4.0 * v : 2.0 * v);
    }
    acc += s * dh / 3.0;
    const double r = (i + 1) * h;
    g_sp.x[i] = (double)(float)(r * r);
    g_sp.f[i] = acc;
  }
  /* second derivatives M: h_{i-1} M_{i-1} + 2 (h_{i-1} + h_i) M_i + h_i M_{i+1}
   * = 6 (slope_i - slope_{i-1}), with S'(x_0) = S'(x_{n-1}) = 0 at the ends */
  double *dg = (double *)malloc(sizeof(double) * n), *up = (double *)malloc(sizeof(double) * n);
  double *lo = (double *)malloc(sizeof(double) * n), *rhs = (double *)malloc(sizeof(double) * n);
  for (int i = 0; i < n; i++) {
    const double hl = i > 0 ? g_sp.x[i] - g_sp.x[i - 1] : 0.0;
    const double hr = i < n - 1 ? g_sp.x[i + 1] - g_sp.x[i] : 0.0;
    const double sl = i > 0 ? (g_sp.f[i] - g_sp.f[i - 1]) / hl : 0.0;
    const double sr = i < n - 1 ? (g_sp.f[i + 1] - g_sp.f[i]) / hr : 0.0;
    lo[i] = hl;
    dg[i] = 2.0 * (hl + hr);
    up[i] = hr;
    rhs[i] = 6.0 * (sr - sl);
  }
  for (int i = 1; i < n; i++) { /* forward elimination */
    const double m = lo[i] / dg[i - 1];
    dg[i] -= m * up[i - 1];
    rhs[i] -= m * rhs[i - 1];
  }
  g_sp.M[n - 1] = rhs[n - 1] / dg[n - 1];
  for (int i = n - 2; i >= 0; i--) g_sp.M[i] = (rhs[i] - up[i] * g_sp.M[i + 1]) / dg[i];
  free(dg);
  free(up);
  free(lo);
  free(rhs);
  g_sp.l2 = l2;
  g_sp.a = a;
  g_sp.n = n;
}

/* builds the table before any parallel region reads it */
static void spline_prepare(const wlo_field *fl) {
  if (fl->profile == WLO_SPLINE) spline_build(fl->lambda2, fl->tubedist, 1000);
}

static double spline_f(double r2, const wlo_field *fl) {
  /* parallel callers prepared the table; single-threaded ones may build here */
  if (g_sp.n != 1000 || g_sp.l2 != fl->lambda2 || g_sp.a != fl->tubedist)
    spline_build(fl->lambda2, fl->tubedist, 1000);
  const int n = g_sp.n;
  const double *x = g_sp.x;
  if (!(r2 < x[n - 1] && r2 > x[0])) return 0.0;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (r2 >= x[mid]) lo = mid;
    else hi = mid;
  }
  const double h = x[hi] - x[lo], A = (x[hi] - r2) / h, B = (r2 - x[lo]) / h;
  return A * g_sp.f[lo] + B * g_sp.f[hi] +
         ((A * A * A - A) * g_sp.M[lo] + (B * B * B - B) * g_sp.M[hi]) * h * h / 6.0;
}

/* f' of the spline profile: the reference kernel's sin(pi sqrt(rho2))
 * (intEV.cu:389-397, no tube spacing) in ref-compat mode, the derivative of
 * the tabulated f, sin(pi sqrt(rho2)/a), in exact mode */
static double spline_fp(double r2, const wlo_field *fl) {
  const double arg = fl->mode == WLO_EXACT ? M_PI / fl->tubedist : M_PI;
  const double s = sin(sqrt(r2) * arg);
  return exp(-s * s / fl->lambda2) / fl->lambda2;
}

void wlo_spline_table(double lambda2, double a, int n, double *x, double *f) {
  spline_build(lambda2, a, n);
  memcpy(x, g_sp.x, sizeof(double) * n);
  memcpy(f, g_sp.f, sizeof(double) * n);
}

double wlo_spline_eval(double r2, const wlo_field *fl) {
  spline_prepare(fl);
  return spline_f(r2, fl);
}

/* ---------------------------------------------------------------- FP64 -- */
#define REAL double
#define SFX(name) d_##name
#define EXP exp
#define LOG log
#define SQRT sqrt
#define FLOOR floor
#define FABS fabs
#define COS cos
#define SIN sin
#define COSH cosh
/* 1 - exp(-x) without cancellation */
#define GAUSS_1MEXP(x) (-expm1(-(x)))
#define EXPINT_EPS 1.0e-15
#include "wl_oracle_body.h"
#undef REAL
#undef SFX
#undef EXP
#undef LOG
#undef SQRT
#undef FLOOR
#undef FABS
#undef COS
#undef SIN
#undef COSH
#undef GAUSS_1MEXP
#undef EXPINT_EPS

/* ---------------------------------------------------------------- FP32 -- */
#define REAL float
#define SFX(name) f_##name
#define EXP expf
#define LOG logf
#define SQRT sqrtf
#define FLOOR floorf
#define FABS fabsf
#define COS cosf
#define SIN sinf
#define COSH coshf
/* the reference evaluates 1 - exp(-x) literally (intEV.cu:283) */
#define GAUSS_1MEXP(x) (1.0f - expf(-(x)))
#define EXPINT_EPS 1.0e-6f
#include "wl_oracle_body.h"

/* ------------------------------------------------------------ exports -- */
double wlo64_flambda(double rho2, const wlo_field *f) {
  spline_prepare(f);
  return d_flambda(rho2, f);
}
double wlo64_fplambda(double rho2, const wlo_field *f) { return d_fplambda(rho2, f); }
double wlo64_fl_over_rho2(double rho2, const wlo_field *f) {
  spline_prepare(f);
  return d_flrho2(rho2, f);
}

void wlo64_idt(double a, double b, double c, const wlo_field *f, double *scalI,
               double *fermI) {
  d_idt(a, b, c, f, scalI, fermI);
}

/* square lattice of Gaussian tubes (see wl_oracle.h) */
static double g_lattice_rcut = WLO_LATTICE_RCUT_L;

void wlo_set_lattice_rcut(double r_over_lambda) { g_lattice_rcut = r_over_lambda; }

static void d_lattice_sums(const float *w, int ppl, double cx, double cy, double rtT,
                           const wlo_field *f, double gs[3], double gf[3]) {
  wlo_field g = *f;
  g.profile = WLO_GAUSSIAN;
  g.mode = WLO_EXACT;
  const double a = f->tubedist, rcut = g_lattice_rcut * sqrt(f->lambda2);
  double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
  for (int i = 0; i < ppl; i++) {
    double x = cx + rtT * (double)w[4 * i], y = cy + rtT * (double)w[4 * i + 1];
    xmin = fmin(xmin, x);
    xmax = fmax(xmax, x);
    ymin = fmin(ymin, y);
    ymax = fmax(ymax, y);
  }
  const double rr = f->rimage / a;
  int m0 = (int)ceil((xmin - rcut) / a), m1 = (int)floor((xmax + rcut) / a);
  int n0 = (int)ceil((ymin - rcut) / a), n1 = (int)floor((ymax + rcut) / a);
  if (g_lattice_rcut <= 0.0) m0 = n0 = -(int)floor(rr), m1 = n1 = (int)floor(rr);
  gs[0] = gs[1] = gs[2] = 0;
  gf[0] = gf[1] = gf[2] = 0;
  for (int m = m0; m <= m1; m++)
    for (int n = n0; n <= n1; n++) {
      if ((double)m * m + (double)n * n > rr * rr * (1.0 + 1e-12)) continue;
      double s3[3], f3[3];
      d_loop_sums_impl(w, ppl, cx - m * a, cy - n * a, rtT, &g, s3, f3);
      for (int k = 0; k < 3; k++) {
        gs[k] += s3[k];
        gf[k] += f3[k];
      }
    }
}

static void d_sums(const float *w, int ppl, double cx, double cy, double rtT, const wlo_field *f,
                   double gs[3], double gf[3]) {
  if (f->profile == WLO_LATTICE)
    d_lattice_sums(w, ppl, cx, cy, rtT, f, gs, gf);
  else
    d_loop_sums_impl(w, ppl, cx, cy, rtT, f, gs, gf);
}

void wlo64_loop_sums(const float *loop, int ppl, double cx, double cy, double rtT,
                     const wlo_field *f, double gs[3], double gf[3]) {
  d_sums(loop, ppl, cx, cy, rtT, f, gs, gf);
}

void wlo32_loop_sums(const float *loop, int ppl, float cx, float cy, float rtT,
                     const wlo_field *f, float gs[3], float gf[3]) {
  f_loop_sums_impl(loop, ppl, cx, cy, rtT, f, gs, gf);
}

/* Wsscal / Wsferm (intEV.cu:553-561): the N/2 exponent is normalised by
 * N/2 segments, the N/4 ones by N/4. */
static void finish_loop(const double gs[3], const double gf[3], double T, double F,
                        int ppl, double scal[3], double ferm[3]) {
  for (int k = 0; k < 3; k++) scal[k] = F * gs[k];
  ferm[0] = 2.0 * F * gf[0] * T / (ppl / 2.0);
  ferm[1] = 2.0 * F * gf[1] * T / (ppl / 4.0);
  ferm[2] = 2.0 * F * gf[2] * T / (ppl / 4.0);
}

void wlo64_loops(const float *loops, int Nl, int ppl, double cx, double cy, double T,
                 double F, const wlo_field *f, double *scal, double *ferm) {
  const double rtT = sqrt(T);
  spline_prepare(f);
#pragma omp parallel for schedule(dynamic, 4)
  for (int l = 0; l < Nl; l++) {
    double gs[3], gf[3];
    d_sums(loops + (size_t)l * ppl * 4, ppl, cx, cy, rtT, f, gs, gf);
    finish_loop(gs, gf, T, F, ppl, scal + 3 * l, ferm + 3 * l);
  }
}

/* C abs() of a double converts it to int (Integrand.c:371): the sentinel
 * fires when |trunc(x)| > 600, i.e. |x| >= 601.  Out-of-range conversions
 * follow x86 (INT_MIN, so no sentinel), the reference's platform.         */
static int sentinel600(double x) {
  double ax = fabs(x);
  return ax >= 601.0 && ax < 2147483648.0;
}

void wlo64_wfactors(const double s[3], const double fm[3], int fermion, double w[3]) {
  double nb4 = s[1] + s[2];
  w[0] = cos(0.5 * s[0] + 0.25 * nb4);
  w[1] = cos(s[0]);
  w[2] = cos(0.5 * nb4);
  if (fermion) {
    double nb4f = fm[1] + fm[2];
    if (sentinel600(nb4f) || sentinel600(fm[0])) {
      w[0] *= 1.0e10;
      w[1] *= 1.0e10;
      w[2] *= 1.0e10;
    } else {
      w[0] *= cosh(0.5 * fm[0] + 0.25 * nb4f);
      w[1] *= cosh(fm[0]);
      w[2] *= cosh(0.5 * nb4f);
    }
  }
}

double wlo64_evmean(const double *scal, const double *ferm, int n, const int *WL,
                    int fermion) {
  double s1 = 0, s2 = 0, s4 = 0;
  for (int i = 0; i < n; i++) {
    double w[3];
    wlo64_wfactors(scal + 3 * WL[i], ferm + 3 * WL[i], fermion, w);
    s1 += w[0];
    s2 += w[1];
    s4 += w[2];
  }
  s1 /= n;
  s2 /= n;
  s4 /= n;
  return 8.0 / 3.0 * s1 - 2.0 * s2 + 1.0 / 3.0 * s4;
}

static void eval_generic(int fp32, const float *loops, int Nl, int ppl, int ninst,
                         const double *cx, const double *cy, const double *T, int nF,
                         const double *F, const wlo_field *f, int group, double *out,
                         double *scale, int nthreads) {
  const int ng = Nl / group;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif
  spline_prepare(f);
  /* one task per (instance, group); loops of a group are summed in order */
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (long task = 0; task < (long)ninst * ng; task++) {
    const int i = (int)(task / ng), g = (int)(task % ng);
    double acc[16][3], aab[16][3];
    memset(acc, 0, sizeof(acc));
    memset(aab, 0, sizeof(aab));
    const double rtT = sqrt(T[i]);
    for (int l = g * group; l < (g + 1) * group; l++) {
      double gs[3], gf[3];
      const float *w = loops + (size_t)l * ppl * 4;
      if (fp32) {
        float s32[3], f32[3];
        f_loop_sums_impl(w, ppl, (float)cx[i], (float)cy[i], (float)rtT, f, s32, f32);
        for (int k = 0; k < 3; k++) {
          gs[k] = s32[k];
          gf[k] = f32[k];
        }
      } else {
        d_sums(w, ppl, cx[i], cy[i], rtT, f, gs, gf);
      }
      for (int j = 0; j < nF && j < 16; j++) {
        double s[3], fm[3], wv[3];
        finish_loop(gs, gf, T[i], F[j], ppl, s, fm);
        wlo64_wfactors(s, fm, f->fermion, wv);
        for (int k = 0; k < 3; k++) {
          acc[j][k] += wv[k];
          aab[j][k] += fabs(wv[k]);
        }
      }
    }
    for (int j = 0; j < nF && j < 16; j++) {
      double m1 = acc[j][0] / group, m2 = acc[j][1] / group, m4 = acc[j][2] / group;
      out[((size_t)i * nF + j) * ng + g] = 8.0 / 3.0 * m1 - 2.0 * m2 + 1.0 / 3.0 * m4;
      if (scale)
        scale[((size_t)i * nF + j) * ng + g] =
            (8.0 / 3.0 * aab[j][0] + 2.0 * aab[j][1] + 1.0 / 3.0 * aab[j][2]) / group;
    }
  }
}

void wlo64_eval(const float *loops, int Nl, int ppl, int ninst, const double *cx,
                const double *cy, const double *T, int nF, const double *F,
                const wlo_field *f, int group, double *out, double *scale, int nthreads) {
  eval_generic(0, loops, Nl, ppl, ninst, cx, cy, T, nF, F, f, group, out, scale, nthreads);
}

void wlo32_eval(const float *loops, int Nl, int ppl, int ninst, const double *cx,
                const double *cy, const double *T, int nF, const double *F,
                const wlo_field *f, int group, double *out, double *scale, int nthreads) {
  eval_generic(1, loops, Nl, ppl, ninst, cx, cy, T, nF, F, f, group, out, scale, nthreads);
}

/* ------------------------------------------------ proper-time integrand -- */
static double d_bumpd(double x) {
  /* Integrand.c:39-46: abs(x) < 1.0 on a double truncates to int first */
  if (fabs(x) < 1.0) return exp(-1.0 / (1.0 - x * x));
  return 0.0;
}

/* Integrand.c:48-56; l and lmlmin are floats there, so they are rounded to
 * float here too (the constant-field integrand cancels catastrophically in B) */
static double d_fixfluxB(double rho2, const wlo_field *f) {
  double a = f->tubedist;
  float lf = (float)sqrt(f->lambda2), af = (float)a, lminf = (float)f->lmin;
  double lml = (float)((lf - lminf) / (af - lminf));
  return 2.0 / (f->lambda2 * WLO_Q2) * (1.0 - 0.75 * lml) *
             d_bumpd(2.0 * sqrt(rho2 / f->lambda2)) +
         3.0 / (a * a) * lml;
}

/* Integrand.c:58-96.  "abs(fmod(rho, a)) < 1e-6" truncates to int, so the
 * branch is taken whenever fmod(rho, a) < 1. */
static double d_periodicB(double rho2, const wlo_field *fl) {
  double a = fl->tubedist, l2 = fl->lambda2;
  double rho = sqrt(rho2), lam = sqrt(l2), f;
  double expr = exp(-rho / lam), flraf = floor(rho / a), ceilraf = ceil(rho / a);
  if (rho < a) {
    double expral = 0.0;
    if ((a - rho) / lam < 10.0) expral = exp(-(rho - a) / lam);
    f = expr / (a * (1.0 + expr) * (1.0 + expr));
    if (rho > 0.0) f += expral / (rho * (1.0 + expral) * (1.0 + expral));
  } else {
    if (fabs(fmod(rho, a)) < 1.0) {
      f = flraf / (4.0 * rho);
    } else {
      double ea = exp(-(rho - flraf * a) / lam), eb = exp(-(rho - ceilraf * a) / lam);
      f = flraf * ea / (rho * (1.0 + ea) * (1.0 + ea)) +
          ceilraf * eb / (rho * (1.0 + eb) * (1.0 + eb));
    }
  }
  return a / (2.0 * log(2.0) * l2) * f;
}

/* Integrand.c:98-140 */
double wlo_magfield(double rho2, double F, const wlo_field *f, const wlo_qed *q) {
  double B = 0.0, l2 = f->lambda2;
  switch (f->profile) {
    case WLO_STEP: B = rho2 < l2 ? 1.0 / l2 : 0.0; break;
    case WLO_SMOOTH: B = l2 / ((l2 + rho2) * (l2 + rho2)); break;
    case WLO_QUADRATIC: B = rho2 < l2 ? 2.0 / l2 * (1.0 - rho2 / l2) : 0.0; break;
    case WLO_GAUSSIAN: B = rho2 < 100.0 * l2 ? 1.0 / (l2 * exp(rho2 / l2)) : 0.0; break;
    case WLO_PERIODIC: B = d_periodicB(rho2, f); break;
    case WLO_SPLINE: {  /* Integrand.c:128-131 */
      const double sr = sin(M_PI * sqrt(rho2) / f->tubedist);
      B = 1.0 / (l2 * exp(sr * sr / l2));
      break;
    }
    case WLO_FIXFLUX: B = d_fixfluxB(rho2, f); break;
    case WLO_LATTICE: {
      /* no reference: the images' Gaussian fields at (sqrt(rho2), 0) */
      const double a = f->tubedist, rr = f->rimage / a, x = sqrt(rho2);
      const int lim = (int)floor(rr);
      for (int m = -lim; m <= lim; m++)
        for (int n = -lim; n <= lim; n++) {
          if ((double)m * m + (double)n * n > rr * rr * (1.0 + 1e-6)) continue;
          double dx = x - m * a, dy = -n * a, d2 = dx * dx + dy * dy;
          if (d2 < 40.0 * l2) B += exp(-d2 / l2) / l2;
        }
      break;
    }
    default: B = 0.0;
  }
  return 2.0 * F / q->e * B;
}

/* Integrand.c:20-37 */
double wlo_exact(double T, double B, int fermion, const wlo_qed *q) {
  double TB = q->e * T * B;
  if (B < 1.0e-40) return 0.0;
  if (fermion) return exp(-q->m2 * T) / (T * T * T) * (TB / tanh(TB) - 1.0 - TB * TB / 3.0);
  if (TB < 50.0) return exp(-q->m2 * T) / (T * T * T) * (TB / sinh(TB) - 1.0 + TB * TB / 6.0);
  return exp(-q->m2 * T) / (T * T * T) * (TB * TB / 6.0 - 1.0);
}

/* Integrand.c:142-155 */
double wlo_smTscal(double B, double T, const wlo_qed *q) {
  double B2 = q->e * q->e * B * B, B4 = B2 * B2, B6 = B2 * B4, m2 = q->m2;
  double T3 = T * T * T, T4 = T3 * T;
  return 7.0 / 360.0 * B4 * T * (1.0 - m2 * T) + (147.0 * B4 * m2 * m2 - 31.0 * B6) / 15120.0 * T3 +
         (31.0 * B6 * m2 - 49.0 * B4 * m2 * m2 * m2) / 15120.0 * T4;
}

/* Integrand.c:157-172 */
double wlo_smTferm(double B, double T, const wlo_qed *q) {
  double B2 = q->e * q->e * B * B, B4 = B2 * B2, B6 = B2 * B4, m2 = q->m2;
  double T3 = T * T * T, T4 = T3 * T;
  return 1.0 / 45.0 * B4 * T * (m2 * T - 1.0) + (2.0 * B6 / 945.0 - B4 * m2 * m2 / 90.0) * T3 +
         (7.0 * B4 * m2 * m2 * m2 - 4.0 * B6 * m2) / 1890.0 * T4;
}

/* regime selection of Tfunc (Integrand.c:215-288) */
int wlo_tfunc_regime(double T, double xcmx, double xcmy, double F, const wlo_field *f,
                     const wlo_qed *q, double *analytic) {
  double rho2 = xcmx * xcmx + xcmy * xcmy, rho = xcmx, l2 = f->lambda2, smallT = 0.0;
  double B = wlo_magfield(rho2, F, f, q), TB = q->e * T * B;
  switch (f->profile) {
    case WLO_STEP: smallT = (double)abs((int)(rho * rho - l2)); break;
    case WLO_SMOOTH:
    case WLO_QUADRATIC:
    case WLO_PERIODIC: smallT = 0.5 * (l2 + rho * rho); break;
    case WLO_GAUSSIAN:
    case WLO_LATTICE: smallT = l2; break;
    case WLO_SPLINE: {  /* Integrand.c:209, 236-240 */
      const double a = f->tubedist, s2 = sin(2.0 * M_PI * rho / a);
      smallT = rho / a > 1.0e-8 ? a * a * l2 / (M_PI * M_PI * s2 * s2) : 1.0e12;
      break;
    }
    case WLO_FIXFLUX:
      smallT = rho * rho < l2 / 4.0 ? 0.25 * l2
                                    : 0.25 * l2 + (rho - sqrt(l2) / 2.0) * (rho - sqrt(l2) / 2.0);
      break;
    default: smallT = 0.0;
  }
  if (T < 0.1 && T < 0.01 * smallT) {
    *analytic = f->fermion ? wlo_smTferm(B, T, q) : wlo_smTscal(B, T, q);
    return 0;
  }
  if (T < 0.01 * smallT) {
    *analytic = TB > 1.0e-6 ? wlo_exact(T, B, f->fermion, q) : 0.0;
    return 1;
  }
  if (T > 49.0) {
    *analytic = f->fermion ? -1.0 * exp(-q->m2 * T) / (3.0 * T) * q->e * q->e * B * B
                           : exp(-q->m2 * T) / (6.0 * T) * q->e * q->e * B * B;
    return 2;
  }
  *analytic = 0.0;
  return 3;
}

/* Integrand.c:298-301 */
double wlo_tfunc_mc(double T, double EVg, double xcmx, double xcmy, double F,
                    const wlo_field *f, const wlo_qed *q) {
  double rho2 = xcmx * xcmx + xcmy * xcmy;
  double B = wlo_magfield(rho2, F, f, q), TB = q->e * T * B;
  if (f->fermion) return exp(-q->m2 * T) / (T * T * T) * (EVg - 1.0 - 1.0 / 3.0 * TB * TB);
  return exp(-q->m2 * T) / (T * T * T) * (EVg - 1.0 + 1.0 / 6.0 * TB * TB);
}

/* transformT + Tfunc for all groups at t (Tint.c:15-33) */
static void tfunc_groups(double t, const float *loops, int ppl, int ng, double xcmx,
                         double xcmy, double F, const wlo_field *f, const wlo_qed *q,
                         double *out, int nthreads) {
  const double T = (1.0 - t) / t;
  double an;
  int reg = wlo_tfunc_regime(T, xcmx, xcmy, F, f, q, &an);
  if (reg != 3) {
    for (int g = 0; g < ng; g++) out[g] = an / t / t;
    return;
  }
  double cx = xcmx, cy = xcmy, TT = T, FF = F;
  wlo64_eval(loops, ng * 128, ppl, 1, &cx, &cy, &TT, 1, &FF, f, 128, out, NULL, nthreads);
  for (int g = 0; g < ng; g++) out[g] = wlo_tfunc_mc(T, out[g], xcmx, xcmy, F, f, q) / t / t;
}

/* Tint.c:100-175.  The reference evaluates its "t" and "t+1" Simpson points
 * at the same abscissa h*(inx+1) (Tint.c:127-130); that rule is reproduced. */
void wlo64_integrateT(const float *loops, int Nl, int ppl, int n, int ng, double xcmx,
                      double xcmy, double F, const wlo_field *f, const wlo_qed *q,
                      double *val, double *leff, double *sem, int nthreads) {
  (void)Nl;
  spline_prepare(f);
  const double h = 1.0 / (double)n;
  double *trt = (double *)malloc(sizeof(double) * ng);
  double *trh = (double *)malloc(sizeof(double) * ng);
  for (int g = 0; g < ng; g++) val[g] = 0.0;
  for (int inx = 0; inx < n; inx++) {
    tfunc_groups(h * ((double)inx + 1.0), loops, ppl, ng, xcmx, xcmy, F, f, q, trt, nthreads);
    tfunc_groups(h * ((double)inx + 0.5), loops, ppl, ng, xcmx, xcmy, F, f, q, trh, nthreads);
    for (int g = 0; g < ng; g++) {
      double a = isinf(trt[g]) ? 0.0 : trt[g];
      double b = isinf(trh[g]) ? 0.0 : trh[g];
      val[g] += h / 6.0 * (a + 4.0 * b + a);
    }
  }
  /* Tintout (Tint.c:51-73) */
  double avg = 0.0, s = 0.0;
  for (int g = 0; g < ng; g++) avg += val[g];
  avg /= ng;
  for (int g = 0; g < ng; g++) s += (val[g] - avg) * (val[g] - avg);
  s = sqrt(s / ((double)ng * ((double)ng - 1.0)));
  if (f->fermion) {
    *leff = avg / (4.0 * M_PI);
    *sem = s / (4.0 * M_PI);
  } else {
    *leff = avg / (-2.0 * M_PI);
    *sem = s / (2.0 * M_PI);
  }
  free(trt);
  free(trh);
}

/* ------------------------------------------------------ loop ensemble -- */
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

void wlo_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

#define WLO_VLOOP_TAG 0x764C6F6Fu /* "vLoo" */

void wlo_vloops(uint64_t seed, int first, int Nl, int ppl, float *out) {
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  const double sigma = sqrt(2.0 / (double)ppl);
  const double two32 = 4294967296.0;
#pragma omp parallel for schedule(static)
  for (int l = 0; l < Nl; l++) {
    double *x = (double *)malloc(sizeof(double) * 4 * (size_t)ppl);
    double y[4] = {0, 0, 0, 0};
    for (int k = 0; k < ppl; k++) {
      uint32_t ctr[4] = {(uint32_t)k, (uint32_t)(first + l), WLO_VLOOP_TAG, 0u}, r[4];
      wlo_philox4x32(ctr, key, r);
      double nrm[4];
      for (int p = 0; p < 2; p++) {
        double u = ((double)r[2 * p] + 0.5) / two32;
        double v = ((double)r[2 * p + 1] + 0.5) / two32;
        double rad = sqrt(-2.0 * log(u)), th = 2.0 * M_PI * v;
        nrm[2 * p] = rad * cos(th);
        nrm[2 * p + 1] = rad * sin(th);
      }
      for (int d = 0; d < 4; d++) {
        x[4 * k + d] = y[d];
        y[d] += sigma * nrm[d];
      }
    }
    /* bridge: remove the closing displacement linearly, then the mean */
    double mean[4] = {0, 0, 0, 0};
    for (int k = 0; k < ppl; k++)
      for (int d = 0; d < 4; d++) {
        x[4 * k + d] -= ((double)k / (double)ppl) * y[d];
        mean[d] += x[4 * k + d];
      }
    for (int d = 0; d < 4; d++) mean[d] /= (double)ppl;
    float *o = out + (size_t)l * ppl * 4;
    for (int k = 0; k < ppl; k++)
      for (int d = 0; d < 4; d++) o[4 * k + d] = (float)(x[4 * k + d] - mean[d]);
    free(x);
  }
}
