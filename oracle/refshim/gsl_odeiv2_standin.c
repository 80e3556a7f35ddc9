/* The stand-in of oracle/refshim/gsl/gsl_odeiv2.h: quadrature steps for
 * y-independent right-hand sides (see that header).  Test infrastructure
 * for oracle/_ref only. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "gsl/gsl_errno.h"
#include "gsl/gsl_odeiv2.h"

static const gsl_odeiv2_step_type rk8pd_standin = {"rk8pd (stand-in: Gauss-Legendre 10)"};
const gsl_odeiv2_step_type *gsl_odeiv2_step_rk8pd = &rk8pd_standin;

enum { kGL = 10 };
static double gl_x[kGL], gl_w[kGL];
static int gl_ready;

/* nodes and weights on [-1, 1]: Newton on P_n from Chebyshev guesses */
static void gl_init(void) {
  if (gl_ready) return;
  for (int i = 0; i < kGL; ++i) {
    double z = cos(M_PI * (i + 0.75) / (kGL + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= kGL; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = kGL * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    gl_x[i] = z;
    gl_w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  gl_ready = 1;
}

gsl_odeiv2_step *gsl_odeiv2_step_alloc(const gsl_odeiv2_step_type *T, size_t dim) {
  gsl_odeiv2_step *s = (gsl_odeiv2_step *)malloc(sizeof(*s));
  s->type = T;
  s->dimension = dim;
  return s;
}
void gsl_odeiv2_step_free(gsl_odeiv2_step *s) { free(s); }

gsl_odeiv2_control *gsl_odeiv2_control_y_new(double eps_abs, double eps_rel) {
  gsl_odeiv2_control *c = (gsl_odeiv2_control *)malloc(sizeof(*c));
  c->eps_abs = eps_abs;
  c->eps_rel = eps_rel;
  return c;
}
void gsl_odeiv2_control_free(gsl_odeiv2_control *c) { free(c); }

gsl_odeiv2_evolve *gsl_odeiv2_evolve_alloc(size_t dim) {
  gsl_odeiv2_evolve *e = (gsl_odeiv2_evolve *)malloc(sizeof(*e));
  e->dimension = dim;
  e->f0 = (double *)malloc(dim * sizeof(double));
  e->f1 = (double *)malloc(dim * sizeof(double));
  e->yt = (double *)malloc(dim * sizeof(double));
  return e;
}
void gsl_odeiv2_evolve_free(gsl_odeiv2_evolve *e) {
  free(e->f0);
  free(e->f1);
  free(e->yt);
  free(e);
}

/* y += integral of f over [t0, t0 + h]; GSL_FAILURE if f depends on y */
static int quad_step(gsl_odeiv2_evolve *e, const gsl_odeiv2_system *sys, double t0, double h,
                     double y[]) {
  const size_t n = sys->dimension;
  gl_init();
  if (sys->function(t0, y, e->f0, sys->params) != GSL_SUCCESS) return GSL_FAILURE;
  for (size_t i = 0; i < n; ++i) e->yt[i] = y[i] + 1.0;
  if (sys->function(t0, e->yt, e->f1, sys->params) != GSL_SUCCESS) return GSL_FAILURE;
  for (size_t i = 0; i < n; ++i)
    if (e->f0[i] != e->f1[i]) {
      fprintf(stderr, "gsl_odeiv2 stand-in: the right-hand side depends on y\n");
      return GSL_FAILURE;
    }
  double acc[16] = {0.0};
  if (n > 16) return GSL_FAILURE;
  for (int k = 0; k < kGL; ++k) {
    if (sys->function(t0 + 0.5 * h * (1.0 + gl_x[k]), y, e->f1, sys->params) != GSL_SUCCESS)
      return GSL_FAILURE;
    for (size_t i = 0; i < n; ++i) acc[i] += gl_w[k] * e->f1[i];
  }
  for (size_t i = 0; i < n; ++i) y[i] += 0.5 * h * acc[i];
  return GSL_SUCCESS;
}

int gsl_odeiv2_evolve_apply_fixed_step(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con,
                                       gsl_odeiv2_step *step, const gsl_odeiv2_system *sys,
                                       double *t, const double h, double y[]) {
  (void)con;
  (void)step;
  const double t0 = *t;
  const int st = quad_step(e, sys, t0, h, y);
  if (st != GSL_SUCCESS) return st;
  *t = t0 + h;
  return GSL_SUCCESS;
}

int gsl_odeiv2_evolve_apply(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con,
                            gsl_odeiv2_step *step, const gsl_odeiv2_system *sys, double *t,
                            double t1, double *h, double y[]) {
  (void)con;
  (void)step;
  const double t0 = *t;
  const double hh = (t1 - t0 < *h) ? t1 - t0 : *h;
  const int st = quad_step(e, sys, t0, hh, y);
  if (st != GSL_SUCCESS) return st;
  *t = (hh == t1 - t0) ? t1 : t0 + hh;
  return GSL_SUCCESS;
}
