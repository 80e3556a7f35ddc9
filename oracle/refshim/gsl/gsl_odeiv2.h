/* Stand-in for the part of GSL's ODE interface (gsl_odeiv2, GSL >= 1.15; the
 * reference pins no version) that periodic.c calls (periodic.c:113-164,
 * 200-247): a stepper "rk8pd", a y-error control, and an evolve object
 * advanced either by fixed steps or up to a target time.  Test
 * infrastructure for oracle/_ref only; GSL is not installed.
 *
 * The stand-in integrates only right-hand sides that do not depend on y --
 * periodic.c's f(rho) = (2/lambda^2) rho exp(-sin^2(pi rho/a)/lambda^2) --
 * where a Runge-Kutta step is a quadrature of f over the step: GSL's rk8pd
 * (the Prince-Dormand 8(7) pair) is an 8th-order one; the stand-in takes a
 * 10-point Gauss-Legendre rule (order 20) instead, which agrees with it to the
 * stepper's own local error (far below the FP32 table the reference builds).
 * A right-hand side that changes with y is refused (GSL_FAILURE).  The error
 * control is accepted and not applied. */
#ifndef WLREF_GSL_ODEIV2_H
#define WLREF_GSL_ODEIV2_H
#include <stddef.h>

typedef struct {
  int (*function)(double t, const double y[], double dydt[], void *params);
  int (*jacobian)(double t, const double y[], double *dfdy, double dfdt[], void *params);
  size_t dimension;
  void *params;
} gsl_odeiv2_system;

typedef struct {
  const char *name;
} gsl_odeiv2_step_type;
typedef struct {
  const gsl_odeiv2_step_type *type;
  size_t dimension;
} gsl_odeiv2_step;
typedef struct {
  double eps_abs, eps_rel;
} gsl_odeiv2_control;
typedef struct {
  size_t dimension;
  double *f0, *f1, *yt;
} gsl_odeiv2_evolve;

extern const gsl_odeiv2_step_type *gsl_odeiv2_step_rk8pd;

gsl_odeiv2_step *gsl_odeiv2_step_alloc(const gsl_odeiv2_step_type *T, size_t dim);
void gsl_odeiv2_step_free(gsl_odeiv2_step *s);
gsl_odeiv2_control *gsl_odeiv2_control_y_new(double eps_abs, double eps_rel);
void gsl_odeiv2_control_free(gsl_odeiv2_control *c);
gsl_odeiv2_evolve *gsl_odeiv2_evolve_alloc(size_t dim);
void gsl_odeiv2_evolve_free(gsl_odeiv2_evolve *e);
int gsl_odeiv2_evolve_apply_fixed_step(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con,
                                       gsl_odeiv2_step *step, const gsl_odeiv2_system *sys,
                                       double *t, const double h, double y[]);
int gsl_odeiv2_evolve_apply(gsl_odeiv2_evolve *e, gsl_odeiv2_control *con,
                            gsl_odeiv2_step *step, const gsl_odeiv2_system *sys, double *t,
                            double t1, double *h, double y[]);
#endif
