// wl_spline.cpp -- the table of the spline profile (host side).
//
// The profile of periodic.c:17-164: f(rho) solves df/drho = (2/lambda^2) rho
// exp(-sin^2(pi rho / a)/lambda^2), f(0) = 0, on knots rho_i = i h, i = 1..n,
// h = 20/n (periodic.c:128-150); the kernel interpolates f in rho^2 with a
// clamped cubic spline (zero slope at both ends) through (rho_i^2, f_i), the
// knots rounded to float as the reference stores them (periodic.c:46-110).
// The right-hand side does not depend on f, so each step is a quadrature:
// here 8-point Gauss-Legendre per step (the reference integrates with an
// 8th-order Runge-Kutta stepper of GSL at the same fixed step).
#include <math.h>
#include <string.h>

#include <vector>

#include "wl_spline.h"

namespace wl {

namespace {

// nodes and weights of n-point Gauss-Legendre on [-1, 1]: Newton's method on
// P_n from the Chebyshev guesses, P_n by the three-term recurrence
void gauss_legendre(int n, double *x, double *w) {
  for (int i = 0; i < n; ++i) {
    double z = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

}  // namespace

int spline_table(double lambda2, double a, int n, float *rho2, float *coef4) {
  if (!(lambda2 > 0.0) || !(a > 0.0) || n < 4 || !rho2 || !coef4) return -1;
  double gx[8], gw[8];
  gauss_legendre(8, gx, gw);
  const double h = 20.0 / n;
  auto rhs = [&](double s) {
    const double sn = sin(M_PI * s / a);
    return 2.0 / lambda2 * s * exp(-sn * sn / lambda2);
  };
  std::vector<double> f(n);
  double acc = 0.0;
  for (int i = 0; i < n; ++i) {  // step [i h, (i + 1) h]
    const double lo = i * h, mid = lo + 0.5 * h;
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += gw[k] * rhs(mid + 0.5 * h * gx[k]);
    acc += 0.5 * h * s;
    f[i] = acc;
    const double r = (i + 1) * h;
    rho2[i] = (float)(r * r);
  }
  // clamped cubic spline in x = rho^2 with zero end slopes (Burden and
  // Faires, algorithm 3.5, as periodic.c:46-110 applies it): S_i(x) = f_i +
  // b_i d + c_i d^2 + d_i d^3, d = x - x_i; c from the tridiagonal system of
  // slope continuity (Crout factorisation).  The knot differences are taken
  // in FP32 as the reference takes them from its float knots, and each c_i
  // is rounded to FP32 before the next row and b_i, d_i use it (the
  // reference back-substitutes through its float table); so the table
  // matches the reference's bit for bit (tests/test_spline_reference.py).
  std::vector<double> hh(n - 1), alpha(n), l(n), mu(n), z(n);
  std::vector<float> c(n);
  for (int i = 0; i < n - 1; ++i) hh[i] = (double)(rho2[i + 1] - rho2[i]);
  alpha[0] = 3.0 * (f[1] - f[0]) / hh[0];
  alpha[n - 1] = -3.0 * (f[n - 1] - f[n - 2]) / hh[n - 2];
  for (int i = 1; i < n - 1; ++i)
    alpha[i] = 3.0 / hh[i] * (f[i + 1] - f[i]) - 3.0 / hh[i - 1] * (f[i] - f[i - 1]);
  l[0] = 2.0 * hh[0];
  mu[0] = 0.5;
  z[0] = alpha[0] / l[0];
  for (int i = 1; i < n - 1; ++i) {
    l[i] = 2.0 * (double)(rho2[i + 1] - rho2[i - 1]) - hh[i - 1] * mu[i - 1];
    mu[i] = hh[i] / l[i];
    z[i] = (alpha[i] - hh[i - 1] * z[i - 1]) / l[i];
  }
  l[n - 1] = hh[n - 2] * (2.0 - mu[n - 2]);
  z[n - 1] = (alpha[n - 1] - hh[n - 2] * z[n - 2]) / l[n - 1];
  c[n - 1] = (float)z[n - 1];
  coef4[4 * (n - 1)] = (float)f[n - 1];
  coef4[4 * (n - 1) + 1] = 0.0f;
  coef4[4 * (n - 1) + 2] = c[n - 1];
  coef4[4 * (n - 1) + 3] = 0.0f;
  for (int i = n - 2; i >= 0; --i) {
    c[i] = (float)(z[i] - mu[i] * (double)c[i + 1]);
    coef4[4 * i] = (float)f[i];
    coef4[4 * i + 1] =
        (float)((f[i + 1] - f[i]) / hh[i] - hh[i] * ((double)c[i + 1] + 2.0 * (double)c[i]) / 3.0);
    coef4[4 * i + 2] = c[i];
    coef4[4 * i + 3] = (float)(((double)c[i + 1] - (double)c[i]) / (3.0 * hh[i]));
  }
  return 0;
}

}  // namespace wl
