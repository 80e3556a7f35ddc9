// wl_spline.h -- the spline profile's table (wl_spline.cpp).
#pragma once

namespace wl {

// knots of the table (the reference's Nspline)
constexpr int kSplineKnots = 1000;

// Knots rho2[n] (float, as the reference stores them) and coefficients
// coef4[n][4] = (f, b, c, d) of S_i(x) = f + b d + c d^2 + d d^3, d = x -
// rho2[i], for lambda^2 and the tube spacing a.  Returns 0, or -1 for
// invalid arguments.
int spline_table(double lambda2, double a, int n, float *rho2, float *coef4);

}  // namespace wl
