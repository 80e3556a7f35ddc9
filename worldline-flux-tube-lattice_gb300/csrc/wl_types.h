// wl_types.h -- types and constants shared by host runtime and kernels.
#pragma once

#include <stdint.h>
#include <vector_types.h>

namespace wl {

enum : int {
  kStep = 0,
  kSmooth = 1,
  kQuadratic = 2,
  kGaussian = 3,
  kPeriodic = 4,
  kSpline = 5,     // tabulated profile of periodic.c (clamped cubic spline)
  kFixflux = 6,
  kFixfluxFF = 7,  // fixflux with the intEVff.cu phi/chi fits
  kLattice = 8     // square lattice of Gaussian tubes (image sum)
};

constexpr int kMaxF = 4;  // flux values sharing one geometric pass

// Field constants of one launch, FP32 (the reference kernel is FP32).
struct FieldDev {
  float l2, inv_l2, lam;  // lambda^2, 1/lambda^2, lambda
  float a, lmin;          // lattice spacing, fixflux minimum width
  float lml, aml;         // fixflux (lam-lmin)/(a-lmin), (a-lam)/(a-lmin)
  // clamps of the segment polynomial: the reference's 1e-8 / 1e-10
  // (intEV.cu:418-422, 439) or -inf / 1e-30 in exact mode
  float clampA, clampB, clampC, clampE, clampI;
  int nint;  // Simpson intervals (used by the run-time-n kernels)
  float h;   // 1.0f / nint
  // lattice: images with m^2 + n^2 <= rimg2 (|R| <= rimage), near-image
  // margin rcut = sqrt(18) lambda around the loop's bounding box (beyond it
  // 1 - e^{-rho^2/lambda^2} rounds to 1 in FP32: the image is pure gauge)
  float rimg2, rcut;
  // spline: knots (rho^2) and cubic coefficients in device memory, the knot
  // spacing in rho, and the argument factor of f' (pi, or pi/a in exact mode)
  const float *sp_rho2;
  const float4 *sp_coef;
  int sp_n;
  float sp_h, sp_piarg;
};

}  // namespace wl
