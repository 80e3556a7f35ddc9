// wl_tint.cu -- FP64 proper-time integral of the effective action density.
//
// From the per-group <W>(rho, T) of a (rho x T) instance grid, for each
// (rho, F, group g):
//   I_g(rho) = int dT igrand_g(T)
// with the integrand of Tfunc (Integrand.c:195-316): small-T series,
// constant-field expression, large-T asymptotics or the Monte Carlo value
//   e^{-m^2 T} / T^3 (<W>_g - 1 + (eTB)^2/6)    scalar QED
//   e^{-m^2 T} / T^3 (<W>_g - 1 - (eTB)^2/3)    spinor QED
// (the free and constant-field counterterms subtracted in FP64, where the
// difference cancels catastrophically at small T), integrated over ln T with
// Simpson weights on the log-spaced grid; then
//   L_eff = <I>/(4 pi) (spinor) or <I>/(-2 pi) (scalar)   (Tint.c:69-72)
// with a jackknife error over nbins bins of groups.
#include <math.h>

#include "wl_internal.h"

namespace wl {



// magnetic field of the profile at rho^2, times 2F/e (Integrand.c:98-140)
__device__ double magfield_d(const TintArgs &A, double rho2, double F) {
  const double l2 = A.l2, a = A.a;
  double B = 0.0;
  switch (A.profile) {
    case kStep: B = rho2 < l2 ? 1.0 / l2 : 0.0; break;
    case kSmooth: B = l2 / ((l2 + rho2) * (l2 + rho2)); break;
    case kQuadratic: B = rho2 < l2 ? 2.0 / l2 * (1.0 - rho2 / l2) : 0.0; break;
    case kGaussian: B = rho2 < 100.0 * l2 ? exp(-rho2 / l2) / l2 : 0.0; break;
    case kPeriodic: {  // Integrand.c:58-96, its int-truncating fmod test included
      const double rho = sqrt(rho2), lam = sqrt(l2);
      const double ex = exp(-rho / lam), fl = floor(rho / a), ce = ceil(rho / a);
      double f;
      if (rho < a) {
        const double eb = (a - rho) / lam < 10.0 ? exp(-(rho - a) / lam) : 0.0;
        f = ex / (a * (1.0 + ex) * (1.0 + ex));
        if (rho > 0.0) f += eb / (rho * (1.0 + eb) * (1.0 + eb));
      } else if (fabs(fmod(rho, a)) < 1.0) {
        f = fl / (4.0 * rho);
      } else {
        const double e1 = exp(-(rho - fl * a) / lam), e2 = exp(-(rho - ce * a) / lam);
        f = fl * e1 / (rho * (1.0 + e1) * (1.0 + e1)) + ce * e2 / (rho * (1.0 + e2) * (1.0 + e2));
      }
      B = a / (2.0 * log(2.0) * l2) * f;
      break;
    }
    case kSpline: {  // Integrand.c:128-131
      const double s = sin(M_PI * sqrt(rho2) / a);
      B = 1.0 / (l2 * exp(s * s / l2));
      break;
    }
    case kFixflux:
    case kFixfluxFF: {  // Integrand.c:39-56 (the width ratio is a float there)
      const float lf = (float)sqrt(l2), af = (float)a, lmf = (float)A.lmin;
      const double lml = (float)((lf - lmf) / (af - lmf));
      const double x = 2.0 * sqrt(rho2 / l2);
      const double bump = fabs(x) < 1.0 ? exp(-1.0 / (1.0 - x * x)) : 0.0;
      B = 2.0 / (l2 * 0.0742478) * (1.0 - 0.75 * lml) * bump + 3.0 / (a * a) * lml;
      break;
    }
    case kLattice: {  // sum of the images' Gaussian fields (|R| <= rimage)
      const double cutoff2 = 40.0 * l2;  // e^-40: beyond, an image adds nothing
      const int lim = (int)floor(sqrt(A.rimg2));
      for (int m = -lim; m <= lim; ++m)
        for (int n = -lim; n <= lim; ++n) {
          if ((double)(m * m + n * n) > A.rimg2) continue;
          const double dx = A.xcm_x - m * a, dy = -n * a;
          const double d2 = dx * dx + dy * dy;
          if (d2 < cutoff2) B += exp(-d2 / l2) / l2;
        }
      (void)rho2;
      break;
    }
    default: B = 0.0;
  }
  return 2.0 * F / A.e * B;
}

// Tfunc's integrand for one group (Integrand.c:215-305)
__device__ double igrand_d(TintArgs A, double rho, double T, double F, double W) {
  const double rho2 = rho * rho, l2 = A.l2, m2 = A.m2, e = A.e;
  A.xcm_x = rho;
  const double B = magfield_d(A, rho2, F), TB = e * T * B;
  double smallT;
  switch (A.profile) {
    case kStep: smallT = (double)abs((int)(rho * rho - l2)); break;
    case kGaussian:
    case kLattice: smallT = l2; break;
    case kSpline: {  // Integrand.c:209, 236-240
      const double s2 = sin(2.0 * M_PI * rho / A.a);
      smallT = rho / A.a > 1.0e-8 ? A.a * A.a * l2 / (M_PI * M_PI * s2 * s2) : 1.0e12;
      break;
    }
    case kFixflux:
    case kFixfluxFF:
      smallT = rho2 < l2 / 4.0 ? 0.25 * l2 : 0.25 * l2 + (rho - sqrt(l2) / 2.0) * (rho - sqrt(l2) / 2.0);
      break;
    default: smallT = 0.5 * (l2 + rho2);
  }
  const double pre = exp(-m2 * T) / (T * T * T);
  if (T < 0.1 && T < 0.01 * smallT) {  // small-T series (Integrand.c:142-172)
    const double B2 = e * e * B * B, B4 = B2 * B2, B6 = B2 * B4;
    const double T3 = T * T * T, T4 = T3 * T;
    if (A.fermion)
      return B4 * T * (m2 * T - 1.0) / 45.0 + (2.0 * B6 / 945.0 - B4 * m2 * m2 / 90.0) * T3 +
             (7.0 * B4 * m2 * m2 * m2 - 4.0 * B6 * m2) / 1890.0 * T4;
    return 7.0 / 360.0 * B4 * T * (1.0 - m2 * T) + (147.0 * B4 * m2 * m2 - 31.0 * B6) / 15120.0 * T3 +
           (31.0 * B6 * m2 - 49.0 * B4 * m2 * m2 * m2) / 15120.0 * T4;
  }
  if (T < 0.01 * smallT) {  // constant field (Integrand.c:20-37)
    if (!(TB > 1.0e-6) || B < 1.0e-40) return 0.0;
    if (A.fermion) return pre * (TB / tanh(TB) - 1.0 - TB * TB / 3.0);
    if (TB < 50.0) return pre * (TB / sinh(TB) - 1.0 + TB * TB / 6.0);
    return pre * (TB * TB / 6.0 - 1.0);
  }
  if (T > 49.0)  // large T (Integrand.c:272-288)
    return A.fermion ? -exp(-m2 * T) / (3.0 * T) * e * e * B * B
                     : exp(-m2 * T) / (6.0 * T) * e * e * B * B;
  return A.fermion ? pre * (W - 1.0 - TB * TB / 3.0) : pre * (W - 1.0 + TB * TB / 6.0);
}

// one thread per (rho, F, group): the T integral
__global__ void tint_kernel(const TintArgs A) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= A.nrho * A.nF * A.ng) return;
  const int g = idx % A.ng, j = (idx / A.ng) % A.nF, r = idx / (A.ng * A.nF);
  const double rho = A.rho[r], F = A.F[j];
  double s = 0.0;
  for (int k = 0; k < A.nT; ++k) {
    const int inst = r * A.nT + k;
    const double W = A.groups[((size_t)inst * A.nF + j) * A.ng + g];
    double v = igrand_d(A, rho, A.T[k], F, W);
    if (isinf(v)) v = 0.0;  // Tint.c:132-149
    if (A.igrand) A.igrand[(((size_t)r * A.nF + j) * A.nT + k) * A.ng + g] = v;
    s += A.w[k] * v;
  }
  A.Ig[((size_t)r * A.nF + j) * A.ng + g] = s;
}

// one thread per (rho, F): L_eff and its jackknife error over nbins bins
__global__ void jackknife_kernel(const TintArgs A) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= A.nrho * A.nF) return;
  const double *I = A.Ig + (size_t)idx * A.ng;
  const int nb = A.nbins, per = A.ng / nb;
  double tot = 0.0;
  for (int g = 0; g < nb * per; ++g) tot += I[g];
  const double n = (double)(nb * per);
  const double mean = tot / n;
  double ss = 0.0;
  for (int b = 0; b < nb; ++b) {
    double sb = 0.0;
    for (int g = b * per; g < (b + 1) * per; ++g) sb += I[g];
    const double loo = (tot - sb) / (n - per);  // leave bin b out
    ss += (loo - mean) * (loo - mean);
  }
  const double jk = nb > 1 ? sqrt((nb - 1.0) / nb * ss) : 0.0;
  const double norm = A.fermion ? 1.0 / (4.0 * M_PI) : -1.0 / (2.0 * M_PI);
  A.leff[idx] = mean * norm;
  A.err[idx] = jk * fabs(norm);
}

cudaError_t launch_tint(const TintArgs &a, cudaStream_t s) {
  const int bs = 128;
  const int n1 = a.nrho * a.nF * a.ng, n2 = a.nrho * a.nF;
  tint_kernel<<<(n1 + bs - 1) / bs, bs, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  jackknife_kernel<<<(n2 + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace wl
