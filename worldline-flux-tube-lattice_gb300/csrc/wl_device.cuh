// wl_device.cuh -- device building blocks of the Wilson-loop kernels (sm_103a).
//
// Field profiles, the Simpson segment integral, the per-loop W factors and
// the bulk-copy / mbarrier primitives used to stage loops in shared memory.
// Reference semantics are cited per function (intEV.cu, intEVff.cu,
// Integrand.c line numbers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wl_types.h"

namespace wl {

// ---------------------------------------------------------------- math --
// Single-instruction MUFU operations, PTX-documented accuracy: rcp.approx
// max 1 ulp; ex2.approx max relative error 2^-22 (ftz: no subnormals).
__device__ __forceinline__ float rcp_fast(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_fast(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// e^-x for x >= 0 through 2^(-x log2 e)
__device__ __forceinline__ float expneg_fast(float x) {
  return ex2_fast(-1.4426950408889634f * x);
}

// 1/d for a positive normal d on the FP32 pipe instead of the MUFU: the
// bit-level initial approximation (integer subtraction from the exponent and
// mantissa bits, Blinn, "Floating-point tricks", IEEE CG&A 17(4), 1997; the
// constant 0x7ef311c2 is the minimax fit of the relative error over two
// binades, 5.1e-2), one Newton-Raphson step x(1 + e) and one third-order step
// x(1 + e + e^2), e = 1 - d x: error 5.1e-2 -> 2.6e-3 -> 1.7e-8, i.e. within
// 0.78 ulp of 1/d (tests/test_device_math.py).  NaN in, NaN out.
__device__ __forceinline__ float rcp_newton(float d) {
  float x = __int_as_float(0x7ef311c2 - __float_as_int(d));
  float e = fmaf(-d, x, 1.0f);
  x = fmaf(x, e, x);
  e = fmaf(-d, x, 1.0f);
  return fmaf(x, fmaf(e, e, e), x);
}

// (1 - e^-x) / x for 0 <= x < 0.5: a degree-5 polynomial fitted to the
// function on [0, 0.5] (iteratively reweighted least squares for the relative
// error on Chebyshev nodes); FP32 Horner evaluation stays within 5.5e-8 of it,
// the FP32 rounding level (checked by tests/test_device_math.py).
// Coefficients c0..c5 (kQ1):
//   1.0f, -0.4999998211860657f, 0.16666224598884583f,
//   -0.041629087179899216f, 0.008187385275959969f, -0.0011216341517865658f
__device__ __forceinline__ float one_minus_expneg_over_x(float x) {
  float p = -0.0011216341517865658f;
  p = fmaf(p, x, 0.008187385275959969f);
  p = fmaf(p, x, -0.041629087179899216f);
  p = fmaf(p, x, 0.16666224598884583f);
  p = fmaf(p, x, -0.4999998211860657f);
  p = fmaf(p, x, 1.0f);
  return p;
}

// ------------------------------------------------------------- profiles --
// Each profile returns, at rho^2 = r2:
//   g  = f_lambda(r2) / r2        (scalar Simpson integrand, intEV.cu:425-449)
//   fp = f'_lambda(r2) / FpScale  (spinor integrand, intEV.cu:430-451)
// fp is scaled so that the per-node work is minimal; the constant factor is
// applied once per loop (fp_scale()).

// exponential integral Ei(x) = -E1(-x), x < -1, by Lentz's continued
// fraction with the reference's stopping rule (intEV.cu:29-61)
__device__ __forceinline__ float expint_lentz(float x) {
  float b = -x + 1.0f, c = 1.0e10f, d = 1.0f / b, h = d;
  for (int i = 1; i <= 400; i++) {
    float an = -(float)i * (float)i;
    b += 2.0f;
    d = 1.0f / (an * d + b);
    c = b + an / c;
    float del = c * d;
    h *= del;
    if (fabsf(del - 1.0f) <= 1.0e-6f) return -h * expf(x);
  }
  return 0.0f;
}

__device__ __forceinline__ float bump_d(float x) {  // intEV.cu:151-159
  return (x * x < 0.999f) ? expf(-1.0f / (1.0f - x * x)) : 0.0f;
}

template <bool FF>
__device__ __forceinline__ float phi_d(float x) {  // intEV.cu:161-174 / intEVff.cu:147-157
  const float onemx2 = 1.0f - x * x;
  if (x < (FF ? 1.0f : 0.999f))
    return 1.0f - (0.5f / 0.0742478f) *
                      (onemx2 * expf(-1.0f / onemx2) + expint_lentz(-1.0f / onemx2));
  return 1.0f;
}

template <bool FF>
__device__ __forceinline__ float chi_d(float x, float n, float lam, float a) {
  // intEV.cu:176-198 (logistic fit) / intEVff.cu:159-176 (cosh-ratio fit)
  const float onemx2 = 1.0f - x * x, x2 = x * x, x4 = x2 * x2;
  if (x <= (FF ? -1.0f : -0.999f)) return 0.0f;
  if (x2 < (FF ? 1.0f : 0.999f)) {
    float ans = 0.5f * (-onemx2 * expf(-1.0f / onemx2) - expint_lentz(-1.0f / onemx2));
    if (FF)
      ans += 2.0f * n * a / lam *
             (0.218f + 0.393f * x * coshf(0.806f * x4 - 0.696f * x2 + 0.0902f) /
                           coshf(0.825f * x2 - 0.0234f * x + 0.375f));
    else
      ans += 2.0f * n * a / lam * 0.444f /
             (1.0f + expf(-(3.31f * x + 5.25f * x * x2 * sinf(x) *
                                            cosf(-0.907f * x2 - 1.29f * x4 * x4)) /
                          cosf(x)));
    return ans;
  }
  return 2.0f * n * a * 0.443991f / lam;
}

template <int P>
struct Profile;

template <>
struct Profile<kSmooth> {  // f = r2/(l2+r2): f/r2 = 1/(l2+r2), f' = l2 (f/r2)^2
  // evaluated on d = l2 + r2: the segment folds l2 into the constant term of
  // its rho^2 polynomial once instead of adding it at every node
  static __device__ __forceinline__ float shift(const FieldDev &F) { return F.l2; }
  static __device__ __forceinline__ void eval(float d, const FieldDev &, float &g, float &fp) {
    g = rcp_fast(d);
    fp = g * g;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &F) { return F.l2; }
  static constexpr bool kHeavy = false;
};

template <>
struct Profile<kStep> {  // intEV.cu:267-272, 368-373
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    const bool in = r2 < F.l2;
    g = in ? F.inv_l2 : rcp_fast(r2);
    fp = in ? 1.0f : 0.0f;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &F) { return F.inv_l2; }
  static constexpr bool kHeavy = false;
};

template <>
struct Profile<kQuadratic> {  // intEV.cu:276-281, 377-382
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    const bool in = r2 < F.l2;
    const float u = r2 * F.inv_l2;
    g = in ? (2.0f - u) * F.inv_l2 : rcp_fast(r2);
    fp = in ? 1.0f - u : 0.0f;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &F) {
    return 2.0f * F.inv_l2;
  }
  static constexpr bool kHeavy = false;
};

template <>
struct Profile<kGaussian> {  // f = 1 - e^{-r2/l2} (intEV.cu:282-284, 383-385)
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    const float x = r2 * F.inv_l2;
    const float e = expneg_fast(x);
    // below x = 0.5 the series avoids the cancellation of 1 - e^-x (both
    // forms are evaluated and one selected: cheaper than a branch here)
    g = (x < 0.5f) ? one_minus_expneg_over_x(x) * F.inv_l2 : (1.0f - e) * rcp_fast(r2);
    fp = e;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &F) { return F.inv_l2; }
  static constexpr bool kHeavy = false;
};

// The lattice profiles below are heavy (loops, several transcendentals per
// node): they are compiled only with a run-time interval count and without
// unrolling, which keeps code size and build time bounded.
template <>
struct Profile<kPeriodic> {  // radial shells, intEV.cu:201-232 and 300-328
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    const float rho = sqrtf(r2), a = F.a, lam = F.lam;
    const float flraf = floorf(rho / a);
    const int i0 = (int)flraf - 2, i1 = (int)flraf + 2;
    float f = (i0 > 0) ? 0.5f * (flraf - 3.0f) * (flraf - 2.0f) : 0.0f;
    float d = 0.0f;
    // The shell at the axis (i = 0, when i0 <= 0 <= i1) comes first in the
    // loop's ascending order: it sets f and d, the shells i > 0 then add to
    // them.  Evaluated before the loop, its exp and log run once per warp
    // instead of once for each iteration at which some lane meets i = 0.
    if (i0 <= 0) {
      const float ex = expf(-rho / lam), ex1 = 1.0f + ex;
      f = -rho / a * (ex / ex1) - lam / a * logf(ex1);
      d = ex / (a * ex1 * ex1);
    }
    for (int i = i0; i <= i1; i++) {
      if (i > 0) {
        const float ea = expf(-(rho - (float)i * a) / lam), ea1 = 1.0f + ea;
        f = f + (float)i / ea1;
        d = d + ((float)i / rho) * ea / (ea1 * ea1);
      }
    }
    const float ln2 = 0.69314718055994531f;
    g = (a / (lam * ln2) * f + 1.0f) / r2;
    fp = a / (2.0f * F.l2 * ln2) * d;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &) { return 1.0f; }
  static constexpr bool kHeavy = true;
};

template <>
struct Profile<kSpline> {  // interp (intEV.cu:64-107), fplambda spline (intEV.cu:389-397)
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    // the interval [rho2[j], rho2[j+1]) of the table; 0 outside, as interp;
    // the knots are near ((j + 1) h)^2, so the guess is within one knot
    float f = 0.0f;
    const int n = F.sp_n;
    if (F.sp_rho2 && n >= 2 && r2 < F.sp_rho2[n - 1] && r2 > F.sp_rho2[0]) {
      int j = min(max((int)(sqrtf(r2) / F.sp_h) - 1, 0), n - 2);
      while (j > 0 && r2 < F.sp_rho2[j]) --j;
      while (j < n - 2 && r2 >= F.sp_rho2[j + 1]) ++j;
      const float d = r2 - F.sp_rho2[j];
      const float4 c = F.sp_coef[j];
      f = c.x + d * (c.y + d * (c.z + d * c.w));
    }
    g = f / r2;
    const float s = sinf(sqrtf(r2) * F.sp_piarg);
    fp = expf(-s * s * F.inv_l2) * F.inv_l2;
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &) { return 1.0f; }
  static constexpr bool kHeavy = true;
};

template <bool FF>
struct FixfluxProfile {  // intEV.cu:236-257, 333-357; intEVff.cu:194-250
  static __device__ __forceinline__ void eval(float r2, const FieldDev &F, float &g,
                                              float &fp) {
    const float a = F.a, lam = F.lam, lml = F.lml, aml = F.aml;
    const float rho = sqrtf(r2);
    const float n = floorf((rho + 0.5f * a) / a);
    float f;
    if (r2 <= 0.25f * a * a) {
      f = (1.0f - 0.75f * lml) * phi_d<FF>(2.0f * sqrtf(r2 * F.inv_l2)) +
          3.0f * r2 / (a * a) * lml;
    } else {
      f = 1.0f + 0.75f * (4.0f * r2 / (a * a) - 1.0f) * lml + 3.0f * n * (n - 1.0f) * aml;
      f += 3.0f * lam / (0.443991f * a) * aml *
           chi_d<FF>(2.0f * (rho - n * a) / lam, n, lam, a);
    }
    g = f / r2;
    const float bbg = 3.0f / (a * a) * lml;
    if (rho <= 0.5f * a)
      fp = bbg + 2.0f / (F.l2 * 0.0742478f) * (1.0f - 0.75f * lml) * bump_d(2.0f * rho / lam);
    else
      fp = bbg + 6.0f / (0.443991f * lam * a) * aml * bump_d(2.0f * (rho - n * a) / lam);
  }
  static __device__ __forceinline__ float fp_scale(const FieldDev &) { return 1.0f; }
  static constexpr bool kHeavy = true;
};
template <>
struct Profile<kFixflux> : FixfluxProfile<false> {};
template <>
struct Profile<kFixfluxFF> : FixfluxProfile<true> {};

// The fixflux profile with its Lentz continued fraction split out.  The
// fraction (up to ~17 iterations of two divisions) is needed only where the
// node lies in a bump region -- about a third of the nodes -- but on almost
// every node some lane of a warp needs it, so evaluated in place the warp
// runs ~16 iterations per node for an average lane need of ~3.  Instead the
// fractions of a batch of nodes are gathered across the warp's lanes and
// evaluated 32 at a time (a lane may evaluate another lane's), then each
// lane finishes its own nodes in the usual order.
//
// fixflux_cf: whether the node at r2 needs a fraction, and its argument
// -1/(1 - x^2) (x as phi_d / chi_d compute it)
template <bool FF>
__device__ __forceinline__ bool fixflux_cf(float r2, const FieldDev &F, float &arg) {
  const float a = F.a;
  float x;
  if (r2 <= 0.25f * a * a) {
    x = 2.0f * sqrtf(r2 * F.inv_l2);
    if (!(x < (FF ? 1.0f : 0.999f))) return false;
  } else {
    const float rho = sqrtf(r2);
    const float n = floorf((rho + 0.5f * a) / a);
    x = 2.0f * (rho - n * a) / F.lam;
    if (x <= (FF ? -1.0f : -0.999f) || !(x * x < (FF ? 1.0f : 0.999f))) return false;
  }
  arg = -1.0f / (1.0f - x * x);
  return true;
}

// FixfluxProfile::eval with the node's fraction value E given (used only
// where fixflux_cf says the node needs it)
template <bool FF>
__device__ __forceinline__ void fixflux_eval(float r2, const FieldDev &F, float E, float &g,
                                             float &fp) {
  const float a = F.a, lam = F.lam, lml = F.lml, aml = F.aml;
  const float rho = sqrtf(r2);
  const float n = floorf((rho + 0.5f * a) / a);
  float f;
  if (r2 <= 0.25f * a * a) {
    const float x = 2.0f * sqrtf(r2 * F.inv_l2);
    float phi = 1.0f;
    if (x < (FF ? 1.0f : 0.999f)) {
      const float onemx2 = 1.0f - x * x;
      phi = 1.0f - (0.5f / 0.0742478f) * (onemx2 * expf(-1.0f / onemx2) + E);
    }
    f = (1.0f - 0.75f * lml) * phi + 3.0f * r2 / (a * a) * lml;
  } else {
    const float x = 2.0f * (rho - n * a) / lam;
    const float onemx2 = 1.0f - x * x, x2 = x * x, x4 = x2 * x2;
    float chi;
    if (x <= (FF ? -1.0f : -0.999f)) {
      chi = 0.0f;
    } else if (x2 < (FF ? 1.0f : 0.999f)) {
      chi = 0.5f * (-onemx2 * expf(-1.0f / onemx2) - E);
      if (FF)
        chi += 2.0f * n * a / lam *
               (0.218f + 0.393f * x * coshf(0.806f * x4 - 0.696f * x2 + 0.0902f) /
                             coshf(0.825f * x2 - 0.0234f * x + 0.375f));
      else
        chi += 2.0f * n * a / lam * 0.444f /
               (1.0f + expf(-(3.31f * x + 5.25f * x * x2 * sinf(x) *
                                              cosf(-0.907f * x2 - 1.29f * x4 * x4)) /
                            cosf(x)));
    } else {
      chi = 2.0f * n * a * 0.443991f / lam;
    }
    f = 1.0f + 0.75f * (4.0f * r2 / (a * a) - 1.0f) * lml + 3.0f * n * (n - 1.0f) * aml;
    f += 3.0f * lam / (0.443991f * a) * aml * chi;
  }
  g = f / r2;
  const float bbg = 3.0f / (a * a) * lml;
  if (rho <= 0.5f * a)
    fp = bbg + 2.0f / (F.l2 * 0.0742478f) * (1.0f - 0.75f * lml) * bump_d(2.0f * rho / lam);
  else
    fp = bbg + 6.0f / (0.443991f * lam * a) * aml * bump_d(2.0f * (rho - n * a) / lam);
}

// nodes per gathering batch of the fixflux segment
constexpr int kFfBatch = 8;
constexpr int kFfWarps = 4;  // warps per CTA of the kernels that call it (128 threads)

// segment<> for the fixflux profiles (run-time interval count), with the
// continued fractions gathered per warp; the same node values and sums as
// segment<> evaluating FixfluxProfile<FF>::eval node by node.  Not inlined:
// one copy for the dozen call sites of the sweep.
template <bool FF, bool FERM>
__device__ __noinline__ float2 segment_fixflux(float zix, float ziy, float zjx, float zjy,
                                               const FieldDev &F, float ph, float sp) {
  __shared__ float cfq[kFfWarps][32 * kFfBatch];  // arguments, then values in place
  __shared__ unsigned cfm[kFfWarps][kFfBatch];     // per node of the batch: lanes needing one
  __shared__ int cfo[kFfWarps][kFfBatch];          // and their first queue slot
  const int w = (threadIdx.x >> 5) & (kFfWarps - 1);
  const int lane = threadIdx.x & 31;
  const unsigned act = __activemask();
  const unsigned lt = (1u << lane) - 1u;
  const int rank = __popc(act & lt), nact = __popc(act);
  const bool leader = rank == 0;

  const float dx = zjx - zix, dy = zjy - ziy;
  float a = fmaf(zix, zix, ziy * ziy);
  float b = fmaf(zix, dx, ziy * dy);
  float c = fmaf(dx, dx, dy * dy);
  const float xyyx = fmaf(zix, zjy, -(ziy * zjx));
  a = fmaxf(a, F.clampA);
  b = fmaxf(b, F.clampB);
  c = fmaxf(c, F.clampC);
  const float b2 = b + b;
  const float as = a;
  const float ae = fmaxf((as + b2) + c, F.clampE);
  const int n = F.nint;
  // node k of the evaluation order 0 (t = 0), n (t = 1), 1 .. n-1
  auto node_j = [&](int k) { return k == 0 ? 0 : (k == 1 ? n : k - 1); };
  auto node_r2 = [&](int j) {
    if (j == 0) return as;
    if (j == n) return ae;
    const float t = (float)j * F.h;
    return fmaxf(fmaf(fmaf(c, t, b2), t, as), F.clampI);
  };
  float g0 = 0.f, f0 = 0.f, g1 = 0.f, f1 = 0.f;
  float so = 0.f, se = 0.f, fo = 0.f, fe = 0.f;
  for (int k0 = 0; k0 <= n; k0 += kFfBatch) {
    int base = 0;
#pragma unroll
    for (int kk = 0; kk < kFfBatch; ++kk) {  // gather the batch's fractions
      const int k = k0 + kk;
      if (k > n) break;
      float arg = 0.0f;
      const bool need = fixflux_cf<FF>(node_r2(node_j(k)), F, arg);
      const unsigned m = __ballot_sync(act, need);
      if (need) cfq[w][base + __popc(m & lt)] = arg;
      if (leader) {
        cfm[w][kk] = m;
        cfo[w][kk] = base;
      }
      base += __popc(m);
    }
    __syncwarp(act);
    for (int q = rank; q < base; q += nact) cfq[w][q] = expint_lentz(cfq[w][q]);
    __syncwarp(act);
#pragma unroll
    for (int kk = 0; kk < kFfBatch; ++kk) {  // each lane's nodes, in order
      const int k = k0 + kk;
      if (k > n) break;
      const int j = node_j(k);
      const unsigned m = cfm[w][kk];
      const float E = (m >> lane) & 1u ? cfq[w][cfo[w][kk] + __popc(m & lt)] : 0.0f;
      float g, fp;
      fixflux_eval<FF>(node_r2(j), F, E, g, fp);
      if (j == 0) {
        g0 = g;
        f0 = fp;
      } else if (j == n) {
        g1 = g;
        f1 = fp;
      } else if (j & 1) {
        so += g;
        if (FERM) fo += fp;
      } else {
        se += g;
        if (FERM) fe += fp;
      }
    }
    __syncwarp(act);  // the queue is rewritten by the next batch
  }
  const float S = fmaf(4.0f, so, fmaf(2.0f, se, g0 + g1));
  ph = fmaf(xyyx, S, ph);
  if (FERM) sp += fmaf(4.0f, fo, fmaf(2.0f, fe, f0 + f1));
  return make_float2(ph, sp);
}

// rho^2 shift folded into the segment polynomial (Profile<P>::shift where a
// profile evaluates on l2 + rho^2, else 0)
template <int P>
__device__ __forceinline__ float profile_shift(const FieldDev &F) {
  if constexpr (P == kSmooth)
    return Profile<P>::shift(F);
  else
    return 0.0f;
}

// The smooth profile at a fixed interval count of 8 or more: one node costs
// 1 MUFU reciprocal against 3 (scalar) or 5 (spinor) FP32 operations, so the
// MUFU (16 per SM per clock, an eighth of the FP32 rate) bounds the segment
// alone.  Every kSoftRcp-th interior node takes its reciprocal from
// rcp_newton (5 FP32 + 1 integer operation) to share the work between the
// two pipes; 0 = every node on the MUFU.
// Periods measured on the GB300 at 50 intervals: one instance per thread,
// scalar 5 (+16 % over no FP32-pipe reciprocal), spinor 12 (+5 %); packed
// pairs, scalar 4 (+20 %), spinor 3 (+13 %).  More FP32-pipe reciprocals
// measured slower: the segment then runs out of issue slots and latency
// hiding before either pipe saturates.
#ifndef WL_SOFT_RCP_SCALAR
#define WL_SOFT_RCP_SCALAR 5
#endif
#ifndef WL_SOFT_RCP_SPINOR
#define WL_SOFT_RCP_SPINOR 12
#endif
#ifndef WL_SOFT_RCP_PAIR_SCALAR
#define WL_SOFT_RCP_PAIR_SCALAR 4
#endif
#ifndef WL_SOFT_RCP_PAIR_SPINOR
#define WL_SOFT_RCP_PAIR_SPINOR 3
#endif
template <int P, bool FERM, int NINT, bool PAIR = false>
constexpr int soft_rcp_period() {
  if constexpr (P == kSmooth && NINT >= 8) {
    if constexpr (PAIR)
      return FERM ? WL_SOFT_RCP_PAIR_SPINOR : WL_SOFT_RCP_PAIR_SCALAR;
    else
      return FERM ? WL_SOFT_RCP_SPINOR : WL_SOFT_RCP_SCALAR;
  } else {
    return 0;
  }
}

// ------------------------------------------------------------- segment --
// One segment z_i -> z_j of a sub-loop (intEV.cu:526-552 with Idt,
// intEV.cu:408-459): rho^2(t) = a + 2bt + ct^2 with a = |z_i|^2,
// b = z_i.(z_j - z_i), c = |z_j - z_i|^2, composite Simpson with NINT
// intervals.  Adds xyyx * sum_w(f/rho^2) to ph and sum_w(f') to sp; the
// Simpson factor h/3 and the f' scale are applied once per loop.
template <int P, bool FERM, int NINT>
__device__ __forceinline__ void segment(float zix, float ziy, float zjx, float zjy,
                                        const FieldDev &F, float &ph, float &sp) {
  static_assert(NINT == 0 || (NINT % 2 == 0 && NINT >= 2), "Simpson needs an even interval count");
  const float dx = zjx - zix, dy = zjy - ziy;
  float a = fmaf(zix, zix, ziy * ziy);
  float b = fmaf(zix, dx, ziy * dy);
  float c = fmaf(dx, dx, dy * dy);
  const float xyyx = fmaf(zix, zjy, -(ziy * zjx));
  a = fmaxf(a, F.clampA);
  b = fmaxf(b, F.clampB);
  c = fmaxf(c, F.clampC);
  const float b2 = b + b;
  // The end-value and interior floors (1e-8, 1e-10 in the reference) can only
  // act on the dividing (lattice) profiles: with a, b, c clamped positive,
  // rho^2(t) = a + 2bt + ct^2 >= a >= 1e-8 for t in [0, 1], and the closed
  // forms of the other profiles are finite at rho^2 -> 0 in exact mode.
  constexpr bool kFloor = Profile<P>::kHeavy;
  const float as = a + profile_shift<P>(F);
  float ae = (as + b2) + c;
  if (kFloor) ae = fmaxf(ae, F.clampE);
  float g0, f0, g1, f1;
  Profile<P>::eval(as, F, g0, f0);
  Profile<P>::eval(ae, F, g1, f1);
  float so = 0.0f, se = 0.0f, fo = 0.0f, fe = 0.0f;
  constexpr int kSoftRcp = soft_rcp_period<P, FERM, NINT>();
  auto node = [&](int j, float t) {
    float r2 = fmaf(fmaf(c, t, b2), t, as);
    if (kFloor) r2 = fmaxf(r2, F.clampI);
    float g, fp;
    if (kSoftRcp > 0 && j % kSoftRcp == kSoftRcp - 1) {  // j is a constant after unrolling
      g = rcp_newton(r2);
      fp = g * g;
    } else {
      Profile<P>::eval(r2, F, g, fp);
    }
    if (j & 1) {
      so += g;
      if (FERM) fo += fp;
    } else {
      se += g;
      if (FERM) fe += fp;
    }
  };
  if constexpr (NINT > 0) {
#pragma unroll
    for (int j = 1; j < NINT; j++)
      // the reference's abscissa (float)j * h with h = 1.0f/n (intEV.cu:416, 436)
      node(j, (float)j * (1.0f / (float)NINT));
  } else {
#pragma unroll 1
    for (int j = 1; j < F.nint; j++) node(j, (float)j * F.h);
  }
  const float S = fmaf(4.0f, so, fmaf(2.0f, se, g0 + g1));
  ph = fmaf(xyyx, S, ph);
  if (FERM) sp += fmaf(4.0f, fo, fmaf(2.0f, fe, f0 + f1));
}

// ------------------------------------------------ packed pairs (f32x2) --
// Two instances per thread: every FP32 operation of the segment runs as one
// packed fma/add/mul.rn.f32x2 on the pair (each half rounds exactly like the
// scalar operation), which halves the issue slots of the FP32 work; the MUFU
// reciprocals and the clamps stay per half.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 max2(float2 a, float b) {
  return make_float2(fmaxf(a.x, b), fmaxf(a.y, b));
}
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(rcp_fast(a.x), rcp_fast(a.y)); }
// rcp_newton on a pair: the seeds per half, the refinement as packed FMAs
__device__ __forceinline__ float2 rcp_newton2(float2 d) {
  const float2 nd = neg2(d);
  float2 x = make_float2(__int_as_float(0x7ef311c2 - __float_as_int(d.x)),
                         __int_as_float(0x7ef311c2 - __float_as_int(d.y)));
  float2 e = fma2(nd, x, f2(1.0f));
  x = fma2(x, e, x);
  e = fma2(nd, x, f2(1.0f));
  return fma2(x, fma2(e, e, e), x);
}

// the light profiles on a pair: g = f/rho^2 and fp = f'/fp_scale as in eval
template <int P>
__device__ __forceinline__ void eval2(float2 r2, const FieldDev &F, float2 &g, float2 &fp) {
  if constexpr (P == kSmooth) {
    g = rcp2(r2);
    fp = mul2(g, g);
  } else if constexpr (P == kGaussian) {  // as Profile<kGaussian>::eval, per half
    const float2 x = mul2(r2, f2(F.inv_l2));
    const float2 a = mul2(x, f2(-1.4426950408889634f));
    const float2 e = make_float2(ex2_fast(a.x), ex2_fast(a.y));
    // the small-x polynomial of one_minus_expneg_over_x, on the pair
    float2 p = f2(-0.0011216341517865658f);
    p = fma2(p, x, f2(0.008187385275959969f));
    p = fma2(p, x, f2(-0.041629087179899216f));
    p = fma2(p, x, f2(0.16666224598884583f));
    p = fma2(p, x, f2(-0.4999998211860657f));
    p = fma2(p, x, f2(1.0f));
    const float2 sm = mul2(p, f2(F.inv_l2));
    const float2 bg = mul2(add2(f2(1.0f), neg2(e)), rcp2(r2));
    g = make_float2(x.x < 0.5f ? sm.x : bg.x, x.y < 0.5f ? sm.y : bg.y);
    fp = e;
  } else {
    Profile<P>::eval(r2.x, F, g.x, fp.x);
    Profile<P>::eval(r2.y, F, g.y, fp.y);
  }
}

// segment() on a pair of instances (same loop segment, two centres / T)
template <int P, bool FERM, int NINT>
__device__ __forceinline__ void segment2(float2 zix, float2 ziy, float2 zjx, float2 zjy,
                                         const FieldDev &F, float2 &ph, float2 &sp) {
  static_assert(!Profile<P>::kHeavy && NINT >= 4, "pairs: light profiles, fixed intervals");
  constexpr int kSoftRcp = soft_rcp_period<P, FERM, NINT, true>();
  const float2 dx = add2(zjx, neg2(zix)), dy = add2(zjy, neg2(ziy));
  float2 a = fma2(zix, zix, mul2(ziy, ziy));
  float2 b = fma2(zix, dx, mul2(ziy, dy));
  float2 c = fma2(dx, dx, mul2(dy, dy));
  const float2 xyyx = fma2(zix, zjy, neg2(mul2(ziy, zjx)));
  a = max2(a, F.clampA);
  b = max2(b, F.clampB);
  c = max2(c, F.clampC);
  const float2 as = add2(a, f2(profile_shift<P>(F)));
  // (as + 2b) + c as the scalar segment rounds it: 2b is exact, so the fma
  // rounds once as the sum does and 2b needs no register or operation
  const float2 ae = add2(fma2(b, f2(2.0f), as), c);
  float2 g0, f0, g1, f1;
  eval2<P>(as, F, g0, f0);
  eval2<P>(ae, F, g1, f1);
  // Simpson sums opened by their first node rather than by 0 + node, two
  // operations fewer per sum.  The smooth profile's f' = g^2 enters its sums
  // as explicit fma (the square of each later node fused into the running
  // sum), so no sum of two products is left for the compiler to contract
  // one way or the other.
  constexpr bool kSq = (P == kSmooth);
  float2 so, se, fo, fe;
#pragma unroll
  for (int j = 1; j < NINT; j++) {
    const float t = (float)j * (1.0f / (float)NINT);
    // as + t (2b + c t) = as + 2t (b + c t/2): halving and doubling are
    // exact, so both fma round as the scalar segment's do
    const float2 r2 = fma2(fma2(c, f2(0.5f * t), b), f2(2.0f * t), as);
    float2 g, fp;
    if (kSoftRcp > 0 && j % kSoftRcp == kSoftRcp - 1) {  // smooth only: g = 1/(l2 + rho^2)
      g = rcp_newton2(r2);
      fp = mul2(g, g);
    } else {
      eval2<P>(r2, F, g, fp);
    }
    if (j & 1) {
      so = j == 1 ? g : add2(so, g);
      if (FERM) fo = j == 1 ? (kSq ? mul2(g, g) : fp) : (kSq ? fma2(g, g, fo) : add2(fo, fp));
    } else {
      se = j == 2 ? g : add2(se, g);
      if (FERM) fe = j == 2 ? (kSq ? mul2(g, g) : fp) : (kSq ? fma2(g, g, fe) : add2(fe, fp));
    }
  }
  const float2 S = fma2(f2(4.0f), so, fma2(f2(2.0f), se, add2(g0, g1)));
  ph = fma2(xyyx, S, ph);
  if (FERM) {
    const float2 f01 = kSq ? fma2(g1, g1, mul2(g0, g0)) : add2(f0, f1);
    sp = add2(sp, fma2(f2(4.0f), fo, fma2(f2(2.0f), fe, f01)));
  }
}

// segment2 as a called function for many intervals: one copy of the long
// node sequence instead of one per call site of the sweep (a dozen), which
// keeps the kernel within the instruction cache; the sums travel by value
#ifndef WL_SEG2_CALL_MIN
#define WL_SEG2_CALL_MIN 8
#endif
template <int P, bool FERM, int NINT>
__device__ __noinline__ float4 segment2_called(float2 zix, float2 ziy, float2 zjx, float2 zjy,
                                               const FieldDev &F, float4 acc) {
  float2 ph = make_float2(acc.x, acc.y), sp = make_float2(acc.z, acc.w);
  segment2<P, FERM, NINT>(zix, ziy, zjx, zjy, F, ph, sp);
  return make_float4(ph.x, ph.y, sp.x, sp.y);
}
template <int P, bool FERM, int NINT>
__device__ __forceinline__ void seg2(float2 zix, float2 ziy, float2 zjx, float2 zjy,
                                     const FieldDev &F, float2 &ph, float2 &sp) {
  if constexpr (NINT >= WL_SEG2_CALL_MIN) {
    const float4 r = segment2_called<P, FERM, NINT>(zix, ziy, zjx, zjy, F,
                                                    make_float4(ph.x, ph.y, sp.x, sp.y));
    ph = make_float2(r.x, r.y);
    sp = make_float2(r.z, r.w);
  } else {
    segment2<P, FERM, NINT>(zix, ziy, zjx, zjy, F, ph, sp);
  }
}

__device__ __forceinline__ void kahan_add2(float2 &sum, float2 &comp, float2 x) {
  const float2 y = add2(x, neg2(comp));
  const float2 t = add2(sum, y);
  comp = add2(add2(t, neg2(sum)), neg2(y));
  sum = t;
}

// ---------------------------------------------------------- lattice --
// Square lattice of Gaussian tubes at R = a(m, n).  Per (loop, instance) the
// images within rcut of the loop's scaled bounding box (and |R| <= rimage)
// are summed; farther images are pure gauge outside the loop and contribute 0.
template <>
struct Profile<kLattice> {  // spin integrand f' = e^{-x}/l2, x = rho^2/l2
  static __device__ __forceinline__ float fp_scale(const FieldDev &F) { return F.inv_l2; }
  static constexpr bool kHeavy = false;
};

struct ImgRange {
  int m0, m1, n0, n1;
  int inside;  // the whole range lies in the disk m^2 + n^2 <= (rimage/a)^2
};

__device__ __forceinline__ ImgRange image_range(float4 bb, float s, float cx, float cy,
                                                const FieldDev &F) {
  const float inva = 1.0f / F.a;
  const int lim = (int)floorf(sqrtf(F.rimg2));
  ImgRange r;
  r.m0 = max(-lim, (int)ceilf((fmaf(s, bb.x, cx) - F.rcut) * inva));
  r.m1 = min(lim, (int)floorf((fmaf(s, bb.y, cx) + F.rcut) * inva));
  r.n0 = max(-lim, (int)ceilf((fmaf(s, bb.z, cy) - F.rcut) * inva));
  r.n1 = min(lim, (int)floorf((fmaf(s, bb.w, cy) + F.rcut) * inva));
  const int mx = max(abs(r.m0), abs(r.m1)), nx = max(abs(r.n0), abs(r.n1));
  r.inside = (float)(mx * mx) + (float)(nx * nx) <= F.rimg2;
  return r;
}

// (1 - e^-x)/x and e^-x for x >= 0 (x slightly below 0 from rounding is fine);
// below x = 0.5 the series avoids the cancellation of 1 - e^-x.  Both forms
// are evaluated and one selected: a warp-uniform branch around the series
// measured 30 % slower on the lattice (it splits the unrolled Simpson nodes).
__device__ __forceinline__ void gauss_q(float x, float &q, float &e) {
  e = expneg_fast(x);
  const float big = (1.0f - e) * rcp_fast(x);
  const float small = one_minus_expneg_over_x(x);
  q = x < 0.5f ? small : big;
}

// gauss_q2 where every x >= 0.5: the large-x form alone, without the small-x
// polynomial.  The form is still taken through a select against a bound no
// node reaches (x < neg1, the caller passing -1 as a run-time value): so
// written, a walk's sums are bit-identical to gauss_q2's on the lattice
// parity cases; with the product returned directly they were not (measured
// on the GB300; the cause was not found in the source), and the lattice
// kernel needs the two walks to agree bit for bit.
__device__ __forceinline__ void gauss_q2_big(float2 x, float2 &q, float2 &e, float neg1) {
  const float2 a = mul2(f2(-1.4426950408889634f), x);
  e = make_float2(ex2_fast(a.x), ex2_fast(a.y));
  const float2 big = mul2(add2(f2(1.0f), neg2(e)), rcp2(x));
  q = make_float2(x.x < neg1 ? 0.0f : big.x, x.y < neg1 ? 0.0f : big.y);
}
// gauss_q on a pair (each half as gauss_q)
__device__ __forceinline__ void gauss_q2(float2 x, float2 &q, float2 &e) {
  const float2 a = mul2(f2(-1.4426950408889634f), x);
  e = make_float2(ex2_fast(a.x), ex2_fast(a.y));
  const float2 big = mul2(add2(f2(1.0f), neg2(e)), rcp2(x));
  float2 p = f2(-0.0011216341517865658f);
  p = fma2(p, x, f2(0.008187385275959969f));
  p = fma2(p, x, f2(-0.041629087179899216f));
  p = fma2(p, x, f2(0.16666224598884583f));
  p = fma2(p, x, f2(-0.4999998211860657f));
  p = fma2(p, x, f2(1.0f));
  q = make_float2(x.x < 0.5f ? p.x : big.x, x.y < 0.5f ? p.y : big.y);
}

// One segment z_i -> z_j against every image of the range: in units of
// x = rho^2/lambda^2, the reference's Gaussian Simpson integral per image,
// exact mode (no clamps).  Adds sum_R (u_R x Delta)/l2 * sum_w q(x) to ph and
// sum_R sum_w e^-x to sp (the f' scale 1/l2 is applied per loop).  Not
// inlined: the image loop with its five node evaluations is large, and one
// copy of it per call site (a dozen in the sweep) overflowed the instruction
// cache (ncu: "no instruction" the top stall); returns the updated (ph, sp).
template <bool FERM, int NINT>
__device__ __noinline__ float2 segment_lattice(float zix, float ziy, float zjx, float zjy,
                                               const FieldDev &F, const ImgRange img,
                                               float ph, float sp) {
  const float dx = zjx - zix, dy = zjy - ziy;
  const float il2 = F.inv_l2;
  const float cs = fmaf(dx, dx, dy * dy) * il2;
  const int nint = NINT > 0 ? NINT : F.nint;
  const float h = NINT > 0 ? 1.0f / (float)NINT : F.h;
  // the whole range inside the disk (the usual case): no per-row trimming
  const bool inside = img.inside;
  for (int m = img.m0; m <= img.m1; ++m) {
    const float ux = fmaf(-(float)m, F.a, zix);
    const float mm = (float)(m * m);
    // this row's images inside the disk (an interval)
    int lo = img.n0, hi = img.n1;
    if (!inside) {
      while (lo <= hi && mm + (float)(lo * lo) > F.rimg2) ++lo;
      while (hi >= lo && mm + (float)(hi * hi) > F.rimg2) --hi;
    }
    int n = lo;
    if constexpr (NINT > 0) {
      // two images per step as packed pairs: every FP32 operation of the two
      // images is one f32x2 operation (each half rounds as the single-image
      // code below) and the sums are added in image order
      for (; n < hi; n += 2) {
        const float2 uy = make_float2(fmaf(-(float)n, F.a, ziy), fmaf(-(float)(n + 1), F.a, ziy));
        const float2 ux2 = f2(ux), dx2 = f2(dx), dy2 = f2(dy), il22 = f2(il2);
        const float2 as = mul2(fma2(ux2, ux2, mul2(uy, uy)), il22);
        const float2 bs2 = mul2(mul2(f2(2.0f), fma2(ux2, dx2, mul2(uy, dy2))), il22);
        const float2 cross = mul2(fma2(ux2, dy2, neg2(mul2(uy, dx2))), il22);
        float2 q0, e0, q1, e1;
        gauss_q2(as, q0, e0);
        gauss_q2(add2(add2(as, bs2), f2(cs)), q1, e1);
        float2 so = f2(0.f), se = f2(0.f), fo = f2(0.f), fe = f2(0.f);
#pragma unroll
        for (int j = 1; j < NINT; j++) {
          const float t = (float)j * (1.0f / (float)NINT);
          float2 q, e;
          gauss_q2(fma2(fma2(f2(cs), f2(t), bs2), f2(t), as), q, e);
          if (j & 1) {
            so = add2(so, q);
            if (FERM) fo = add2(fo, e);
          } else {
            se = add2(se, q);
            if (FERM) fe = add2(fe, e);
          }
        }
        const float2 S = fma2(f2(4.0f), so, fma2(f2(2.0f), se, add2(q0, q1)));
        ph = fmaf(cross.x, S.x, ph);
        ph = fmaf(cross.y, S.y, ph);
        if (FERM) {
          const float2 SP = fma2(f2(4.0f), fo, fma2(f2(2.0f), fe, add2(e0, e1)));
          sp += SP.x;
          sp += SP.y;
        }
      }
    }
    for (; n <= hi; ++n) {
      const float uy = fmaf(-(float)n, F.a, ziy);
      const float as = fmaf(ux, ux, uy * uy) * il2;
      const float bs2 = 2.0f * fmaf(ux, dx, uy * dy) * il2;
      const float cross = fmaf(ux, dy, -(uy * dx)) * il2;  // (z_i - R) x (z_j - R) / l2
      float q0, e0, q1, e1;
      gauss_q(as, q0, e0);
      gauss_q((as + bs2) + cs, q1, e1);
      float so = 0.f, se = 0.f, fo = 0.f, fe = 0.f;
      auto node = [&](int j, float t) {
        float q, e;
        gauss_q(fmaf(fmaf(cs, t, bs2), t, as), q, e);
        if (j & 1) {
          so += q;
          if (FERM) fo += e;
        } else {
          se += q;
          if (FERM) fe += e;
        }
      };
      if constexpr (NINT > 0) {
#pragma unroll
        for (int j = 1; j < NINT; j++) node(j, (float)j * (1.0f / (float)NINT));
      } else {
#pragma unroll 1
        for (int j = 1; j < nint; j++) node(j, (float)j * h);
      }
      ph = fmaf(cross, fmaf(4.0f, so, fmaf(2.0f, se, q0 + q1)), ph);
      if (FERM) sp += fmaf(4.0f, fo, fmaf(2.0f, fe, e0 + e1));
    }
  }
  return make_float2(ph, sp);
}

// the segment of profile P (the image range is used by the lattice only)
template <int P, bool FERM, int NINT>
__device__ __forceinline__ void seg(float zix, float ziy, float zjx, float zjy,
                                    const FieldDev &F, const ImgRange &img, float &ph,
                                    float &sp) {
  if constexpr (P == kLattice) {
    const float2 r = segment_lattice<FERM, NINT>(zix, ziy, zjx, zjy, F, img, ph, sp);
    ph = r.x;
    sp = r.y;
  } else if constexpr ((P == kFixflux || P == kFixfluxFF) && NINT == 0) {
    const float2 r =
        segment_fixflux<P == kFixfluxFF, FERM>(zix, ziy, zjx, zjy, F, ph, sp);
    ph = r.x;
    sp = r.y;
  } else {
    segment<P, FERM, NINT>(zix, ziy, zjx, zjy, F, ph, sp);
  }
}

// Kahan compensated accumulation: sum - comp is the running total.
__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
  const float y = x - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// ------------------------------------------------- double-float (FP32 pairs) --
// The per-loop phases and spin exponents reach |x| ~ 1e2-1e3; FP32 rounding of
// their scale factors would shift every loop coherently (relative 1e-7, i.e.
// 1e-5 in cosh(60)).  The per-loop epilogue therefore works on unevaluated
// sums hi + lo of two floats (error-free transformations of Knuth / Dekker).
struct df {
  float hi, lo;
};
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df df_mul(df x, df y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + x.lo + y.lo);
}
__device__ __forceinline__ df df_scale2(df x, float p2) { return {x.hi * p2, x.lo * p2}; }

// cos(x.hi + x.lo) - 1, accurate relative to the deviation itself (small
// phases give W - 1 ~ 1e-9 that the proper-time integrand needs, Tint.c).
// Cody-Waite reduction by 2 pi = C1 + C2 + C3 (Cody and Waite, Software
// Manual for the Elementary Functions, 1980): C1 = 6.28125 has 8 significant
// bits, so k*C1 is exact for |k| < 2^16 and x.hi - k*C1 is exact (Sterbenz);
// then with s, c = sin, cos of r/2:  cos(r + e) - 1 = -2 s^2 - 2 s c e.
__device__ __forceinline__ float cosm1_df(df x) {
  const float k = rintf(x.hi * 0.15915494f);
  const float t = fmaf(-k, 6.28125f, x.hi);
  const float u = fmaf(-k, 1.9353071693331003e-3f, x.lo);
  df r = two_sum(t, u);
  r.lo = fmaf(-k, 1.0253131677018246e-11f, r.lo);
  float sn, cs;
  sincosf(0.5f * r.hi, &sn, &cs);
  return -2.0f * sn * fmaf(cs, r.lo, sn);
}

// The reference's sentinel: C abs() of a double truncates to int
// (Integrand.c:371), so it fires for |x| >= 601; conversions beyond the int
// range give INT_MIN on x86 (no sentinel), which is mirrored.
__device__ __forceinline__ bool sentinel600(float x) {
  const float ax = fabsf(x);
  return ax >= 601.0f && ax < 2147483648.0f;
}

// cosh(x.hi + x.lo) - 1 in FP64 range.  Below |x| = 80 from FP32:
// cosh(a + e) - 1 = 2 sinh^2(a/2) + e sinh a, accurate for small a; above,
// FP64 exp (FP32 overflows near 89 while the reference's FP64 cosh is finite
// up to 710).
__device__ __forceinline__ double coshm1_df(df x) {
  const float a = fabsf(x.hi), e = x.hi < 0.0f ? -x.lo : x.lo;
  if (a < 80.0f) {
    const float sh = sinhf(0.5f * a);
    const float ch = sqrtf(fmaf(sh, sh, 1.0f));
    // sinh a = 2 sinh(a/2) cosh(a/2)
    return (double)fmaf(2.0f * sh * ch, e, 2.0f * sh * sh);
  }
  return 0.5 * exp((double)a + (double)e) - 1.0;
}

// Per-loop factors of EVMean (Integrand.c:352-390) from the sub-loop phases
// p[k] and spin exponents q[k] (k: N/2, N/4b, N/4a), returned as deviations
// d = w - 1 (the sums of deviations keep <W> - 1 accurate):
//   w0 = W_N   = cos(p0/2 + (p1+p2)/4) [* cosh(same of q)]
//   w1 = W_N/2 = cos(p0)                [* cosh(q0)]
//   w2 = W_N/4 = cos((p1+p2)/2)         [* cosh(same of q)]
// with the reference's 1e10 sentinel when a spin exponent truncates above 600.
template <bool FERM>
__device__ __forceinline__ void wfactors(const df p[3], const df q[3], double &d0, double &d1,
                                         double &d2) {
  const df nb4 = df_add(p[1], p[2]);
  const float c0 = cosm1_df(df_add(df_scale2(p[0], 0.5f), df_scale2(nb4, 0.25f)));
  const float c1 = cosm1_df(p[0]);
  const float c2 = cosm1_df(df_scale2(nb4, 0.5f));
  d0 = c0;
  d1 = c1;
  d2 = c2;
  if (FERM) {
    const df nb4f = df_add(q[1], q[2]);
    if (sentinel600(nb4f.hi) || sentinel600(q[0].hi)) {
      d0 = (1.0 + (double)c0) * 1.0e10 - 1.0;
      d1 = (1.0 + (double)c1) * 1.0e10 - 1.0;
      d2 = (1.0 + (double)c2) * 1.0e10 - 1.0;
    } else {
      // cos * cosh - 1 = (cos - 1) cosh + (cosh - 1)
      const double h0 = coshm1_df(df_add(df_scale2(q[0], 0.5f), df_scale2(nb4f, 0.25f)));
      const double h1 = coshm1_df(q[0]);
      const double h2 = coshm1_df(df_scale2(nb4f, 0.5f));
      d0 = (double)c0 * (1.0 + h0) + h0;
      d1 = (double)c1 * (1.0 + h1) + h1;
      d2 = (double)c2 * (1.0 + h2) + h2;
    }
  }
}

// Finishes one loop at one instance (intEV.cu:553-561 with the EVMean
// factors).  G[k], H[k]: the loop's Simpson sums of xyyx f/rho^2 and of f'
// (without h/3 and the f' scale).  Per flux value j, cph_j = F_j h/3 and
// csp_j = F_j h/3 fp_scale are double-float constants and tq = 4T/N is the
// instance's, so the phase is F G h/3 and the spin exponent 2 F T sum/(N/2)
// (N/2 loop) or 2 F T sum/(N/4) (N/4 loops).  add(j, d0, d1, d2) receives the
// W factors minus one (accumulated in FP64 by the caller).
template <bool FERM, class Add>
__device__ __forceinline__ void loop_epilogue(const df G[3], const df H[3], const float *cph_hi,
                                              const float *cph_lo, const float *csp_hi,
                                              const float *csp_lo, df tq, int nF, Add &&add) {
#pragma unroll
  for (int j = 0; j < kMaxF; ++j) {
    if (j < nF) {
      const df cph = {cph_hi[j], cph_lo[j]};
      df p[3], q[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) p[k] = df_mul(cph, G[k]);
      if (FERM) {
        const df csp = df_mul(df{csp_hi[j], csp_lo[j]}, tq);
        q[0] = df_mul(csp, H[0]);
        q[1] = df_scale2(df_mul(csp, H[1]), 2.0f);
        q[2] = df_scale2(df_mul(csp, H[2]), 2.0f);
      } else {
        q[0] = q[1] = q[2] = df{0.0f, 0.0f};
      }
      double w0, w1, w2;
      wfactors<FERM>(p, q, w0, w1, w2);
      add(j, w0, w1, w2);
    }
  }
}

// ------------------------------------------ bulk copy + mbarrier (PTX) --
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "{ .reg .b64 st; mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1; }" ::"r"(
          smem_addr(bar)),
      "r"(bytes)
      : "memory");
}
// global -> shared bulk copy (non-tensor TMA); addresses 16-byte aligned,
// size a multiple of 16 bytes; completion is signalled on bar.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Bounded wait on an mbarrier phase: returns false when max_tries polls
// (each a hardware-suspended try_wait) did not see the phase complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint32_t max_tries) {
  const uint32_t addr = smem_addr(bar);
  for (uint32_t it = 0; it < max_tries; ++it) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, "
        "1, 0, p; }"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace wl
