/*
 * wl_oracle.h -- CPU restatement of the reference's Wilson-loop path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker of the GPU path: the
 * tests, the smoke check and the CPU-baseline leg of the benchmark call it;
 * the product library never links it.
 *
 * Two precisions of the same restatement are exported:
 *   wlo64_*  all-FP64 (the accuracy oracle),
 *   wlo32_*  FP32 (the reference formula as plain C, used as the CPU baseline).
 *
 * Sources restated (reference file:line):
 *   profiles f_lambda, f'_lambda ............ intEV.cu:151-406, intEVff.cu:134-250
 *   Simpson segment integral Idt ............ intEV.cu:408-459, intEVff.cu:253-297
 *   successor index getzp1 .................. intEV.cu:461-506
 *   per-loop phases WilsonLoop .............. intEV.cu:508-571, intEVff.cu:346-406
 *   group mean + Richardson EVMean .......... Integrand.c:325-407
 *   MagField / Exact / small-T / Tfunc ...... Integrand.c:20-172, 195-316
 *   integrateT / Tintout .................... Tint.c:15-33, 51-73, 100-175
 */
#ifndef WL_ORACLE_H
#define WL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* profile ids: the values of the reconstructed intT.h macros */
enum { WLO_STEP = 0, WLO_SMOOTH = 1, WLO_QUADRATIC = 2, WLO_GAUSSIAN = 3,
       WLO_PERIODIC = 4, WLO_SPLINE = 5, WLO_FIXFLUX = 6,
       /* square lattice of Gaussian tubes: no reference implementation */
       WLO_LATTICE = 8 };

/* clamp modes: 0 reproduces the reference clamps (intEV.cu:418-422, 439),
 * 1 evaluates the segment polynomial exactly (only a 1e-30 floor on rho^2
 * where the profile divides by it).                                           */
enum { WLO_REFCOMPAT = 0, WLO_EXACT = 1 };

typedef struct {
  int profile;     /* WLO_* profile id                                         */
  int fermion;     /* 1: also integrate f' for the spin factor                 */
  int nint;        /* Simpson intervals per segment (even; the reference: 50)  */
  int mode;        /* WLO_REFCOMPAT or WLO_EXACT                               */
  int ff_variant;  /* fixflux: 0 = intEV.cu phi/chi, 1 = intEVff.cu phi/chi   */
  int pad_;
  double lambda2;  /* lambda^2                                                 */
  double tubedist; /* lattice spacing a (periodic, fixflux)                    */
  double lmin;     /* fixflux minimum width (0.1 a in the reference runs)      */
  double rimage;   /* lattice: images R = a(m, n) with |R| <= rimage            */
} wlo_field;

/* Square lattice of identical Gaussian flux tubes (WLO_LATTICE).  No
 * reference implementation: each image tube at R = a(m, n), |R| <= rimage,
 * contributes the single-tube Gaussian segment integral (intEV.cu:408-459 with
 * f = 1 - exp(-rho^2/lambda^2), intEV.cu:282-284) in coordinates relative to
 * R, in exact mode (no clamps: the reference's b >= 1e-8 clamp would break
 * the pure-gauge cancellation of distant images).  Images farther than
 * rcut = sqrt(18) lambda from the loop's bounding box see x = rho^2/lambda^2
 * >= 18 along the whole loop, where f = 1 - e^-x rounds to 1 in FP32 (e^-18 <
 * 2^-25): pure gauge, and the loop does not wind around them, so their
 * continuum contribution is zero and they are skipped.
 * wlo_set_lattice_rcut(r) sets rcut / lambda (r <= 0: sum every image with
 * |R| <= rimage), which the tests use to check the selection.              */
#define WLO_LATTICE_RCUT_L 4.242640687119285 /* sqrt(18) */

/* the spline profile's table (knots x = rho^2 as float values, f at the
 * knots) for lambda^2 and a with n knots, and its interpolant at rho2 */
void wlo_spline_table(double lambda2, double a, int n, double *x, double *f);
double wlo_spline_eval(double rho2, const wlo_field *f);
void wlo_set_lattice_rcut(double r_over_lambda);

/* ---- profiles (FP64) -------------------------------------------------- */
double wlo64_flambda(double rho2, const wlo_field *f);
double wlo64_fplambda(double rho2, const wlo_field *f);
/* f_lambda(rho2)/rho2 as the Simpson integrand uses it */
double wlo64_fl_over_rho2(double rho2, const wlo_field *f);

/* ---- one segment: Simpson integrals of f/rho^2 and f' over t in [0,1]
 *      of rho^2(t) = a + 2 b t + c t^2 (intEV.cu:408-459)                 */
void wlo64_idt(double a, double b, double c, const wlo_field *f,
               double *scalI, double *fermI);

/* ---- one loop: geometric sums with F = 1.
 *   gs[k] = sum over the sub-loop's segments of xyyx * scalI
 *   gf[k] = sum of fermI
 * k = 0: N/2 loop (odd points), 1: N/4b loop (i = 2 mod 4), 2: N/4a loop
 * (i = 0 mod 4) -- the .x/.y/.z slots of Wsscal (intEV.cu:538-551).
 * loop is [ppl][4] float (x, y, z, w); the centre of mass is (cx, cy).     */
void wlo64_loop_sums(const float *loop, int ppl, double cx, double cy,
                     double rtT, const wlo_field *f, double gs[3], double gf[3]);
void wlo32_loop_sums(const float *loop, int ppl, float cx, float cy,
                     float rtT, const wlo_field *f, float gs[3], float gf[3]);

/* ---- per-loop reference outputs: Wsscal / Wsferm of intEV.cu:553-561.
 * scal[l*3+k] = F * gs[k];  ferm[l*3+k] = 2 F T gf[k] / (N/2 or N/4).      */
void wlo64_loops(const float *loops, int Nl, int ppl, double cx, double cy,
                 double T, double F, const wlo_field *f, double *scal,
                 double *ferm);

/* ---- the three per-loop factors of EVMean (Integrand.c:352-390):
 * w[0] = W_N, w[1] = W_N/2, w[2] = W_N/4 (cos, times cosh for spinors, with
 * the 1e10 sentinel when a spin exponent truncates to more than 600).      */
void wlo64_wfactors(const double scal[3], const double ferm[3], int fermion,
                    double w[3]);
/* EVMean over a list of n loop indices (Integrand.c:325-407) */
double wlo64_evmean(const double *scal, const double *ferm, int n,
                    const int *WL, int fermion);

/* ---- many instances: per-group <W> (Richardson-combined).
 * Instances are (cx[i], cy[i], T[i]); all share the field; nF flux values.
 * out[(i*nF + j)*ng + g] = <W> of group g (loops g*G .. g*G+G-1), G = group.
 * scale (may be NULL), same layout: S = 8/3 <|w_N|> + 2 <|w_N/2|> +
 * 1/3 <|w_N/4|>, the magnitude of the Richardson sum's terms (the error
 * scale of the estimator).  nthreads <= 0 uses all OpenMP threads.       */
void wlo64_eval(const float *loops, int Nl, int ppl, int ninst,
                const double *cx, const double *cy, const double *T, int nF,
                const double *F, const wlo_field *f, int group, double *out,
                double *scale, int nthreads);
void wlo32_eval(const float *loops, int Nl, int ppl, int ninst,
                const double *cx, const double *cy, const double *T, int nF,
                const double *F, const wlo_field *f, int group, double *out,
                double *scale, int nthreads);

/* ---- proper-time integrand and integral (FP64) ------------------------ */
typedef struct {
  double m2;       /* electron mass squared (Integrand.c:12)                   */
  double e;        /* electron charge (Integrand.c:14)                         */
} wlo_qed;

double wlo_magfield(double rho2, double F, const wlo_field *f, const wlo_qed *q);
double wlo_exact(double T, double B, int fermion, const wlo_qed *q);
double wlo_smTscal(double B, double T, const wlo_qed *q);
double wlo_smTferm(double B, double T, const wlo_qed *q);
/* regime of Tfunc at (T, rho): 0 small-T series, 1 constant-field exact,
 * 2 large-T asymptotic, 3 Monte Carlo.  *analytic receives the value of the
 * analytic regimes.                                                        */
int wlo_tfunc_regime(double T, double xcmx, double xcmy, double F,
                     const wlo_field *f, const wlo_qed *q, double *analytic);
/* Monte Carlo integrand from a group's <W> (Integrand.c:298-301) */
double wlo_tfunc_mc(double T, double EVg, double xcmx, double xcmy, double F,
                    const wlo_field *f, const wlo_qed *q);
/* integrateT(n) of Tint.c:100-175 on an ensemble: ng groups of 128 loops.
 * val[g] is the T integral of group g; leff/sem receive Tintout's values.  */
void wlo64_integrateT(const float *loops, int Nl, int ppl, int n, int ng,
                      double xcmx, double xcmy, double F, const wlo_field *f,
                      const wlo_qed *q, double *val, double *leff, double *sem,
                      int nthreads);

/* ---- seeded unit-loop ensemble --------------------------------------- */
/* Philox4x32-10 block (Salmon et al., SC'11) */
void wlo_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* loops [Nl][ppl][4] float: closed Brownian bridges of unit proper time,
 * per-component step variance 2/ppl, centre of mass at the origin; loop l
 * uses the draws keyed by (seed, first + l).                               */
void wlo_vloops(uint64_t seed, int first, int Nl, int ppl, float *out);

#ifdef __cplusplus
}
#endif

#endif /* WL_ORACLE_H */
