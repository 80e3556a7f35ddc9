/*
 * wl_legacy.h -- the legacy host ABI of the Wilson-loop path, without macros.
 *
 * The reference's own header intT.h is not in its source tree (it is included by
 * EffAct.c:5, intEV.cu:7, Tint.c:11, Integrand.c:7, testT.c:5 and listed as a
 * Makefile dependency, Makefile:3-28).  This header restates the one type every
 * caller shares, struct Wparams, from how the fields are used:
 *   EffAct.c:399-413, 454-455   (filled by main)
 *   intEV.cu:115, 123-125       (read by value in EV, passed to the kernel)
 *   Integrand.c:198-208         (read by Tfunc / MagField)
 *   Tint.c:110-126, EffAct.c:21-25  (ng, Nl, xcm)
 * and declares the legacy entry points with their reference signatures.
 *
 * Library code includes this header; legacy C host code includes intT.h, which
 * adds the reference's profile macros and constants on top of it.
 */
#ifndef WL_LEGACY_H
#define WL_LEGACY_H

#include <vector_types.h> /* float4 (CUDA's plain-C vector types, no device code) */

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters of one Wilson-loop evaluation, shared by the legacy callers.
 * Ownership follows EffAct.c:368-395: the caller allocates every buffer.     */
struct Wparams {
  int Nl;            /* number of loops in the ensemble                        */
  int Nppl;          /* points per loop (must be a multiple of 4)              */
  double F;          /* flux parameter F (Phi = 2 pi F f_lambda)               */
  double l2;         /* lambda^2, the tube width squared                       */
  float4 xcm;        /* centre of mass of the loops (x, y used)                */
  float4 *Wsscal_h;  /* host   [Nl]: scalar phases of the N/2, N/4b, N/4a loops */
  float4 *Wsscal_d;  /* device [Nl]: same, written by the kernel              */
  float4 *Wsferm_h;  /* host   [Nl]: spin-factor exponents (fermion only)      */
  float4 *Wsferm_d;  /* device [Nl]                                            */
  float4 *worldlines;/* device [Nl*Nppl] unit loops, AoS float4 (x, y, z, w)   */
  double SE;         /* unused by the path (set to 0 by EffAct.c:409)          */
  int nBlocks;       /* launch geometry of the reference kernel (ignored here) */
  int nThreads;
  int ng;            /* number of loop groups of 128 (Integrand.c:204, 249)    */
  int fermion;       /* 1 = spinor QED (spin factor), 0 = scalar QED           */
  float4 *flcoefs;   /* spline profile coefficients (spline profile only)      */
  float *rho2sp;     /* spline profile knots (spline profile only)             */
};

/* <W> of one group of 128 loops at proper time T (intEV.cu:111-148).
 * p points at a struct Wparams; WLlist holds the 128 loop indices of the group. */
double EV(double T, void *p, int *WLlist);

/* Proper-time integrand per group (Integrand.c:195-316) and its Simpson
 * integral over T in (0, inf) (Tint.c:100-175).  Both return malloc'd arrays of
 * length ng that the caller frees.                                            */
double *Tfunc(double T, void *p, int *order);
double *integrateT(int n, void *p);

/* Text reader of a loop ensemble (getwl.c:6-40).  Per loop: Nppl x values, then
 * Nppl y values (Dim > 1), then Nppl z values (Dim > 2).                      */
int getwl(float4 *worldlines, char *filename, int Nl, int Nppl, int Dim);

#ifdef __cplusplus
}
#endif

#endif /* WL_LEGACY_H */
