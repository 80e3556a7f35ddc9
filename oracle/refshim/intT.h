/*
 * oracle/refshim/intT.h -- configuration header used only to compile the
 * reference's own sources into oracle/_ref/ (test infrastructure).
 *
 * The reference tree has no intT.h; this one supplies what its sources use
 * (the same reconstruction as include/intT.h) plus two build switches:
 *
 *  WLREF_HOSTCALL  (host pass only) makes the reference's __device__
 *                  functions callable from the host, so that WilsonLoop,
 *                  Idt and the profiles of intEV.cu / intEVff.cu run on the
 *                  CPU exactly as written, with the CUDA-only intrinsics
 *                  __expf / __sinf mapped to expf / sinf.
 *  WLREF_FF        declare the 11-argument kernel of intEVff.cu instead of
 *                  the 12-argument one of intEV.cu.
 *
 * tubedist is a run-time variable on the host (wlref_tubedist) so that one
 * build covers every lattice spacing; device code sees WLREF_TUBEDIST.
 */
#ifndef WLREF_INTT_H
#define WLREF_INTT_H

#include "../../include/wl_legacy.h"

#define step 0
#define smooth 1
#define quadratic 2
#define gaussian 3
#define periodic 4
#define spline 5
#define fixflux 6
#ifndef profile
#define profile smooth
#endif

#define pi 3.14159265358979323846

#ifdef __cplusplus
extern "C" {
#endif
extern float wlref_tubedist;
#ifdef __cplusplus
}
#endif

#if defined(__CUDA_ARCH__)
#ifndef WLREF_TUBEDIST
#define WLREF_TUBEDIST 1.0f
#endif
#define tubedist WLREF_TUBEDIST
#else
#define tubedist wlref_tubedist
#endif

#define lmin (0.1f * tubedist)
#define q1 0.443991f
#define q2 0.0742478f
#define Nspline 1000
#ifndef verbosity
#define verbosity 0
#endif

#if defined(__CUDACC__)
#if defined(WLREF_HOSTCALL)
/* every __device__ function below this point is also compiled for the host */
#undef __device__
#define __device__ __location__(device) __location__(host)
#if !defined(__CUDA_ARCH__)
#define __expf(x) expf(x)
#define __sinf(x) sinf(x)
#endif
#endif
#ifdef WLREF_FF
__global__ void ExpectValue(float4 *Wsscal, float4 *Wsferm, float4 *worldlines,
                            float4 xcm, float F, float l2, float rtT, int Nl,
                            int Nppl, float4 *flcoefs, float *rho2sp);
#else
__global__ void ExpectValue(float4 *Wsscal, float4 *Wsferm, float4 *worldlines,
                            float4 xcm, float F, float l2, float rtT, int Nl,
                            int Nppl, float4 *flcoefs, float *rho2sp, int fermion);
#endif
#endif

#endif /* WLREF_INTT_H */
