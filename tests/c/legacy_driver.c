/*
 * legacy_driver.c -- a C driver in the reference's own style, built against
 * include/intT.h and linked with libwlhost.so + libwlgpu.so, for
 * tests/test_gpu_tint.py.  It sets up struct Wparams as EffAct.c:368-413 does
 * (text ensemble read by getwl, device buffers by cudaMalloc / cudaMemcpy),
 * configures the profile the reference fixes at compile time, and calls
 * integrateT (Tint.c:100-175) for one centre of mass, printing the per-group
 * proper-time integrals after the Leffvsrho line integrateT itself prints.
 *
 *   legacy_driver <loops.txt> <Nl> <Nppl> <rho> <F> <lambda2> <fermion> <nint> <panels>
 */
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "intT.h"
#include "wl_host.h"
#include "wlgpu.h"

int main(int argc, char **argv) {
  if (argc != 10) {
    fprintf(stderr, "usage: %s loops.txt Nl Nppl rho F lambda2 fermion nint panels\n", argv[0]);
    return 2;
  }
  const int Nl = atoi(argv[2]), Nppl = atoi(argv[3]);
  const double rho = atof(argv[4]), F = atof(argv[5]), l2 = atof(argv[6]);
  const int fermion = atoi(argv[7]), nint = atoi(argv[8]), panels = atoi(argv[9]);
  const size_t npts = (size_t)Nl * Nppl;
  float4 *wl_h = (float4 *)calloc(npts, sizeof(float4));
  if (!wl_h || getwl(wl_h, argv[1], Nl, Nppl, 2) != 0) return 3;  /* x then y per loop */
  struct Wparams params = {0};
  params.Nl = Nl;
  params.Nppl = Nppl;
  params.F = F;
  params.l2 = l2;
  params.xcm.x = (float)rho;
  params.xcm.y = 0.0f;
  params.fermion = fermion;
  params.ng = Nl / 128;
  params.Wsscal_h = (float4 *)calloc((size_t)Nl, sizeof(float4));
  params.Wsferm_h = (float4 *)calloc((size_t)Nl, sizeof(float4));
  if (cudaMalloc((void **)&params.worldlines, npts * sizeof(float4)) != cudaSuccess ||
      cudaMalloc((void **)&params.Wsscal_d, (size_t)Nl * sizeof(float4)) != cudaSuccess ||
      cudaMalloc((void **)&params.Wsferm_d, (size_t)Nl * sizeof(float4)) != cudaSuccess)
    return 4;
  cudaMemcpy(params.worldlines, wl_h, npts * sizeof(float4), cudaMemcpyHostToDevice);
  if (wl_legacy_configure(profile, tubedist, lmin, nint, WL_MODE_REFCOMPAT) != WL_OK) return 5;
  double *I = integrateT(panels, &params);
  if (!I) return 6;
  for (int g = 0; g < params.ng; g++) printf("I %d %.17g\n", g, I[g]);
  free(I);
  cudaFree(params.worldlines);
  cudaFree(params.Wsscal_d);
  cudaFree(params.Wsferm_d);
  free(params.Wsscal_h);
  free(params.Wsferm_h);
  free(wl_h);
  return 0;
}
