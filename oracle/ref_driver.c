/*
 * ref_driver.c -- runs the reference's own code on the CPU to produce golden
 * vectors.  TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.sh into
 * oracle/_ref/, never shipped, never linked by the product).
 *
 * Linked with, compiled unmodified from the reference tree:
 *   intEV.cu (or intEVff.cu)  with its __device__ functions made host-callable
 *                             (refshim/intT.h, WLREF_HOSTCALL),
 *   Integrand.c, Tint.c       (EVMean, Tfunc, MagField, Exact, integrateT ...).
 * This file supplies what the reference gets from elsewhere:
 *   - EV(): the body of intEV.cu:111-148 with the kernel launch replaced by a
 *     host loop of the reference's WilsonLoop over all loops (the kernel is one
 *     thread per loop, intEV.cu:573-582), then the reference's EVMean;
 *   - main(): a command-line front end writing raw little-endian results.
 *
 * Usage (all numbers decimal; loops file = raw float32 [Nl][ppl][4]):
 *   ref_driver loops  Nl ppl cx cy T F l2 fermion a loops.bin out.bin
 *       -> float32 [Nl][8]: Wsscal (x,y,z,w) then Wsferm (x,y,z,w)
 *   ref_driver ev     Nl ppl cx cy T F l2 fermion a loops.bin out.bin
 *       -> float64 [Nl/128]: EV() of each identity-ordered group of 128
 *   ref_driver tfunc  Nl ppl cx cy T F l2 fermion a loops.bin out.bin
 *       -> float64 [Nl/128]: Tfunc(T)
 *   ref_driver intT   Nl ppl cx cy n F l2 fermion a loops.bin out.bin
 *       -> float64 [Nl/128]: integrateT(n)
 *   ref_driver funcs  l2 F fermion a in.bin out.bin
 *       in: float64 pairs (rho2, T); out: float64 [k][6]:
 *       flambda(rho2), fplambda(rho2), MagField(rho2), Exact(T, B(rho2)),
 *       smTscal(B, T), smTferm(B, T)
 */
#define _GNU_SOURCE
#include <fenv.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/wl_legacy.h"

float wlref_tubedist = 1.0f;

/* reference symbols (extern "C" in intEV.cu / intEVff.cu; C in Integrand.c) */
#ifdef WLREF_FF
void WilsonLoop(float4 *worldlines, float4 *Wsscal, float4 *Wsferm, float4 xcm,
                int inx, float F, float l2, float rtT, int Nppl, float4 *flcoefs,
                float *rho2sp);
#else
void WilsonLoop(float4 *worldlines, float4 *Wsscal, float4 *Wsferm, float4 xcm,
                int inx, float F, float l2, float rtT, int Nppl, float4 *flcoefs,
                float *rho2sp, int fermion);
#endif
#ifdef WLREF_FF
/* intEVff.cu has no flambda/fplambda dispatch: its profile functions are
 * called directly (intEVff.cu:194-250) */
float ffixflux(float rho2, float lambda2);
float fpfixflux(float rho2, float lambda2);
#define flambda(r2, l2, c, s) ffixflux(r2, l2)
#define fplambda(r2, l2, c, s) fpfixflux(r2, l2)
#else
float flambda(float rho2, float lambda2, float4 *flcoefs, float *rho2sp);
float fplambda(float rho2, float lambda2, float4 *flcoefs, float *rho2sp);
#endif
void EVMean(double *EV, float4 *Wsscal_h, float4 *Wsferm_h, int n, int *WL, double T,
            int fermion);
double MagField(double rho2, void *p);
double Exact(double T, double B, int fermion);
double smTscal(double B, double T);
double smTferm(double B, double T);

/* all loops at (T, xcm) as the kernel would compute them */
static void run_loops(struct Wparams *pp, double T) {
  float rtT = (float)sqrt(T);
  /* device code raises no floating-point traps; EVMean enables them for the
   * host code that follows it (Integrand.c:339) */
  fedisableexcept(FE_ALL_EXCEPT);
  for (int inx = 0; inx < pp->Nl; inx++) {
#ifdef WLREF_FF
    WilsonLoop(pp->worldlines, pp->Wsscal_h, pp->Wsferm_h, pp->xcm, inx, (float)pp->F,
               (float)pp->l2, rtT, pp->Nppl, pp->flcoefs, pp->rho2sp);
#else
    WilsonLoop(pp->worldlines, pp->Wsscal_h, pp->Wsferm_h, pp->xcm, inx, (float)pp->F,
               (float)pp->l2, rtT, pp->Nppl, pp->flcoefs, pp->rho2sp, pp->fermion);
#endif
  }
}

double EV(double T, void *p, int *WLlist) {
  struct Wparams params = *(struct Wparams *)p;
  double ev = 0.0;
  run_loops(&params, T);
  EVMean(&ev, params.Wsscal_h, params.Wsferm_h, 128, WLlist, T, params.fermion);
  return ev;
}

static float4 *read_loops(const char *path, size_t n) {
  float4 *w = (float4 *)calloc(n, sizeof(float4));
  FILE *fp = fopen(path, "rb");
  if (!w || !fp || fread(w, sizeof(float4), n, fp) != n) {
    fprintf(stderr, "ref_driver: cannot read %s\n", path);
    exit(2);
  }
  fclose(fp);
  return w;
}

static void write_out(const char *path, const void *buf, size_t bytes) {
  FILE *fp = fopen(path, "wb");
  if (!fp || fwrite(buf, 1, bytes, fp) != bytes) {
    fprintf(stderr, "ref_driver: cannot write %s\n", path);
    exit(2);
  }
  fclose(fp);
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  const char *mode = argv[1];
  if (!strcmp(mode, "funcs")) {
    if (argc != 8) return 2;
    struct Wparams params;
    memset(&params, 0, sizeof(params));
    params.l2 = atof(argv[2]);
    params.F = atof(argv[3]);
    params.fermion = atoi(argv[4]);
    wlref_tubedist = (float)atof(argv[5]);
    FILE *fp = fopen(argv[6], "rb");
    if (!fp) return 2;
    fseek(fp, 0, SEEK_END);
    long bytes = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    int k = (int)(bytes / (2 * sizeof(double)));
    double *in = (double *)malloc(bytes), *out = (double *)malloc(sizeof(double) * 6 * k);
    if (fread(in, 1, bytes, fp) != (size_t)bytes) return 2;
    fclose(fp);
    for (int i = 0; i < k; i++) {
      double r2 = in[2 * i], T = in[2 * i + 1];
      out[6 * i + 0] = flambda((float)r2, (float)params.l2, NULL, NULL);
      out[6 * i + 1] = fplambda((float)r2, (float)params.l2, NULL, NULL);
      double B = MagField(r2, &params);
      out[6 * i + 2] = B;
      out[6 * i + 3] = Exact(T, B, params.fermion);
      out[6 * i + 4] = smTscal(B, T);
      out[6 * i + 5] = smTferm(B, T);
    }
    write_out(argv[7], out, sizeof(double) * 6 * k);
    return 0;
  }
  if (argc != 13) return 2;
  struct Wparams params;
  memset(&params, 0, sizeof(params));
  params.Nl = atoi(argv[2]);
  params.Nppl = atoi(argv[3]);
  params.xcm.x = (float)atof(argv[4]);
  params.xcm.y = (float)atof(argv[5]);
  double Tn = atof(argv[6]);
  params.F = atof(argv[7]);
  params.l2 = atof(argv[8]);
  params.fermion = atoi(argv[9]);
  wlref_tubedist = (float)atof(argv[10]);
  params.ng = params.Nl / 128;
  size_t npts = (size_t)params.Nl * params.Nppl;
  params.worldlines = read_loops(argv[11], npts);
  params.Wsscal_h = (float4 *)calloc(params.Nl, sizeof(float4));
  params.Wsferm_h = (float4 *)calloc(params.Nl, sizeof(float4));
  if (!strcmp(mode, "loops")) {
    run_loops(&params, Tn);
    float *out = (float *)malloc(sizeof(float) * 8 * params.Nl);
    for (int l = 0; l < params.Nl; l++) {
      memcpy(out + 8 * l, &params.Wsscal_h[l], sizeof(float4));
      memcpy(out + 8 * l + 4, &params.Wsferm_h[l], sizeof(float4));
    }
    write_out(argv[12], out, sizeof(float) * 8 * params.Nl);
    return 0;
  }
  double *res = NULL;
  if (!strcmp(mode, "ev")) {
    res = (double *)malloc(sizeof(double) * params.ng);
    int WL[128];
    for (int g = 0; g < params.ng; g++) {
      for (int j = 0; j < 128; j++) WL[j] = g * 128 + j;
      res[g] = EV(Tn, &params, WL);
    }
  } else if (!strcmp(mode, "tfunc")) {
    int *order = (int *)malloc(sizeof(int) * params.Nl);
    for (int i = 0; i < params.Nl; i++) order[i] = i;
    res = Tfunc(Tn, &params, order);
  } else if (!strcmp(mode, "intT")) {
    res = integrateT((int)Tn, &params);
  } else {
    return 2;
  }
  fedisableexcept(FE_ALL_EXCEPT);
  write_out(argv[12], res, sizeof(double) * params.ng);
  return 0;
}
