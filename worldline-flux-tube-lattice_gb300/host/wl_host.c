/*
 * wl_host.c -- the C host layer above the Wilson-loop C ABI (libwlhost.so).
 *
 * Keeps the reference's host calling convention (wl_legacy.h) so that a
 * driver written against it (EffAct.c:15-40 calls integrateT; testT.c:88
 * likewise) runs unchanged on libwlgpu.so:
 *   getwl       text ensemble reader                   (getwl.c:6-40)
 *   Tfunc       proper-time integrand per loop group   (Integrand.c:195-316)
 *   integrateT  Simpson over t in (0,1], T = (1-t)/t   (Tint.c:15-33, 100-175)
 * and, without counterpart in the reference (wl_host.h), the writer of the
 * text format and a binary ensemble file format.
 * The field profile is the one EV() uses (wl_legacy_configure / _query).
 * Physical constants follow Integrand.c:11-14 (m^2 = 1, e = 0.30282212).
 *
 * Simpson rule of integrateT: with the clamp mode WL_MODE_REFCOMPAT the
 * reference's rule is kept, which evaluates its first and last Simpson
 * points at the same abscissa h*(inx+1) (Tint.c:127-130); WL_MODE_EXACT uses
 * the proper composite rule on [h*inx, h*(inx+1)], with the t -> 0 end point
 * (T -> infinity) taken as 0.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/wl_host.h"
#include "../../include/wl_legacy.h"
#include "../../include/wlgpu.h"

#define WLH_API __attribute__((visibility("default")))

static const double wlh_m2 = 1.0;        /* Integrand.c:12 */
static const double wlh_e = 0.30282212;  /* Integrand.c:14 */
static const double wlh_q1 = 0.443991, wlh_q2 = 0.0742478;
static const double wlh_pi = 3.14159265358979323846;

typedef struct {
  int profile, nint, mode;
  double a, lmin;
} wlh_cfg;

static wlh_cfg wlh_config(void) {
  wlh_cfg c = {WL_PROFILE_SMOOTH, 50, WL_MODE_REFCOMPAT, 1.0, 0.1};
  wl_legacy_query(&c.profile, &c.a, &c.lmin, &c.nint, &c.mode);
  return c;
}

/* magnetic field shape of each profile, times 2F/e (Integrand.c:98-140) */
static double wlh_magfield(double rho2, double F, double l2, const wlh_cfg *c) {
  double B = 0.0, a = c->a;
  switch (c->profile) {
    case WL_PROFILE_STEP: B = rho2 < l2 ? 1.0 / l2 : 0.0; break;
    case WL_PROFILE_SMOOTH: B = l2 / ((l2 + rho2) * (l2 + rho2)); break;
    case WL_PROFILE_QUADRATIC: B = rho2 < l2 ? 2.0 / l2 * (1.0 - rho2 / l2) : 0.0; break;
    case WL_PROFILE_GAUSSIAN: B = rho2 < 100.0 * l2 ? exp(-rho2 / l2) / l2 : 0.0; break;
    case WL_PROFILE_PERIODIC: {
      /* Integrand.c:58-96, including its int-truncating abs(fmod(...)) test */
      double rho = sqrt(rho2), lam = sqrt(l2), f;
      double ex = exp(-rho / lam), fl = floor(rho / a), ce = ceil(rho / a);
      if (rho < a) {
        double eb = (a - rho) / lam < 10.0 ? exp(-(rho - a) / lam) : 0.0;
        f = ex / (a * (1.0 + ex) * (1.0 + ex));
        if (rho > 0.0) f += eb / (rho * (1.0 + eb) * (1.0 + eb));
      } else if (fabs(fmod(rho, a)) < 1.0) {
        f = fl / (4.0 * rho);
      } else {
        double e1 = exp(-(rho - fl * a) / lam), e2 = exp(-(rho - ce * a) / lam);
        f = fl * e1 / (rho * (1.0 + e1) * (1.0 + e1)) + ce * e2 / (rho * (1.0 + e2) * (1.0 + e2));
      }
      B = a / (2.0 * log(2.0) * l2) * f;
      break;
    }
    case WL_PROFILE_SPLINE: { /* Integrand.c:128-131 */
      const double s = sin(wlh_pi * sqrt(rho2) / c->a);
      B = 1.0 / (l2 * exp(s * s / l2));
      break;
    }
    case WL_PROFILE_FIXFLUX: {
      /* Integrand.c:39-56: the width ratio is a float there */
      float lf = (float)sqrt(l2), af = (float)a, lmf = (float)c->lmin;
      double lml = (float)((lf - lmf) / (af - lmf));
      double x = 2.0 * sqrt(rho2 / l2);
      double bump = fabs(x) < 1.0 ? exp(-1.0 / (1.0 - x * x)) : 0.0;
      B = 2.0 / (l2 * wlh_q2) * (1.0 - 0.75 * lml) * bump + 3.0 / (a * a) * lml;
      break;
    }
    default: B = 0.0;
  }
  (void)wlh_q1;
  return 2.0 * F / wlh_e * B;
}

/* Integrand.c:20-37 */
static double wlh_exact(double T, double B, int fermion) {
  double TB = wlh_e * T * B, pre = exp(-wlh_m2 * T) / (T * T * T);
  if (B < 1.0e-40) return 0.0;
  if (fermion) return pre * (TB / tanh(TB) - 1.0 - TB * TB / 3.0);
  if (TB < 50.0) return pre * (TB / sinh(TB) - 1.0 + TB * TB / 6.0);
  return pre * (TB * TB / 6.0 - 1.0);
}

/* Integrand.c:142-172 */
static double wlh_small_t(double B, double T, int fermion) {
  double B2 = wlh_e * wlh_e * B * B, B4 = B2 * B2, B6 = B2 * B4, m2 = wlh_m2;
  double T3 = T * T * T, T4 = T3 * T;
  if (fermion)
    return B4 * T * (m2 * T - 1.0) / 45.0 + (2.0 * B6 / 945.0 - B4 * m2 * m2 / 90.0) * T3 +
           (7.0 * B4 * m2 * m2 * m2 - 4.0 * B6 * m2) / 1890.0 * T4;
  return 7.0 / 360.0 * B4 * T * (1.0 - m2 * T) + (147.0 * B4 * m2 * m2 - 31.0 * B6) / 15120.0 * T3 +
         (31.0 * B6 * m2 - 49.0 * B4 * m2 * m2 * m2) / 15120.0 * T4;
}

WLH_API double *Tfunc(double T, void *p, int *order) {
  struct Wparams *params = (struct Wparams *)p;
  const wlh_cfg c = wlh_config();
  const int groupsize = 128; /* Integrand.c:204 */
  double *igrand = (double *)malloc(sizeof(double) * (size_t)(params->ng > 0 ? params->ng : 1));
  int WL[128];
  const double rho2 = (double)params->xcm.x * params->xcm.x + (double)params->xcm.y * params->xcm.y;
  const double rho = params->xcm.x, l2 = params->l2;
  const double B = wlh_magfield(rho2, params->F, l2, &c), TB = wlh_e * T * B;
  double smallT;
  if (!igrand) return NULL;
  switch (c.profile) { /* Integrand.c:219-248 */
    case WL_PROFILE_STEP: smallT = (double)abs((int)(rho * rho - l2)); break;
    case WL_PROFILE_GAUSSIAN: smallT = l2; break;
    case WL_PROFILE_SPLINE: { /* Integrand.c:209, 236-240 */
      const double s2 = sin(2.0 * wlh_pi * rho / c.a);
      smallT = rho / c.a > 1.0e-8 ? c.a * c.a * l2 / (wlh_pi * wlh_pi * s2 * s2) : 1.0e12;
      break;
    }
    case WL_PROFILE_FIXFLUX:
      smallT = rho * rho < l2 / 4.0 ? 0.25 * l2
                                    : 0.25 * l2 + (rho - sqrt(l2) / 2.0) * (rho - sqrt(l2) / 2.0);
      break;
    default: smallT = 0.5 * (l2 + rho * rho);
  }
  for (int i = 0; i < params->ng; i++) {
    if (T < 0.1 && T < 0.01 * smallT) {
      igrand[i] = wlh_small_t(B, T, params->fermion);
    } else if (T < 0.01 * smallT) {
      igrand[i] = TB > 1.0e-6 ? wlh_exact(T, B, params->fermion) : 0.0;
    } else if (T > 49.0) {
      igrand[i] = params->fermion ? -exp(-wlh_m2 * T) / (3.0 * T) * wlh_e * wlh_e * B * B
                                  : exp(-wlh_m2 * T) / (6.0 * T) * wlh_e * wlh_e * B * B;
    } else {
      for (int j = 0; j < groupsize; j++) WL[j] = order[j + i * groupsize];
      double ev = EV(T, p, WL);
      igrand[i] = params->fermion ? exp(-wlh_m2 * T) / (T * T * T) * (ev - 1.0 - TB * TB / 3.0)
                                  : exp(-wlh_m2 * T) / (T * T * T) * (ev - 1.0 + TB * TB / 6.0);
    }
  }
  return igrand;
}

/* Tfunc at T = (1 - t)/t times the Jacobian 1/t^2 (Tint.c:15-33); infinite
 * values are replaced by 0 as Tint.c:132-149 does. */
static double *wlh_transform(double t, void *p, int *order) {
  struct Wparams *params = (struct Wparams *)p;
  double *f = Tfunc((1.0 - t) / t, p, order);
  if (!f) return NULL;
  for (int g = 0; g < params->ng; g++) {
    f[g] = f[g] / t / t;
    if (isinf(f[g])) f[g] = 0.0;
  }
  return f;
}

WLH_API double *integrateT(int n, void *p) {
  struct Wparams *params = (struct Wparams *)p;
  const wlh_cfg c = wlh_config();
  const int ng = params->ng;
  const double h = 1.0 / (double)n;
  double *val = (double *)calloc((size_t)(ng > 0 ? ng : 1), sizeof(double));
  int *order = (int *)malloc(sizeof(int) * (size_t)(params->Nl > 0 ? params->Nl : 1));
  if (!val || !order) {
    free(val);
    free(order);
    return NULL;
  }
  for (int i = 0; i < params->Nl; i++) order[i] = i; /* Tint.c:76-96, no shuffle */
  for (int inx = 0; inx < n; inx++) {
    double *hi = wlh_transform(h * ((double)inx + 1.0), p, order);
    double *mid = wlh_transform(h * ((double)inx + 0.5), p, order);
    double *lo = NULL;
    if (c.mode == WL_MODE_EXACT && inx > 0) lo = wlh_transform(h * (double)inx, p, order);
    if (!hi || !mid) {
      free(hi);
      free(mid);
      free(lo);
      break;
    }
    for (int g = 0; g < ng; g++) {
      /* ref-compat: both outer points at h*(inx+1) (Tint.c:127-154) */
      double flo = c.mode == WL_MODE_EXACT ? (lo ? lo[g] : 0.0) : hi[g];
      val[g] += h / 6.0 * (flo + 4.0 * mid[g] + hi[g]);
    }
    free(hi);
    free(mid);
    free(lo);
  }
  free(order);
  /* Tintout (Tint.c:51-73): the stdout tag the analysis scripts parse */
  double avg = 0.0, sem = 0.0;
  for (int g = 0; g < ng; g++) avg += val[g];
  avg /= ng;
  for (int g = 0; g < ng; g++) sem += (val[g] - avg) * (val[g] - avg);
  sem = ng > 1 ? sqrt(sem / ((double)ng * ((double)ng - 1.0))) : 0.0;
  if (params->fermion == 1)
    printf("Leffvsrho: %e %e %e\n", (double)params->xcm.x, avg / (4.0 * wlh_pi), sem / (4.0 * wlh_pi));
  else
    printf("Leffvsrho: %e %e %e\n", (double)params->xcm.x, avg / (-2.0 * wlh_pi), sem / (2.0 * wlh_pi));
  return val;
}

/* getwl.c:6-40: per loop Nppl x values, then Nppl y values (Dim > 1), then
 * Nppl z values (Dim > 2), whitespace separated.  Returns 0, or -1 when the
 * file cannot be opened or ends early (the reference prints and returns 0). */
WLH_API int getwl(float4 *worldlines, char *filename, int Nl, int Nppl, int Dim) {
  FILE *fp = fopen(filename, "rb");
  if (!fp) {
    fprintf(stderr, "getwl: cannot open %s\n", filename);
    return -1;
  }
  int ok = 1;
  for (int i = 0; i < Nl && ok; i++) {
    for (int d = 0; d < Dim && d < 3 && ok; d++) {
      for (int j = 0; j < Nppl; j++) {
        float v;
        if (fscanf(fp, "%f ", &v) != 1) {
          ok = 0;
          break;
        }
        float4 *w = &worldlines[(size_t)i * Nppl + j];
        if (d == 0) w->x = v;
        else if (d == 1) w->y = v;
        else w->z = v;
      }
    }
  }
  fclose(fp);
  return ok ? 0 : -1;
}

/* writer of the same text format (for ensembles generated here) */
WLH_API int wlh_putwl(const float4 *worldlines, const char *filename, int Nl, int Nppl, int Dim) {
  FILE *fp = fopen(filename, "wb");
  if (!fp) return -1;
  for (int i = 0; i < Nl; i++)
    for (int d = 0; d < Dim && d < 3; d++) {
      for (int j = 0; j < Nppl; j++) {
        const float4 *w = &worldlines[(size_t)i * Nppl + j];
        fprintf(fp, "%.9g ", d == 0 ? w->x : (d == 1 ? w->y : w->z));
      }
      fputc('\n', fp);
    }
  return fclose(fp) == 0 ? 0 : -1;
}

/* ---- binary ensemble files --------------------------------------------- */
/* Layout (little-endian): bytes 0-7 the magic "WLENSv1" + NUL, 8-11 Nl,
 * 12-15 ppl, 16-23 the generator seed (0 if none), 24-27 the values per point
 * (4: the float4 x, y, z, w), 28-31 zero; then Nl * ppl points of four IEEE-754
 * binary32 values, loop-major, as the device holds them. */
static const char wlh_magic[8] = {'W', 'L', 'E', 'N', 'S', 'v', '1', 0};

static void wlh_put32(unsigned char *b, uint32_t v) {
  for (int i = 0; i < 4; i++) b[i] = (unsigned char)(v >> (8 * i));
}
static uint32_t wlh_get32(const unsigned char *b) {
  uint32_t v = 0;
  for (int i = 0; i < 4; i++) v |= (uint32_t)b[i] << (8 * i);
  return v;
}
static int wlh_little_endian(void) {
  const uint32_t one = 1;
  unsigned char c;
  memcpy(&c, &one, 1);
  return c == 1;
}
static void wlh_swap_floats(float *v, size_t n) {
  for (size_t i = 0; i < n; i++) {
    uint32_t u;
    memcpy(&u, &v[i], 4);
    u = (u >> 24) | ((u >> 8) & 0xff00u) | ((u << 8) & 0xff0000u) | (u << 24);
    memcpy(&v[i], &u, 4);
  }
}

WLH_API int wlh_write_ensemble(const char *path, const float4 *loops, int Nl, int ppl,
                               uint64_t seed) {
  if (!path || !loops || Nl < 1 || ppl < 1) return -1;
  FILE *fp = fopen(path, "wb");
  if (!fp) return -1;
  unsigned char hdr[32] = {0};
  memcpy(hdr, wlh_magic, 8);
  wlh_put32(hdr + 8, (uint32_t)Nl);
  wlh_put32(hdr + 12, (uint32_t)ppl);
  wlh_put32(hdr + 16, (uint32_t)seed);
  wlh_put32(hdr + 20, (uint32_t)(seed >> 32));
  wlh_put32(hdr + 24, 4u);
  int ok = fwrite(hdr, 1, 32, fp) == 32;
  const size_t n = (size_t)Nl * ppl * 4;
  if (ok && wlh_little_endian()) {
    ok = fwrite(loops, sizeof(float), n, fp) == n;
  } else if (ok) {
    float buf[1024];
    const float *src = (const float *)loops;
    for (size_t i = 0; i < n && ok; i += 1024) {
      const size_t m = n - i < 1024 ? n - i : 1024;
      memcpy(buf, src + i, m * sizeof(float));
      wlh_swap_floats(buf, m);
      ok = fwrite(buf, sizeof(float), m, fp) == m;
    }
  }
  if (fclose(fp) != 0) ok = 0;
  return ok ? 0 : -1;
}

/* header of an ensemble file: 0, or -1 (unreadable, not an ensemble file) */
WLH_API int wlh_ensemble_file_info(const char *path, int *Nl, int *ppl, uint64_t *seed) {
  if (!path) return -1;
  FILE *fp = fopen(path, "rb");
  if (!fp) return -1;
  unsigned char hdr[32];
  const int ok = fread(hdr, 1, 32, fp) == 32 && memcmp(hdr, wlh_magic, 8) == 0 &&
                 wlh_get32(hdr + 24) == 4u;
  fclose(fp);
  if (!ok) return -1;
  const uint32_t nl = wlh_get32(hdr + 8), pp = wlh_get32(hdr + 12);
  if (nl < 1 || pp < 1 || nl > 0x7fffffffu || pp > 0x7fffffffu) return -1;
  if (Nl) *Nl = (int)nl;
  if (ppl) *ppl = (int)pp;
  if (seed) *seed = (uint64_t)wlh_get32(hdr + 16) | ((uint64_t)wlh_get32(hdr + 20) << 32);
  return 0;
}

/* reads the points into loops[Nl * ppl] (sizes from wlh_ensemble_file_info):
 * 0, or -1 if the file is unreadable, of another shape or short */
WLH_API int wlh_read_ensemble(const char *path, float4 *loops, int Nl, int ppl) {
  int fn = 0, fp_ = 0;
  if (!loops || wlh_ensemble_file_info(path, &fn, &fp_, NULL) || fn != Nl || fp_ != ppl)
    return -1;
  FILE *fp = fopen(path, "rb");
  if (!fp) return -1;
  const size_t n = (size_t)Nl * ppl * 4;
  int ok = fseek(fp, 32, SEEK_SET) == 0 && fread(loops, sizeof(float), n, fp) == n;
  fclose(fp);
  if (ok && !wlh_little_endian()) wlh_swap_floats((float *)loops, n);
  return ok ? 0 : -1;
}

