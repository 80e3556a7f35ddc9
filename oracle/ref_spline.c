/* Runs the reference's own spline-table builder, getspline (periodic.c:113-164,
 * the table EffAct.c:423 builds with Nspline knots), compiled from the
 * reference's source with the GSL stand-in of refshim/ (test infrastructure:
 * golden-vector generation only; built into oracle/_ref by build_ref.sh).
 *
 *   ref_spline LAMBDA2 A N  >  table.bin
 *
 * writes the N knots rho^2 (float32) and then the N float4 coefficients
 * (f, b, c, d of the clamped spline; the last knot's b and d are never set by
 * periodic.c and are written as 0 here). */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <builtin_types.h>

float4 *getspline(float *rho2, double lambda2, double a, int Npoints);

/* testspline (periodic.c:200-247) calls the kernel's interp (intEV.cu:65);
 * the driver never calls testspline */
int interp() { return 0; }

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: ref_spline LAMBDA2 A N\n");
    return 2;
  }
  const double lambda2 = atof(argv[1]), a = atof(argv[2]);
  const int n = atoi(argv[3]);
  if (n < 4) return 2;
  float *rho2 = (float *)calloc((size_t)n, sizeof(float));
  float4 *c = getspline(rho2, lambda2, a, n);
  c[n - 1].y = 0.0f;  /* unset by periodic.c (malloc'd) */
  c[n - 1].w = 0.0f;
  fwrite(rho2, sizeof(float), (size_t)n, stdout);
  fwrite(c, sizeof(float4), (size_t)n, stdout);
  free(rho2);
  free(c);
  return 0;
}
