/* Minimal stand-in for the GSL matrix names periodic.c's Jacobian uses
 * (periodic.c:33-39: a 1 x 1 view on the caller's array and one set).  Test
 * infrastructure for oracle/_ref only; GSL is not installed. */
#ifndef WLREF_GSL_MATRIX_H
#define WLREF_GSL_MATRIX_H
#include <stddef.h>
typedef struct {
  size_t size1, size2, tda;
  double *data;
} gsl_matrix;
typedef struct {
  gsl_matrix matrix;
} gsl_matrix_view;
static inline gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2) {
  gsl_matrix_view v;
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = n2;
  v.matrix.data = base;
  return v;
}
static inline void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x) {
  m->data[i * m->tda + j] = x;
}
#endif
