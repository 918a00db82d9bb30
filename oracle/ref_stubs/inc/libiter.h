/* Minimal stand-in for the external iterative-solver library ("libiter",
 * not shipped with the reference). Only what the reference's stokes.c needs
 * to compile is declared; the solver itself is never reached by the
 * mobility product, the dense builder or the Chebyshev routines. */
#ifndef ORACLE_STUB_LIBITER_H
#define ORACLE_STUB_LIBITER_H
#include <stdio.h>
struct iter {
  char *solver;
  int max;
  int restart;
  double eps;
  int debug;
  FILE *out;
};
struct iter *iter_init (const char *solver, int max, int restart, double eps,
                        int n, const double *guess, int flag_guess,
                        int debug, FILE *out);
void iter_free (struct iter *it);
void solve_iter (int n, const double *b, double *x,
                 void (*atimes) (int, const double *, double *, void *),
                 void *user_data, struct iter *it);
#endif
