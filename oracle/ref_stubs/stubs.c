/* Link stubs for the external libraries the reference links against
 * (libiter, LAPACK/BLAS Fortran symbols, ARPACK). None of them is reached by
 * the code paths the oracle calls; each one aborts loudly if it ever is. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "libiter.h"

struct iter *
iter_init (const char *solver, int max, int restart, double eps,
           int n, const double *guess, int flag_guess, int debug, FILE *out)
{
  (void) n; (void) guess; (void) flag_guess;
  struct iter *it = (struct iter *) calloc (1, sizeof (struct iter));
  if (it == NULL) { fprintf (stderr, "iter_init: out of memory\n"); exit (1); }
  it->solver = strdup (solver != NULL ? solver : "gmres");
  it->max = max;
  it->restart = restart;
  it->eps = eps;
  it->debug = debug;
  it->out = out;
  return it;
}

void
iter_free (struct iter *it)
{
  if (it == NULL) return;
  free (it->solver);
  free (it);
}

#define ORACLE_ABORT_STUB(name) \
  void name (void) { fprintf (stderr, "oracle stub: %s called\n", #name); abort (); }

void
solve_iter (int n, const double *b, double *x,
            void (*atimes) (int, const double *, double *, void *),
            void *user_data, struct iter *it)
{
  (void) n; (void) b; (void) x; (void) atimes; (void) user_data; (void) it;
  fprintf (stderr, "oracle stub: solve_iter called\n");
  abort ();
}

ORACLE_ABORT_STUB (dcopy_)
ORACLE_ABORT_STUB (dgetrf_)
ORACLE_ABORT_STUB (dgetri_)
ORACLE_ABORT_STUB (dgetrs_)

/* ARPACK, the LAPACK/BLAS routines of the matrix-noise branch and the
 * bead-rod constraints: linked by the reference's Brownian-dynamics sources,
 * never reached when the Chebyshev bounds are preset and no constraints are
 * given. */
ORACLE_ABORT_STUB (dnaupd_)
ORACLE_ABORT_STUB (dneupd_)
ORACLE_ABORT_STUB (dsaupd_)
ORACLE_ABORT_STUB (dseupd_)
ORACLE_ABORT_STUB (dgeev_)
ORACLE_ABORT_STUB (dpotrf_)
ORACLE_ABORT_STUB (dpotf2_)
ORACLE_ABORT_STUB (dgemv_)
ORACLE_ABORT_STUB (dgemm_)
ORACLE_ABORT_STUB (BeadRod_set_coefs)
ORACLE_ABORT_STUB (BeadRod_adjust_by_constraints)
ORACLE_ABORT_STUB (BeadRod_bead_to_connector)
