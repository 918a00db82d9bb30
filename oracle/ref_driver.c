/* ref_driver.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A flat C entry layer over the reference library itself (compiled from the
 * reference sources by oracle/Makefile.ref into oracle/_ref/).  It exposes the
 * same calls as oracle/oracle_ewald.c (ref_* instead of oracle_*), so the
 * fixture generator can run the reference and the restatement on identical
 * inputs.  It only calls the reference's public functions
 * (stokes_init, stokes_set_np/l/xi, stokes_set_radius/slip,
 * atimes_ewald_3all, make_matrix_mob_ewald_3all, chebyshev_*) and sets struct
 * members the way the reference's own tests do (test/check-ewald.c:73-125).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "stokes.h"
#include "ewald.h"
#include "non-ewald.h"
#include "matrix.h"
#include "chebyshev.h"
#include "libiter.h"

void *
ref_new (int version, int np, const double *pos, double lx, double ly,
         double lz)
{
  struct stokes *sys = stokes_init ();
  sys->version = version;
  stokes_set_np (sys, np, np);
  memcpy (sys->pos, pos, sizeof (double) * 3 * np);
  sys->periodic = 1;
  stokes_set_l (sys, lx, ly, lz);
  /* struct iter is only read by stokes_copy; give it one like the tests do */
  stokes_set_iter (sys, "gmres", 2000, 20, 1.0e-6, 0, stderr);
  return sys;
}

void ref_free (void *h) { stokes_free ((struct stokes *) h); }

void
ref_set_pos (void *h, const double *pos)
{
  struct stokes *sys = h;
  memcpy (sys->pos, pos, sizeof (double) * 3 * sys->np);
}

void ref_set_split (void *h, double xi, double eps) { stokes_set_xi (h, xi, eps); }

double
ref_xi_by_tratio (void *h, double tratio)
{
  return xi_by_tratio ((struct stokes *) h, tratio);
}

/* same override as oracle_set_cube: full image cube and full k cube */
void
ref_set_cube (void *h, int nr_shell, int nk_shell)
{
  struct stokes *sys = h;
  int side = 2 * nr_shell + 1, cap = side * side * side;
  sys->nr = 0;
  sys->rlx = realloc (sys->rlx, sizeof (double) * cap);
  sys->rly = realloc (sys->rly, sizeof (double) * cap);
  sys->rlz = realloc (sys->rlz, sizeof (double) * cap);
  sys->rmx = realloc (sys->rmx, sizeof (int) * cap);
  sys->rmy = realloc (sys->rmy, sizeof (int) * cap);
  sys->rmz = realloc (sys->rmz, sizeof (int) * cap);
  for (int m1 = -nr_shell; m1 <= nr_shell; m1++)
    for (int m2 = -nr_shell; m2 <= nr_shell; m2++)
      for (int m3 = -nr_shell; m3 <= nr_shell; m3++)
        {
          int q = sys->nr++;
          sys->rlx[q] = sys->lx * m1; sys->rly[q] = sys->ly * m2;
          sys->rlz[q] = sys->lz * m3;
          sys->rmx[q] = m1; sys->rmy[q] = m2; sys->rmz[q] = m3;
        }
  sys->rmax2 = INFINITY;
  sys->kmaxx = sys->kmaxy = sys->kmaxz = nk_shell;
  sys->kmax = 0.0;
}

void ref_set_radius (void *h, const double *a)
{
  if (a == NULL) stokes_unset_radius (h);
  else stokes_set_radius (h, a);
}

void ref_set_slip (void *h, const double *g)
{
  if (g == NULL) stokes_unset_slip (h);
  else stokes_set_slip (h, g);
}

void
ref_set_misc (void *h, double rmin, int shear_mode, double shear_shift)
{
  struct stokes *sys = h;
  sys->rmin = rmin;
  sys->shear_mode = shear_mode;
  sys->shear_shift = shear_shift;
}

void
ref_get_split (void *h, double *out)
{
  struct stokes *s = h;
  out[0] = s->xi; out[1] = s->rmax2; out[2] = s->kmax;
  out[3] = s->self_a; out[4] = s->self_c; out[5] = s->self_m;
  out[6] = s->pivol; out[7] = s->nr;
  out[8] = s->kmaxx * 10000 + s->kmaxy * 100 + s->kmaxz;
}

void
ref_get_table (void *h, double *rl, int *rm)
{
  struct stokes *s = h;
  for (int q = 0; q < s->nr; q++)
    {
      rl[3 * q] = s->rlx[q]; rl[3 * q + 1] = s->rly[q]; rl[3 * q + 2] = s->rlz[q];
      rm[3 * q] = s->rmx[q]; rm[3 * q + 1] = s->rmy[q]; rm[3 * q + 2] = s->rmz[q];
    }
}

void
ref_atimes (void *h, const double *x, double *y)
{
  struct stokes *s = h;
  int c = s->version == 0 ? 3 : (s->version == 1 ? 6 : 11);
  atimes_ewald_3all (c * s->np, x, y, s);
}

void ref_atimes_notbl (void *h, const double *x, double *y)
{
  struct stokes *s = h;
  int c = s->version == 0 ? 3 : (s->version == 1 ? 6 : 11);
  atimes_ewald_3all_notbl (c * s->np, x, y, s);
}

void ref_matrix (void *h, double *mat) { make_matrix_mob_ewald_3all (h, mat); }

void ref_matrix_notbl (void *h, double *mat)
{
  make_matrix_mob_ewald_3all_notbl (h, mat);
}

/* the free-space operator (src/non-ewald.c); periodic is cleared as the
 * reference's own dispatcher atimes_3all would require */
void
ref_atimes_nonewald (void *h, const double *x, double *y)
{
  struct stokes *s = h;
  int c = s->version == 0 ? 3 : (s->version == 1 ? 6 : 11);
  atimes_nonewald_3all (c * s->np, x, y, s);
}

void ref_matrix_nonewald (void *h, double *mat) { make_matrix_mob_nonewald_3all (h, mat); }

/* sys->periodic: 0 makes the dispatchers (atimes_3all, make_matrix_mob_3all)
 * and the BD routines take the free-space branch */
void ref_set_periodic (void *h, int p) { ((struct stokes *) h)->periodic = p; }

void
ref_matvec (int version, int np, const double *mat, const double *x, double *y)
{
  int c = version == 0 ? 3 : (version == 1 ? 6 : 11);
  if (version == 2) multiply_extmat_with_extvec_3fts (np, mat, x, y);
  else dot_prod_matrix (mat, c * np, c * np, x, y);
}

void ref_cpu_times (void *h, double *out)
{
  struct stokes *s = h;
  out[0] = s->cpu1; out[1] = s->cpu2; out[2] = s->cpu3;
}

/* Chebyshev helpers on a dense symmetric matrix operator */
typedef struct { int n; const double *m; } densop;

static void
dense_atimes (int n, const double *x, double *y, void *u)
{
  densop *d = u;
  for (int i = 0; i < n; i++)
    {
      double acc = 0.0;
      for (int j = 0; j < n; j++) acc += d->m[i * n + j] * x[j];
      y[i] = acc;
    }
}

static double f_invsqrt (double x) { return 1.0 / sqrt (x); }
static double f_sqrt (double x) { return sqrt (x); }

void
ref_cheb_coef (int ncheb, int which, double x0, double x1, double *a)
{
  chebyshev_coef (ncheb, which == 0 ? f_invsqrt : f_sqrt, x0, x1, a);
}

double
ref_cheb_eval (int ncheb, const double *a, double x0, double x1, double x)
{
  return chebyshev_eval (ncheb, a, x0, x1, x);
}

void
ref_cheb_eval_dense (int ncheb, const double *a, int n, const double *m,
                     const double *y, double *z, double e0, double e1,
                     double *err)
{
  densop d = {n, m};
  chebyshev_eval_atimes (ncheb, a, n, y, z, e0, e1, dense_atimes, &d);
  *err = chebyshev_error_minvsqrt (n, y, z, dense_atimes, &d);
}

/* Chebyshev on the reference's own Ewald operator */
void
ref_cheb_eval_ewald (void *h, int ncheb, const double *a, const double *y,
                     double *z, double e0, double e1, double *err)
{
  struct stokes *s = h;
  int c = s->version == 0 ? 3 : (s->version == 1 ? 6 : 11);
  int n = c * s->np;
  chebyshev_eval_atimes (ncheb, a, n, y, z, e0, e1, atimes_ewald_3all, s);
  *err = chebyshev_error_minvsqrt (n, y, z, atimes_ewald_3all, s);
}
