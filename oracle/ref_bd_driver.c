/* ref_bd_driver.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A flat entry over the reference's own Brownian-dynamics routines
 * (BD_params_init, BD_calc_FB, BD_evolve_mid of src/brownian.c, the EV_LJ
 * repulsion of src/ev-LJ.c), compiled from the reference sources by
 * oracle/Makefile.ref into oracle/_ref/libstokes_ref_bd.so, for the fixture
 * generator.  ARPACK is not available: the eigenvalue bounds are preset
 * (eig_minv[0] != eig_minv[1]), a_minv is fitted by the reference's own
 * chebyshev_coef, and BD->eps is chosen by the caller so that the
 * re-estimate branch (src/brownian.c:1710-1727) is not taken.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "stokes.h"
#include "brownian.h"
#include "chebyshev.h"
#include "ev-LJ.h"
#include "KIrand.h"

static double inv_sqrt (double x) { return 1.0 / sqrt (x); }

static struct BD_params *
make_bd (struct stokes *sys, unsigned long seed, double peclet, int n_minv, double eig0,
         double eig1, double bd_eps, const double *lj_e, const double *lj_r0, int lj_flag,
         double bd_rmin, double dt_lim, double t0, double s0, const double *F,
         const double *T, struct EV_LJ **lj_out)
{
  const int nm = sys->nm;
  double *Fb = calloc ((size_t) nm * 3, sizeof (double));
  double *Tb = calloc ((size_t) nm * 3, sizeof (double));
  double *Eb = calloc ((size_t) nm * 5, sizeof (double));
  if (F) memcpy (Fb, F, sizeof (double) * nm * 3);
  if (T) memcpy (Tb, T, sizeof (double) * nm * 3);
  struct EV_LJ *lj = NULL;
  if (lj_e)
    {
      lj = EV_LJ_init (sys->np);
      for (int i = 0; i < sys->np; i++)
        {
          lj->flag[i] = lj_flag;
          lj->e[i] = lj_e[i];
          lj->r0[i] = lj_r0[i];
        }
    }
  struct BD_params *BD = BD_params_init (sys, seed, Fb, Tb, Eb, NULL, NULL, NULL,
                                         0 /* noHI */, 0 /* lub */, 0 /* mat */, 0.0 /* st */,
                                         NULL, NULL, 1.0, NULL, NULL, NULL, lj, NULL,
                                         0 /* flag_Q */, peclet, bd_eps, n_minv, 0,
                                         0 /* mid-point */, 0.0, bd_rmin, dt_lim);
  BD->t0 = t0;
  BD->s0 = s0;
  BD->eig_minv[0] = eig0;
  BD->eig_minv[1] = eig1;
  chebyshev_coef (n_minv, inv_sqrt, eig0, eig1, BD->a_minv);
  *lj_out = lj;
  return BD;
}

static void
free_bd (struct BD_params *BD, struct EV_LJ *lj)
{
  free (BD->F);
  free (BD->T);
  free (BD->E);
  BD_params_free (BD);
  if (lj) EV_LJ_free (lj);
}

/* simple shear of the given mode and rate (imposed flow set as the
 * reference's stokes_set_shear does) */
void refbd_set_shear (void *h, int mode, double rate) { stokes_set_shear (h, mode, rate); }

/* z = BD_calc_FB at the system's current positions (n = BD_get_n values) */
int
refbd_calc_fb (void *h, unsigned long seed, double peclet, int n_minv, double eig0,
               double eig1, double bd_eps, double *z)
{
  struct EV_LJ *lj;
  struct BD_params *BD = make_bd (h, seed, peclet, n_minv, eig0, eig1, bd_eps, NULL, NULL, 0,
                                  0.0, 1e-12, 0.0, 0.0, NULL, NULL, &lj);
  BD_calc_FB (BD, z);
  free_bd (BD, lj);
  return BD_get_n (h);
}

/* z = BD_calc_FB with the lubrication noise (flag_lub_B = 1, the Chebyshev
 * form n_lub > 0, src/brownian.c:1734-1849) at the given lubmin2 / lubmax.
 * The bounds of L are preset (eig_lub[0] != eig_lub[1]: ARPACK is absent)
 * and a_lub is fitted by the reference's chebyshev_coef of sqrt; bd_eps
 * keeps both re-estimate branches off. */
static double sqrt_fn (double x) { return sqrt (x); }
int
refbd_calc_fb_lub (void *h, unsigned long seed, double peclet, int n_minv, double eig0,
                   double eig1, int n_lub, double eigl0, double eigl1, double bd_eps,
                   double lubmin2, double lubmax, double *z)
{
  struct stokes *sys = h;
  sys->lubmin2 = lubmin2;
  sys->lubmax = lubmax;
  const int nm = sys->nm;
  double *Fb = calloc ((size_t) nm * 3, sizeof (double));
  double *Tb = calloc ((size_t) nm * 3, sizeof (double));
  double *Eb = calloc ((size_t) nm * 5, sizeof (double));
  struct BD_params *BD = BD_params_init (sys, seed, Fb, Tb, Eb, NULL, NULL, NULL,
                                         0 /* noHI */, 1 /* lub */, 0 /* mat */, 0.0 /* st */,
                                         NULL, NULL, 1.0, NULL, NULL, NULL, NULL, NULL,
                                         0 /* flag_Q */, peclet, bd_eps, n_minv, n_lub,
                                         0 /* mid-point */, 0.0, 0.0, 1e-12);
  BD->flag_lub_B = 1;
  BD->eig_minv[0] = eig0;
  BD->eig_minv[1] = eig1;
  chebyshev_coef (n_minv, inv_sqrt, eig0, eig1, BD->a_minv);
  BD->eig_lub[0] = eigl0;
  BD->eig_lub[1] = eigl1;
  chebyshev_coef (n_lub, sqrt_fn, eigl0, eigl1, BD->a_lub);
  BD_calc_FB (BD, z);
  free_bd (BD, NULL);
  return BD_get_n (h);
}

/* nsteps BD_evolve_mid steps from time t0; x (nm*3) and q (nm*4 or NULL)
 * are advanced in place, x_traj[s] holds x after step s, dts[s] the dt done */
int
refbd_run (void *h, unsigned long seed, double peclet, double dt, int nsteps, int n_minv,
           double eig0, double eig1, double bd_eps, const double *lj_e, const double *lj_r0,
           int lj_flag, double bd_rmin, double dt_lim, double t0, double s0, const double *F,
           const double *T, double *x, double *q, double *x_traj, double *dts)
{
  struct stokes *sys = h;
  struct EV_LJ *lj;
  struct BD_params *BD = make_bd (sys, seed, peclet, n_minv, eig0, eig1, bd_eps, lj_e, lj_r0,
                                  lj_flag, bd_rmin, dt_lim, t0, s0, F, T, &lj);
  double t = t0;
  for (int s = 0; s < nsteps; s++)
    {
      dts[s] = BD_evolve_mid (t, BD, x, q, dt);
      t += dts[s];
      memcpy (x_traj + (size_t) s * 3 * sys->nm, x, sizeof (double) * 3 * sys->nm);
    }
  free_bd (BD, lj);
  return 0;
}

/* f = L u, the reference's lubrication correction (src/lub.c:164-575) at
 * the given lubmin2 / lubmax; version 0 (F) or 1 (FT) from the system */
#include "lub.h"
void
refbd_calc_lub (void *h, double lubmin2, double lubmax, const double *u, double *f)
{
  struct stokes *sys = h;
  sys->lubmin2 = lubmin2;
  sys->lubmax = lubmax;
  if (sys->version == 0) calc_lub_3f (sys, u, f);
  else if (sys->version == 1) calc_lub_3ft (sys, u, f);
  else calc_lub_3fts (sys, u, f);
}

/* the reference's dense lubrication matrix (src/lub-matrix.c:76-507) at
 * the given lubmin2 / lubmax, n = np * {3, 6, 11} rows, row-major */
#include "lub-matrix.h"
void
refbd_matrix_lub (void *h, double lubmin2, double lubmax, double *mat)
{
  struct stokes *sys = h;
  sys->lubmin2 = lubmin2;
  sys->lubmax = lubmax;
  if (sys->version == 0) make_matrix_lub_3f (sys, mat);
  else if (sys->version == 1) make_matrix_lub_3ft (sys, mat);
  else make_matrix_lub_3fts (sys, mat);
}

/* the reference's two-body lubrication-form functions and (M^inf)^-1 */
#include "two-body-res.h"
void ref_res2b (double s, double *res) { scalar_two_body_res (s, res); }
void scalar_minv_f (double s, double *r);
void scalar_minv_ft (double s, double *r);
void scalar_minv_fts (double s, double *r);
void ref_minv (int version, double s, double *r)
{
  if (version == 0) scalar_minv_f (s, r);
  else if (version == 1) scalar_minv_ft (s, r);
  else scalar_minv_fts (s, r);
}
