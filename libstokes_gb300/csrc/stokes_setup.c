/* stokes_setup.c -- system set-up of libstokes_gb300 (host C, FP64).
 *
 * Replaces the part of libstokes' src/stokes.c that the Ewald mobility path
 * consumes: struct allocation, particle arrays, box, imposed flow, shear,
 * and the Ewald split with its cutoff search and image table.  The numbers
 * produced are the reference's: same self constants (src/stokes.c:714-716),
 * same cutoff search with safety factor 1.15 and shrink factor 0.99
 * (src/stokes.c:655-700, 726-758), same image-table rule
 * (src/stokes.c:193-233) -- tests/test_abi.py checks them against the
 * reference bit for bit.
 *
 * Not rebuilt here: the lubrication tables (poly_table, twobody_f_list,
 * slip_table); the mobility kernels do not read them.  The iterative-solver
 * settings (stokes_set_iter) go to this library's iter_init (krylov.cu).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "stokes_gpu.h"
#include "stokes_iter.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void *
must_alloc (size_t bytes, const char *who)
{
  void *p = malloc (bytes > 0 ? bytes : 1);
  if (p == NULL)
    {
      fprintf (stderr, "libstokes_gb300 %s: out of memory\n", who);
      exit (1);
    }
  return p;
}

static void
free_tables (struct stokes *sys)
{
  double **dd[] = {&sys->rlx, &sys->rly, &sys->rlz, &sys->ex, &sys->ey, &sys->ez,
                   &sys->k, &sys->k1, &sys->k2, &sys->k3, &sys->ya, &sys->yb,
                   &sys->yc, &sys->yg, &sys->yh, &sys->ym};
  for (size_t q = 0; q < sizeof dd / sizeof dd[0]; q++)
    {
      free (*dd[q]);
      *dd[q] = NULL;
    }
  free (sys->rmx); free (sys->rmy); free (sys->rmz);
  sys->rmx = sys->rmy = sys->rmz = NULL;
  sys->nr = 0;
  sys->nk = 0;
  sys->flag_table = 0;
}

struct stokes *
stokes_init (void)
{
  struct stokes *sys = (struct stokes *) calloc (1, sizeof (struct stokes));
  if (sys == NULL)
    {
      fprintf (stderr, "libstokes_gb300 stokes_init: out of memory\n");
      exit (1);
    }
  /* every member starts at zero / NULL, as in src/stokes.c:317-418, except: */
  sys->twobody_nmax = 100;
  sys->twobody_lub = 1;
  return sys;
}

void
stokes_free (struct stokes *sys)
{
  if (sys == NULL) return;
  stokes_gpu_release (sys);
  free (sys->pos);
  stokes_unset_radius (sys);
  stokes_unset_slip (sys);
  free_tables (sys);
  /* the iterative-solver settings (src/stokes.c:440) */
  if (sys->it != NULL) iter_free (sys->it);
  free (sys);
}

/* iterative-solver settings (src/stokes.c:790-812): the guess is kept
 * between solves (flag_guess 1, zero at first) */
void
stokes_set_iter (struct stokes *sys, const char *solver, int max, int restart, double eps,
                 int debug, FILE *out)
{
  int n;
  if (sys->version == 0) n = sys->np * 3;
  else if (sys->version == 1) n = sys->np * 6;
  else if (sys->version == 2) n = sys->np * 11;
  else
    {
      fprintf (stderr, "libstokes stokes_set_iter : invalid version %d\n", sys->version);
      exit (1);
    }
  if (sys->it != NULL) iter_free (sys->it);
  sys->it = iter_init (solver, max, restart, eps, n, NULL, 1, debug, out);
}

void
stokes_set_np (struct stokes *sys, int np, int nm)
{
  sys->np = np;
  sys->nm = nm;
  free (sys->pos);
  sys->pos = (double *) must_alloc (sizeof (double) * 3 * (size_t) (np > 0 ? np : 0),
                                    "stokes_set_np");
}

void
stokes_set_Ui (struct stokes *sys, double uix, double uiy, double uiz)
{
  sys->Ui[0] = uix; sys->Ui[1] = uiy; sys->Ui[2] = uiz;
}

void
stokes_set_Oi (struct stokes *sys, double oix, double oiy, double oiz)
{
  sys->Oi[0] = oix; sys->Oi[1] = oiy; sys->Oi[2] = oiz;
}

void
stokes_set_Ei (struct stokes *sys, double eixx, double eixy, double eixz,
               double eiyz, double eiyy)
{
  sys->Ei[0] = eixx; sys->Ei[1] = eixy; sys->Ei[2] = eixz;
  sys->Ei[3] = eiyz; sys->Ei[4] = eiyy;
}

/* simple shear: overwrite the imposed flow (src/stokes.c:506-543) */
void
stokes_set_shear (struct stokes *sys, int shear_mode, double shear_rate)
{
  sys->shear_mode = shear_mode;
  sys->shear_rate = shear_rate;
  memset (sys->Ui, 0, sizeof sys->Ui);
  memset (sys->Oi, 0, sizeof sys->Oi);
  memset (sys->Ei, 0, sizeof sys->Ei);
  if (shear_mode == 1)
    {
      sys->Oi[2] = -0.5 * shear_rate;
      sys->Ei[1] = +0.5 * shear_rate;
    }
  else if (shear_mode == 2)
    {
      sys->Oi[1] = +0.5 * shear_rate;
      sys->Ei[2] = +0.5 * shear_rate;
    }
  else if (shear_mode != 0)
    fprintf (stderr, "stokes_set_shear(): invalid shear_mode %d\n", shear_mode);
}

/* Lees-Edwards shift at time t, folded into [-lx/2, lx/2)
 * (src/stokes.c:554-589) */
double
stokes_get_shear_shift (struct stokes *sys, double t, double t0, double s0)
{
  if (sys->periodic == 0 || sys->shear_mode == 0) return 0.0;
  double h;
  if (sys->shear_mode == 1) h = sys->ly;
  else if (sys->shear_mode == 2) h = sys->lz;
  else
    {
      fprintf (stderr, "stokes_set_shear(): invalid shear_mode %d\n", sys->shear_mode);
      return 0.0;
    }
  double shift = s0 + h * sys->shear_rate * (t - t0);
  while (shift < -0.5 * sys->lx) shift += sys->lx;
  while (shift >= 0.5 * sys->lx) shift -= sys->lx;
  return shift;
}

void
stokes_set_shear_shift (struct stokes *sys, double t, double t0, double s0)
{
  sys->shear_shift = stokes_get_shear_shift (sys, t, t0, s0);
}

/* box, pi/V and the 27-cell neighbour table (src/stokes.c:607-651).  The
 * table order is the reference's: primary cell, the 8 in-plane (xy)
 * neighbours, then the z = -1 and z = +1 layers. */
void
stokes_set_l (struct stokes *sys, double lx, double ly, double lz)
{
  static const int cx[9] = {0, -1, 0, +1, 0, -1, -1, +1, +1};
  static const int cy[9] = {0, 0, -1, 0, +1, -1, +1, -1, +1};
  sys->pivol = M_PI / lx / ly / lz;
  sys->lx = lx;
  sys->ly = ly;
  sys->lz = lz;
  for (int layer = 0; layer < 3; layer++)
    {
      static const int cz[3] = {0, -1, +1};
      for (int q = 0; q < 9; q++)
        {
          int i = layer * 9 + q;
          sys->ilx[i] = cx[q];
          sys->ily[i] = cy[q];
          sys->ilz[i] = cz[layer];
        }
    }
}

/* cutoff estimators of the reference (src/stokes.c:655-700): the error of
 * the last real-space / reciprocal shell with a 1.15 safety factor */
static double
est_real (double r, double xi)
{
  const double u = xi * r / 1.15;
  const double u2 = u * u;
  const double r2 = r * r;
  return erfc (u) * (0.75 + 1.5 / r2) / r
    + exp (-u2) * xi / sqrt (M_PI)
      * (4.5 + 3.0 * u2 + (3.0 + u2 * (14.0 + u2 * (4.0 + u2))) / r2);
}

static double
est_recip (double k, double xi)
{
  const double u = k / xi / 1.15;
  const double u2 = u * u;
  const double k2 = k * k;
  return 6.0 * M_PI * exp (-u2 / 4.0) * (1.0 + k2 / 3.0) / k2
    * (1.0 + u2 * (1.0 / 4.0 + u2 / 8.0));
}

/* Cutoffs of the reference's search for a given split xi and tolerance eps
 * (same estimators and shrink rule as stokes_set_xi).  Internal: the mixed
 * path uses it to size its own, re-tuned split. */
void
lsg_ewald_cutoffs (double xi, double eps, double lmin, double lmax, double *rmax_out,
                   double *kmax_out)
{
  const double shrink = 0.99;
  double rmax = 10.0 * sqrt (-log (eps)) / xi;
  while (est_real (rmax * shrink, xi) + 6.0 * est_real (rmax * shrink + lmin, xi) < eps)
    rmax *= shrink;
  const double dk = 2.0 * M_PI / lmax;
  double kmax = 10.0 * sqrt (-log (eps)) * 2.0 * xi;
  while (est_recip (kmax * shrink, xi) + 6.0 * est_recip (kmax * shrink + dk, xi) < eps)
    kmax *= shrink;
  *rmax_out = rmax;
  *kmax_out = kmax;
}

/* The reciprocal table (ex..ym, src/stokes.c:236-307) is filled as in the
 * reference for callers that read it; the GPU product does not. */
static void
fill_k_table (struct stokes *sys)
{
  int cap = (2 * sys->kmaxx + 1) * (2 * sys->kmaxy + 1) * (2 * sys->kmaxz + 1);
  double **cols[] = {&sys->ex, &sys->ey, &sys->ez, &sys->k, &sys->k1, &sys->k2,
                     &sys->k3, &sys->ya, &sys->yb, &sys->yc, &sys->yg, &sys->yh,
                     &sys->ym};
  for (size_t q = 0; q < sizeof cols / sizeof cols[0]; q++)
    *cols[q] = (double *) must_alloc (sizeof (double) * (size_t) cap, "stokes_set_xi");
  int nk = 0;
  for (int m1 = -sys->kmaxx; m1 <= sys->kmaxx; m1++)
    for (int m2 = -sys->kmaxy; m2 <= sys->kmaxy; m2++)
      for (int m3 = -sys->kmaxz; m3 <= sys->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          double k1 = 2.0 * M_PI * (double) m1 / sys->lx;
          double k2 = 2.0 * M_PI * (double) m2 / sys->ly;
          double k3 = 2.0 * M_PI * (double) m3 / sys->lz;
          double kk = k1 * k1 + k2 * k2 + k3 * k3;
          double k = sqrt (kk);
          if (k > sys->kmax) continue;
          double k4z = kk / 4.0 / sys->xi2;
          double kexp = sys->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          sys->ex[nk] = k1 / k; sys->ey[nk] = k2 / k; sys->ez[nk] = k3 / k;
          sys->k[nk] = k; sys->k1[nk] = k1; sys->k2[nk] = k2; sys->k3[nk] = k3;
          sys->ya[nk] = 6.0 * (1.0 - kk / 3.0) * kexp;
          sys->yb[nk] = sys->version >= 1 ? 3.0 * k * kexp : 0.0;
          sys->yc[nk] = sys->version >= 1 ? 1.5 * kk * kexp : 0.0;
          sys->yg[nk] = sys->version >= 2 ? 3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp : 0.0;
          sys->yh[nk] = sys->version >= 2 ? 1.5 * kk * kexp : 0.0;
          sys->ym[nk] = sys->version >= 2 ? 3.0 * (1.0 - kk / 5.0) * kk * kexp : 0.0;
          nk++;
        }
  sys->nk = nk;
}

void
stokes_set_xi (struct stokes *sys, double xi, double ewald_eps)
{
  sys->ewald_eps = ewald_eps;
  sys->xi = xi;
  sys->xi2 = xi * xi;
  sys->xia2 = sys->xi2;
  sys->xiaspi = xi / sqrt (M_PI);

  sys->self_a = 1.0 - sys->xiaspi * (6.0 - 40.0 / 3.0 * sys->xia2);
  sys->self_c = 0.75 - sys->xiaspi * sys->xia2 * 10.0;
  sys->self_m = 0.9 - sys->xiaspi * sys->xia2 * (12.0 - 30.24 * sys->xia2);

  const double shrink = 0.99;
  double lmin = sys->lx, lmax = sys->lx;
  if (sys->ly < lmin) lmin = sys->ly;
  if (sys->lz < lmin) lmin = sys->lz;
  if (sys->ly > lmax) lmax = sys->ly;
  if (sys->lz > lmax) lmax = sys->lz;

  /* real space: start far out and shrink while the last shell stays < eps */
  double rmax = 10.0 * sqrt (-log (ewald_eps)) / xi;
  while (est_real (rmax * shrink, xi) + 6.0 * est_real (rmax * shrink + lmin, xi)
         < ewald_eps)
    rmax *= shrink;
  sys->rmax2 = rmax * rmax;
  sys->rmaxx = (int) (rmax / sys->lx) + 1;
  sys->rmaxy = (int) (rmax / sys->ly) + 1;
  sys->rmaxz = (int) (rmax / sys->lz) + 1;

  /* reciprocal space, same rule with the shell width 2 pi / lmax */
  const double dk = 2.0 * M_PI / lmax;
  double kmax = 10.0 * sqrt (-log (ewald_eps)) * 2.0 * xi;
  while (est_recip (kmax * shrink, xi) + 6.0 * est_recip (kmax * shrink + dk, xi)
         < ewald_eps)
    kmax *= shrink;
  sys->kmax = kmax;
  sys->kmaxx = (int) (kmax * sys->lx / 2.0 / M_PI);
  sys->kmaxy = (int) (kmax * sys->ly / 2.0 / M_PI);
  sys->kmaxz = (int) (kmax * sys->lz / 2.0 / M_PI);

  /* image table: every cell whose point nearest to the primary cell lies
   * within rmax + |box diagonal| */
  free_tables (sys);
  int cap = (2 * sys->rmaxx + 1) * (2 * sys->rmaxy + 1) * (2 * sys->rmaxz + 1);
  sys->rlx = (double *) must_alloc (sizeof (double) * (size_t) cap, "stokes_set_xi");
  sys->rly = (double *) must_alloc (sizeof (double) * (size_t) cap, "stokes_set_xi");
  sys->rlz = (double *) must_alloc (sizeof (double) * (size_t) cap, "stokes_set_xi");
  sys->rmx = (int *) must_alloc (sizeof (int) * (size_t) cap, "stokes_set_xi");
  sys->rmy = (int *) must_alloc (sizeof (int) * (size_t) cap, "stokes_set_xi");
  sys->rmz = (int *) must_alloc (sizeof (int) * (size_t) cap, "stokes_set_xi");
  const double lim = rmax + sqrt (sys->lx * sys->lx + sys->ly * sys->ly + sys->lz * sys->lz);
  int nr = 0;
  for (int m1 = -sys->rmaxx; m1 <= sys->rmaxx; m1++)
    {
      const double cx = sys->lx * (double) m1;
      const double nx = cx - (m1 > 0 ? 0.5 * sys->lx : 0.0) + (m1 < 0 ? 0.5 * sys->lx : 0.0);
      for (int m2 = -sys->rmaxy; m2 <= sys->rmaxy; m2++)
        {
          const double cy = sys->ly * (double) m2;
          const double ny = cy - (m2 > 0 ? 0.5 * sys->ly : 0.0) + (m2 < 0 ? 0.5 * sys->ly : 0.0);
          for (int m3 = -sys->rmaxz; m3 <= sys->rmaxz; m3++)
            {
              const double cz = sys->lz * (double) m3;
              const double nz = cz - (m3 > 0 ? 0.5 * sys->lz : 0.0) + (m3 < 0 ? 0.5 * sys->lz : 0.0);
              if (sqrt (nx * nx + ny * ny + nz * nz) <= lim)
                {
                  sys->rlx[nr] = cx; sys->rly[nr] = cy; sys->rlz[nr] = cz;
                  sys->rmx[nr] = m1; sys->rmy[nr] = m2; sys->rmz[nr] = m3;
                  nr++;
                }
            }
        }
    }
  sys->nr = nr;
  fill_k_table (sys);
  sys->flag_table = 1;
  stokes_gpu_note_split (sys);
}

double
xi_by_tratio (struct stokes *sys, double tratio)
{
  return pow (tratio, 1.0 / 6.0) * sqrt (M_PI) / pow (sys->lx * sys->ly * sys->lz, 1.0 / 3.0);
}

void
stokes_set_pos (struct stokes *sys, const double *pos)
{
  memcpy (sys->pos, pos, sizeof (double) * 3 * (size_t) sys->np);
}

void
stokes_set_pos_mobile (struct stokes *sys, const double *pos)
{
  memcpy (sys->pos, pos, sizeof (double) * 3 * (size_t) sys->nm);
}

void
stokes_set_pos_fixed (struct stokes *sys, const double *pos)
{
  memcpy (sys->pos + 3 * sys->nm, pos, sizeof (double) * 3 * (size_t) (sys->np - sys->nm));
}

void
stokes_set_radius (struct stokes *sys, const double *a)
{
  stokes_unset_radius (sys);
  sys->a = (double *) must_alloc (sizeof (double) * (size_t) sys->np, "stokes_set_radius");
  memcpy (sys->a, a, sizeof (double) * (size_t) sys->np);
}

void
stokes_unset_radius (struct stokes *sys)
{
  free (sys->a);
  sys->a = NULL;
  /* the lubrication tables are libstokes' to free; this library never
   * builds them, so a struct made here has them NULL */
  sys->poly_table = NULL;
  sys->twobody_f_list = NULL;
}

/* slip factors Lambda(3,2), Lambda(3,0), Lambda(5,2) and the effective
 * Laplacian radius a / sqrt(1 + 2 gamma/a) (src/stokes.c:1109-1180) */
void
stokes_set_slip (struct stokes *sys, const double *gamma)
{
  stokes_unset_slip (sys);
  size_t n = (size_t) sys->np;
  sys->slip = (double *) must_alloc (sizeof (double) * n, "stokes_set_slip");
  sys->slip_a = (double *) must_alloc (sizeof (double) * n, "stokes_set_slip");
  sys->slip_G32 = (double *) must_alloc (sizeof (double) * n, "stokes_set_slip");
  sys->slip_G30 = (double *) must_alloc (sizeof (double) * n, "stokes_set_slip");
  sys->slip_G52 = (double *) must_alloc (sizeof (double) * n, "stokes_set_slip");
  for (size_t i = 0; i < n; i++)
    {
      double ai = sys->a ? sys->a[i] : 1.0;
      double g = sys->a ? gamma[i] / ai : gamma[i];
      double l2 = 1.0 + 2.0 * g, l3 = 1.0 + 3.0 * g, l5 = 1.0 + 5.0 * g;
      sys->slip[i] = gamma[i];
      sys->slip_a[i] = ai * sqrt (1.0 / l2);
      sys->slip_G32[i] = l3 / l2;
      sys->slip_G30[i] = l3;
      sys->slip_G52[i] = l5 / l2;
    }
}

void
stokes_unset_slip (struct stokes *sys)
{
  free (sys->slip); free (sys->slip_a); free (sys->slip_G32);
  free (sys->slip_G30); free (sys->slip_G52);
  sys->slip = sys->slip_a = sys->slip_G32 = sys->slip_G30 = sys->slip_G52 = NULL;
  sys->slip_table = NULL;
  sys->twobody_slip_f_list = NULL;
}
