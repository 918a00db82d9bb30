/* oracle_ewald.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C FP64 restatement of the libstokes 0.4.1 Ewald-summed mobility
 * path, used by tests/ (as the checker of the CUDA kernels), by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product
 * (libstokes_gb300) never links, loads or calls this file.
 *
 * It is written from the mathematics of the reference, not from its code:
 *  - the Ewald real-space scalar functions and the reciprocal weights are the
 *    closed forms that the reference evaluates (they must be alike to give
 *    the same numbers): src/ewald.c:49-186 (mono), :204-359 (poly),
 *    :383-420 (SD scaling), :955-958 and :978-1025 (reciprocal);
 *  - the pair tensors A, B, C, G, H, M are applied in vector form
 *    (u += ya F + (xa-ya)(e.F) e, ...), from the definitions that
 *    src/f.c:71-147, src/ft.c:100-267 and src/fts.c:137-1023 spell out
 *    entry by entry; the 5-component stresslet is mapped to a 3x3 tensor
 *    whose full contraction reproduces the extracted-form z-transform of
 *    src/fts.c:664-670 and src/matrix.c:447-478;
 *  - the loops follow src/ewald.c:519-1081 (atimes) and :1092-1677 (dense):
 *    self term, real space over (i, j, image table), reciprocal space over
 *    the k cube and all pairs (i, j), with the rr==0 exclusion, the rmax2
 *    cut, the rmin clamp and the Lees-Edwards shear shifts;
 *  - the set-up (self constants, cutoff search, image table) follows
 *    src/stokes.c:173-310 and :655-776.
 *
 * Parity of this restatement is pinned in tests/ against vectors produced by
 * the reference library itself (tests/golden/, generated by
 * tests/golden/make_golden.py from oracle/_ref).
 *
 * The O(N^2 * images) loop structure is kept on purpose: timed on the host
 * cores it stands for the reference's CPU cost (bench.py cpu_baseline).
 * Loops over target particles i are OpenMP-parallel (each i owns its output).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------------- */
/* oracle system description (independent of the product's struct stokes) */
/* ---------------------------------------------------------------------- */
typedef struct {
  int version;            /* 0 F, 1 FT, 2 FTS */
  int np;
  double *pos;            /* np*3 */
  double *a;              /* NULL = mono */
  double *slip;           /* NULL = no-slip */
  double *slip_a, *slip_G32, *slip_G30, *slip_G52;
  double rmin;
  int shear_mode;
  double shear_shift;
  double lx, ly, lz, pivol;
  double xi, xi2, xiaspi;
  double self_a, self_c, self_m;
  double rmax2;
  int rmaxx, rmaxy, rmaxz;
  double kmax;
  int kmaxx, kmaxy, kmaxz;
  int nr;
  double *rlx, *rly, *rlz;
  int *rmx, *rmy, *rmz;
  int nthreads;
  int open;          /* oracle_atimes evaluates the free-space operator */
} osys;

static int
ncomp (int version)
{
  return version == 0 ? 3 : (version == 1 ? 6 : 11);
}

static void *
xmalloc (size_t n)
{
  void *p = malloc (n > 0 ? n : 1);
  if (p == NULL) { fprintf (stderr, "oracle: out of memory\n"); exit (1); }
  return p;
}

/* real-space error estimate of the cutoff search (src/stokes.c:655-683) */
static double
est_real (double r, double xi)
{
  double u = xi * r / 1.15;
  double u2 = u * u;
  double r2 = r * r;
  return erfc (u) * (0.75 + 1.5 / r2) / r
    + exp (-u2) * xi / sqrt (M_PI)
      * (4.5 + 3.0 * u2 + (3.0 + u2 * (14.0 + u2 * (4.0 + u2))) / r2);
}

/* reciprocal error estimate of the cutoff search (src/stokes.c:685-700) */
static double
est_recip (double k, double xi)
{
  double u = k / xi / 1.15;
  double u2 = u * u;
  double k2 = k * k;
  return 6.0 * M_PI * exp (-u2 / 4.0) * (1.0 + k2 / 3.0) / k2
    * (1.0 + u2 * (1.0 / 4.0 + u2 / 8.0));
}

static void
free_table (osys *s)
{
  free (s->rlx); free (s->rly); free (s->rlz);
  free (s->rmx); free (s->rmy); free (s->rmz);
  s->rlx = s->rly = s->rlz = NULL;
  s->rmx = s->rmy = s->rmz = NULL;
  s->nr = 0;
}

/* Ewald split, self terms, cutoff search and image table
 * (src/stokes.c:703-762 and :173-233). */
static void
setup_split (osys *s, double xi, double eps)
{
  s->xi = xi;
  s->xi2 = xi * xi;
  s->xiaspi = xi / sqrt (M_PI);
  double x2 = s->xi2;
  s->self_a = 1.0 - s->xiaspi * (6.0 - 40.0 / 3.0 * x2);
  s->self_c = 0.75 - s->xiaspi * x2 * 10.0;
  s->self_m = 0.9 - s->xiaspi * x2 * (12.0 - 30.24 * x2);

  double lmin = fmin (s->lx, fmin (s->ly, s->lz));
  double lmax = fmax (s->lx, fmax (s->ly, s->lz));
  const double shrink = 0.99;

  double rmax = 10.0 * sqrt (-log (eps)) / xi;
  while (est_real (rmax * shrink, xi) + 6.0 * est_real (rmax * shrink + lmin, xi)
         < eps)
    rmax *= shrink;
  s->rmax2 = rmax * rmax;
  s->rmaxx = (int) (rmax / s->lx) + 1;
  s->rmaxy = (int) (rmax / s->ly) + 1;
  s->rmaxz = (int) (rmax / s->lz) + 1;

  double dk = 2.0 * M_PI / lmax;
  double kmax = 10.0 * sqrt (-log (eps)) * 2.0 * xi;
  while (est_recip (kmax * shrink, xi) + 6.0 * est_recip (kmax * shrink + dk, xi)
         < eps)
    kmax *= shrink;
  s->kmax = kmax;
  s->kmaxx = (int) (kmax * s->lx / 2.0 / M_PI);
  s->kmaxy = (int) (kmax * s->ly / 2.0 / M_PI);
  s->kmaxz = (int) (kmax * s->lz / 2.0 / M_PI);

  /* image table: cells whose nearest point to the primary cell lies within
   * rmax + |diagonal| */
  free_table (s);
  int cap = (2 * s->rmaxx + 1) * (2 * s->rmaxy + 1) * (2 * s->rmaxz + 1);
  s->rlx = xmalloc (sizeof (double) * cap);
  s->rly = xmalloc (sizeof (double) * cap);
  s->rlz = xmalloc (sizeof (double) * cap);
  s->rmx = xmalloc (sizeof (int) * cap);
  s->rmy = xmalloc (sizeof (int) * cap);
  s->rmz = xmalloc (sizeof (int) * cap);
  double diag = sqrt (s->lx * s->lx + s->ly * s->ly + s->lz * s->lz);
  double lim = sqrt (s->rmax2) + diag;
  for (int m1 = -s->rmaxx; m1 <= s->rmaxx; m1++)
    {
      double cx = s->lx * m1;
      double nx = cx - (m1 > 0 ? 0.5 * s->lx : 0.0) + (m1 < 0 ? 0.5 * s->lx : 0.0);
      for (int m2 = -s->rmaxy; m2 <= s->rmaxy; m2++)
        {
          double cy = s->ly * m2;
          double ny = cy - (m2 > 0 ? 0.5 * s->ly : 0.0) + (m2 < 0 ? 0.5 * s->ly : 0.0);
          for (int m3 = -s->rmaxz; m3 <= s->rmaxz; m3++)
            {
              double cz = s->lz * m3;
              double nz = cz - (m3 > 0 ? 0.5 * s->lz : 0.0) + (m3 < 0 ? 0.5 * s->lz : 0.0);
              if (sqrt (nx * nx + ny * ny + nz * nz) <= lim)
                {
                  int q = s->nr++;
                  s->rlx[q] = cx; s->rly[q] = cy; s->rlz[q] = cz;
                  s->rmx[q] = m1; s->rmy[q] = m2; s->rmz[q] = m3;
                }
            }
        }
    }
}

/* ---------------------------------------------------------------------- */
/* scalar functions                                                        */
/* ---------------------------------------------------------------------- */
/* s[0..10] = xa ya yb xc yc xg yg yh xm ym zm */
enum { XA, YA, YB, XC, YC, XG, YG, YH, XM, YM, ZM, NSC };

/* monodisperse real-space scalars at distance r, unit radius
 * (closed forms evaluated by src/ewald.c:49-186) */
static void
scalars_real_mono (int version, double xi, double r, double *s)
{
  for (int q = 0; q < NSC; q++) s[q] = 0.0;
  double u2 = (xi * r) * (xi * r);
  double r2 = r * r;
  double ec = erfc (xi * r);
  double ex = xi / sqrt (M_PI) * exp (-u2);

  double a1 = (0.75 + 0.5 / r2) / r * ec
    + ((1.0 + u2 * (14.0 + 4.0 * u2 * (u2 - 5.0))) / r2 - 4.5 + 3.0 * u2) * ex;
  double a2 = (0.75 - 1.5 / r2) / r * ec
    + ((-3.0 + u2 * (-2.0 + 4.0 * u2 * (4.0 - u2))) / r2 + 1.5 - 3.0 * u2) * ex;
  s[YA] = a1;
  s[XA] = a1 + a2;
  if (version == 0) return;

  s[YB] = -0.75 / r2 * ec
    - 1.5 * (1.0 + u2 * (-6.0 + 2.0 * u2)) / r * ex;
  double c1 = -0.375 / (r2 * r) * ec
    - 0.75 * (1.0 + u2 * (14.0 + u2 * (-20.0 + 4.0 * u2))) / r2 * ex;
  double c2 = 1.125 / (r2 * r) * ec
    - 0.75 * (-3.0 + u2 * (-2.0 + u2 * (16.0 - 4.0 * u2))) / r2 * ex;
  s[YC] = c1;
  s[XC] = c1 + c2;
  if (version == 1) return;

  s[XG] = (2.25 - 3.6 / r2) / r2 * ec
    + (-1.5 * (-3.0 + 6.0 * u2)
       - 0.8 * (9.0 + u2 * (6.0 + u2 * (-48.0 + 12.0 * u2))) / r2) / r * ex;
  s[YG] = 1.2 / (r2 * r2) * ec
    + (-3.0 * u2 * (2.0 - u2)
       - 0.8 * (-3.0 + u2 * (-2.0 + u2 * (-26.0 + u2 * (26.0 - 4.0 * u2))))
         / r2) / r * ex;
  s[YH] = -1.125 / (r2 * r) * ec
    + 1.5 * (-1.5 + u2 * (-1.0 + u2 * (8.0 - 2.0 * u2))) / r2 * ex;
  s[XM] = (-4.5 + 10.8 / r2) / (r * r2) * ec
    + (1.5 * (-6.0 + u2 * (-12.0 + 12.0 * u2))
       + 1.2 * (18.0 + u2 * (12.0 + u2 * (30.0 + u2 * (-66.0 + 12.0 * u2))))
         / r2) / r2 * ex;
  s[YM] = (2.25 - 7.2 / r2) / (r * r2) * ec
    + (-1.5 * (-3.0 + u2 * (6.0 + u2 * (-12.0 + 4.0 * u2)))
       - 1.2 * (12.0 + u2 * (8.0 + u2 * (-22.0 + u2 * (58.0 + u2 * (-34.0 + 4.0 * u2)))))
         / r2) / r2 * ex;
  s[ZM] = 1.8 / (r2 * r * r2) * ec
    + (-1.5 * u2 * (8.0 - 4.0 * u2)
       - 1.2 * (-3.0 + u2 * (-2.0 + u2 * (-26.0 + u2 * (26.0 - 4.0 * u2))))
         / r2) / r2 * ex;
}

/* polydisperse real-space scalars for radii aa (target) and ab (source),
 * in dimensional form (src/ewald.c:204-359): built from the screened
 * Oseen kernels a(r), b(r) and their radial derivatives */
static void
scalars_real_poly (int version, double xi, double r, double aa, double ab,
                   double *s)
{
  for (int q = 0; q < NSC; q++) s[q] = 0.0;
  double u2 = (xi * r) * (xi * r);
  double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r3 * r2;
  double ec = erfc (xi * r);
  double ex = xi / sqrt (M_PI) * exp (-u2);
  double sa2 = aa * aa + ab * ab;

  double k0 = 2.0 * (-3.0 + 2.0 * u2) * ex + ec / r;
  double k0d = -2.0 / r * (1.0 + u2 * (-10.0 + 4.0 * u2)) * ex - ec / r2;
  double k0dd = 4.0 / r2 * (1.0 + u2 * (6.0 + u2 * (-16.0 + 4.0 * u2))) * ex
    + 2.0 / r3 * ec;
  double h0 = 2.0 * (1.0 - 2.0 * u2) * ex + ec / r;
  double h0d = -2.0 / r * (1.0 + u2 * (6.0 - 4.0 * u2)) * ex - ec / r2;
  double k2 = 4.0 / r2 * (1.0 + u2 * (14.0 + u2 * (-20.0 + 4.0 * u2))) * ex
    + 2.0 / r3 * ec;
  double k2d = -4.0 / r3 * (3.0 + u2 * (2.0 + u2 * (68.0 + u2 * (-56.0 + 8.0 * u2)))) * ex
    - 6.0 / r4 * ec;
  double k2dd = 16.0 / r4
    * (3.0 + u2 * (2.0 + u2 * (-16.0 + u2 * (76.0 + u2 * (-38.0 + 4.0 * u2))))) * ex
    + 24.0 / r5 * ec;
  double h2 = -4.0 / r2 * (3.0 + u2 * (2.0 + u2 * (-16.0 + 4.0 * u2))) * ex
    - 6.0 / r3 * ec;
  double h2d = 4.0 / r3 * (9.0 + u2 * (6.0 + u2 * (36.0 + u2 * (-48.0 + 8.0 * u2)))) * ex
    + 18.0 / r4 * ec;

  s[YA] = 0.75 * (k0 + k2 * sa2 / 6.0);
  s[XA] = 0.75 * (h0 + h2 * sa2 / 6.0) + s[YA];
  if (version == 0) return;

  s[YB] = -0.375 * (-k0d + h0 / r);
  s[YC] = 0.1875 * (-k0dd + (-k0d + h0d) / r);
  s[XC] = 0.1875 * (k0dd + (-k0d - h0d + 2.0 * h0 / r) / r) + s[YC];
  if (version == 1) return;

  double wg = aa * aa / 10.0 + ab * ab / 6.0;
  s[XG] = -3.0 * (-0.75 / r * h0 - 0.75 / r * h2 * wg);
  s[YG] = -0.375 * (k0d + h0 / r) - 0.375 * (k2d + h2 / r) * wg;
  s[YH] = -0.1875 * (k0dd + (-k0d - h0d + 2.0 * h0 / r) / r);
  double m5 = -0.375 * (k0d + h0 / r) / r - 0.375 * (k2d + h2 / r) / r * sa2 / 10.0;
  s[ZM] = 2.0 * m5;
  double m3 = -0.75 * h0 / r2 - 0.75 * h2 / r2 * sa2 / 10.0;
  s[XM] = 6.0 * m3 + 3.0 * s[ZM];
  double m4 = -0.1875 * (k0dd + (-k0d + 3.0 * h0d - 6.0 * h0 / r) / r)
    - 0.1875 * (k2dd + (-k2d + 3.0 * h2d - 6.0 * h2 / r) / r) * sa2 / 10.0;
  s[YM] = 2.0 * m4 + s[ZM];
}

/* dimensional -> SD scaling by the target radius (src/ewald.c:383-420) */
static void
scale_sd (int version, double a1, double *s)
{
  s[XA] *= a1; s[YA] *= a1;
  if (version == 0) return;
  double a2 = a1 * a1, a3 = a2 * a1;
  s[YB] *= a2; s[XC] *= a3; s[YC] *= a3;
  if (version == 1) return;
  s[XG] *= a2; s[YG] *= a2; s[YH] *= a3;
  s[XM] *= a3; s[YM] *= a3; s[ZM] *= a3;
}

/* ---------------------------------------------------------------------- */
/* pair tensors in vector form                                             */
/* ---------------------------------------------------------------------- */
static inline double dot3 (const double *u, const double *v)
{ return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; }
static inline void cross3 (const double *u, const double *v, double *w)
{
  w[0] = u[1] * v[2] - u[2] * v[1];
  w[1] = u[2] * v[0] - u[0] * v[2];
  w[2] = u[0] * v[1] - u[1] * v[0];
}

/* Apply the pair block (target i <- source j, unit vector e from i to j,
 * scalars s) to the source generalised force and ADD into the target.
 *  F[3], T[3]  : force and torque of the source
 *  S[3][3]     : stresslet of the source (full symmetric 3x3; trace terms
 *                are kept so a non-traceless unit tensor yields the single
 *                extracted-form column the dense builder stores)
 *  U[3], W[3], E[3][3] : velocity, angular velocity, strain (accumulated)
 *  sgn_bt, sgn_gt : +1 for the operator (and for i != j); the dense builder
 *                uses -1 on its i == j blocks (src/ft.c:61-75, fts.c:72-104)
 */
static void
pair_apply (int version, const double *e, const double *s,
            const double *F, const double *T, double S[3][3],
            double *U, double *W, double E[3][3],
            double sgn_bt, double sgn_gt)
{
  double eF = dot3 (e, F);
  for (int a = 0; a < 3; a++)
    U[a] += s[YA] * F[a] + (s[XA] - s[YA]) * eF * e[a];
  if (version == 0) return;

  double Fxe[3], Txe[3];
  cross3 (F, e, Fxe);
  cross3 (T, e, Txe);
  double eT = dot3 (e, T);
  for (int a = 0; a < 3; a++)
    {
      U[a] += sgn_bt * s[YB] * Txe[a];
      W[a] += s[YB] * Fxe[a] + s[YC] * T[a] + (s[XC] - s[YC]) * eT * e[a];
    }
  if (version == 1) return;

  double g1 = -s[XG] / 3.0, g2 = s[YG], g3 = s[XG] - 2.0 * s[YG];
  double m1 = 1.5 * s[XM] - 2.0 * s[YM] + 0.5 * s[ZM];
  double m2 = -0.5 * s[XM] + 0.5 * s[ZM];
  double m3 = s[XM] / 6.0 - 0.5 * s[ZM];
  double m4 = 0.5 * s[YM] - 0.5 * s[ZM];
  double m5 = 0.5 * s[ZM];

  double Se[3], eS[3], trS = S[0][0] + S[1][1] + S[2][2];
  for (int a = 0; a < 3; a++)
    {
      Se[a] = S[a][0] * e[0] + S[a][1] * e[1] + S[a][2] * e[2];
      eS[a] = e[0] * S[0][a] + e[1] * S[1][a] + e[2] * S[2][a];
    }
  double eSe = dot3 (e, Se);
  double Sym[3];                    /* (S + S^T) e */
  for (int a = 0; a < 3; a++) Sym[a] = Se[a] + eS[a];

  /* U <- G^T S  (G_(ab)c = g1 d_ab e_c + g2 (e_a d_bc + e_b d_ac) + g3 e_a e_b e_c) */
  for (int c = 0; c < 3; c++)
    {
      double gs = g1 * trS * e[c] + g2 * Sym[c] + g3 * eSe * e[c];
      U[c] += sgn_gt * (-gs);
    }
  /* W <- H^T S  (H_(ab)c = yh (e_a eps_bcl e_l + e_b eps_acl e_l)) */
  {
    double v1[3], v2[3];
    cross3 (e, Se, v1);             /* sum_ab e_a S_ab eps_bcl e_l -> -(Se x e) */
    cross3 (e, eS, v2);
    for (int c = 0; c < 3; c++) W[c] += s[YH] * (v1[c] + v2[c]);
  }
  /* E <- G F + H T + M S */
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      {
        double dab = (a == b) ? 1.0 : 0.0;
        double g = g1 * dab * eF + g2 * (e[a] * F[b] + e[b] * F[a])
          + g3 * e[a] * e[b] * eF;
        double h = s[YH] * (e[a] * Txe[b] + e[b] * Txe[a]);
        double m = m1 * e[a] * e[b] * eSe
          + m2 * (dab * eSe + e[a] * e[b] * trS)
          + m3 * dab * trS
          + m4 * (e[a] * Sym[b] + e[b] * Sym[a])
          + m5 * (S[a][b] + S[b][a]);
        E[a][b] += g + h + m;
      }
}

/* Map a 5-component stresslet (xx,xy,xz,yz,yy) to the 3x3 tensor S' whose
 * full contraction with a pair tensor equals the extracted-form product of
 * src/fts.c:664-670 / src/matrix.c:447-478 (z = (2xx+yy, 2xy, 2xz, 2yz,
 * 2yy+xx) against the five stored components).  For a traceless pair tensor
 * this is the contraction with the traceless S (Szz = -Sxx-Syy); S' also
 * reproduces the reference when the rmin clamp makes |e| < 1 and the pair
 * tensors lose their tracelessness. */
static void
stress_full (const double *x5, double S[3][3])
{
  S[0][0] = 2.0 * x5[0] + x5[4]; S[0][1] = x5[1]; S[0][2] = x5[2];
  S[1][0] = x5[1]; S[1][1] = 2.0 * x5[4] + x5[0]; S[1][2] = x5[3];
  S[2][0] = x5[2]; S[2][1] = x5[3]; S[2][2] = 0.0;
}

/* accumulate the generalised velocity of the target into y[c] */
static void
store_out (int version, const double *U, const double *W, double E[3][3],
           double *y)
{
  y[0] += U[0]; y[1] += U[1]; y[2] += U[2];
  if (version == 0) return;
  y[3] += W[0]; y[4] += W[1]; y[5] += W[2];
  if (version == 1) return;
  y[6] += E[0][0]; y[7] += E[0][1]; y[8] += E[0][2];
  y[9] += E[1][2]; y[10] += E[1][1];
}

/* one pair term on vectors: y_i += block(e, s) . x_j.  Same algebra as
 * pair_apply, unrolled for the symmetric S' of the product so that the CPU
 * cost per term stays close to the reference's. */
static void
pair_vec (int version, const double *e, const double *s, const double *xj,
          double *yi)
{
  const double *F = xj;
  double eF = dot3 (e, F);
  double a2 = s[XA] - s[YA];
  yi[0] += s[YA] * F[0] + a2 * eF * e[0];
  yi[1] += s[YA] * F[1] + a2 * eF * e[1];
  yi[2] += s[YA] * F[2] + a2 * eF * e[2];
  if (version == 0) return;

  const double *T = xj + 3;
  double Fxe[3], Txe[3];
  cross3 (F, e, Fxe);
  cross3 (T, e, Txe);
  double eT = dot3 (e, T);
  double c2 = s[XC] - s[YC];
  for (int a = 0; a < 3; a++)
    {
      yi[a] += s[YB] * Txe[a];
      yi[3 + a] += s[YB] * Fxe[a] + s[YC] * T[a] + c2 * eT * e[a];
    }
  if (version == 1) return;

  double S[3][3];
  stress_full (xj + 6, S);
  double Se[3];
  for (int a = 0; a < 3; a++) Se[a] = S[a][0] * e[0] + S[a][1] * e[1] + S[a][2] * e[2];
  double eSe = dot3 (e, Se), trS = S[0][0] + S[1][1];
  double g1 = -s[XG] / 3.0, g2 = s[YG], g3 = s[XG] - 2.0 * s[YG];
  double m1 = 1.5 * s[XM] - 2.0 * s[YM] + 0.5 * s[ZM];
  double m2 = -0.5 * s[XM] + 0.5 * s[ZM];
  double m3 = s[XM] / 6.0 - 0.5 * s[ZM];
  double m4 = 0.5 * s[YM] - 0.5 * s[ZM];
  double m5 = 0.5 * s[ZM];
  double v[3];
  cross3 (e, Se, v);
  double gu = g1 * trS + g3 * eSe;
  double d = g1 * eF + m2 * eSe + m3 * trS;     /* delta_ab coefficient */
  double q = g3 * eF + m1 * eSe + m2 * trS;     /* e_a e_b coefficient */
  double V[3];                                  /* e_a V_b + e_b V_a */
  for (int a = 0; a < 3; a++)
    {
      yi[a] -= gu * e[a] + 2.0 * g2 * Se[a];
      yi[3 + a] += 2.0 * s[YH] * v[a];
      V[a] = g2 * F[a] + s[YH] * Txe[a] + 2.0 * m4 * Se[a];
    }
  static const int ia[5] = {0, 0, 0, 1, 1}, ib[5] = {0, 1, 2, 2, 1};
  for (int k = 0; k < 5; k++)
    {
      int a = ia[k], b = ib[k];
      yi[6 + k] += (a == b ? d : 0.0) + q * e[a] * e[b] + e[a] * V[b] + e[b] * V[a]
        + 2.0 * m5 * S[a][b];
    }
}

/* one pair term on the dense matrix: block (i, j) += block(e, s), written
 * column by column in the extracted form */
static void
pair_mat (int version, int same, const double *e, const double *s,
          double *blk, int ld)
{
  int c = ncomp (version);
  double sgn = same ? -1.0 : 1.0;
  for (int col = 0; col < c; col++)
    {
      double F[3] = {0, 0, 0}, T[3] = {0, 0, 0}, S[3][3] = {{0}};
      if (col < 3) F[col] = 1.0;
      else if (col < 6) T[col - 3] = 1.0;
      else
        {
          /* extracted-form column: unit weight on one tensor component */
          static const int ia[5] = {0, 0, 0, 1, 1};
          static const int ib[5] = {0, 1, 2, 2, 1};
          int q = col - 6;
          if (ia[q] == ib[q]) S[ia[q]][ib[q]] = 1.0;
          else { S[ia[q]][ib[q]] = 0.5; S[ib[q]][ia[q]] = 0.5; }
        }
      double U[3] = {0, 0, 0}, W[3] = {0, 0, 0}, E[3][3] = {{0}};
      pair_apply (version, e, s, F, T, S, U, W, E, sgn, sgn);
      double out[11] = {0};
      store_out (version, U, W, E, out);
      for (int row = 0; row < c; row++) blk[row * ld + col] += out[row];
    }
}

/* ---------------------------------------------------------------------- */
/* per-particle constants                                                  */
/* ---------------------------------------------------------------------- */
static double rad (const osys *s, int i) { return s->a ? s->a[i] : 1.0; }

/* self scalars of particle i (src/ewald.c:540-643) */
static void
self_scalars (const osys *s, int i, double *sc)
{
  for (int q = 0; q < NSC; q++) sc[q] = 0.0;
  if (s->a == NULL && s->slip == NULL)
    {
      sc[XA] = sc[YA] = s->self_a;
      sc[XC] = sc[YC] = s->self_c;
      sc[XM] = sc[YM] = sc[ZM] = s->self_m;
      return;
    }
  double a = rad (s, i), a2 = a * a, a3 = a2 * a;
  double fa = 1.0, fc = 1.0, fm = 1.0;
  if (s->slip != NULL)
    { fa = s->slip_G32[i]; fc = s->slip_G30[i]; fm = s->slip_G52[i]; }
  double sa = 1.0 * fa - a * s->xiaspi * (6.0 - 40.0 / 3.0 * s->xi2 * a2);
  double scc = 0.75 * fc - a3 * s->xiaspi * s->xi2 * 10.0;
  double sm = 0.9 * fm - a3 * s->xiaspi * s->xi2 * (12.0 - 30.24 * s->xi2 * a2);
  sc[XA] = sc[YA] = sa;
  sc[XC] = sc[YC] = scc;
  sc[XM] = sc[YM] = sc[ZM] = sm;
}

/* real-space scalars for the pair (i, j) at distance r, SD form */
static void
real_scalars (const osys *s, int i, int j, double r, double *sc)
{
  if (s->a == NULL && s->slip == NULL)
    {
      scalars_real_mono (s->version, s->xi, r, sc);
      return;
    }
  if (s->slip == NULL)
    scalars_real_poly (s->version, s->xi, r, s->a[i], s->a[j], sc);
  else
    scalars_real_poly (s->version, s->xi, r, s->slip_a[i], s->slip_a[j], sc);
  scale_sd (s->version, rad (s, i), sc);
}

/* reciprocal weights for pair (i, j): y-functions times kexp
 * (src/ewald.c:955-958, 978-1025) */
static void
recip_scalars (const osys *s, int i, int j, double k, double kk, double kexp,
               double cf, double sf, double *sc)
{
  double ya, yb, yc, yg, yh, ym;
  if (s->a == NULL && s->slip == NULL)
    {
      ya = 6.0 * (1.0 - kk / 3.0) * kexp;
      yb = 3.0 * k * kexp;
      yc = 1.5 * kk * kexp;
      yg = 3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp;
      yh = 1.5 * kk * kexp;
      ym = 3.0 * (1.0 - kk / 5.0) * kk * kexp;
    }
  else
    {
      double aa = rad (s, i), aa2 = aa * aa, aa3 = aa2 * aa;
      double qa, qb;
      if (s->slip == NULL) { qa = aa2; qb = rad (s, j) * rad (s, j); }
      else { qa = s->slip_a[i] * s->slip_a[i]; qb = s->slip_a[j] * s->slip_a[j]; }
      ya = aa * 6.0 * (1.0 - kk * (qa + qb) / 6.0) * kexp;
      yb = aa2 * 3.0 * k * kexp;
      yc = aa3 * 1.5 * kk * kexp;
      yg = aa2 * 3.0 * (1.0 - kk * (qa / 10.0 + qb / 6.0)) * k * kexp;
      yh = aa3 * 1.5 * kk * kexp;
      ym = aa3 * 3.0 * (1.0 - kk * (qa + qb) / 10.0) * kk * kexp;
    }
  for (int q = 0; q < NSC; q++) sc[q] = 0.0;
  sc[YA] = cf * ya;
  sc[YB] = sf * yb;
  sc[YC] = cf * yc;
  sc[YG] = sf * yg;
  sc[YH] = cf * yh;
  sc[YM] = cf * ym;
}

/* reciprocal vector (m1, m2, m3) with shear; returns 0 when outside kmax */
static int
kvec (const osys *s, int m1, int m2, int m3, double *kv, double *k, double *kk)
{
  double k0x = 2.0 * M_PI / s->lx, k0y = 2.0 * M_PI / s->ly, k0z = 2.0 * M_PI / s->lz;
  double sl = s->shear_shift / s->lx;
  kv[0] = k0x * m1;
  kv[1] = k0y * m2;
  kv[2] = k0z * m3;
  if (s->shear_mode == 1) kv[1] = k0y * ((double) m2 - sl * (double) m1);
  else if (s->shear_mode == 2) kv[2] = k0z * ((double) m3 - sl * (double) m1);
  *kk = dot3 (kv, kv);
  *k = sqrt (*kk);
  if (s->kmax != 0.0 && *k > s->kmax) return 0;
  return 1;
}

/* ---------------------------------------------------------------------- */
/* exported oracle API                                                     */
/* ---------------------------------------------------------------------- */
void *
oracle_new (int version, int np, const double *pos, double lx, double ly,
            double lz)
{
  osys *s = calloc (1, sizeof (osys));
  s->version = version;
  s->np = np;
  s->pos = xmalloc (sizeof (double) * 3 * np);
  memcpy (s->pos, pos, sizeof (double) * 3 * np);
  s->lx = lx; s->ly = ly; s->lz = lz;
  s->pivol = M_PI / lx / ly / lz;
  s->nthreads = 1;
  return s;
}

void
oracle_free (void *h)
{
  osys *s = h;
  if (s == NULL) return;
  free_table (s);
  free (s->pos); free (s->a); free (s->slip);
  free (s->slip_a); free (s->slip_G32); free (s->slip_G30); free (s->slip_G52);
  free (s);
}

void oracle_set_threads (void *h, int n) { ((osys *) h)->nthreads = n > 0 ? n : 1; }

void
oracle_set_pos (void *h, const double *pos)
{
  osys *s = h;
  memcpy (s->pos, pos, sizeof (double) * 3 * s->np);
}

void
oracle_set_split (void *h, double xi, double eps)
{
  setup_split ((osys *) h, xi, eps);
}

/* xi from the time ratio (src/stokes.c:766-776) */
double
oracle_xi_by_tratio (double lx, double ly, double lz, double tratio)
{
  return pow (tratio, 1.0 / 6.0) * sqrt (M_PI) / pow (lx * ly * lz, 1.0 / 3.0);
}

/* replace the image table by the full cube |m_i| <= nr_shell, take every
 * image (rmax2 = +inf) and the whole k cube |m_i| <= nk_shell (kmax = 0) */
void
oracle_set_cube (void *h, int nr_shell, int nk_shell)
{
  osys *s = h;
  free_table (s);
  int side = 2 * nr_shell + 1, cap = side * side * side;
  s->rlx = xmalloc (sizeof (double) * cap);
  s->rly = xmalloc (sizeof (double) * cap);
  s->rlz = xmalloc (sizeof (double) * cap);
  s->rmx = xmalloc (sizeof (int) * cap);
  s->rmy = xmalloc (sizeof (int) * cap);
  s->rmz = xmalloc (sizeof (int) * cap);
  for (int m1 = -nr_shell; m1 <= nr_shell; m1++)
    for (int m2 = -nr_shell; m2 <= nr_shell; m2++)
      for (int m3 = -nr_shell; m3 <= nr_shell; m3++)
        {
          int q = s->nr++;
          s->rlx[q] = s->lx * m1; s->rly[q] = s->ly * m2; s->rlz[q] = s->lz * m3;
          s->rmx[q] = m1; s->rmy[q] = m2; s->rmz[q] = m3;
        }
  s->rmax2 = INFINITY;
  s->kmaxx = s->kmaxy = s->kmaxz = nk_shell;
  s->kmax = 0.0;
}

void
oracle_set_radius (void *h, const double *a)
{
  osys *s = h;
  free (s->a);
  s->a = NULL;
  if (a == NULL) return;
  s->a = xmalloc (sizeof (double) * s->np);
  memcpy (s->a, a, sizeof (double) * s->np);
}

/* slip factors (src/stokes.c:1109-1180) */
void
oracle_set_slip (void *h, const double *gamma)
{
  osys *s = h;
  free (s->slip); free (s->slip_a); free (s->slip_G32); free (s->slip_G30);
  free (s->slip_G52);
  s->slip = s->slip_a = s->slip_G32 = s->slip_G30 = s->slip_G52 = NULL;
  if (gamma == NULL) return;
  int n = s->np;
  s->slip = xmalloc (sizeof (double) * n);
  s->slip_a = xmalloc (sizeof (double) * n);
  s->slip_G32 = xmalloc (sizeof (double) * n);
  s->slip_G30 = xmalloc (sizeof (double) * n);
  s->slip_G52 = xmalloc (sizeof (double) * n);
  for (int i = 0; i < n; i++)
    {
      double a = rad (s, i);
      double g = gamma[i] / (s->a ? a : 1.0);
      double l2 = 1.0 + 2.0 * g, l3 = 1.0 + 3.0 * g, l5 = 1.0 + 5.0 * g;
      s->slip[i] = gamma[i];
      s->slip_a[i] = a * sqrt (1.0 / l2);
      s->slip_G32[i] = l3 / l2;
      s->slip_G30[i] = l3;
      s->slip_G52[i] = l5 / l2;
    }
}

void
oracle_set_misc (void *h, double rmin, int shear_mode, double shear_shift)
{
  osys *s = h;
  s->rmin = rmin;
  s->shear_mode = shear_mode;
  s->shear_shift = shear_shift;
}

/* query the split: out[0..8] = xi, rmax2, kmax, self_a, self_c, self_m,
 * pivol, nr, (kmaxx*10000 + kmaxy*100 + kmaxz) */
void
oracle_get_split (void *h, double *out)
{
  osys *s = h;
  out[0] = s->xi; out[1] = s->rmax2; out[2] = s->kmax;
  out[3] = s->self_a; out[4] = s->self_c; out[5] = s->self_m;
  out[6] = s->pivol; out[7] = s->nr;
  out[8] = s->kmaxx * 10000 + s->kmaxy * 100 + s->kmaxz;
}

void
oracle_get_table (void *h, double *rl, int *rm)
{
  osys *s = h;
  for (int q = 0; q < s->nr; q++)
    {
      rl[3 * q] = s->rlx[q]; rl[3 * q + 1] = s->rly[q]; rl[3 * q + 2] = s->rlz[q];
      rm[3 * q] = s->rmx[q]; rm[3 * q + 1] = s->rmy[q]; rm[3 * q + 2] = s->rmz[q];
    }
}

/* count of real-space terms (i, j, image) inside the cutoff */
long long
oracle_count_real_terms (void *h)
{
  osys *s = h;
  long long cnt = 0;
  for (int i = 0; i < s->np; i++)
    for (int j = 0; j < s->np; j++)
      for (int m = 0; m < s->nr; m++)
        {
          double d[3];
          d[0] = s->pos[3 * j] - s->pos[3 * i] + s->rlx[m];
          d[1] = s->pos[3 * j + 1] - s->pos[3 * i + 1] + s->rly[m];
          d[2] = s->pos[3 * j + 2] - s->pos[3 * i + 2] + s->rlz[m];
          if (s->shear_mode == 1) d[0] += s->rmy[m] * s->shear_shift;
          else if (s->shear_mode == 2) d[0] += s->rmz[m] * s->shear_shift;
          double rr = dot3 (d, d);
          if (rr == 0.0 || rr > s->rmax2) continue;
          cnt++;
        }
  return cnt;
}

/* number of reciprocal vectors taken */
int
oracle_count_k (void *h)
{
  osys *s = h;
  int cnt = 0;
  for (int m1 = -s->kmaxx; m1 <= s->kmaxx; m1++)
    for (int m2 = -s->kmaxy; m2 <= s->kmaxy; m2++)
      for (int m3 = -s->kmaxz; m3 <= s->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          double kv[3], k, kk;
          if (kvec (s, m1, m2, m3, kv, &k, &kk)) cnt++;
        }
  return cnt;
}

/* y = M x  (restates src/ewald.c:519-1081) for the target rows [i0, i1).
 * part: 1 = self + real space only, 2 = reciprocal only, 3 = full */
static void
atimes_rows (osys *s, const double *x, double *y, int part, int i0, int i1)
{
  int c = ncomp (s->version);
  memset (y, 0, sizeof (double) * c * s->np);

  /* reciprocal vectors and weights, shared by all i */
  int kcap = (2 * s->kmaxx + 1) * (2 * s->kmaxy + 1) * (2 * s->kmaxz + 1);
  double *kt = xmalloc (sizeof (double) * 6 * kcap);
  int nk = 0;
  for (int m1 = -s->kmaxx; m1 <= s->kmaxx; m1++)
    for (int m2 = -s->kmaxy; m2 <= s->kmaxy; m2++)
      for (int m3 = -s->kmaxz; m3 <= s->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          double kv[3], k, kk;
          if (!kvec (s, m1, m2, m3, kv, &k, &kk)) continue;
          double k4z = kk / 4.0 / s->xi2;
          double kexp = s->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          double *t = kt + 6 * nk++;
          t[0] = kv[0]; t[1] = kv[1]; t[2] = kv[2]; t[3] = k; t[4] = kk; t[5] = kexp;
        }

  int np = s->np;
#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads)
  for (int i = i0; i < i1; i++)
    {
      double *yi = y + c * i;
      double sc[NSC], e[3];
      if (part & 1)
        {
          double e0[3] = {0, 0, 0};
          self_scalars (s, i, sc);
          pair_vec (s->version, e0, sc, x + c * i, yi);

          double ai = rad (s, i);
          for (int j = 0; j < np; j++)
            {
              double aj = rad (s, j);
              for (int m = 0; m < s->nr; m++)
                {
                  double d[3];
                  d[0] = s->pos[3 * j] - s->pos[3 * i] + s->rlx[m];
                  d[1] = s->pos[3 * j + 1] - s->pos[3 * i + 1] + s->rly[m];
                  d[2] = s->pos[3 * j + 2] - s->pos[3 * i + 2] + s->rlz[m];
                  if (s->shear_mode == 1) d[0] += s->rmy[m] * s->shear_shift;
                  else if (s->shear_mode == 2) d[0] += s->rmz[m] * s->shear_shift;
                  double rr = dot3 (d, d);
                  if (rr == 0.0 || rr > s->rmax2) continue;
                  double r = sqrt (rr);
                  double rm = (ai + aj) * s->rmin;
                  if (r < rm) r = rm;
                  e[0] = d[0] / r; e[1] = d[1] / r; e[2] = d[2] / r;
                  real_scalars (s, i, j, r, sc);
                  pair_vec (s->version, e, sc, x + c * j, yi);
                }
            }
        }
      if (part & 2)
        {
          for (int q = 0; q < nk; q++)
            {
              const double *t = kt + 6 * q;
              double k = t[3];
              e[0] = t[0] / k; e[1] = t[1] / k; e[2] = t[2] / k;
              for (int j = 0; j < np; j++)
                {
                  double ph = t[0] * (s->pos[3 * j] - s->pos[3 * i])
                    + t[1] * (s->pos[3 * j + 1] - s->pos[3 * i + 1])
                    + t[2] * (s->pos[3 * j + 2] - s->pos[3 * i + 2]);
                  recip_scalars (s, i, j, k, t[4], t[5], cos (ph), -sin (ph), sc);
                  pair_vec (s->version, e, sc, x + c * j, yi);
                }
            }
        }
    }
  free (kt);
}

void
oracle_atimes_part (void *h, const double *x, double *y, int part)
{
  osys *s = h;
  atimes_rows (s, x, y, part, 0, s->np);
}

/* rows [i0, i1) only: a bounded sample of the full product's CPU cost */
void
oracle_atimes_rows (void *h, const double *x, double *y, int i0, int i1)
{
  osys *s = h;
  atimes_rows (s, x, y, 3, i0 < 0 ? 0 : i0, i1 > s->np ? s->np : i1);
}

void oracle_atimes_nonewald (void *h, const double *x, double *y);

/* the operator of the system: the Ewald sum, or the free-space sum once
 * oracle_set_open (h, 1) was called (src/ewald.c:433-447 on periodic) */
void
oracle_atimes (void *h, const double *x, double *y)
{
  if (((osys *) h)->open)
    oracle_atimes_nonewald (h, x, y);
  else
    oracle_atimes_part (h, x, y, 3);
}

void oracle_set_open (void *h, int open) { ((osys *) h)->open = open; }

/* dense mobility matrix, extracted form (restates src/ewald.c:1092-1677) */
void
oracle_matrix (void *h, double *mat)
{
  osys *s = h;
  int c = ncomp (s->version);
  int np = s->np, n = c * np;
  memset (mat, 0, sizeof (double) * (size_t) n * n);

  int kcap = (2 * s->kmaxx + 1) * (2 * s->kmaxy + 1) * (2 * s->kmaxz + 1);
  double *kt = xmalloc (sizeof (double) * 6 * kcap);
  int nk = 0;
  for (int m1 = -s->kmaxx; m1 <= s->kmaxx; m1++)
    for (int m2 = -s->kmaxy; m2 <= s->kmaxy; m2++)
      for (int m3 = -s->kmaxz; m3 <= s->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          double kv[3], k, kk;
          if (!kvec (s, m1, m2, m3, kv, &k, &kk)) continue;
          double k4z = kk / 4.0 / s->xi2;
          double kexp = s->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          double *t = kt + 6 * nk++;
          t[0] = kv[0]; t[1] = kv[1]; t[2] = kv[2]; t[3] = k; t[4] = kk; t[5] = kexp;
        }

#pragma omp parallel for schedule(dynamic, 1) num_threads(s->nthreads)
  for (int i = 0; i < np; i++)
    {
      double sc[NSC], e[3];
      double e0[3] = {0, 0, 0};
      self_scalars (s, i, sc);
      pair_mat (s->version, 1, e0, sc, mat + (size_t) (c * i) * n + c * i, n);
      double ai = rad (s, i);
      for (int j = 0; j < np; j++)
        {
          double *blk = mat + (size_t) (c * i) * n + c * j;
          double aj = rad (s, j);
          for (int m = 0; m < s->nr; m++)
            {
              double d[3];
              d[0] = s->pos[3 * j] - s->pos[3 * i] + s->rlx[m];
              d[1] = s->pos[3 * j + 1] - s->pos[3 * i + 1] + s->rly[m];
              d[2] = s->pos[3 * j + 2] - s->pos[3 * i + 2] + s->rlz[m];
              if (s->shear_mode == 1) d[0] += s->rmy[m] * s->shear_shift;
              else if (s->shear_mode == 2) d[0] += s->rmz[m] * s->shear_shift;
              double rr = dot3 (d, d);
              if (rr == 0.0 || rr > s->rmax2) continue;
              double r = sqrt (rr);
              double rm = (ai + aj) * s->rmin;
              if (r < rm) r = rm;
              e[0] = d[0] / r; e[1] = d[1] / r; e[2] = d[2] / r;
              real_scalars (s, i, j, r, sc);
              pair_mat (s->version, i == j, e, sc, blk, n);
            }
          for (int q = 0; q < nk; q++)
            {
              const double *t = kt + 6 * q;
              double k = t[3];
              e[0] = t[0] / k; e[1] = t[1] / k; e[2] = t[2] / k;
              double ph = t[0] * (s->pos[3 * j] - s->pos[3 * i])
                + t[1] * (s->pos[3 * j + 1] - s->pos[3 * i + 1])
                + t[2] * (s->pos[3 * j + 2] - s->pos[3 * i + 2]);
              recip_scalars (s, i, j, k, t[4], t[5], cos (ph), -sin (ph), sc);
              pair_mat (s->version, i == j, e, sc, blk, n);
            }
        }
    }
  free (kt);
}

/* free-space (non-periodic) Rotne-Prager-Yamakawa scalars at distance r for
 * radii aa, ab in dimensional form (src/non-ewald.c:49-152; equal spheres
 * are aa = ab = 1) */
static void
scalars_open (int version, double r, double aa, double ab, double *sc)
{
  for (int q = 0; q < NSC; q++) sc[q] = 0.0;
  double r2 = r * r, s2 = aa * aa + ab * ab;
  sc[XA] = (1.5 - 0.5 * s2 / r2) / r;
  sc[YA] = (0.75 + 0.25 * s2 / r2) / r;
  if (version == 0) return;
  sc[YB] = -0.75 / r2;
  sc[XC] = 0.75 / r2 / r;
  sc[YC] = -0.375 / r2 / r;
  if (version == 1) return;
  double q = aa * aa / 10.0 + ab * ab / 6.0;
  sc[XG] = (2.25 - 13.5 * q / r2) / r2;
  sc[YG] = 4.5 * q / r2 / r2;
  sc[YH] = -1.125 / r2 / r;
  sc[XM] = (-4.5 + 5.4 * s2 / r2) / r2 / r;
  sc[YM] = (2.25 - 3.6 * s2 / r2) / r2 / r;
  sc[ZM] = 0.9 * s2 / r2 / r2 / r;
}

/* self and pair scalars of the free-space operator (src/non-ewald.c:344-471):
 * self 1, 3/4, 9/10 (times the slip factors); pairs in the SD form scaled by
 * the target's radius, with the slip-effective radii under slip */
static void
open_self (const osys *s, int i, double *sc)
{
  for (int q = 0; q < NSC; q++) sc[q] = 0.0;
  double fa = 1.0, fc = 1.0, fm = 1.0;
  if (s->slip != NULL) { fa = s->slip_G32[i]; fc = s->slip_G30[i]; fm = s->slip_G52[i]; }
  sc[XA] = sc[YA] = 1.0 * fa;
  sc[XC] = sc[YC] = 0.75 * fc;
  sc[XM] = sc[YM] = sc[ZM] = 0.9 * fm;
}

static void
open_pair (const osys *s, int i, int j, double r, double *sc)
{
  if (s->a == NULL && s->slip == NULL)
    {
      scalars_open (s->version, r, 1.0, 1.0, sc);
      return;
    }
  if (s->slip == NULL)
    scalars_open (s->version, r, s->a[i], s->a[j], sc);
  else
    scalars_open (s->version, r, s->slip_a[i], s->slip_a[j], sc);
  scale_sd (s->version, rad (s, i), sc);
}

/* y = M x of the free-space operator: every pair j != i once, positions as
 * given (no periodic images), rmin clamp (src/non-ewald.c:330-475) */
void
oracle_atimes_nonewald (void *h, const double *x, double *y)
{
  osys *s = h;
  int c = ncomp (s->version), np = s->np;
  memset (y, 0, sizeof (double) * (size_t) c * np);
#pragma omp parallel for schedule(dynamic, 4) num_threads(s->nthreads)
  for (int i = 0; i < np; i++)
    {
      double sc[NSC], e[3], e0[3] = {0, 0, 0};
      double *yi = y + c * i;
      open_self (s, i, sc);
      pair_vec (s->version, e0, sc, x + c * i, yi);
      double ai = rad (s, i);
      for (int j = 0; j < np; j++)
        {
          if (j == i) continue;
          double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                         s->pos[3 * j + 2] - s->pos[3 * i + 2]};
          double r = sqrt (dot3 (d, d));
          double rm = (ai + rad (s, j)) * s->rmin;
          if (r < rm) r = rm;
          e[0] = d[0] / r; e[1] = d[1] / r; e[2] = d[2] / r;
          open_pair (s, i, j, r, sc);
          pair_vec (s->version, e, sc, x + c * j, yi);
        }
    }
}

/* dense free-space matrix, extracted form (src/non-ewald.c:494-666) */
void
oracle_matrix_nonewald (void *h, double *mat)
{
  osys *s = h;
  int c = ncomp (s->version), np = s->np, n = c * np;
  memset (mat, 0, sizeof (double) * (size_t) n * n);
#pragma omp parallel for schedule(dynamic, 4) num_threads(s->nthreads)
  for (int i = 0; i < np; i++)
    {
      double sc[NSC], e[3], e0[3] = {0, 0, 0};
      open_self (s, i, sc);
      pair_mat (s->version, 1, e0, sc, mat + (size_t) (c * i) * n + c * i, n);
      double ai = rad (s, i);
      for (int j = 0; j < np; j++)
        {
          if (j == i) continue;
          double d[3] = {s->pos[3 * j] - s->pos[3 * i], s->pos[3 * j + 1] - s->pos[3 * i + 1],
                         s->pos[3 * j + 2] - s->pos[3 * i + 2]};
          double r = sqrt (dot3 (d, d));
          double rm = (ai + rad (s, j)) * s->rmin;
          if (r < rm) r = rm;
          e[0] = d[0] / r; e[1] = d[1] / r; e[2] = d[2] / r;
          open_pair (s, i, j, r, sc);
          pair_mat (s->version, 0, e, sc, mat + (size_t) (c * i) * n + c * j, n);
        }
    }
}

/* extracted-form FTS product (src/matrix.c:447-478) and plain GEMV */
void
oracle_matvec (int version, int np, const double *mat, const double *x, double *y)
{
  int c = ncomp (version), n = c * np;
  double *z = xmalloc (sizeof (double) * n);
  memcpy (z, x, sizeof (double) * n);
  if (version == 2)
    for (int j = 0; j < np; j++)
      {
        const double *xj = x + 11 * j;
        double *zj = z + 11 * j;
        zj[6] = 2.0 * xj[6] + xj[10];
        zj[7] = 2.0 * xj[7];
        zj[8] = 2.0 * xj[8];
        zj[9] = 2.0 * xj[9];
        zj[10] = 2.0 * xj[10] + xj[6];
      }
  for (int i = 0; i < n; i++)
    {
      double acc = 0.0;
      const double *row = mat + (size_t) i * n;
      for (int j = 0; j < n; j++) acc += row[j] * z[j];
      y[i] = acc;
    }
  free (z);
}
