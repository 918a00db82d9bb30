/* oracle_lub.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of libstokes' lubrication correction for equal
 * spheres, F and FT versions, used by tests/ as the checker of the CUDA
 * lubrication kernel.  The product (libstokes_gb300) never links, loads or
 * calls this file.
 *
 * What it restates:
 *  - the exact two-sphere resistance functions X^A, Y^A, Y^B, X^C, Y^C of
 *    Jeffrey & Onishi, J. Fluid Mech. 139 (1984) 261-290: the coefficients
 *    f_k(lambda) come from their recurrences for the P, V, Q multipole
 *    coefficients (axisymmetric and asymmetric translation, axisymmetric and
 *    asymmetric rotation), evaluated here at lambda = 1 in long double;
 *  - the lubrication form of src/two-body-res.c:31 (scalar_two_body_res):
 *    each function is its near-contact singular part, written with
 *    s1 = 1 - 4/s^2, ln s1 and ln((s+2)/(s-2)) and the published
 *    lubrication constants at lambda = 1, plus a power series in 1/s^2 (odd
 *    functions: times 1/s) truncated where libstokes truncates it (1/s^50
 *    and 1/s^49).  The series coefficients are the coefficients of the exact
 *    far-field series minus those of the singular part, derived here;
 *  - the two-sphere far-field resistance (M^inf)^-1 of src/f.c:183 and
 *    src/ft.c:414: the inverse of the Rotne-Prager two-sphere mobility, in
 *    closed form;
 *  - the pair loop of src/lub.c:164-575 and the pair application of
 *    src/f.c:234 and src/ft.c:494: pairs j >= i, lattice images in the cube
 *    |n_x,y,z| <= lubmax / L + 1 (with its accumulating Lees-Edwards shift),
 *    the lubmax cut, the lubmin2 clamp, and the (res - minv) scalars applied
 *    to both particles.
 *
 * Its parity is pinned in tests/ against the reference library itself
 * (oracle/_ref) and against committed vectors (tests/golden/).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OL_NMAX 51          /* f_k up to k = 51 (series to 1/s^50 and 1/s^49) */
#define OL_NN (OL_NMAX + 2)
#define OL_NP (OL_NMAX + 1)
#define OL_IDX(n, p, q) (((size_t) (n) * OL_NP + (size_t) (p)) * OL_NP + (size_t) (q))

typedef long double LD;

static LD
ol_binom (int a, int b)
{
  if (b < 0 || b > a) return 0.0L;
  LD r = 1.0L;
  for (int k = 1; k <= b; k++) r = r * (LD) (a - b + k) / (LD) k;
  return r;
}

static LD
ol_get (const LD *T, int n, int p, int q)
{
  if (n < 1 || n >= OL_NN || p < 0 || q < 0 || p >= OL_NP || q >= OL_NP) return 0.0L;
  return T[OL_IDX (n, p, q)];
}

/* axisymmetric translation (X^A): P, V with P_100 = V_100 = 1 */
static void
ol_family_xa (LD *P, LD *V)
{
  P[OL_IDX (1, 0, 0)] = 1.0L;
  V[OL_IDX (1, 0, 0)] = 1.0L;
  for (int m = 1; m <= OL_NMAX; m++)
    for (int q = 0; q <= m; q++)
      {
        const int p = m - q;
        for (int n = 1; n < OL_NN; n++)
          {
            LD sp = 0.0L, sv = 0.0L;
            for (int s = 1; s <= q; s++)
              {
                const LD c = ol_binom (n + s, n);
                sp += c * ((LD) (n * (2 * n + 1) * (2 * n * s - n - s + 2))
                             / (LD) (2 * (n + 1) * (2 * s - 1) * (n + s))
                             * ol_get (P, s, q - s, p - n + 1)
                           - (LD) (n * (2 * n - 1)) / (LD) (2 * (n + 1))
                             * ol_get (P, s, q - s, p - n - 1)
                           - (LD) (n * (4 * n * n - 1)) / (LD) (2 * (n + 1) * (2 * s + 1))
                             * ol_get (V, s, q - s - 2, p - n + 1));
                sv += c * ol_get (P, s, q - s, p - n - 1);
              }
            P[OL_IDX (n, p, q)] = sp;
            V[OL_IDX (n, p, q)] = sp - (LD) (2 * n) / (LD) ((n + 1) * (2 * n + 3)) * sv;
          }
      }
}

/* asymmetric problems (Y^A, Y^B with P_100 = V_100 = 1; Y^C with Q_100 = 1) */
static void
ol_family_y (LD *P, LD *V, LD *Q, int rotation)
{
  if (rotation)
    Q[OL_IDX (1, 0, 0)] = 1.0L;
  else
    {
      P[OL_IDX (1, 0, 0)] = 1.0L;
      V[OL_IDX (1, 0, 0)] = 1.0L;
    }
  for (int m = 1; m <= OL_NMAX; m++)
    for (int q = 0; q <= m; q++)
      {
        const int p = m - q;
        for (int n = 1; n < OL_NN; n++)
          {
            LD sp = 0.0L, sq = 0.0L, sv = 0.0L, qq = 0.0L;
            for (int s = 1; s <= q; s++)
              {
                const LD c = ol_binom (n + s, n + 1);
                const LD w = (LD) (3 * (n + s) - (n * s + 1) * (2 * n * s - s - n + 2))
                             / (LD) (s * (n + s) * (2 * s - 1));
                sp += c * ((LD) (2 * n + 1) / (LD) (2 * (n + 1)) * w
                             * ol_get (P, s, q - s, p - n + 1)
                           + (LD) (n * (2 * n - 1)) / (LD) (2 * (n + 1))
                             * ol_get (P, s, q - s, p - n - 1)
                           + (LD) (n * (4 * n * n - 1)) / (LD) (2 * (n + 1) * (2 * s + 1))
                             * ol_get (V, s, q - s - 2, p - n + 1));
                sq += c * ol_get (Q, s, q - s - 1, p - n + 1);
                sv += c * ol_get (P, s, q - s, p - n - 1);
                qq += c * ((LD) s / (LD) (n + 1) * ol_get (Q, s, q - s - 1, p - n)
                           - (LD) 3 / (LD) (2 * n * s * (n + 1)) * ol_get (P, s, q - s, p - n));
              }
            const LD pv = sp - (LD) (2 * (4 * n * n - 1)) / (LD) (3 * (n + 1)) * sq;
            P[OL_IDX (n, p, q)] = pv;
            V[OL_IDX (n, p, q)] = pv + (LD) (2 * n) / (LD) ((n + 1) * (2 * n + 3)) * sv;
            Q[OL_IDX (n, p, q)] = qq;
          }
      }
}

/* axisymmetric rotation (X^C): Q only, Q_100 = 1 */
static void
ol_family_xc (LD *Q)
{
  Q[OL_IDX (1, 0, 0)] = 1.0L;
  for (int m = 1; m <= OL_NMAX; m++)
    for (int q = 0; q <= m; q++)
      {
        const int p = m - q;
        for (int n = 1; n < OL_NN; n++)
          {
            LD v = 0.0L;
            for (int s = 1; s <= q; s++)
              v += ol_binom (n + s, n + 1) * ol_get (Q, s, q - s - 1, p - n);
            Q[OL_IDX (n, p, q)] = v;
          }
      }
}

/* f_k(1) = 2^k sum_q T_{1, k-q, q} */
static void
ol_fk (const LD *T, LD scale, LD *f)
{
  for (int k = 0; k <= OL_NMAX; k++)
    {
      LD v = 0.0L;
      for (int q = 0; q <= k; q++) v += ol_get (T, 1, k - q, q);
      f[k] = scale * ldexpl (v, k);
    }
}

/* ---- lubrication forms ---------------------------------------------------
 * Ten functions, in the order of src/two-body-res.c's output:
 * x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c.  Each is
 *   S(s) + u^par sum_{m=0}^{M} c_m u^(2m),   u = 1/s,
 * with par 0 (M = 25) or 1 (M = 24).  Building blocks of S, as series in u:
 *   L1 = ln(1 - 4u^2), L2 = ln((1+2u)/(1-2u)), IS1 = 1/(1 - 4u^2),
 *   S1 = 1 - 4u^2 (multiplies L1 or L2), U = u. */
#define OL_J (OL_NMAX + 2)
enum { B_L1, B_L2, B_IS1, B_S1L1, B_S1L2, B_UIS1, B_UL1, B_UL2, B_U, B_ONE, B_N };

static void
ol_blocks (LD blk[B_N][OL_J])
{
  memset (blk, 0, sizeof (LD) * B_N * OL_J);
  for (int j = 0; j < OL_J; j++)
    {
      if (j % 2 == 0 && j >= 2) blk[B_L1][j] = -powl (4.0L, j / 2) / (LD) (j / 2);
      if (j % 2 == 1) blk[B_L2][j] = 2.0L * powl (2.0L, j) / (LD) j;
      if (j % 2 == 0) blk[B_IS1][j] = powl (4.0L, j / 2);
    }
  for (int j = 0; j < OL_J; j++)
    {
      blk[B_S1L1][j] = blk[B_L1][j] - (j >= 2 ? 4.0L * blk[B_L1][j - 2] : 0.0L);
      blk[B_S1L2][j] = blk[B_L2][j] - (j >= 2 ? 4.0L * blk[B_L2][j - 2] : 0.0L);
      if (j >= 1)
        {
          blk[B_UIS1][j] = blk[B_IS1][j - 1];
          blk[B_UL1][j] = blk[B_L1][j - 1];
          blk[B_UL2][j] = blk[B_L2][j - 1];
        }
    }
  blk[B_U][1] = 1.0L;
  blk[B_ONE][0] = 1.0L;
}

/* singular parts at lambda = 1: (block, coefficient) pairs */
typedef struct { int b; LD c; } OLTerm;
typedef struct { int par; int nt; OLTerm t[4]; LD esc; } OLForm;

static const OLForm ol_forms[10] = {
  /* x11a */ {0, 3, {{B_IS1, 1.0L / 4}, {B_L1, -9.0L / 40}, {B_S1L1, -3.0L / 112}}, 1.0L},
  /* x12a */ {1, 4, {{B_UIS1, -1.0L / 2}, {B_L2, -9.0L / 40}, {B_S1L2, -3.0L / 112},
                     {B_U, -12.0L / 112}}, -1.0L},
  /* y11a */ {0, 1, {{B_L1, -1.0L / 6}}, 1.0L},
  /* y12a */ {1, 1, {{B_L2, -1.0L / 6}}, -1.0L},
  /* y11b */ {1, 3, {{B_L2, -2.0L / 3 / 4}, {B_S1L2, -2.0L / 3 / 8}, {B_U, -2.0L / 3 / 2}},
              2.0L / 3},
  /* y12b */ {0, 2, {{B_L1, -2.0L / 3 / 4}, {B_S1L1, -2.0L / 3 / 8}}, -2.0L / 3},
  /* x11c */ {0, 3, {{B_L1, 4.0L / 3 / 4}, {B_UL2, 4.0L / 3 / 2}, {B_ONE, 4.0L / 3}}, 4.0L / 3},
  /* x12c */ {1, 3, {{B_L2, 4.0L / 3 / 4}, {B_UL1, 4.0L / 3 / 2}, {B_U, -4.0L / 3}}, -4.0L / 3},
  /* y11c */ {0, 3, {{B_L1, -4.0L / 3 / 5}, {B_S1L1, -4.0L / 3 * 47 / 250}, {B_ONE, 4.0L / 3}},
              4.0L / 3},
  /* y12c */ {1, 3, {{B_L2, 4.0L / 3 / 20}, {B_S1L2, 4.0L / 3 * 31 / 250},
                     {B_U, 4.0L / 3 * 62 / 125}}, 4.0L / 3},
};

static double ol_coef[10][26];
static int ol_ready = 0;

static void
ol_init (void)
{
  if (ol_ready) return;
  const size_t sz = (size_t) OL_NN * OL_NP * OL_NP;
  LD *P = calloc (sz, sizeof (LD)), *V = calloc (sz, sizeof (LD)), *Q = calloc (sz, sizeof (LD));
  LD fXA[OL_NMAX + 1], fYA[OL_NMAX + 1], fYB[OL_NMAX + 1], fXC[OL_NMAX + 1], fYC[OL_NMAX + 1];
  ol_family_xa (P, V);
  ol_fk (P, 1.0L, fXA);
  memset (P, 0, sz * sizeof (LD)); memset (V, 0, sz * sizeof (LD)); memset (Q, 0, sz * sizeof (LD));
  ol_family_y (P, V, Q, 0);
  ol_fk (P, 1.0L, fYA);
  ol_fk (Q, 2.0L, fYB);
  memset (P, 0, sz * sizeof (LD)); memset (V, 0, sz * sizeof (LD)); memset (Q, 0, sz * sizeof (LD));
  ol_family_y (P, V, Q, 1);
  ol_fk (Q, 1.0L, fYC);
  memset (Q, 0, sz * sizeof (LD));
  ol_family_xc (Q);
  ol_fk (Q, 1.0L, fXC);
  free (P); free (V); free (Q);
  const LD *fam[10] = {fXA, fXA, fYA, fYA, fYB, fYB, fXC, fXC, fYC, fYC};
  static LD blk[B_N][OL_J];
  ol_blocks (blk);
  for (int g = 0; g < 10; g++)
    {
      const OLForm *F = &ol_forms[g];
      const int M = F->par ? 24 : 25;
      for (int m = 0; m <= M; m++)
        {
          const int j = 2 * m + F->par;
          /* exact series: esc * f_j / 2^j u^j on the function's parity */
          LD v = F->esc * ldexpl (fam[g][j], -j);
          for (int t = 0; t < F->nt; t++) v -= F->t[t].c * blk[F->t[t].b][j];
          ol_coef[g][m] = (double) v;
        }
    }
  ol_ready = 1;
}

/* the series coefficients, out[10 * 26] */
void
oracle_lub_coef (double *out)
{
  ol_init ();
  memcpy (out, ol_coef, sizeof ol_coef);
}

/* res[10]: the lubrication-form resistance functions at distance s */
void
oracle_lub_res2b (double s, double *res)
{
  ol_init ();
  const double u = 1.0 / s, u2 = u * u, s1 = 1.0 - 4.0 * u2;
  const double l1 = log (s1), l2 = log ((s + 2.0) / (s - 2.0));
  const double bv[B_N] = {l1, l2, 1.0 / s1, s1 * l1, s1 * l2, u / s1, u * l1, u * l2, u, 1.0};
  for (int g = 0; g < 10; g++)
    {
      const OLForm *F = &ol_forms[g];
      double v = 0.0;
      for (int t = 0; t < F->nt; t++) v += (double) F->t[t].c * bv[F->t[t].b];
      const int M = F->par ? 24 : 25;
      double p = 0.0;
      for (int m = M; m >= 0; m--) p = p * u2 + ol_coef[g][m];
      res[g] = v + (F->par ? p * u : p);
    }
}

/* (M^inf)^-1 of two spheres: F (4 values) and FT (10 values), the inverse
 * of the Rotne-Prager two-sphere mobility at distance s */
void
oracle_lub_minv (int version, double s, double *r)
{
  const double s2 = s * s, s3 = s2 * s, s6 = s3 * s3;
  const double dx = (2.0 * s3 - 3.0 * s2 + 2.0) * (2.0 * s3 + 3.0 * s2 - 2.0);
  r[0] = 4.0 * s6 / dx;
  r[1] = -2.0 * s3 * (3.0 * s2 - 2.0) / dx;
  if (version == 0)
    {
      const double dy = 16.0 * s6 - (3.0 * s2 + 2.0) * (3.0 * s2 + 2.0);
      r[2] = 16.0 * s6 / dy;
      r[3] = -4.0 * s3 * (3.0 * s2 + 2.0) / dy;
      return;
    }
  const double s5 = s3 * s2;
  const double dy = (8.0 * s6 - 6.0 * s5 - 8.0 * s3 - 3.0 * s2 + 2.0)
                    * (8.0 * s6 + 6.0 * s5 + 8.0 * s3 - 3.0 * s2 + 2.0);
  r[2] = 16.0 * s6 * (s2 - 1.0) * (2.0 * s2 + 1.0) * (2.0 * s2 + 1.0) / dy;
  r[3] = -4.0 * s3 * (12.0 * s6 * s2 + 8.0 * s6 + 3.0 * s2 - 2.0) / dy;
  r[4] = -16.0 * s6 * s * (3.0 * s2 + 4.0) / dy;
  r[5] = 8.0 * s2 * s2 * (8.0 * s6 - 3.0 * s2 + 2.0) / dy;
  r[6] = 4.0 * s6 / (3.0 * (s6 - 1.0));
  r[7] = -4.0 * s3 / (3.0 * (s6 - 1.0));
  r[8] = 16.0 * s6 * (16.0 * s6 - 9.0 * s2 * s2 - 24.0 * s2 - 4.0) / (3.0 * dy);
  r[9] = 8.0 * s3 * (16.0 * s6 + 9.0 * s2 * s2 - 4.0) / (3.0 * dy);
}

/* y += block(e; x) for one particle pair: A = xa ee + ya (1 - ee) on the
 * force part; FT adds torque <- force b (F x e), force <- torque
 * sgn b (T x e) (sgn -1 for the self block of a pair, src/ft.c:305-343),
 * and C = xc ee + yc (1 - ee) on the torque part */
static void
ol_apply (int version, const double e[3], const double *sc, int self, const double *x,
          double *y)
{
  const double xa = sc[0], ya = sc[1];
  const double eF = e[0] * x[0] + e[1] * x[1] + e[2] * x[2];
  for (int d = 0; d < 3; d++) y[d] += ya * x[d] + (xa - ya) * eF * e[d];
  if (version == 0) return;
  const double yb = sc[2], xc = sc[3], yc = sc[4];
  const double *T = x + 3;
  const double eT = e[0] * T[0] + e[1] * T[1] + e[2] * T[2];
  const double Fxe[3] = {x[1] * e[2] - x[2] * e[1], x[2] * e[0] - x[0] * e[2],
                         x[0] * e[1] - x[1] * e[0]};
  const double Txe[3] = {T[1] * e[2] - T[2] * e[1], T[2] * e[0] - T[0] * e[2],
                         T[0] * e[1] - T[1] * e[0]};
  const double sg = self ? -1.0 : 1.0;
  for (int d = 0; d < 3; d++)
    {
      y[d] += sg * yb * Txe[d];
      y[3 + d] += yb * Fxe[d] + yc * T[d] + (xc - yc) * eT * e[d];
    }
}

/* one pair (1 at x1, 2 at x2) to both particles, src/f.c:234 / src/ft.c:494 */
static void
ol_pair (int version, double lubmin2, const double *x1, const double *x2, const double *u1,
         const double *u2, double *f1, double *f2)
{
  const double d[3] = {x2[0] - x1[0], x2[1] - x1[1], x2[2] - x1[2]};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (r2 < lubmin2) r2 = lubmin2;
  const double r = sqrt (r2);
  const double e[3] = {d[0] / r, d[1] / r, d[2] / r}, me[3] = {-e[0], -e[1], -e[2]};
  double res[10], inf[10];
  oracle_lub_res2b (r, res);
  oracle_lub_minv (version, r, inf);
  /* (xa, ya, yb, xc, yc) for the self (11) and cross (12) blocks */
  double s11[5], s12[5];
  s11[0] = res[0] - inf[0]; s12[0] = res[1] - inf[1];
  s11[1] = res[2] - inf[2]; s12[1] = res[3] - inf[3];
  if (version == 1)
    {
      s11[2] = res[4] - inf[4]; s12[2] = res[5] - inf[5];
      s11[3] = res[6] - inf[6]; s12[3] = res[7] - inf[7];
      s11[4] = res[8] - inf[8]; s12[4] = res[9] - inf[9];
    }
  ol_apply (version, e, s11, 1, u1, f1);
  ol_apply (version, e, s12, 0, u2, f1);
  ol_apply (version, me, s11, 1, u2, f2);
  ol_apply (version, me, s12, 0, u1, f2);
}

/* f = L u over all pairs, src/lub.c:164-575 (equal spheres, no slip) */
void
oracle_calc_lub (int version, int np, const double *pos, int periodic, double lx, double ly,
                 double lz, int shear_mode, double shear_shift, double lubmin2, double lubmax,
                 const double *u, double *f)
{
  const int c = version == 0 ? 3 : 6;
  memset (f, 0, sizeof (double) * (size_t) c * np);
  const double lubmax2 = lubmax * lubmax;
  int imx = 0, imy = 0, imz = 0;
  if (periodic)
    {
      double lm = lubmax;
      if (lubmax <= 0.0) lm = fmax (lx, fmax (ly, lz));
      imx = (int) (lm / lx) + 1;
      imy = (int) (lm / ly) + 1;
      imz = (int) (lm / lz) + 1;
    }
  for (int i = 0; i < np; i++)
    for (int j = i; j < np; j++)
      {
        const double *xi = pos + 3 * i;
        for (int ix = -imx; ix <= imx; ix++)
          {
            double t0 = pos[3 * j] + lx * ix;
            for (int iy = -imy; iy <= imy; iy++)
              {
                const double t1 = pos[3 * j + 1] + ly * iy;
                for (int iz = -imz; iz <= imz; iz++)
                  {
                    const double t2 = pos[3 * j + 2] + lz * iz;
                    /* the shift accumulates over the loop, as in the reference */
                    if (shear_mode == 1) t0 += iy * shear_shift;
                    else if (shear_mode == 2) t0 += iz * shear_shift;
                    const double xj[3] = {t0, t1, t2};
                    const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 != 0.0 && (lubmax2 <= 0.0 || r2 < lubmax2))
                      ol_pair (version, lubmin2, xi, xj, u + c * i, u + c * j, f + c * i,
                               f + c * j);
                  }
              }
            if (!periodic) break;
          }
      }
}
