/* oracle_lub.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of libstokes' lubrication correction for equal
 * spheres, F, FT and FTS versions, used by tests/ as the checker of the CUDA
 * lubrication kernel.  The product (libstokes_gb300) never links, loads or
 * calls this file.
 *
 * What it restates:
 *  - the exact two-sphere resistance functions X^A, Y^A, Y^B, X^C, Y^C of
 *    Jeffrey & Onishi, J. Fluid Mech. 139 (1984) 261-290, and X^G, Y^G,
 *    Y^H, X^M, Y^M, Z^M of Jeffrey, Phys. Fluids A 4 (1992) 16-29: the
 *    coefficients f_k(lambda) come from the recurrences for the P, V, Q
 *    multipole coefficients (azimuthal orders 0, 1, 2; translation,
 *    rotation and straining), evaluated here at lambda = 1 in long double;
 *  - the lubrication form of src/two-body-res.c:31 (scalar_two_body_res):
 *    each function is its near-contact singular part, written with
 *    s1 = 1 - 4/s^2, ln s1 and ln((s+2)/(s-2)) and the published
 *    lubrication constants at lambda = 1, plus a power series in 1/s^2 (odd
 *    functions: times 1/s) truncated where libstokes truncates it (1/s^50
 *    and 1/s^49).  The series coefficients are the coefficients of the exact
 *    far-field series minus those of the singular part, derived here;
 *  - the two-sphere far-field resistance (M^inf)^-1 of src/f.c:183,
 *    src/ft.c:414 and src/fts.c:1491: the inverse of the Rotne-Prager
 *    two-sphere mobility, in closed form;
 *  - the pair loop of src/lub.c:164-768 and the pair application of
 *    src/f.c:234, src/ft.c:494 and src/fts.c:1755: pairs j >= i, lattice
 *    images in the cube
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

#define OL_NMAX 51          /* f_k up to k = 51 (series to 1/s^50) */
#define OL_NN (OL_NMAX + 2)
#define OL_NP (OL_NMAX + 1)
#define OL_IDX(n, p, q) (((size_t) (n) * OL_NP + (size_t) (p)) * OL_NP + (size_t) (q))
#define OL_NF 22
#define OL_NC 26

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

/* The multipole recurrences of two spheres for azimuthal order m (0: the X
 * functions, 1: Y, 2: Z), started from a force-type (P_n0,0,0 = V_n0,0,0 =
 * 1) or a rotation-type (Q_n0,0,0 = 1) singularity on sphere 1; n0 = 1 for
 * the A, B, C, G, H problems, 2 for the straining (M) problems.  For m = 0
 * and 1 these are the recurrences of Jeffrey & Onishi (1984); one
 * expression in m covers both, and at m = 2 it gives the Z^M coefficients
 * of Jeffrey (1992). */
static void
ol_family (int m, int n0, int rotation, LD *P, LD *V, LD *Q)
{
  const size_t sz = (size_t) OL_NN * OL_NP * OL_NP;
  memset (P, 0, sz * sizeof (LD));
  memset (V, 0, sz * sizeof (LD));
  memset (Q, 0, sz * sizeof (LD));
  if (rotation)
    Q[OL_IDX (n0, 0, 0)] = 1.0L;
  else
    P[OL_IDX (n0, 0, 0)] = V[OL_IDX (n0, 0, 0)] = 1.0L;
  const LD sg = m == 0 ? 1.0L : -1.0L;   /* the sign convention of the m > 0 modes */
  for (int lv = 1; lv <= OL_NMAX; lv++)
    for (int q = 0; q <= lv; q++)
      {
        const int p = lv - q;
        for (int n = 1; n < OL_NN; n++)
          {
            LD sp = 0.0L, sq = 0.0L, sv = 0.0L, qq = 0.0L;
            for (int s = 1; s <= q; s++)
              {
                const LD c = ol_binom (n + s, n + m);
                if (c == 0.0L) continue;
                const int X = 2 * n * s - n - s + 2;
                const LD A = sg * (LD) (2 * n + 1) * (LD) (n * s * X + m * m * (X - 3 * (n + s)))
                             / (LD) (2 * (n + 1) * s * (n + s) * (2 * s - 1));
                sp += c * (A * ol_get (P, s, q - s, p - n + 1)
                           + sg * (-(LD) (n * (2 * n - 1)) / (LD) (2 * (n + 1))
                                     * ol_get (P, s, q - s, p - n - 1)
                                   - (LD) (n * (4 * n * n - 1)) / (LD) (2 * (n + 1) * (2 * s + 1))
                                     * ol_get (V, s, q - s - 2, p - n + 1)));
                sq += c * ol_get (Q, s, q - s - 1, p - n + 1);
                sv += c * ol_get (P, s, q - s, p - n - 1);
                qq += c * ((LD) s / (LD) (n + 1) * ol_get (Q, s, q - s - 1, p - n)
                           - (LD) (3 * m) / (LD) (2 * n * s * (n + 1)) * ol_get (P, s, q - s, p - n));
              }
            const LD pv = sp - (LD) (2 * m * (4 * n * n - 1)) / (LD) (3 * (n + 1)) * sq;
            P[OL_IDX (n, p, q)] = pv;
            V[OL_IDX (n, p, q)] = pv - sg * (LD) (2 * n) / (LD) ((n + 1) * (2 * n + 3)) * sv;
            Q[OL_IDX (n, p, q)] = qq;
          }
      }
}

/* f_k(1) = scale 2^k sum_q T_{n, k-q, q} */
static void
ol_fk (const LD *T, int n, LD scale, LD *f)
{
  for (int k = 0; k <= OL_NMAX; k++)
    {
      LD v = 0.0L;
      for (int q = 0; q <= k; q++) v += ol_get (T, n, k - q, q);
      f[k] = scale * ldexpl (v, k);
    }
}

/* ---- lubrication forms ---------------------------------------------------
 * Twenty-two functions, in the order of src/two-body-res.c's output:
 * x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c x11g x12g y11g y12g
 * y11h y12h x11m x12m y11m y12m z11m z12m.  Each is
 *   S(s) + u^par sum_{m=0}^{M} c_m u^(2m),   u = 1/s,
 * with M = 25 (even) or 24 (odd), where libstokes truncates.  Blocks of S,
 * as series in u: L1 = ln(1 - 4u^2), L2 = ln((1+2u)/(1-2u)),
 * IS1 = 1/(1 - 4u^2), S1 = 1 - 4u^2, s5 = s^2/4 - 1; S5L2M = s5 L2 - s
 * (whose 1/u terms cancel). */
#define OL_J (OL_NMAX + 3)
enum { B_L1, B_L2, B_IS1, B_S1L1, B_S1L2, B_UIS1, B_UL1, B_UL2, B_U, B_ONE, B_U2IS1, B_S5L1,
       B_S5L2M, B_N };

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
      if (j >= 2) blk[B_U2IS1][j] = blk[B_IS1][j - 2];
      if (j + 2 < OL_J)
        {
          blk[B_S5L1][j] = blk[B_L1][j + 2] / 4.0L - blk[B_L1][j];
          blk[B_S5L2M][j] = blk[B_L2][j + 2] / 4.0L - blk[B_L2][j];
        }
    }
  blk[B_U][1] = 1.0L;
  blk[B_ONE][0] = 1.0L;
}

/* singular parts at lambda = 1 (the published lubrication constants), the
 * scale and sign of the exact series (libstokes' SD form), its family */
enum { F_XA, F_YA, F_YB, F_XC, F_YC, F_XG, F_YG, F_YH, F_XM, F_YM, F_ZM, F_N };
typedef struct { int b; LD c; } OLTerm;
typedef struct { int par, M, nt; OLTerm t[4]; LD esc; int fam; } OLForm;

static const OLForm ol_forms[OL_NF] = {
  /* x11a */ {0, 25, 3, {{B_IS1, 1.0L / 4}, {B_L1, -9.0L / 40}, {B_S1L1, -3.0L / 112}}, 1.0L, F_XA},
  /* x12a */ {1, 24, 4, {{B_UIS1, -1.0L / 2}, {B_L2, -9.0L / 40}, {B_S1L2, -3.0L / 112},
                         {B_U, -12.0L / 112}}, -1.0L, F_XA},
  /* y11a */ {0, 25, 1, {{B_L1, -1.0L / 6}}, 1.0L, F_YA},
  /* y12a */ {1, 24, 1, {{B_L2, -1.0L / 6}}, -1.0L, F_YA},
  /* y11b */ {1, 24, 3, {{B_L2, -1.0L / 6}, {B_S1L2, -1.0L / 12}, {B_U, -1.0L / 3}}, 2.0L / 3, F_YB},
  /* y12b */ {0, 25, 2, {{B_L1, -1.0L / 6}, {B_S1L1, -1.0L / 12}}, -2.0L / 3, F_YB},
  /* x11c */ {0, 25, 3, {{B_L1, 1.0L / 3}, {B_UL2, 2.0L / 3}, {B_ONE, 4.0L / 3}}, 4.0L / 3, F_XC},
  /* x12c */ {1, 24, 3, {{B_L2, 1.0L / 3}, {B_UL1, 2.0L / 3}, {B_U, -4.0L / 3}}, -4.0L / 3, F_XC},
  /* y11c */ {0, 25, 3, {{B_L1, -4.0L / 15}, {B_S1L1, -4.0L * 47 / 750}, {B_ONE, 4.0L / 3}},
              4.0L / 3, F_YC},
  /* y12c */ {1, 24, 3, {{B_L2, 4.0L / 60}, {B_S1L2, 4.0L * 31 / 750}, {B_U, 4.0L * 62 / 375}},
              4.0L / 3, F_YC},
  /* x11g */ {1, 24, 3, {{B_UIS1, 1.0L / 2}, {B_L2, 9.0L / 40}, {B_S5L2M, 39.0L / 280}},
              2.0L / 3, F_XG},
  /* x12g */ {0, 25, 3, {{B_U2IS1, -1.0L}, {B_L1, 9.0L / 40}, {B_S5L1, 39.0L / 280}},
              -2.0L / 3, F_XG},
  /* y11g */ {1, 24, 2, {{B_L2, 1.0L / 12}, {B_S5L2M, 1.0L / 24}}, 2.0L / 3, F_YG},
  /* y12g */ {0, 25, 2, {{B_L1, 1.0L / 12}, {B_S5L1, 1.0L / 24}}, -2.0L / 3, F_YG},
  /* y11h */ {0, 25, 2, {{B_L1, -1.0L / 30}, {B_S5L1, -137.0L / 1500}}, 4.0L / 3, F_YH},
  /* y12h */ {1, 24, 2, {{B_L2, 2.0L / 15}, {B_S5L2M, 113.0L / 1500}}, 4.0L / 3, F_YH},
  /* x11m */ {0, 25, 3, {{B_U2IS1, 2.0L / 3}, {B_L1, -3.0L / 20}, {B_S5L1, -353.0L / 2520}},
              10.0L / 9, F_XM},
  /* x12m */ {1, 24, 3, {{B_UIS1, 1.0L / 3}, {B_L2, 3.0L / 20}, {B_S5L2M, 493.0L / 2520}},
              10.0L / 9, F_XM},
  /* y11m */ {0, 25, 2, {{B_L1, -2.0L / 15}, {B_S5L1, -19.0L / 750}}, 10.0L / 9, F_YM},
  /* y12m */ {1, 24, 2, {{B_L2, 1.0L / 30}, {B_S5L2M, 37.0L / 250}}, 10.0L / 9, F_YM},
  /* z11m */ {0, 25, 1, {{B_S5L1, 1.0L / 12}}, 10.0L / 9, F_ZM},
  /* z12m */ {1, 24, 1, {{B_S5L2M, 1.0L / 12}}, -10.0L / 9, F_ZM},
};

static double ol_coef[OL_NF][OL_NC];
static int ol_ready = 0;

static void
ol_init (void)
{
  if (ol_ready) return;
  const size_t sz = (size_t) OL_NN * OL_NP * OL_NP;
  LD *P = calloc (sz, sizeof (LD)), *V = calloc (sz, sizeof (LD)), *Q = calloc (sz, sizeof (LD));
  static LD f[F_N][OL_NMAX + 1];
  ol_family (0, 1, 0, P, V, Q);           /* X^A, X^G */
  ol_fk (P, 1, 1.0L, f[F_XA]);
  ol_fk (P, 2, 0.75L, f[F_XG]);
  ol_family (1, 1, 0, P, V, Q);           /* Y^A, Y^B, Y^G */
  ol_fk (P, 1, 1.0L, f[F_YA]);
  ol_fk (Q, 1, 2.0L, f[F_YB]);
  ol_fk (P, 2, 0.75L, f[F_YG]);
  ol_family (1, 1, 1, P, V, Q);           /* Y^C, Y^H */
  ol_fk (Q, 1, 1.0L, f[F_YC]);
  ol_fk (P, 2, -0.375L, f[F_YH]);
  ol_family (0, 1, 1, P, V, Q);           /* X^C */
  ol_fk (Q, 1, 1.0L, f[F_XC]);
  ol_family (0, 2, 0, P, V, Q);           /* X^M */
  ol_fk (P, 2, 1.0L, f[F_XM]);
  ol_family (1, 2, 0, P, V, Q);           /* Y^M */
  ol_fk (P, 2, 1.0L, f[F_YM]);
  ol_family (2, 2, 0, P, V, Q);           /* Z^M */
  ol_fk (P, 2, 1.0L, f[F_ZM]);
  free (P); free (V); free (Q);
  static LD blk[B_N][OL_J];
  ol_blocks (blk);
  for (int g = 0; g < OL_NF; g++)
    {
      const OLForm *F = &ol_forms[g];
      for (int m = 0; m <= F->M; m++)
        {
          const int j = 2 * m + F->par;
          /* exact series: esc * f_j / 2^j u^j on the function's parity */
          LD v = F->esc * ldexpl (f[F->fam][j], -j);
          for (int t = 0; t < F->nt; t++) v -= F->t[t].c * blk[F->t[t].b][j];
          ol_coef[g][m] = (double) v;
        }
      for (int m = F->M + 1; m < OL_NC; m++) ol_coef[g][m] = 0.0;
    }
  ol_ready = 1;
}

/* the series coefficients, out[22 * 26] */
void
oracle_lub_coef (double *out)
{
  ol_init ();
  memcpy (out, ol_coef, sizeof ol_coef);
}

/* res[22]: the lubrication-form resistance functions at distance s */
void
oracle_lub_res2b (double s, double *res)
{
  ol_init ();
  const double u = 1.0 / s, u2 = u * u, s1 = 1.0 - 4.0 * u2, s5 = 0.25 * s * s - 1.0;
  const double l1 = log (s1), l2 = log ((s + 2.0) / (s - 2.0));
  const double bv[B_N] = {l1,      l2,     1.0 / s1, s1 * l1, s1 * l2, u / s1, u * l1,
                          u * l2,  u,      1.0,      u2 / s1, s5 * l1, s5 * l2 - s};
  for (int g = 0; g < OL_NF; g++)
    {
      const OLForm *F = &ol_forms[g];
      double v = 0.0;
      for (int t = 0; t < F->nt; t++) v += (double) F->t[t].c * bv[F->t[t].b];
      double p = 0.0;
      for (int m = F->M; m >= 0; m--) p = p * u2 + ol_coef[g][m];
      res[g] = v + (F->par ? p * u : p);
    }
}

/* (M^inf)^-1 of two spheres: F (4 values) and FT (10 values), the inverse
 * of the Rotne-Prager two-sphere mobility at distance s */
/* FTS: the block form (the 22 scalars of the self and cross blocks) of the
 * inverse of the Rotne-Prager two-sphere mobility with stresslets, as
 * rational functions of s (derived with a computer-algebra inversion of the
 * two-sphere matrix at e = z, mode by mode) */
static void
ol_minv_fts (double s, double *r)
{
  double p[11];
  p[0] = 1.0;
  for (int k = 1; k <= 10; k++) p[k] = p[k - 1] * s;
  r[0] = (p[6]*(p[2]*(p[2]*(p[2]*(400.0*p[4] - 1500.0) - 5200.0) + 44160.0) - 57600.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(400.0*p[2] - 900.0) - 1800.0) - 800.0) + 45945.0) - 90600.0) + 55600.0) - 21120.0) + 2304.0);   /* xa11 */
  r[1] = (p[3]*(p[2]*(p[2]*(p[2]*(p[4]*(400.0 - 600.0*p[2]) + 7500.0) - 40000.0) + 57600.0) - 11520.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(400.0*p[2] - 900.0) - 1800.0) - 800.0) + 45945.0) - 90600.0) + 55600.0) - 21120.0) + 2304.0);   /* xa12 */
  r[2] = (p[6]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[4] - 1200.0) - 22400.0) + 58880.0) - 90400.0) + 11200.0) - 43520.0) + 25600.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[2] - 900.0) - 3600.0) - 22800.0) + 66360.0) - 112600.0) + 14880.0) - 16505.0) + 29624.0) + 2000.0) - 640.0) - 256.0);   /* ya11 */
  r[3] = (p[3]*(p[4]*(p[2]*(p[2]*(p[2]*(p[2]*(p[4]*(-1200.0*p[2] - 800.0) + 16200.0) - 46400.0) + 57600.0) - 4760.0) + 16000.0) - 2560.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[2] - 900.0) - 3600.0) - 22800.0) + 66360.0) - 112600.0) + 14880.0) - 16505.0) + 29624.0) + 2000.0) - 640.0) - 256.0);   /* ya12 */
  r[4] = (p[7]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(-1200.0*p[2] - 1600.0) - 6400.0) + 12000.0) - 15200.0) - 19840.0) + 30720.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[2] - 900.0) - 3600.0) - 22800.0) + 66360.0) - 112600.0) + 14880.0) - 16505.0) + 29624.0) + 2000.0) - 640.0) - 256.0);   /* yb11 */
  r[5] = (p[4]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[4] - 600.0) - 10800.0) + 49280.0) - 58700.0) + 14000.0) - 1600.0) - 2560.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0*p[2] - 900.0) - 3600.0) - 22800.0) + 66360.0) - 112600.0) + 14880.0) - 16505.0) + 29624.0) + 2000.0) - 640.0) - 256.0);   /* yb12 */
  r[6] = (4.0*p[6])
         / (3.0*p[6] - 3.0);   /* xc11 */
  r[7] = (-4.0*p[3])
         / (3.0*p[6] - 3.0);   /* xc12 */
  r[8] = (p[6]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(6400.0*p[2] - 3600.0) - 9600.0) - 65600.0) + 251040.0) - 504400.0) + 31360.0) + 125440.0) + 4096.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yc11 */
  r[9] = (p[3]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[4]*(3200.0*p[2] + 1800.0) - 42400.0) + 322020.0) - 267800.0) + 800.0) + 14720.0) + 2048.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yc12 */
  r[10] = (p[7]*(p[2]*(p[2]*(1500.0*p[2] + 1600.0) - 18400.0) + 19200.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(400.0*p[2] - 900.0) - 1800.0) - 800.0) + 45945.0) - 90600.0) + 55600.0) - 21120.0) + 2304.0);   /* xg11 */
  r[11] = (p[4]*(p[2]*(p[2]*(p[2]*(p[2]*(1600.0 - 1000.0*p[2]) - 3750.0) + 17000.0) - 20000.0) + 3840.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(400.0*p[2] - 900.0) - 1800.0) - 800.0) + 45945.0) - 90600.0) + 55600.0) - 21120.0) + 2304.0);   /* xg12 */
  r[12] = (p[7]*(p[2]*(p[2]*(p[2]*(p[2]*(10800.0*p[2] - 12800.0) + 37700.0) - 4800.0) + 32000.0) - 12800.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yg11 */
  r[13] = (p[4]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(-6400.0*p[2] - 4500.0) + 25800.0) - 52800.0) + 6130.0) - 9000.0) - 800.0) + 1280.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yg12 */
  r[14] = (p[8]*(p[2]*(p[2]*(p[2]*(77500.0 - 9600.0*p[2]) - 20400.0) - 24800.0) + 14720.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yh11 */
  r[15] = (p[5]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(8000.0*p[2] - 4500.0) - 7200.0) - 51600.0) + 68850.0) - 7500.0) - 1200.0) + 960.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(4800.0*p[2] - 2700.0) - 10800.0) - 68400.0) + 199080.0) - 337800.0) + 44640.0) - 49515.0) + 88872.0) + 6000.0) - 1920.0) - 768.0);   /* yh12 */
  r[16] = (p[8]*(p[2]*(p[2]*(p[2]*(4000.0*p[2] - 9000.0) - 3000.0) + 44000.0) - 38400.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(3600.0*p[2] - 8100.0) - 16200.0) - 7200.0) + 413505.0) - 815400.0) + 500400.0) - 190080.0) + 20736.0);   /* xm11 */
  r[17] = (p[5]*(p[2]*(p[2]*(p[2]*(20000.0*p[2] - 70500.0) + 81000.0) - 58400.0) + 9600.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(3600.0*p[2] - 8100.0) - 16200.0) - 7200.0) + 413505.0) - 815400.0) + 500400.0) - 190080.0) + 20736.0);   /* xm12 */
  r[18] = (p[8]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(16000.0*p[2] - 9000.0) - 36000.0) - 68000.0) - 15200.0) + 15000.0) - 41600.0) + 12800.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(14400.0*p[2] - 8100.0) - 32400.0) - 205200.0) + 597240.0) - 1013400.0) + 133920.0) - 148545.0) + 266616.0) + 18000.0) - 5760.0) - 2304.0);   /* ym11 */
  r[19] = (p[5]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(150500.0 - 40000.0*p[2]) + 18000.0) - 103600.0) - 27150.0) - 10500.0) - 400.0) + 1600.0))
         / (p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(p[2]*(14400.0*p[2] - 8100.0) - 32400.0) - 205200.0) + 597240.0) - 1013400.0) + 133920.0) - 148545.0) + 266616.0) + 18000.0) - 5760.0) - 2304.0);   /* ym12 */
  r[20] = (10.0*p[10])
         / (9.0*p[10] - 36.0);   /* zm11 */
  r[21] = (-20.0*p[5])
         / (9.0*p[10] - 36.0);   /* zm12 */
}

void
oracle_lub_minv (int version, double s, double *r)
{
  if (version == 2)
    {
      ol_minv_fts (s, r);
      return;
    }
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
/* the stresslet part of a block (FTS), the vector form of src/fts.c:626-1023
 * with the extracted 5-component stresslet: S' = (2 sxx + syy, 2 syy + sxx,
 * sxy, sxz, syz) and S'zz = 0; the self block of a pair flips the
 * force-from-stresslet coupling, as it flips the force-from-torque one */
static void
ol_apply_s (const double e[3], const double *sc, double sg, const double *x, double *y)
{
  const double xg = sc[5], yg = sc[6], yh = sc[7], xm = sc[8], ym = sc[9], zm = sc[10];
  const double *F = x, *T = x + 3;
  const double S[3][3] = {{2.0 * x[6] + x[10], x[7], x[8]},
                          {x[7], 2.0 * x[10] + x[6], x[9]},
                          {x[8], x[9], 0.0}};
  double Se[3];
  for (int a = 0; a < 3; a++) Se[a] = S[a][0] * e[0] + S[a][1] * e[1] + S[a][2] * e[2];
  const double eSe = e[0] * Se[0] + e[1] * Se[1] + e[2] * Se[2];
  const double trS = S[0][0] + S[1][1];
  const double eF = e[0] * F[0] + e[1] * F[1] + e[2] * F[2];
  const double Txe[3] = {T[1] * e[2] - T[2] * e[1], T[2] * e[0] - T[0] * e[2],
                         T[0] * e[1] - T[1] * e[0]};
  const double g1 = -xg / 3.0, g2 = yg, g3 = xg - 2.0 * yg;
  const double m1 = 1.5 * xm - 2.0 * ym + 0.5 * zm, m2 = -0.5 * xm + 0.5 * zm;
  const double m3 = xm / 6.0 - 0.5 * zm, m4x2 = ym - zm, m5x2 = zm;
  const double gu = g1 * trS + g3 * eSe;
  for (int d = 0; d < 3; d++) y[d] -= sg * (gu * e[d] + 2.0 * g2 * Se[d]);
  y[3] += 2.0 * yh * (e[1] * Se[2] - e[2] * Se[1]);
  y[4] += 2.0 * yh * (e[2] * Se[0] - e[0] * Se[2]);
  y[5] += 2.0 * yh * (e[0] * Se[1] - e[1] * Se[0]);
  const double dE = g1 * eF + m2 * eSe + m3 * trS, eeE = g3 * eF + m1 * eSe + m2 * trS;
  double V[3];
  for (int d = 0; d < 3; d++) V[d] = g2 * F[d] + yh * Txe[d] + m4x2 * Se[d];
  y[6] += dE + eeE * e[0] * e[0] + 2.0 * e[0] * V[0] + m5x2 * S[0][0];
  y[7] += eeE * e[0] * e[1] + e[0] * V[1] + e[1] * V[0] + m5x2 * S[0][1];
  y[8] += eeE * e[0] * e[2] + e[0] * V[2] + e[2] * V[0] + m5x2 * S[0][2];
  y[9] += eeE * e[1] * e[2] + e[1] * V[2] + e[2] * V[1] + m5x2 * S[1][2];
  y[10] += dE + eeE * e[1] * e[1] + 2.0 * e[1] * V[1] + m5x2 * S[1][1];
}

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
  if (version == 2) ol_apply_s (e, sc, sg, x, y);
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
  double res[22], inf[22];
  oracle_lub_res2b (r, res);
  oracle_lub_minv (version, r, inf);
  /* (xa, ya, yb, xc, yc) for the self (11) and cross (12) blocks */
  /* (xa, ya, yb, xc, yc, xg, yg, yh, xm, ym, zm) of the self (11) and cross
     (12) blocks: the 11 and 12 entries of each function alternate */
  double s11[11] = {0}, s12[11] = {0};
  const int nsc = version == 0 ? 2 : (version == 1 ? 5 : 11);
  for (int k = 0; k < nsc; k++)
    {
      s11[k] = res[2 * k] - inf[2 * k];
      s12[k] = res[2 * k + 1] - inf[2 * k + 1];
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
  const int c = version == 0 ? 3 : (version == 1 ? 6 : 11);
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
