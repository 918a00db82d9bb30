// lub.cu -- the lubrication correction f = L u for equal spheres, F, FT and
// FTS (the drop-in for src/lub.c:164-768; unequal or slip spheres are
// refused), in FP64 on the device.
//
// L is the sum over close pairs (r < lubmax, images in the cube |n| <=
// lubmax / L + 1) of the two-sphere resistance minus its far-field part,
// R2(r) - (M^inf)^-1(r) (src/f.c:234, src/ft.c:494).  R2 is the exact
// two-sphere resistance in libstokes' lubrication form
// (src/two-body-res.c:31): a near-contact singular part in s1 = 1 - 4/s^2,
// ln s1 and ln((s+2)/(s-2)) plus a power series in 1/s^2 truncated at
// 1/s^50.  The series coefficients are generated here, at start-up, from
// the Jeffrey & Onishi (1984) and Jeffrey (1992) recurrences for the
// multipole coefficients of two spheres (translation, rotation and
// straining, azimuthal orders 0, 1, 2) and the expansion of the singular
// part; (M^inf)^-1 is the closed-form inverse of the Rotne-Prager
// two-sphere mobility.
//
// Each target i is one warp: the lanes take the sources j, reject those
// whose minimum image is beyond lubmax (unsheared boxes), walk the image
// cube of the others in the reference's order (its Lees-Edwards shift
// accumulates along the loop, so the image set of a pair is taken from the
// pair's lower index, as the reference's j >= i loop takes it), and sum
// their blocks; a particle and its own image give both halves of the pair
// to the same particle, as in the reference.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "engine.h"
#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "stokes_abi.h"
#include "stokes_gpu.h"
#include "stokes_lub.h"

namespace lsg {

// ---- series coefficients ---------------------------------------------------
namespace {

constexpr int JO_K = 51;                 // f_k up to k = 51
constexpr int LUB_NF = 22;   // x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c x11g x12g
                             // y11g y12g y11h y12h x11m x12m y11m y12m z11m z12m
constexpr int LUB_NC = 26;

// the multipole coefficients P, V, Q of one problem, n in [1, K + 1],
// p + q <= K
struct JO {
  std::vector<double> P, V, Q;
  static size_t at (int n, int p, int q) { return ((size_t) n * (JO_K + 1) + p) * (JO_K + 1) + q; }
  JO () : P (at (JO_K + 2, 0, 0), 0.0), V (P), Q (P) {}
  static double get (const std::vector<double> &T, int n, int p, int q)
  {
    if (n < 1 || n > JO_K + 1 || p < 0 || q < 0 || p > JO_K || q > JO_K) return 0.0;
    return T[at (n, p, q)];
  }
  // f_k(1) = scale 2^k sum_q T_n,(k-q),q
  void fk (const std::vector<double> &T, int n, double scale, double *f) const
  {
    for (int k = 0; k <= JO_K; k++)
      {
        double v = 0.0;
        for (int q = 0; q <= k; q++) v += get (T, n, k - q, q);
        f[k] = scale * std::ldexp (v, k);
      }
  }
};

double
binom (int a, int b)
{
  if (b < 0 || b > a) return 0.0;
  double r = 1.0;
  for (int k = 1; k <= b; k++) r = r * (a - b + k) / k;
  return r;
}

// the recurrence of azimuthal order m (0: X, 1: Y, 2: Z functions) started
// from a force-type (P = V = 1 at n0) or rotation-type (Q = 1 at n0)
// singularity: Jeffrey & Onishi (1984) for m = 0, 1 written as one
// expression in m, which at m = 2 gives Jeffrey's (1992) Z^M coefficients
void
jo_family (JO &J, int m, int n0, bool rotation)
{
  std::fill (J.P.begin (), J.P.end (), 0.0);
  std::fill (J.V.begin (), J.V.end (), 0.0);
  std::fill (J.Q.begin (), J.Q.end (), 0.0);
  if (rotation) J.Q[JO::at (n0, 0, 0)] = 1.0;
  else J.P[JO::at (n0, 0, 0)] = J.V[JO::at (n0, 0, 0)] = 1.0;
  const double sg = m == 0 ? 1.0 : -1.0;
  for (int lv = 1; lv <= JO_K; lv++)
    for (int q = 0; q <= lv; q++)
      for (int n = 1; n <= JO_K + 1; n++)
        {
          const int p = lv - q;
          double a = 0.0, bq = 0.0, bv = 0.0, qq = 0.0;
          for (int s = 1; s <= q; s++)
            {
              const double c = binom (n + s, n + m);
              if (c == 0.0) continue;
              const double X = 2.0 * n * s - n - s + 2;
              const double A = sg * (2.0 * n + 1) * (n * s * X + m * m * (X - 3.0 * (n + s)))
                               / (2.0 * (n + 1) * s * (n + s) * (2 * s - 1));
              a += c * (A * JO::get (J.P, s, q - s, p - n + 1)
                        + sg * (-(double) n * (2 * n - 1) / (2.0 * (n + 1))
                                  * JO::get (J.P, s, q - s, p - n - 1)
                                - (double) n * (4 * n * n - 1) / (2.0 * (n + 1) * (2 * s + 1))
                                  * JO::get (J.V, s, q - s - 2, p - n + 1)));
              bq += c * JO::get (J.Q, s, q - s - 1, p - n + 1);
              bv += c * JO::get (J.P, s, q - s, p - n - 1);
              qq += c * ((double) s / (n + 1) * JO::get (J.Q, s, q - s - 1, p - n)
                         - 3.0 * m / (2.0 * n * s * (n + 1)) * JO::get (J.P, s, q - s, p - n));
            }
          const double pv = a - 2.0 * m * (4.0 * n * n - 1) / (3.0 * (n + 1)) * bq;
          J.P[JO::at (n, p, q)] = pv;
          J.V[JO::at (n, p, q)] = pv - sg * 2.0 * n / ((n + 1.0) * (2 * n + 3)) * bv;
          J.Q[JO::at (n, p, q)] = qq;
        }
}

// singular-part building blocks as series in u = 1/s; s5 = s^2/4 - 1 and
// S5L2M = s5 L2 - s (its 1/u terms cancel)
enum { SB_L1, SB_L2, SB_IS1, SB_S1L1, SB_S1L2, SB_UIS1, SB_UL1, SB_UL2, SB_U, SB_ONE, SB_U2IS1,
       SB_S5L1, SB_S5L2M, SB_N };
enum { FA_XA, FA_YA, FA_YB, FA_XC, FA_YC, FA_XG, FA_YG, FA_YH, FA_XM, FA_YM, FA_ZM, FA_N };
struct Term { int b; double c; };
struct Form { int par, M, nt; Term t[4]; double esc; int fam; };

// libstokes' lubrication forms at lambda = 1: parity, truncation, singular
// part (the published lubrication constants), the factor of the exact series
// (the SD scaling and sign of each function) and its family
const Form kForms[LUB_NF] = {
  {0, 25, 3, {{SB_IS1, 0.25}, {SB_L1, -0.225}, {SB_S1L1, -3.0 / 112}}, 1.0, FA_XA},
  {1, 24, 4, {{SB_UIS1, -0.5}, {SB_L2, -0.225}, {SB_S1L2, -3.0 / 112}, {SB_U, -12.0 / 112}}, -1.0, FA_XA},
  {0, 25, 1, {{SB_L1, -1.0 / 6}}, 1.0, FA_YA},
  {1, 24, 1, {{SB_L2, -1.0 / 6}}, -1.0, FA_YA},
  {1, 24, 3, {{SB_L2, -2.0 / 12}, {SB_S1L2, -2.0 / 24}, {SB_U, -2.0 / 6}}, 2.0 / 3, FA_YB},
  {0, 25, 2, {{SB_L1, -2.0 / 12}, {SB_S1L1, -2.0 / 24}}, -2.0 / 3, FA_YB},
  {0, 25, 3, {{SB_L1, 4.0 / 12}, {SB_UL2, 4.0 / 6}, {SB_ONE, 4.0 / 3}}, 4.0 / 3, FA_XC},
  {1, 24, 3, {{SB_L2, 4.0 / 12}, {SB_UL1, 4.0 / 6}, {SB_U, -4.0 / 3}}, -4.0 / 3, FA_XC},
  {0, 25, 3, {{SB_L1, -4.0 / 15}, {SB_S1L1, -4.0 * 47 / 750}, {SB_ONE, 4.0 / 3}}, 4.0 / 3, FA_YC},
  {1, 24, 3, {{SB_L2, 4.0 / 60}, {SB_S1L2, 4.0 * 31 / 750}, {SB_U, 4.0 * 62 / 375}}, 4.0 / 3, FA_YC},
  {1, 24, 3, {{SB_UIS1, 0.5}, {SB_L2, 0.225}, {SB_S5L2M, 39.0 / 280}}, 2.0 / 3, FA_XG},
  {0, 25, 3, {{SB_U2IS1, -1.0}, {SB_L1, 0.225}, {SB_S5L1, 39.0 / 280}}, -2.0 / 3, FA_XG},
  {1, 24, 2, {{SB_L2, 1.0 / 12}, {SB_S5L2M, 1.0 / 24}}, 2.0 / 3, FA_YG},
  {0, 25, 2, {{SB_L1, 1.0 / 12}, {SB_S5L1, 1.0 / 24}}, -2.0 / 3, FA_YG},
  {0, 25, 2, {{SB_L1, -1.0 / 30}, {SB_S5L1, -137.0 / 1500}}, 4.0 / 3, FA_YH},
  {1, 24, 2, {{SB_L2, 2.0 / 15}, {SB_S5L2M, 113.0 / 1500}}, 4.0 / 3, FA_YH},
  {0, 25, 3, {{SB_U2IS1, 2.0 / 3}, {SB_L1, -0.15}, {SB_S5L1, -353.0 / 2520}}, 10.0 / 9, FA_XM},
  {1, 24, 3, {{SB_UIS1, 1.0 / 3}, {SB_L2, 0.15}, {SB_S5L2M, 493.0 / 2520}}, 10.0 / 9, FA_XM},
  {0, 25, 2, {{SB_L1, -2.0 / 15}, {SB_S5L1, -19.0 / 750}}, 10.0 / 9, FA_YM},
  {1, 24, 2, {{SB_L2, 1.0 / 30}, {SB_S5L2M, 37.0 / 250}}, 10.0 / 9, FA_YM},
  {0, 25, 1, {{SB_S5L1, 1.0 / 12}}, 10.0 / 9, FA_ZM},
  {1, 24, 1, {{SB_S5L2M, 1.0 / 12}}, -10.0 / 9, FA_ZM},
};

struct LubCoef { double c[LUB_NF][LUB_NC]; };

LubCoef
make_coefficients ()
{
  static double f[FA_N][JO_K + 1];
  JO J;
  jo_family (J, 0, 1, false);           // X^A, X^G (the n = 2 coefficients)
  J.fk (J.P, 1, 1.0, f[FA_XA]);
  J.fk (J.P, 2, 0.75, f[FA_XG]);
  jo_family (J, 1, 1, false);           // Y^A, Y^B, Y^G
  J.fk (J.P, 1, 1.0, f[FA_YA]);
  J.fk (J.Q, 1, 2.0, f[FA_YB]);
  J.fk (J.P, 2, 0.75, f[FA_YG]);
  jo_family (J, 1, 1, true);            // Y^C, Y^H
  J.fk (J.Q, 1, 1.0, f[FA_YC]);
  J.fk (J.P, 2, -0.375, f[FA_YH]);
  jo_family (J, 0, 1, true);            // X^C
  J.fk (J.Q, 1, 1.0, f[FA_XC]);
  jo_family (J, 0, 2, false);           // X^M
  J.fk (J.P, 2, 1.0, f[FA_XM]);
  jo_family (J, 1, 2, false);           // Y^M
  J.fk (J.P, 2, 1.0, f[FA_YM]);
  jo_family (J, 2, 2, false);           // Z^M
  J.fk (J.P, 2, 1.0, f[FA_ZM]);
  constexpr int NJ = JO_K + 3;
  static double blk[SB_N][NJ];
  memset (blk, 0, sizeof blk);
  for (int j = 0; j < NJ; j++)
    {
      if (j % 2 == 0 && j >= 2) blk[SB_L1][j] = -std::pow (4.0, j / 2) / (j / 2);
      if (j % 2 == 1) blk[SB_L2][j] = 2.0 * std::ldexp (1.0, j) / j;
      if (j % 2 == 0) blk[SB_IS1][j] = std::pow (4.0, j / 2);
    }
  for (int j = 0; j < NJ; j++)
    {
      blk[SB_S1L1][j] = blk[SB_L1][j] - (j >= 2 ? 4.0 * blk[SB_L1][j - 2] : 0.0);
      blk[SB_S1L2][j] = blk[SB_L2][j] - (j >= 2 ? 4.0 * blk[SB_L2][j - 2] : 0.0);
      if (j >= 1)
        {
          blk[SB_UIS1][j] = blk[SB_IS1][j - 1];
          blk[SB_UL1][j] = blk[SB_L1][j - 1];
          blk[SB_UL2][j] = blk[SB_L2][j - 1];
        }
      if (j >= 2) blk[SB_U2IS1][j] = blk[SB_IS1][j - 2];
      if (j + 2 < NJ)
        {
          blk[SB_S5L1][j] = blk[SB_L1][j + 2] / 4.0 - blk[SB_L1][j];
          blk[SB_S5L2M][j] = blk[SB_L2][j + 2] / 4.0 - blk[SB_L2][j];
        }
    }
  blk[SB_U][1] = 1.0;
  blk[SB_ONE][0] = 1.0;
  LubCoef C;
  memset (&C, 0, sizeof C);
  for (int g = 0; g < LUB_NF; g++)
    {
      const Form &F = kForms[g];
      for (int m = 0; m <= F.M; m++)
        {
          const int j = 2 * m + F.par;
          double v = F.esc * std::ldexp (f[F.fam][j], -j);
          for (int t = 0; t < F.nt; t++) v -= F.t[t].c * blk[F.t[t].b][j];
          C.c[g][m] = v;
        }
    }
  return C;
}

}  // namespace

__constant__ double c_lub[LUB_NF][LUB_NC];
__constant__ Form c_forms[LUB_NF];

// ---- device side -------------------------------------------------------------
struct LubArgs {
  const double *pos, *u;
  double *f;
  int np, periodic;
  double lx, ly, lz;
  int imx, imy, imz;
  int shear_mode;
  double shift;
  double lubmin2, lubmax2;
};

// the ten lubrication-form functions at distance s (first nf of them)
__device__ __forceinline__ void
lub_res (double s, int nf, double *res)
{
  const double u = 1.0 / s, u2 = u * u, s1 = 1.0 - 4.0 * u2, s5 = 0.25 * s * s - 1.0;
  const double l1 = log (s1), l2 = log ((s + 2.0) / (s - 2.0));
  const double bv[SB_N] = {l1,     l2, 1.0 / s1, s1 * l1,  s1 * l2, u / s1,      u * l1,
                           u * l2, u,  1.0,      u2 / s1,  s5 * l1, s5 * l2 - s};
  for (int g = 0; g < nf; g++)
    {
      const Form &F = c_forms[g];
      double v = 0.0;
      for (int t = 0; t < F.nt; t++) v += F.t[t].c * bv[F.t[t].b];
      double p = 0.0;
      for (int m = F.M; m >= 0; m--) p = fma (p, u2, c_lub[g][m]);
      res[g] = v + (F.par ? p * u : p);
    }
}

// (M^inf)^-1 of two spheres, F (4 values) or FT (10 values)
// FTS: the block form of the inverse of the Rotne-Prager two-sphere mobility
// with stresslets, as rational functions of s (a computer-algebra inversion
// of the two-sphere matrix at e = z, mode by mode)
__device__ __noinline__ void
lub_minv_fts (double s, double *r)
{
  double p[11];
  p[0] = 1.0;
#pragma unroll
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

template <int V>
__device__ __forceinline__ void
lub_minv (double s, double *r)
{
  if (V == 2)
    {
      lub_minv_fts (s, r);
      return;
    }
  const double s2 = s * s, s3 = s2 * s, s6 = s3 * s3;
  const double dx = (2.0 * s3 - 3.0 * s2 + 2.0) * (2.0 * s3 + 3.0 * s2 - 2.0);
  r[0] = 4.0 * s6 / dx;
  r[1] = -2.0 * s3 * (3.0 * s2 - 2.0) / dx;
  if (V == 0)
    {
      const double b = 3.0 * s2 + 2.0, dy = 16.0 * s6 - b * b;
      r[2] = 16.0 * s6 / dy;
      r[3] = -4.0 * s3 * b / dy;
      return;
    }
  const double s5 = s3 * s2;
  const double dy = (8.0 * s6 - 6.0 * s5 - 8.0 * s3 - 3.0 * s2 + 2.0)
                    * (8.0 * s6 + 6.0 * s5 + 8.0 * s3 - 3.0 * s2 + 2.0);
  const double q = 2.0 * s2 + 1.0;
  r[2] = 16.0 * s6 * (s2 - 1.0) * q * q / dy;
  r[3] = -4.0 * s3 * ((12.0 * s2 + 8.0) * s6 + 3.0 * s2 - 2.0) / dy;
  r[4] = -16.0 * s6 * s * (3.0 * s2 + 4.0) / dy;
  r[5] = 8.0 * s2 * s2 * (8.0 * s6 - 3.0 * s2 + 2.0) / dy;
  r[6] = 4.0 * s6 / (3.0 * (s6 - 1.0));
  r[7] = -4.0 * s3 / (3.0 * (s6 - 1.0));
  r[8] = 16.0 * s6 * (16.0 * s6 - 9.0 * s2 * s2 - 24.0 * s2 - 4.0) / (3.0 * dy);
  r[9] = 8.0 * s3 * (16.0 * s6 + 9.0 * s2 * s2 - 4.0) / (3.0 * dy);
}

// y += w * block(e) x; sc = (xa, ya[, yb, xc, yc]); the self block of a pair
// takes the force-from-torque coupling with the opposite sign
template <int V>
__device__ __forceinline__ void
lub_apply (const double e[3], const double *sc, bool self, double w, const double *x, double *y)
{
  const double xa = w * sc[0], ya = w * sc[1];
  const double eF = e[0] * x[0] + e[1] * x[1] + e[2] * x[2];
#pragma unroll
  for (int d = 0; d < 3; d++) y[d] += ya * x[d] + (xa - ya) * eF * e[d];
  if (V == 0) return;
  const double yb = w * sc[2], xc = w * sc[3], yc = w * sc[4];
  const double *T = x + 3;
  const double eT = e[0] * T[0] + e[1] * T[1] + e[2] * T[2];
  const double Fxe[3] = {x[1] * e[2] - x[2] * e[1], x[2] * e[0] - x[0] * e[2],
                         x[0] * e[1] - x[1] * e[0]};
  const double Txe[3] = {T[1] * e[2] - T[2] * e[1], T[2] * e[0] - T[0] * e[2],
                         T[0] * e[1] - T[1] * e[0]};
  const double sg = self ? -yb : yb;
#pragma unroll
  for (int d = 0; d < 3; d++)
    {
      y[d] += sg * Txe[d];
      y[3 + d] += yb * Fxe[d] + yc * T[d] + (xc - yc) * eT * e[d];
    }
  if (V < 2) return;
  // the stresslet couplings (src/fts.c:626-1023 in vector form, the
  // extracted stresslet as S' = (2 sxx + syy, 2 syy + sxx, sxy, sxz, syz),
  // S'zz = 0); the self block flips the force-from-stresslet coupling
  const double xg = w * sc[5], yg = w * sc[6], yh = w * sc[7];
  const double xm = w * sc[8], ym = w * sc[9], zm = w * sc[10];
  const double S00 = 2.0 * x[6] + x[10], S11 = 2.0 * x[10] + x[6], S01 = x[7], S02 = x[8],
               S12 = x[9];
  const double Se[3] = {S00 * e[0] + S01 * e[1] + S02 * e[2], S01 * e[0] + S11 * e[1] + S12 * e[2],
                        S02 * e[0] + S12 * e[1]};
  const double eSe = e[0] * Se[0] + e[1] * Se[1] + e[2] * Se[2], trS = S00 + S11;
  const double g1 = -xg / 3.0, g2 = yg, g3 = xg - 2.0 * yg;
  const double m1 = 1.5 * xm - 2.0 * ym + 0.5 * zm, m2 = 0.5 * (zm - xm);
  const double m3 = xm / 6.0 - 0.5 * zm, m4x2 = ym - zm, m5x2 = zm;
  const double gu = g1 * trS + g3 * eSe, sgg = self ? -1.0 : 1.0;
#pragma unroll
  for (int d = 0; d < 3; d++) y[d] -= sgg * (gu * e[d] + 2.0 * g2 * Se[d]);
  y[3] += 2.0 * yh * (e[1] * Se[2] - e[2] * Se[1]);
  y[4] += 2.0 * yh * (e[2] * Se[0] - e[0] * Se[2]);
  y[5] += 2.0 * yh * (e[0] * Se[1] - e[1] * Se[0]);
  const double dE = g1 * eF + m2 * eSe + m3 * trS, eeE = g3 * eF + m1 * eSe + m2 * trS;
  double Vv[3];
#pragma unroll
  for (int d = 0; d < 3; d++) Vv[d] = g2 * x[d] + yh * Txe[d] + m4x2 * Se[d];
  y[6] += dE + eeE * e[0] * e[0] + 2.0 * e[0] * Vv[0] + m5x2 * S00;
  y[7] += eeE * e[0] * e[1] + e[0] * Vv[1] + e[1] * Vv[0] + m5x2 * S01;
  y[8] += eeE * e[0] * e[2] + e[0] * Vv[2] + e[2] * Vv[0] + m5x2 * S02;
  y[9] += eeE * e[1] * e[2] + e[1] * Vv[2] + e[2] * Vv[1] + m5x2 * S12;
  y[10] += dE + eeE * e[1] * e[1] + 2.0 * e[1] * Vv[1] + m5x2 * S11;
}

// one pair image (separation d, source velocity uj) into the target's sums;
// self: the particle's own image (both halves of the pair)
// the unit separation e and the scalars (xa, ya[, yb, xc, yc[, xg, yg, yh,
// xm, ym, zm]]) of the self (11) and cross (12) blocks of one pair image:
// lubrication form minus far-field part, r clamped at sqrt(lubmin2)
template <int V>
__device__ __forceinline__ void
lub_scalars (const LubArgs &a, const double d[3], double e[3], double *s11, double *s12)
{
  constexpr int NF = V == 0 ? 4 : (V == 1 ? 10 : 22);
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (r2 < a.lubmin2) r2 = a.lubmin2;
  const double r = sqrt (r2), ri = 1.0 / r;
  e[0] = d[0] * ri;
  e[1] = d[1] * ri;
  e[2] = d[2] * ri;
  double res[NF], inf[NF];
  lub_res (r, NF, res);
  lub_minv<V> (r, inf);
  // the 11 and 12 entries of each function alternate
#pragma unroll
  for (int k = 0; k < NF / 2; k++)
    {
      s11[k] = res[2 * k] - inf[2 * k];
      s12[k] = res[2 * k + 1] - inf[2 * k + 1];
    }
}

template <int V>
__device__ __forceinline__ void
lub_pair (const LubArgs &a, const double d[3], const double *ui, const double *uj, bool self,
          double *acc)
{
  constexpr int NF = V == 0 ? 4 : (V == 1 ? 10 : 22);
  double e[3], s11[NF / 2], s12[NF / 2];
  lub_scalars<V> (a, d, e, s11, s12);
  lub_apply<V> (e, s11, true, 1.0, ui, acc);
  lub_apply<V> (e, s12, false, 1.0, uj, acc);
  if (self)
    {
      const double me[3] = {-e[0], -e[1], -e[2]};
      lub_apply<V> (me, s11, true, 1.0, ui, acc);
      lub_apply<V> (me, s12, false, 1.0, ui, acc);
    }
}

constexpr int LUB_QCAP = 64;

// every pair image of (i, j) within lubmax that the reference visits, as
// separation d = x_j(image) - x_i: fn (d).  single: the unsheared periodic
// box with lubmax below half the box, where only the minimum image can be
// within lubmax (taken if the reference's cube holds it).  Otherwise the
// reference's cube: it visits the pair once, from its lower index, with the
// image offsets o(n) of its loop (which need not be symmetric under a shift
// that accumulates): d = x_j + o - x_i for j > i, the negated separation
// x_j - o - x_i for j < i, and both signs for j == i (the caller's fn
// handles the j == i pair as both halves)
template <class Fn>
__device__ __forceinline__ void
lub_images (const LubArgs &a, int i, int j, const double xi[3], bool single, Fn &&fn)
{
  const double r0[3] = {a.pos[3 * j] - xi[0], a.pos[3 * j + 1] - xi[1], a.pos[3 * j + 2] - xi[2]};
  if (single)
    {
      const double n0 = -rint (r0[0] / a.lx), n1 = -rint (r0[1] / a.ly), n2 = -rint (r0[2] / a.lz);
      if (fabs (n0) > a.imx || fabs (n1) > a.imy || fabs (n2) > a.imz) return;
      const double d[3] = {r0[0] + n0 * a.lx, r0[1] + n1 * a.ly, r0[2] + n2 * a.lz};
      const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (r2 == 0.0 || !(r2 < a.lubmax2)) return;
      fn (d);
      return;
    }
  const double sg = (j >= i) ? 1.0 : -1.0;
  for (int ix = -a.imx; ix <= a.imx; ix++)
    {
      double ox = a.lx * ix;
      for (int iy = -a.imy; iy <= a.imy; iy++)
        {
          const double oy = a.ly * iy;
          for (int iz = -a.imz; iz <= a.imz; iz++)
            {
              const double oz = a.lz * iz;
              if (a.shear_mode == 1) ox += iy * a.shift;
              else if (a.shear_mode == 2) ox += iz * a.shift;
              const double d[3] = {r0[0] + sg * ox, r0[1] + sg * oy, r0[2] + sg * oz};
              const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
              if (r2 == 0.0 || (a.lubmax2 > 0.0 && !(r2 < a.lubmax2))) continue;
              fn (d);
            }
        }
    }
}

// the candidate scan of a warp over the sources: the lanes test the
// sources in FP32 (minimum-image distance within lubmax, with a margin for
// the rounding; every source when there is no such test) and queue them in
// q; each full batch of 32 and the remainder go to batch (q, count)
template <class Batch>
__device__ __forceinline__ void
lub_scan (const LubArgs &a, const double xi[3], bool test, int *q, Batch &&batch)
{
  const int lane = threadIdx.x & 31;
  const float cut2 = (float) a.lubmax2 * 1.0001f + 1e-6f;
  const float lxf = (float) a.lx, lyf = (float) a.ly, lzf = (float) a.lz;
  const float ilxf = 1.0f / lxf, ilyf = 1.0f / lyf, ilzf = 1.0f / lzf;
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  for (int jb = 0; jb < a.np; jb += 32)
    {
      const int j = jb + lane;
      bool cand = j < a.np;
      if (cand && test)
        {
          float dx = (float) (a.pos[3 * j] - xi[0]), dy = (float) (a.pos[3 * j + 1] - xi[1]),
                dz = (float) (a.pos[3 * j + 2] - xi[2]);
          if (a.periodic)
            {
              dx -= lxf * rintf (dx * ilxf);
              dy -= lyf * rintf (dy * ilyf);
              dz -= lzf * rintf (dz * ilzf);
            }
          cand = dx * dx + dy * dy + dz * dz < cut2;
        }
      const unsigned b = __ballot_sync (0xffffffffu, cand);
      if (cand) q[qn + __popc (b & lt)] = j;
      qn += __popc (b);
      __syncwarp ();
      if (qn >= 32)
        {
          batch (q + qn - 32, 32);
          qn -= 32;
          __syncwarp ();
        }
    }
  if (qn > 0) batch (q, qn);
  __syncwarp ();
}

// A warp per target i.  The lanes scan the sources in FP32 (the FP64 pipe of
// this GPU is 1/64 of FP32) and queue the candidates; 32 queued candidates
// are then evaluated in FP64 at once, one per lane.  With a periodic,
// unsheared box and lubmax below half the box, a pair has at most one image
// within lubmax: the candidate test is its minimum image (with a margin for
// the FP32 rounding) and the evaluation takes that image alone, if the
// reference's image cube holds it.  Otherwise every source is a candidate
// (or those whose minimum image is within lubmax, unsheared) and its whole
// image cube is walked in FP64.
constexpr int LUB_WPB = 4;   // warps per CTA of k_lub: N = 1000 fills all 152 SMs

template <int V>
__global__ void __launch_bounds__ (LUB_WPB * 32, 2)
k_lub (LubArgs a)
{
  constexpr int C = V == 0 ? 3 : (V == 1 ? 6 : 11);
  __shared__ int s_q[LUB_WPB][LUB_QCAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i = blockIdx.x * LUB_WPB + wib;
  if (i >= a.np) return;   // uniform over the warp
  int *q = s_q[wib];
  const double xi[3] = {a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]};
  double ui[C], acc[C];
#pragma unroll
  for (int k = 0; k < C; k++)
    {
      ui[k] = a.u[C * i + k];
      acc[k] = 0.0;
    }
  const bool unsheared = a.periodic && a.shear_mode == 0;
  const double lmin = fmin (a.lx, fmin (a.ly, a.lz));
  const bool single = unsheared && a.lubmax2 > 0.0 && 4.0 * a.lubmax2 <= lmin * lmin;
  const bool test = a.lubmax2 > 0.0 && (unsheared || !a.periodic);
  // one queued candidate per lane, in FP64
  lub_scan (a, xi, test, q, [&] (const int *qb, int count) {
    if (lane >= count) return;
    const int j = qb[lane];
    double uj[C];
#pragma unroll
    for (int k = 0; k < C; k++) uj[k] = a.u[C * j + k];
    lub_images (a, i, j, xi, single,
                [&] (const double d[3]) { lub_pair<V> (a, d, ui, uj, j == i, acc); });
  });
#pragma unroll
  for (int k = 0; k < C; k++)
    {
      const double v = warp_sum (acc[k]);
      if (lane == 0) a.f[C * i + k] = v;
    }
}

// Dense L (src/lub-matrix.c:76-507), row block i per warp.  Candidates as
// in k_lub, taken one at a time: lane b < C applies the pair's blocks to the
// input t_b, so that it holds column b of the self and the cross block of
// (i, j).  t_b is the unit vector e_b for F and FT; for FTS it is column b
// of T^-1, T being the map through which libstokes' FTS matrices act on the
// strain (2 E0 + E4, 2 E1, 2 E2, 2 E3, E0 + 2 E4; src/matrix.c:447-478), so
// that M T = L.  The cross block is added into (i, j) at once and the self
// block into (i, i) at the end: a warp writes only its own rows and one
// candidate at a time, so no two threads write one entry.  The matrix is
// cleared before the launch.
template <int V>
__global__ void __launch_bounds__ (256)
k_lub_matrix (LubArgs a, double *mat)
{
  constexpr int C = V == 0 ? 3 : (V == 1 ? 6 : 11);
  constexpr int NF = V == 0 ? 4 : (V == 1 ? 10 : 22);
  __shared__ int s_q[8][LUB_QCAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i = blockIdx.x * 8 + wib;
  if (i >= a.np) return;   // uniform over the warp
  int *q = s_q[wib];
  const double xi[3] = {a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]};
  const size_t n = (size_t) C * a.np;
  double tb[C], sacc[C];
#pragma unroll
  for (int k = 0; k < C; k++)
    {
      tb[k] = (k == lane) ? 1.0 : 0.0;
      sacc[k] = 0.0;
    }
  if constexpr (V == 2)
    {
      if (lane == 6) { tb[6] = 2.0 / 3.0; tb[C - 1] = -1.0 / 3.0; }
      else if (lane == 10) { tb[6] = -1.0 / 3.0; tb[C - 1] = 2.0 / 3.0; }
      else if (lane >= 7 && lane <= 9) tb[lane] = 0.5;
    }
  const bool unsheared = a.periodic && a.shear_mode == 0;
  const double lmin = fmin (a.lx, fmin (a.ly, a.lz));
  const bool single = unsheared && a.lubmax2 > 0.0 && 4.0 * a.lubmax2 <= lmin * lmin;
  const bool test = a.lubmax2 > 0.0 && (unsheared || !a.periodic);
  double *rows = mat + (size_t) C * i * n;
  lub_scan (a, xi, test, q, [&] (const int *qb, int count) {
    if (lane >= C) return;
    for (int t = 0; t < count; t++)
      {
        const int j = qb[t];
        double xacc[C];
#pragma unroll
        for (int k = 0; k < C; k++) xacc[k] = 0.0;
        lub_images (a, i, j, xi, single, [&] (const double d[3]) {
          double e[3], s11[NF / 2], s12[NF / 2];
          lub_scalars<V> (a, d, e, s11, s12);
          lub_apply<V> (e, s11, true, 1.0, tb, sacc);
          lub_apply<V> (e, s12, false, 1.0, tb, xacc);
          if (j == i)
            {
              const double me[3] = {-e[0], -e[1], -e[2]};
              lub_apply<V> (me, s11, true, 1.0, tb, sacc);
              lub_apply<V> (me, s12, false, 1.0, tb, xacc);
            }
        });
        double *col = rows + (size_t) C * j + lane;
#pragma unroll
        for (int k = 0; k < C; k++) col[k * n] += xacc[k];
      }
  });
  if (lane < C)
    {
      double *col = rows + (size_t) C * i + lane;
#pragma unroll
      for (int k = 0; k < C; k++) col[k * n] += sacc[k];
    }
}

// ---- host side ---------------------------------------------------------------
static int
lub_upload ()
{
  static std::once_flag once;
  static LubCoef coef;
  std::call_once (once, [] { coef = make_coefficients (); });
  static int done_dev = -1;
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice (&dev);
  std::lock_guard<std::mutex> lk (mu);
  if (done_dev == dev) return STOKES_GPU_OK;
  cudaError_t e = cudaMemcpyToSymbol (c_lub, coef.c, sizeof coef.c);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol (c_forms, kForms, sizeof kForms);
  if (e != cudaSuccess) return cuda_fail (e, "lubrication tables");
  done_dev = dev;
  return STOKES_GPU_OK;
}

static int
lub_check (const struct stokes *sys, int version)
{
  if (!sys) return set_error (STOKES_GPU_EINVAL, "NULL system");
  if (sys->np <= 0) return set_error (STOKES_GPU_EINVAL, "no particles");
  if (version < 0 || version > 2) return set_error (STOKES_GPU_EINVAL, "version %d", version);
  if (sys->a || sys->slip)
    return set_error (STOKES_GPU_EINVAL,
                      "the lubrication correction serves equal spheres without slip");
  if (sys->periodic && (!(sys->lx > 0.0) || !(sys->ly > 0.0) || !(sys->lz > 0.0)))
    return set_error (STOKES_GPU_EINVAL, "periodic box not set");
  return STOKES_GPU_OK;
}

// the kernels' arguments for sys (image cube of src/lub.c:129-157)
static int
lub_args (const struct stokes *sys, int version, const double *d_pos, LubArgs &a)
{
  int rc = lub_check (sys, version);
  if (!rc) rc = lub_upload ();
  if (rc) return rc;
  a.pos = d_pos;
  a.u = nullptr;
  a.f = nullptr;
  a.np = sys->np;
  a.periodic = sys->periodic ? 1 : 0;
  a.lx = sys->lx;
  a.ly = sys->ly;
  a.lz = sys->lz;
  a.imx = a.imy = a.imz = 0;
  if (a.periodic)
    {
      const double lm = sys->lubmax > 0.0 ? sys->lubmax : std::fmax (a.lx, std::fmax (a.ly, a.lz));
      // a cube of more than 33^3 images per pair is refused (the loop is
      // per pair and would run for minutes)
      if (!(lm / a.lx < 16.0 && lm / a.ly < 16.0 && lm / a.lz < 16.0))
        return set_error (STOKES_GPU_EINVAL, "lubmax %g spans more than 16 boxes", lm);
      a.imx = (int) (lm / a.lx) + 1;
      a.imy = (int) (lm / a.ly) + 1;
      a.imz = (int) (lm / a.lz) + 1;
    }
  a.shear_mode = a.periodic ? sys->shear_mode : 0;
  a.shift = sys->shear_shift;
  a.lubmin2 = sys->lubmin2;
  a.lubmax2 = sys->lubmax * sys->lubmax;
  return STOKES_GPU_OK;
}

// f = L u on device buffers, version 0 (F, 3 per particle), 1 (FT, 6) or 2
int
lub_dev (const struct stokes *sys, int version, const double *d_pos, const double *d_u,
         double *d_f, cudaStream_t st)
{
  LubArgs a;
  int rc = lub_args (sys, version, d_pos, a);
  if (rc) return rc;
  a.u = d_u;
  a.f = d_f;
  const int grid = (sys->np + LUB_WPB - 1) / LUB_WPB;
  if (version == 0) k_lub<0><<<grid, LUB_WPB * 32, 0, st>>> (a);
  else if (version == 1) k_lub<1><<<grid, LUB_WPB * 32, 0, st>>> (a);
  else k_lub<2><<<grid, LUB_WPB * 32, 0, st>>> (a);
  cudaError_t e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "lubrication kernel");
}

// the dense L on a device buffer d_mat [n n], n = np {3, 6, 11}, row-major
// (FTS in libstokes' extracted form)
static int
lub_matrix_dev (const struct stokes *sys, int version, const double *d_pos, double *d_mat,
                cudaStream_t st)
{
  LubArgs a;
  int rc = lub_args (sys, version, d_pos, a);
  if (rc) return rc;
  const size_t n = (size_t) (version == 0 ? 3 : (version == 1 ? 6 : 11)) * sys->np;
  cudaError_t e = cudaMemsetAsync (d_mat, 0, sizeof (double) * n * n, st);
  if (e != cudaSuccess) return cuda_fail (e, "lubrication matrix");
  const int grid = (sys->np + 7) / 8;
  if (version == 0) k_lub_matrix<0><<<grid, 256, 0, st>>> (a, d_mat);
  else if (version == 1) k_lub_matrix<1><<<grid, 256, 0, st>>> (a, d_mat);
  else k_lub_matrix<2><<<grid, 256, 0, st>>> (a, d_mat);
  e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "lubrication matrix kernel");
}

// the dense L into host memory
static int
lub_matrix_host (struct stokes *sys, int version, double *mat)
{
  clear_error ();
  if (!mat) return set_error (STOKES_GPU_EINVAL, "NULL matrix");
  int rc = lub_check (sys, version);
  if (rc) return rc;
  if ((rc = check_positions (sys->pos, sys->np))) return rc;
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  const int np = sys->np;
  const size_t n = (size_t) (version == 0 ? 3 : (version == 1 ? 6 : 11)) * np;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess
      || (e = c->mat.ensure (sizeof (double) * n * n)) != cudaSuccess)
    return cuda_fail (e, "lubrication matrix buffers");
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice,
                   c->stream);
  rc = lub_matrix_dev (sys, version, (const double *) c->pos.p, (double *) c->mat.p, c->stream);
  if (rc) return rc;
  e = cudaMemcpyAsync (mat, c->mat.p, sizeof (double) * n * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "lubrication matrix");
}

// f = L u with host vectors
static int
lub_host (struct stokes *sys, int version, const double *u, double *f)
{
  clear_error ();
  if (!u || !f) return set_error (STOKES_GPU_EINVAL, "NULL vector");
  int rc = lub_check (sys, version);
  if (rc) return rc;
  if ((rc = check_positions (sys->pos, sys->np))) return rc;
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  const int np = sys->np;
  const size_t n = (size_t) (version == 0 ? 3 : (version == 1 ? 6 : 11)) * np;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess
      || (e = c->x.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = c->y.ensure (sizeof (double) * n)) != cudaSuccess)
    return cuda_fail (e, "lubrication buffers");
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice,
                   c->stream);
  cudaMemcpyAsync (c->x.p, u, sizeof (double) * n, cudaMemcpyHostToDevice, c->stream);
  rc = lub_dev (sys, version, (const double *) c->pos.p, (const double *) c->x.p,
                (double *) c->y.p, c->stream);
  if (rc) return rc;
  e = cudaMemcpyAsync (f, c->y.p, sizeof (double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "lubrication result");
}

}  // namespace lsg

using namespace lsg;

extern "C" {

// src/lub.c:164 (calc_lub_3f), :370 (calc_lub_3ft), :576 (calc_lub_3fts)
void
calc_lub_3f (struct stokes *sys, const double *u, double *f)
{
  if (lub_host (sys, 0, u, f)) dropin_failed ("calc_lub_3f", f, f && sys ? 3 * (size_t) sys->np : 0);
}

void
calc_lub_3ft (struct stokes *sys, const double *uo, double *ft)
{
  if (lub_host (sys, 1, uo, ft))
    dropin_failed ("calc_lub_3ft", ft, ft && sys ? 6 * (size_t) sys->np : 0);
}

void
calc_lub_3fts (struct stokes *sys, const double *uoe, double *fts)
{
  if (lub_host (sys, 2, uoe, fts))
    dropin_failed ("calc_lub_3fts", fts, fts && sys ? 11 * (size_t) sys->np : 0);
}

// the series coefficients (10 functions x 26, host memory; no GPU needed)
int
stokes_gpu_lub_coefficients (double *out)
{
  clear_error ();
  if (!out) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  const LubCoef c = make_coefficients ();
  memcpy (out, c.c, sizeof c.c);
  return STOKES_GPU_OK;
}

int
stokes_gpu_lub (struct stokes *sys, int version, const double *u, double *f)
{
  return lub_host (sys, version, u, f);
}

// src/lub-matrix.c:76 (make_matrix_lub_3f), :225 (3ft), :373 (3fts)
void
make_matrix_lub_3f (struct stokes *sys, double *mat)
{
  if (lub_matrix_host (sys, 0, mat))
    dropin_failed ("make_matrix_lub_3f", mat, mat && sys ? 9 * (size_t) sys->np * sys->np : 0);
}

void
make_matrix_lub_3ft (struct stokes *sys, double *mat)
{
  if (lub_matrix_host (sys, 1, mat))
    dropin_failed ("make_matrix_lub_3ft", mat, mat && sys ? 36 * (size_t) sys->np * sys->np : 0);
}

void
make_matrix_lub_3fts (struct stokes *sys, double *mat)
{
  if (lub_matrix_host (sys, 2, mat))
    dropin_failed ("make_matrix_lub_3fts", mat,
                   mat && sys ? 121 * (size_t) sys->np * sys->np : 0);
}

int
stokes_gpu_lub_matrix (struct stokes *sys, int version, double *mat)
{
  return lub_matrix_host (sys, version, mat);
}

int
stokes_gpu_lub_matrix_dev (struct stokes *sys, int version, const double *d_pos, double *d_mat,
                           void *stream)
{
  clear_error ();
  if (!d_pos || !d_mat) return set_error (STOKES_GPU_EINVAL, "NULL buffer");
  return lub_matrix_dev (sys, version, d_pos, d_mat, (cudaStream_t) stream);
}

int
stokes_gpu_lub_dev (struct stokes *sys, int version, const double *d_pos, const double *d_u,
                    double *d_f, void *stream)
{
  clear_error ();
  if (!d_pos || !d_u || !d_f) return set_error (STOKES_GPU_EINVAL, "NULL vector");
  return lub_dev (sys, version, d_pos, d_u, d_f, (cudaStream_t) stream);
}

}  // extern "C"
