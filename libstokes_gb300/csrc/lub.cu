// lub.cu -- the lubrication correction f = L u for equal spheres, F and FT
// (the drop-in for src/lub.c:164-575; FTS and unequal or slip spheres are
// refused), in FP64 on the device.
//
// L is the sum over close pairs (r < lubmax, images in the cube |n| <=
// lubmax / L + 1) of the two-sphere resistance minus its far-field part,
// R2(r) - (M^inf)^-1(r) (src/f.c:234, src/ft.c:494).  R2 is the exact
// two-sphere resistance in libstokes' lubrication form
// (src/two-body-res.c:31): a near-contact singular part in s1 = 1 - 4/s^2,
// ln s1 and ln((s+2)/(s-2)) plus a power series in 1/s^2 truncated at
// 1/s^50.  The series coefficients are generated here, at start-up, from
// the Jeffrey & Onishi (1984) recurrences for the multipole coefficients of
// two spheres (axisymmetric and asymmetric translation and rotation) and
// the expansion of the singular part; (M^inf)^-1 is the closed-form inverse
// of the Rotne-Prager two-sphere mobility.
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
constexpr int LUB_NF = 10;               // x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c
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
  // f_k(1) = 2^k sum_q T_1,(k-q),q
  void fk (const std::vector<double> &T, double scale, double *f) const
  {
    for (int k = 0; k <= JO_K; k++)
      {
        double v = 0.0;
        for (int q = 0; q <= k; q++) v += get (T, 1, k - q, q);
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

// translation along the line of centres (X^A)
void
jo_xa (JO &J)
{
  J.P[JO::at (1, 0, 0)] = J.V[JO::at (1, 0, 0)] = 1.0;
  for (int m = 1; m <= JO_K; m++)
    for (int q = 0; q <= m; q++)
      for (int n = 1; n <= JO_K + 1; n++)
        {
          const int p = m - q;
          double a = 0.0, b = 0.0;
          for (int s = 1; s <= q; s++)
            {
              const double c = binom (n + s, n);
              a += c * ((double) n * (2 * n + 1) * (2 * n * s - n - s + 2)
                          / (2.0 * (n + 1) * (2 * s - 1) * (n + s)) * JO::get (J.P, s, q - s, p - n + 1)
                        - (double) n * (2 * n - 1) / (2.0 * (n + 1)) * JO::get (J.P, s, q - s, p - n - 1)
                        - (double) n * (4 * n * n - 1) / (2.0 * (n + 1) * (2 * s + 1))
                            * JO::get (J.V, s, q - s - 2, p - n + 1));
              b += c * JO::get (J.P, s, q - s, p - n - 1);
            }
          J.P[JO::at (n, p, q)] = a;
          J.V[JO::at (n, p, q)] = a - 2.0 * n / ((n + 1.0) * (2 * n + 3)) * b;
        }
}

// translation (rot = 0) or rotation (rot = 1) across the line of centres
void
jo_y (JO &J, int rot)
{
  if (rot) J.Q[JO::at (1, 0, 0)] = 1.0;
  else J.P[JO::at (1, 0, 0)] = J.V[JO::at (1, 0, 0)] = 1.0;
  for (int m = 1; m <= JO_K; m++)
    for (int q = 0; q <= m; q++)
      for (int n = 1; n <= JO_K + 1; n++)
        {
          const int p = m - q;
          double a = 0.0, bq = 0.0, bv = 0.0, qq = 0.0;
          for (int s = 1; s <= q; s++)
            {
              const double c = binom (n + s, n + 1);
              const double w = (3.0 * (n + s) - (double) (n * s + 1) * (2 * n * s - s - n + 2))
                               / ((double) s * (n + s) * (2 * s - 1));
              a += c * ((2.0 * n + 1) / (2.0 * (n + 1)) * w * JO::get (J.P, s, q - s, p - n + 1)
                        + (double) n * (2 * n - 1) / (2.0 * (n + 1)) * JO::get (J.P, s, q - s, p - n - 1)
                        + (double) n * (4 * n * n - 1) / (2.0 * (n + 1) * (2 * s + 1))
                            * JO::get (J.V, s, q - s - 2, p - n + 1));
              bq += c * JO::get (J.Q, s, q - s - 1, p - n + 1);
              bv += c * JO::get (J.P, s, q - s, p - n - 1);
              qq += c * ((double) s / (n + 1) * JO::get (J.Q, s, q - s - 1, p - n)
                         - 3.0 / (2.0 * n * s * (n + 1)) * JO::get (J.P, s, q - s, p - n));
            }
          const double pv = a - 2.0 * (4.0 * n * n - 1) / (3.0 * (n + 1)) * bq;
          J.P[JO::at (n, p, q)] = pv;
          J.V[JO::at (n, p, q)] = pv + 2.0 * n / ((n + 1.0) * (2 * n + 3)) * bv;
          J.Q[JO::at (n, p, q)] = qq;
        }
}

// rotation about the line of centres (X^C)
void
jo_xc (JO &J)
{
  J.Q[JO::at (1, 0, 0)] = 1.0;
  for (int m = 1; m <= JO_K; m++)
    for (int q = 0; q <= m; q++)
      for (int n = 1; n <= JO_K + 1; n++)
        {
          const int p = m - q;
          double v = 0.0;
          for (int s = 1; s <= q; s++) v += binom (n + s, n + 1) * JO::get (J.Q, s, q - s - 1, p - n);
          J.Q[JO::at (n, p, q)] = v;
        }
}

// singular-part building blocks as series in u = 1/s
enum { SB_L1, SB_L2, SB_IS1, SB_S1L1, SB_S1L2, SB_UIS1, SB_UL1, SB_UL2, SB_U, SB_ONE, SB_N };
struct Term { int b; double c; };
struct Form { int par, nt; Term t[4]; double esc; };

// libstokes' lubrication forms at lambda = 1: parity, singular part, and the
// factor of the exact series (the SD scaling and sign of each function)
const Form kForms[LUB_NF] = {
  {0, 3, {{SB_IS1, 0.25}, {SB_L1, -0.225}, {SB_S1L1, -3.0 / 112}}, 1.0},
  {1, 4, {{SB_UIS1, -0.5}, {SB_L2, -0.225}, {SB_S1L2, -3.0 / 112}, {SB_U, -12.0 / 112}}, -1.0},
  {0, 1, {{SB_L1, -1.0 / 6}}, 1.0},
  {1, 1, {{SB_L2, -1.0 / 6}}, -1.0},
  {1, 3, {{SB_L2, -2.0 / 12}, {SB_S1L2, -2.0 / 24}, {SB_U, -2.0 / 6}}, 2.0 / 3},
  {0, 2, {{SB_L1, -2.0 / 12}, {SB_S1L1, -2.0 / 24}}, -2.0 / 3},
  {0, 3, {{SB_L1, 4.0 / 12}, {SB_UL2, 4.0 / 6}, {SB_ONE, 4.0 / 3}}, 4.0 / 3},
  {1, 3, {{SB_L2, 4.0 / 12}, {SB_UL1, 4.0 / 6}, {SB_U, -4.0 / 3}}, -4.0 / 3},
  {0, 3, {{SB_L1, -4.0 / 15}, {SB_S1L1, -4.0 * 47 / 750}, {SB_ONE, 4.0 / 3}}, 4.0 / 3},
  {1, 3, {{SB_L2, 4.0 / 60}, {SB_S1L2, 4.0 * 31 / 750}, {SB_U, 4.0 * 62 / 375}}, 4.0 / 3},
};

struct LubCoef { double c[LUB_NF][LUB_NC]; };

LubCoef
make_coefficients ()
{
  double f[5][JO_K + 1];   // XA, YA, YB, XC, YC
  {
    JO J;
    jo_xa (J);
    J.fk (J.P, 1.0, f[0]);
  }
  {
    JO J;
    jo_y (J, 0);
    J.fk (J.P, 1.0, f[1]);
    J.fk (J.Q, 2.0, f[2]);
  }
  {
    JO J;
    jo_xc (J);
    J.fk (J.Q, 1.0, f[3]);
  }
  {
    JO J;
    jo_y (J, 1);
    J.fk (J.Q, 1.0, f[4]);
  }
  const int fam[LUB_NF] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4};
  constexpr int NJ = JO_K + 2;
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
    }
  blk[SB_U][1] = 1.0;
  blk[SB_ONE][0] = 1.0;
  LubCoef C;
  memset (&C, 0, sizeof C);
  for (int g = 0; g < LUB_NF; g++)
    {
      const Form &F = kForms[g];
      const int M = F.par ? 24 : 25;
      for (int m = 0; m <= M; m++)
        {
          const int j = 2 * m + F.par;
          double v = F.esc * std::ldexp (f[fam[g]][j], -j);
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
  const double u = 1.0 / s, u2 = u * u, s1 = 1.0 - 4.0 * u2;
  const double l1 = log (s1), l2 = log ((s + 2.0) / (s - 2.0));
  const double bv[SB_N] = {l1, l2, 1.0 / s1, s1 * l1, s1 * l2, u / s1, u * l1, u * l2, u, 1.0};
  for (int g = 0; g < nf; g++)
    {
      const Form &F = c_forms[g];
      double v = 0.0;
      for (int t = 0; t < F.nt; t++) v += F.t[t].c * bv[F.t[t].b];
      double p = 0.0;
      for (int m = F.par ? 24 : 25; m >= 0; m--) p = fma (p, u2, c_lub[g][m]);
      res[g] = v + (F.par ? p * u : p);
    }
}

// (M^inf)^-1 of two spheres, F (4 values) or FT (10 values)
template <int V>
__device__ __forceinline__ void
lub_minv (double s, double *r)
{
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
}

// one pair image (separation d, source velocity uj) into the target's sums;
// self: the particle's own image (both halves of the pair)
template <int V>
__device__ __forceinline__ void
lub_pair (const LubArgs &a, const double d[3], const double *ui, const double *uj, bool self,
          double *acc)
{
  constexpr int NF = V == 0 ? 4 : 10;
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  if (r2 < a.lubmin2) r2 = a.lubmin2;
  const double r = sqrt (r2), ri = 1.0 / r;
  const double e[3] = {d[0] * ri, d[1] * ri, d[2] * ri};
  double res[NF], inf[NF];
  lub_res (r, NF, res);
  lub_minv<V> (r, inf);
  double s11[5], s12[5];
  s11[0] = res[0] - inf[0];
  s12[0] = res[1] - inf[1];
  s11[1] = res[2] - inf[2];
  s12[1] = res[3] - inf[3];
  if (V == 1)
    {
      s11[2] = res[4] - inf[4];
      s12[2] = res[5] - inf[5];
      s11[3] = res[6] - inf[6];
      s12[3] = res[7] - inf[7];
      s11[4] = res[8] - inf[8];
      s12[4] = res[9] - inf[9];
    }
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

// A warp per target i.  The lanes scan the sources in FP32 (the FP64 pipe of
// this GPU is 1/64 of FP32) and queue the candidates; 32 queued candidates
// are then evaluated in FP64 at once, one per lane.  With a periodic,
// unsheared box and lubmax below half the box, a pair has at most one image
// within lubmax: the candidate test is its minimum image (with a margin for
// the FP32 rounding) and the evaluation takes that image alone, if the
// reference's image cube holds it.  Otherwise every source is a candidate
// (or those whose minimum image is within lubmax, unsheared) and its whole
// image cube is walked in FP64.
template <int V>
__global__ void __launch_bounds__ (256)
k_lub (LubArgs a)
{
  constexpr int C = V == 0 ? 3 : 6;
  __shared__ int s_q[8][LUB_QCAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i = blockIdx.x * 8 + wib;
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
  const float cut2 = (float) a.lubmax2 * 1.0001f + 1e-6f;
  const float lxf = (float) a.lx, lyf = (float) a.ly, lzf = (float) a.lz;
  const float ilxf = 1.0f / lxf, ilyf = 1.0f / lyf, ilzf = 1.0f / lzf;
  const unsigned lt = (1u << lane) - 1u;

  auto evaluate = [&] (int j) {
    double uj[C];
#pragma unroll
    for (int k = 0; k < C; k++) uj[k] = a.u[C * j + k];
    const double r0[3] = {a.pos[3 * j] - xi[0], a.pos[3 * j + 1] - xi[1], a.pos[3 * j + 2] - xi[2]};
    if (single)
      {
        // the one image within lubmax, if the reference's cube holds it
        const double n0 = -rint (r0[0] / a.lx), n1 = -rint (r0[1] / a.ly),
                     n2 = -rint (r0[2] / a.lz);
        if (fabs (n0) > a.imx || fabs (n1) > a.imy || fabs (n2) > a.imz) return;
        const double d[3] = {r0[0] + n0 * a.lx, r0[1] + n1 * a.ly, r0[2] + n2 * a.lz};
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (r2 == 0.0 || !(r2 < a.lubmax2)) return;
        lub_pair<V> (a, d, ui, uj, j == i, acc);
        return;
      }
    // the reference visits the pair once, from its lower index, with the
    // image offsets o(n) of its loop (which need not be symmetric under a
    // shift that accumulates): d = x_j + o - x_i for j > i, the negated
    // separation x_j - o - x_i for j < i, and both signs for j == i
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
                lub_pair<V> (a, d, ui, uj, j == i, acc);
              }
          }
      }
  };

  int qn = 0;
  for (int jb = 0; jb < a.np; jb += 32)
    {
      const int j = jb + lane;
      bool cand = j < a.np;
      if (cand && test)
        {
          // FP32 minimum-image distance (the box wrap only when periodic)
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
          evaluate (q[qn - 32 + lane]);
          qn -= 32;
          __syncwarp ();
        }
    }
  if (lane < qn) evaluate (q[lane]);
#pragma unroll
  for (int k = 0; k < C; k++)
    {
      const double v = warp_sum (acc[k]);
      if (lane == 0) a.f[C * i + k] = v;
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
  if (version > 1)
    return set_error (STOKES_GPU_EINVAL, "the FTS lubrication correction is not built");
  if (sys->a || sys->slip)
    return set_error (STOKES_GPU_EINVAL,
                      "the lubrication correction serves equal spheres without slip");
  if (sys->periodic && (!(sys->lx > 0.0) || !(sys->ly > 0.0) || !(sys->lz > 0.0)))
    return set_error (STOKES_GPU_EINVAL, "periodic box not set");
  return STOKES_GPU_OK;
}

// f = L u on device buffers, version 0 (F, 3 per particle) or 1 (FT, 6)
int
lub_dev (const struct stokes *sys, int version, const double *d_pos, const double *d_u,
         double *d_f, cudaStream_t st)
{
  int rc = lub_check (sys, version);
  if (!rc) rc = lub_upload ();
  if (rc) return rc;
  LubArgs a;
  a.pos = d_pos;
  a.u = d_u;
  a.f = d_f;
  a.np = sys->np;
  a.periodic = sys->periodic ? 1 : 0;
  a.lx = sys->lx;
  a.ly = sys->ly;
  a.lz = sys->lz;
  a.imx = a.imy = a.imz = 0;
  if (a.periodic)
    {
      // the image cube of src/lub.c:129-157
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
  const int grid = (sys->np + 7) / 8;
  if (version == 0) k_lub<0><<<grid, 256, 0, st>>> (a);
  else k_lub<1><<<grid, 256, 0, st>>> (a);
  cudaError_t e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "lubrication kernel");
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
  const size_t n = (size_t) (version == 0 ? 3 : 6) * np;
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
  (void) uoe;
  clear_error ();
  set_error (STOKES_GPU_EINVAL, "the FTS lubrication correction is not built");
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

int
stokes_gpu_lub_dev (struct stokes *sys, int version, const double *d_pos, const double *d_u,
                    double *d_f, void *stream)
{
  clear_error ();
  if (!d_pos || !d_u || !d_f) return set_error (STOKES_GPU_EINVAL, "NULL vector");
  return lub_dev (sys, version, d_pos, d_u, d_f, (cudaStream_t) stream);
}

}  // extern "C"
