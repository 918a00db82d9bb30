// ewald_device.cuh -- device-side building blocks of the Ewald mobility.
//
// Everything here is templated on the arithmetic type R (double for the FP64
// path, float for the mixed path), so the same formulas serve both.
//
// Conventions (libstokes, src/f.c:30-41, src/fts.c:33-45):
//  * a pair term maps the generalised force of the SOURCE particle j to the
//    generalised velocity of the TARGET particle i;  e = (r_j - r_i) / r;
//  * per particle: F | FT | FTS with the stresslet stored as the five
//    components (xx, xy, xz, yz, yy); velocities U | UO | UOE likewise;
//  * the stresslet input enters through the extracted-form transform
//    z = (2xx+yy, 2xy, 2xz, 2yz, 2yy+xx) (src/fts.c:664-670), which is the
//    full contraction with the tensor S' = [[2xx+yy, xy, xz], [xy, 2yy+xx,
//    yz], [xz, yz, 0]].  S' is what the kernels carry.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "engine.h"

namespace lsg {

enum Version { V_F = 0, V_FT = 1, V_FTS = 2 };

template <int V> struct NComp;
template <> struct NComp<0> { static constexpr int value = 3; };
template <> struct NComp<1> { static constexpr int value = 6; };
template <> struct NComp<2> { static constexpr int value = 11; };

// scalar functions of one pair term
template <typename R> struct PairScalars {
  R xa, ya, yb, xc, yc, xg, yg, yh, xm, ym, zm;
};

template <typename R> __device__ __forceinline__ R dev_erfc (R x);
template <> __device__ __forceinline__ double dev_erfc<double> (double x) { return erfc (x); }
template <> __device__ __forceinline__ float dev_erfc<float> (float x) { return erfcf (x); }
template <typename R> __device__ __forceinline__ R dev_exp (R x);
template <> __device__ __forceinline__ double dev_exp<double> (double x) { return exp (x); }
template <> __device__ __forceinline__ float dev_exp<float> (float x) { return expf (x); }
template <typename R> __device__ __forceinline__ R dev_sqrt (R x);
template <> __device__ __forceinline__ double dev_sqrt<double> (double x) { return sqrt (x); }
template <> __device__ __forceinline__ float dev_sqrt<float> (float x) { return sqrtf (x); }

// erfc(x) and exp(-x^2) for x >= 0, x2 = x^2 (the two transcendentals of
// every real-space term)
template <typename R>
__device__ __forceinline__ void
erfc_exp (R x, R x2, R &ec, R &e)
{
  ec = dev_erfc<R> (x);
  e = dev_exp<R> (-x2);
}

// FP32: one exponential for both.  erfc(x) = exp(-x^2) R(x) with the smooth
// R(x) = exp(x^2) erfc(x) approximated as t Q(u), t = 1 / (1 + x / 2) (the
// variable of the rational erfc approximation in Press et al., Numerical
// Recipes, "erfcc"), u = (t - 0.2222) / 0.3889 mapping x in [0, 7] to
// [-1, 1], Q of degree 9 with coefficients fitted here (weighted least
// squares on the relative error, 3500 points against a 40-digit evaluation):
// approximation error 7e-9, 3e-7 worst case with the FP32 arithmetic, about
// the error of the library erfcf.  Beyond x = 7 erfc < 5e-23 and the terms
// it enters are negligible.  exp: the hardware exponential (__expf), whose
// relative error grows as |x2| 6e-8; where that matters (x2 >> 1) the term
// itself is negligible.
template <>
__device__ __forceinline__ void
erfc_exp<float> (float x, float x2, float &ec, float &e)
{
  e = __expf (-x2);
  const float t = __frcp_rn (fmaf (0.5f, x, 1.0f));
  const float u = fmaf (2.5714285714285714f, t, -1.5714285714285716f);
  float q = 4.768114822208366e-06f;
  q = fmaf (q, u, -2.873052176671487e-05f);
  q = fmaf (q, u, -1.653469624654579e-05f);
  q = fmaf (q, u, 0.0003848538656271584f);
  q = fmaf (q, u, -0.00027154337201642197f);
  q = fmaf (q, u, -0.004794785092242448f);
  q = fmaf (q, u, 0.0034944894230291255f);
  q = fmaf (q, u, 0.08977352324023499f);
  q = fmaf (q, u, 0.31723869625882506f);
  q = fmaf (q, u, 0.594215256210305f);
  ec = e * (t * q);
}

// Monodisperse real-space scalars (unit radius) at distance r for splitting
// parameter xi: the closed forms of src/ewald.c:49-186, arranged in Horner
// form in u2 = (xi r)^2.  xisp = xi / sqrt(pi).  ri = 1 / r.
template <int V, typename R>
__device__ __forceinline__ void
real_scalars_mono_ri (R xi, R xisp, R r, R ri, PairScalars<R> &s)
{
  const R u2 = (xi * r) * (xi * r);
  const R ri2 = ri * ri;
  R ec, eg;
  erfc_exp<R> (xi * r, u2, ec, eg);
  const R ex = xisp * eg;

  const R a1 = (R (0.75) + R (0.5) * ri2) * ri * ec
    + ((R (1) + u2 * (R (14) + R (4) * u2 * (u2 - R (5)))) * ri2 - R (4.5) + R (3) * u2) * ex;
  const R a2 = (R (0.75) - R (1.5) * ri2) * ri * ec
    + ((R (-3) + u2 * (R (-2) + R (4) * u2 * (R (4) - u2))) * ri2 + R (1.5) - R (3) * u2) * ex;
  s.ya = a1;
  s.xa = a1 + a2;
  s.yb = s.xc = s.yc = s.xg = s.yg = s.yh = s.xm = s.ym = s.zm = R (0);
  if (V == V_F) return;

  const R ri3 = ri2 * ri;
  s.yb = R (-0.75) * ri2 * ec - R (1.5) * (R (1) + u2 * (R (-6) + R (2) * u2)) * ri * ex;
  const R c1 = R (-0.375) * ri3 * ec
    - R (0.75) * (R (1) + u2 * (R (14) + u2 * (R (-20) + R (4) * u2))) * ri2 * ex;
  const R c2 = R (1.125) * ri3 * ec
    - R (0.75) * (R (-3) + u2 * (R (-2) + u2 * (R (16) - R (4) * u2))) * ri2 * ex;
  s.yc = c1;
  s.xc = c1 + c2;
  if (V == V_FT) return;

  const R ri4 = ri2 * ri2;
  s.xg = (R (2.25) - R (3.6) * ri2) * ri2 * ec
    + (R (-1.5) * (R (-3) + R (6) * u2)
       - R (0.8) * (R (9) + u2 * (R (6) + u2 * (R (-48) + R (12) * u2))) * ri2) * ri * ex;
  s.yg = R (1.2) * ri4 * ec
    + (R (-3) * u2 * (R (2) - u2)
       - R (0.8) * (R (-3) + u2 * (R (-2) + u2 * (R (-26) + u2 * (R (26) - R (4) * u2)))) * ri2)
      * ri * ex;
  s.yh = R (-1.125) * ri3 * ec
    + R (1.5) * (R (-1.5) + u2 * (R (-1) + u2 * (R (8) - R (2) * u2))) * ri2 * ex;
  s.xm = (R (-4.5) + R (10.8) * ri2) * ri3 * ec
    + (R (1.5) * (R (-6) + u2 * (R (-12) + R (12) * u2))
       + R (1.2) * (R (18) + u2 * (R (12) + u2 * (R (30) + u2 * (R (-66) + R (12) * u2)))) * ri2)
      * ri2 * ex;
  s.ym = (R (2.25) - R (7.2) * ri2) * ri3 * ec
    + (R (-1.5) * (R (-3) + u2 * (R (6) + u2 * (R (-12) + R (4) * u2)))
       - R (1.2) * (R (12) + u2 * (R (8) + u2 * (R (-22) + u2 * (R (58) + u2 * (R (-34) + R (4) * u2))))) * ri2)
      * ri2 * ex;
  s.zm = R (1.8) * ri4 * ri * ec
    + (R (-1.5) * u2 * (R (8) - R (4) * u2)
       - R (1.2) * (R (-3) + u2 * (R (-2) + u2 * (R (-26) + u2 * (R (26) - R (4) * u2)))) * ri2)
      * ri2 * ex;
}

template <int V, typename R>
__device__ __forceinline__ void
real_scalars_mono (R xi, R xisp, R r, PairScalars<R> &s)
{
  real_scalars_mono_ri<V, R> (xi, xisp, r, R (1) / r, s);
}

// Difference of the monodisperse real-space scalars between two splits,
// ds = s_xi2(r) - s_xi1(r), without cancellation at small r.  Each scalar
// has d s / d xi = exp(-xi^2 r^2) / sqrt(pi) * Q(xi, r), Q a polynomial in
// xi and r (differentiating the closed forms above, the r^-k terms of the
// erfc and Gaussian parts cancel identically), so ds is the integral of a
// smooth function over [xi1, xi2], taken by 12-point Gauss-Legendre
// quadrature (relative error 2e-15 for xi r <= 1.5 against a 50-digit
// evaluation of the closed forms).  t = xi^2, p = r^2.
template <int V, typename R>
__device__ __forceinline__ void
split_diff (R xi1, R xi2, R r, PairScalars<R> &ds)
{
  // nodes x_k > 0 and weights of the 12-point rule on [-1, 1] (symmetric)
  const R gx[6] = {R (0.1252334085114689), R (0.3678314989981802), R (0.5873179542866175),
                   R (0.7699026741943047), R (0.9041172563704748), R (0.9815606342467192)};
  const R gw[6] = {R (0.2491470458134027), R (0.2334925365383546), R (0.20316742672306573),
                   R (0.16007832854334642), R (0.10693932599531907), R (0.04717533638651141)};
  const R h = R (0.5) * (xi2 - xi1), m = R (0.5) * (xi2 + xi1), p = r * r;
  ds.xa = ds.ya = ds.yb = ds.xc = ds.yc = ds.xg = ds.yg = ds.yh = ds.xm = ds.ym = ds.zm = R (0);
#pragma unroll 1
  for (int k = 0; k < 12; k++)
    {
      const R x = (k < 6) ? -gx[5 - k] : gx[k - 6];
      const R w = (k < 6) ? gw[5 - k] : gw[k - 6];
      const R xi = m + h * x, t = xi * xi, q = t * p;     // q = (xi r)^2
      const R g = w * dev_exp<R> (-q);
      ds.ya += g * (t * (((R (-8) * q + R (68)) * q - R (128)) * q + R (40))
                    + ((R (-6) * q + R (18)) * q - R (6)));
      ds.xa += g * (t * ((R (8) * q - R (44)) * q + R (40)) + R (6) * q - R (6));
      if (V == V_F) continue;
      ds.yb += g * r * t * ((R (6) * q - R (33)) * q + R (30));
      ds.yc += g * t * (((R (6) * q - R (51)) * q + R (96)) * q - R (30));
      ds.xc += g * t * ((R (-6) * q + R (33)) * q - R (30));
      if (V == V_FT) continue;
      ds.xg += g * r * t * (t * ((R (19.2) * q - R (144)) * q + R (201.6)) + R (18) * q - R (36));
      ds.yg += g * r * t * (t * (((R (-6.4) * q + R (70.4)) * q - R (187.2)) * q + R (100.8))
                            + ((R (-6) * q + R (27)) * q - R (18)));
      ds.yh += g * t * q * ((R (6) * q - R (45)) * q + R (63));
      ds.xm += g * t * (t * (((R (-28.8) * q + R (288)) * q - R (626.4)) * q + R (151.2))
                        + ((R (-36) * q + R (126)) * q - R (36)));
      ds.ym += g * t * (t * ((((R (9.6) * q - R (134.4)) * q + R (506.4)) * q - R (540)) * q
                             + R (151.2))
                        + (((R (12) * q - R (78)) * q + R (108)) * q - R (36)));
      ds.zm += g * t * (t * (((R (-9.6) * q + R (105.6)) * q - R (280.8)) * q + R (151.2))
                        + ((R (-12) * q + R (54)) * q - R (36)));
    }
  const R f = h * R (0.56418958354775628);    // 1 / sqrt(pi)
  ds.xa *= f; ds.ya *= f; ds.yb *= f; ds.xc *= f; ds.yc *= f; ds.xg *= f; ds.yg *= f;
  ds.yh *= f; ds.xm *= f; ds.ym *= f; ds.zm *= f;
}

// Unequal-radius real-space scalars in SD form (src/ewald.c:204-359 followed
// by the scaling of :383-420).  aa, ab are the radii entering the Laplacian
// terms (a_i, a_j, or the slip-effective radii); asd is the SD scale of the
// target particle.  Built from the screened Oseen kernels k(r), h(r) and
// their radial derivatives.
template <int V, typename R>
__device__ __forceinline__ void
real_scalars_poly (R xi, R xisp, R r, R aa, R ab, R asd, PairScalars<R> &s)
{
  const R u2 = (xi * r) * (xi * r);
  const R ri = R (1) / r;
  const R ri2 = ri * ri, ri3 = ri2 * ri, ri4 = ri2 * ri2, ri5 = ri3 * ri2;
  R ec, eg;
  erfc_exp<R> (xi * r, u2, ec, eg);
  const R ex = xisp * eg;
  const R sa2 = aa * aa + ab * ab;

  const R k0 = R (2) * (R (-3) + R (2) * u2) * ex + ec * ri;
  const R k0d = R (-2) * ri * (R (1) + u2 * (R (-10) + R (4) * u2)) * ex - ec * ri2;
  const R h0 = R (2) * (R (1) - R (2) * u2) * ex + ec * ri;
  const R k2 = R (4) * ri2 * (R (1) + u2 * (R (14) + u2 * (R (-20) + R (4) * u2))) * ex
    + R (2) * ri3 * ec;
  const R h2 = R (-4) * ri2 * (R (3) + u2 * (R (2) + u2 * (R (-16) + R (4) * u2))) * ex
    - R (6) * ri3 * ec;

  s.ya = R (0.75) * (k0 + k2 * sa2 * R (1.0 / 6.0));
  s.xa = R (0.75) * (h0 + h2 * sa2 * R (1.0 / 6.0)) + s.ya;
  s.yb = s.xc = s.yc = s.xg = s.yg = s.yh = s.xm = s.ym = s.zm = R (0);
  s.xa *= asd;
  s.ya *= asd;
  if (V == V_F) return;

  const R k0dd = R (4) * ri2 * (R (1) + u2 * (R (6) + u2 * (R (-16) + R (4) * u2))) * ex
    + R (2) * ri3 * ec;
  const R h0d = R (-2) * ri * (R (1) + u2 * (R (6) - R (4) * u2)) * ex - ec * ri2;
  const R asd2 = asd * asd, asd3 = asd2 * asd;
  s.yb = R (-0.375) * (-k0d + h0 * ri) * asd2;
  const R yc = R (0.1875) * (-k0dd + (-k0d + h0d) * ri);
  s.yc = yc * asd3;
  s.xc = (R (0.1875) * (k0dd + (-k0d - h0d + R (2) * h0 * ri) * ri) + yc) * asd3;
  if (V == V_FT) return;

  const R k2d = R (-4) * ri3 * (R (3) + u2 * (R (2) + u2 * (R (68) + u2 * (R (-56) + R (8) * u2)))) * ex
    - R (6) * ri4 * ec;
  const R k2dd = R (16) * ri4
    * (R (3) + u2 * (R (2) + u2 * (R (-16) + u2 * (R (76) + u2 * (R (-38) + R (4) * u2))))) * ex
    + R (24) * ri5 * ec;
  const R h2d = R (4) * ri3 * (R (9) + u2 * (R (6) + u2 * (R (36) + u2 * (R (-48) + R (8) * u2)))) * ex
    + R (18) * ri4 * ec;
  const R wg = aa * aa * R (0.1) + ab * ab * R (1.0 / 6.0);
  s.xg = R (-3) * (R (-0.75) * ri * h0 - R (0.75) * ri * h2 * wg) * asd2;
  s.yg = (R (-0.375) * (k0d + h0 * ri) - R (0.375) * (k2d + h2 * ri) * wg) * asd2;
  s.yh = R (-0.1875) * (k0dd + (-k0d - h0d + R (2) * h0 * ri) * ri) * asd3;
  const R m5 = R (-0.375) * (k0d + h0 * ri) * ri - R (0.375) * (k2d + h2 * ri) * ri * sa2 * R (0.1);
  const R zm = R (2) * m5;
  const R m3 = R (-0.75) * h0 * ri2 - R (0.75) * h2 * ri2 * sa2 * R (0.1);
  const R xm = R (6) * m3 + R (3) * zm;
  const R m4 = R (-0.1875) * (k0dd + (-k0d + R (3) * h0d - R (6) * h0 * ri) * ri)
    - R (0.1875) * (k2dd + (-k2d + R (3) * h2d - R (6) * h2 * ri) * ri) * sa2 * R (0.1);
  const R ym = R (2) * m4 + zm;
  s.zm = zm * asd3;
  s.xm = xm * asd3;
  s.ym = ym * asd3;
}

// Generalised force of one particle, in registers.
template <int V, typename R> struct GenF {
  R F[3];
  R T[3];
  R S[6];   // S' (xx, yy, xy, xz, yz); S'zz = 0
};

template <int V, typename R>
__device__ __forceinline__ void
load_genf (const R *x, GenF<V, R> &g)
{
  g.F[0] = x[0]; g.F[1] = x[1]; g.F[2] = x[2];
  if (V >= V_FT) { g.T[0] = x[3]; g.T[1] = x[4]; g.T[2] = x[5]; }
  if (V == V_FTS)
    {
      const R sxx = x[6], sxy = x[7], sxz = x[8], syz = x[9], syy = x[10];
      g.S[0] = R (2) * sxx + syy;
      g.S[1] = R (2) * syy + sxx;
      g.S[2] = sxy;
      g.S[3] = sxz;
      g.S[4] = syz;
    }
}

// Generalised velocity accumulator: U, W (angular), E (xx, xy, xz, yz, yy).
template <int V, typename R> struct GenU {
  R v[NComp<V>::value];
  __device__ __forceinline__ void zero ()
  {
#pragma unroll
    for (int q = 0; q < NComp<V>::value; q++) v[q] = R (0);
  }
};

// Free-space (non-periodic) Rotne-Prager-Yamakawa mobility scalars of a pair
// at distance r, for radii aa (target) and ab (source), in the SD form scaled
// by the target's radius a1: the functions of src/non-ewald.c:110-152 scaled
// as src/non-ewald.c:172-210.  Equal spheres are aa = ab = a1 = 1, which
// reduces exactly to src/non-ewald.c:49-108; with slip, aa and ab are the
// slip-effective radii and a1 the real one (src/non-ewald.c:443-456).
template <int V, typename R>
__device__ __forceinline__ void
open_scalars (R r, R aa, R ab, R a1, PairScalars<R> &s)
{
  const R ri = R (1) / r, r2i = ri * ri;
  const R s2 = aa * aa + ab * ab;
  s.xa = (R (1.5) - R (0.5) * s2 * r2i) * ri * a1;
  s.ya = (R (0.75) + R (0.25) * s2 * r2i) * ri * a1;
  s.yb = s.xc = s.yc = s.xg = s.yg = s.yh = s.xm = s.ym = s.zm = R (0);
  if (V == V_F) return;
  const R a12 = a1 * a1, a13 = a12 * a1;
  s.yb = R (-0.75) * r2i * a12;
  s.xc = R (0.75) * r2i * ri * a13;
  s.yc = R (-0.375) * r2i * ri * a13;
  if (V == V_FT) return;
  const R q = aa * aa * R (0.1) + ab * ab * R (1.0 / 6.0);
  s.xg = (R (2.25) - R (13.5) * q * r2i) * r2i * a12;
  s.yg = R (4.5) * q * r2i * r2i * a12;
  s.yh = R (-1.125) * r2i * ri * a13;
  s.xm = (R (-4.5) + R (5.4) * s2 * r2i) * r2i * ri * a13;
  s.ym = (R (2.25) - R (3.6) * s2 * r2i) * r2i * ri * a13;
  s.zm = R (0.9) * s2 * r2i * r2i * ri * a13;
}

// y_i += block(e, s) . x_j for one real-space (or self) term, in vector form.
// The block is the non-self one used by the matrix-free product
// (src/f.c:115-147, src/ft.c:179-267, src/fts.c:626-1023).
template <int V, typename R>
__device__ __forceinline__ void
pair_apply (const R e[3], const PairScalars<R> &s, const GenF<V, R> &g, GenU<V, R> &y)
{
  const R eF = e[0] * g.F[0] + e[1] * g.F[1] + e[2] * g.F[2];
  const R a2 = s.xa - s.ya;
  y.v[0] += s.ya * g.F[0] + a2 * eF * e[0];
  y.v[1] += s.ya * g.F[1] + a2 * eF * e[1];
  y.v[2] += s.ya * g.F[2] + a2 * eF * e[2];
  if (V == V_F) return;

  const R eT = e[0] * g.T[0] + e[1] * g.T[1] + e[2] * g.T[2];
  const R Txe0 = g.T[1] * e[2] - g.T[2] * e[1];
  const R Txe1 = g.T[2] * e[0] - g.T[0] * e[2];
  const R Txe2 = g.T[0] * e[1] - g.T[1] * e[0];
  const R Fxe0 = g.F[1] * e[2] - g.F[2] * e[1];
  const R Fxe1 = g.F[2] * e[0] - g.F[0] * e[2];
  const R Fxe2 = g.F[0] * e[1] - g.F[1] * e[0];
  const R c2 = s.xc - s.yc;
  y.v[0] += s.yb * Txe0;
  y.v[1] += s.yb * Txe1;
  y.v[2] += s.yb * Txe2;
  y.v[3] += s.yb * Fxe0 + s.yc * g.T[0] + c2 * eT * e[0];
  y.v[4] += s.yb * Fxe1 + s.yc * g.T[1] + c2 * eT * e[1];
  y.v[5] += s.yb * Fxe2 + s.yc * g.T[2] + c2 * eT * e[2];
  if (V == V_FT) return;

  // S' e and e.S'.e (S' symmetric, S'zz = 0)
  const R Sxx = g.S[0], Syy = g.S[1], Sxy = g.S[2], Sxz = g.S[3], Syz = g.S[4];
  const R Se0 = Sxx * e[0] + Sxy * e[1] + Sxz * e[2];
  const R Se1 = Sxy * e[0] + Syy * e[1] + Syz * e[2];
  const R Se2 = Sxz * e[0] + Syz * e[1];
  const R eSe = e[0] * Se0 + e[1] * Se1 + e[2] * Se2;
  const R trS = Sxx + Syy;
  const R g1 = -s.xg * R (1.0 / 3.0), g2 = s.yg, g3 = s.xg - R (2) * s.yg;
  const R m1 = R (1.5) * s.xm - R (2) * s.ym + R (0.5) * s.zm;
  const R m2 = R (-0.5) * s.xm + R (0.5) * s.zm;
  const R m3 = s.xm * R (1.0 / 6.0) - R (0.5) * s.zm;
  const R m4x2 = s.ym - s.zm;          // 2 m4
  const R m5x2 = s.zm;                 // 2 m5

  // U -= G^T S'
  const R gu = g1 * trS + g3 * eSe;
  y.v[0] -= gu * e[0] + R (2) * g2 * Se0;
  y.v[1] -= gu * e[1] + R (2) * g2 * Se1;
  y.v[2] -= gu * e[2] + R (2) * g2 * Se2;
  // W += H^T S' = 2 yh e x (S'e)
  const R h2 = R (2) * s.yh;
  y.v[3] += h2 * (e[1] * Se2 - e[2] * Se1);
  y.v[4] += h2 * (e[2] * Se0 - e[0] * Se2);
  y.v[5] += h2 * (e[0] * Se1 - e[1] * Se0);
  // E += G F + H T + M S'
  const R dE = g1 * eF + m2 * eSe + m3 * trS;           // delta_ab part
  const R eeE = g3 * eF + m1 * eSe + m2 * trS;          // e_a e_b part
  // e_a V_b + e_b V_a part with V = g2 F + yh (T x e) + 2 m4 S'e
  const R V0 = g2 * g.F[0] + s.yh * Txe0 + m4x2 * Se0;
  const R V1 = g2 * g.F[1] + s.yh * Txe1 + m4x2 * Se1;
  const R V2 = g2 * g.F[2] + s.yh * Txe2 + m4x2 * Se2;
  y.v[6] += dE + eeE * e[0] * e[0] + R (2) * e[0] * V0 + m5x2 * Sxx;
  y.v[7] += eeE * e[0] * e[1] + e[0] * V1 + e[1] * V0 + m5x2 * Sxy;
  y.v[8] += eeE * e[0] * e[2] + e[0] * V2 + e[2] * V0 + m5x2 * Sxz;
  y.v[9] += eeE * e[1] * e[2] + e[1] * V2 + e[2] * V1 + m5x2 * Syz;
  y.v[10] += dE + eeE * e[1] * e[1] + R (2) * e[1] * V1 + m5x2 * Syy;
}

// Reciprocal-space term with unit vector e = k/|k| and weights
// ya..ym (src/ewald.c:978-1070, where xa = xc = xg = xm = zm = 0):
//   y += Bc(e) . v1 + Bs(e) . v2
// Bc is the part carried by cos(k.r) (ya, yc, yh, ym); Bs the part carried
// by -sin(k.r) (yb, yg).  v1, v2 are generalised forces (S' form).
template <int V, typename R>
__device__ __forceinline__ void
recip_apply (const R e[3], R ya, R yb, R yc, R yg, R yh, R ym,
             const GenF<V, R> &v1, const GenF<V, R> &v2, GenU<V, R> &y)
{
  const R eF1 = e[0] * v1.F[0] + e[1] * v1.F[1] + e[2] * v1.F[2];
  y.v[0] += ya * (v1.F[0] - eF1 * e[0]);
  y.v[1] += ya * (v1.F[1] - eF1 * e[1]);
  y.v[2] += ya * (v1.F[2] - eF1 * e[2]);
  if (V == V_F) return;

  const R eT1 = e[0] * v1.T[0] + e[1] * v1.T[1] + e[2] * v1.T[2];
  const R Txe0 = v2.T[1] * e[2] - v2.T[2] * e[1];
  const R Txe1 = v2.T[2] * e[0] - v2.T[0] * e[2];
  const R Txe2 = v2.T[0] * e[1] - v2.T[1] * e[0];
  const R Fxe0 = v2.F[1] * e[2] - v2.F[2] * e[1];
  const R Fxe1 = v2.F[2] * e[0] - v2.F[0] * e[2];
  const R Fxe2 = v2.F[0] * e[1] - v2.F[1] * e[0];
  y.v[0] += yb * Txe0;
  y.v[1] += yb * Txe1;
  y.v[2] += yb * Txe2;
  y.v[3] += yb * Fxe0 + yc * (v1.T[0] - eT1 * e[0]);
  y.v[4] += yb * Fxe1 + yc * (v1.T[1] - eT1 * e[1]);
  y.v[5] += yb * Fxe2 + yc * (v1.T[2] - eT1 * e[2]);
  if (V == V_FT) return;

  // S'2 e, e S'2 e for the G^T (sin) part; S'1 e, e S'1 e for H^T and M (cos)
  const R Se20 = v2.S[0] * e[0] + v2.S[2] * e[1] + v2.S[3] * e[2];
  const R Se21 = v2.S[2] * e[0] + v2.S[1] * e[1] + v2.S[4] * e[2];
  const R Se22 = v2.S[3] * e[0] + v2.S[4] * e[1];
  const R eSe2 = e[0] * Se20 + e[1] * Se21 + e[2] * Se22;
  const R Se10 = v1.S[0] * e[0] + v1.S[2] * e[1] + v1.S[3] * e[2];
  const R Se11 = v1.S[2] * e[0] + v1.S[1] * e[1] + v1.S[4] * e[2];
  const R Se12 = v1.S[3] * e[0] + v1.S[4] * e[1];
  const R eSe1 = e[0] * Se10 + e[1] * Se11 + e[2] * Se12;
  const R yg2 = R (2) * yg;
  // U -= G^T S'2 with g1 = 0, g2 = yg, g3 = -2 yg
  y.v[0] -= yg2 * (Se20 - eSe2 * e[0]);
  y.v[1] -= yg2 * (Se21 - eSe2 * e[1]);
  y.v[2] -= yg2 * (Se22 - eSe2 * e[2]);
  // W += 2 yh e x (S'1 e)
  const R h2 = R (2) * yh;
  y.v[3] += h2 * (e[1] * Se12 - e[2] * Se11);
  y.v[4] += h2 * (e[2] * Se10 - e[0] * Se12);
  y.v[5] += h2 * (e[0] * Se11 - e[1] * Se10);
  // E += G F2 + H T1 + M S'1, with m1 = -2 ym, 2 m4 = ym
  const R T1xe0 = v1.T[1] * e[2] - v1.T[2] * e[1];
  const R T1xe1 = v1.T[2] * e[0] - v1.T[0] * e[2];
  const R T1xe2 = v1.T[0] * e[1] - v1.T[1] * e[0];
  const R eF2 = e[0] * v2.F[0] + e[1] * v2.F[1] + e[2] * v2.F[2];
  const R eeE = R (-2) * yg * eF2 - R (2) * ym * eSe1;
  const R V0 = yg * v2.F[0] + yh * T1xe0 + ym * Se10;
  const R V1 = yg * v2.F[1] + yh * T1xe1 + ym * Se11;
  const R V2 = yg * v2.F[2] + yh * T1xe2 + ym * Se12;
  y.v[6] += eeE * e[0] * e[0] + R (2) * e[0] * V0;
  y.v[7] += eeE * e[0] * e[1] + e[0] * V1 + e[1] * V0;
  y.v[8] += eeE * e[0] * e[2] + e[0] * V2 + e[2] * V0;
  y.v[9] += eeE * e[1] * e[2] + e[1] * V2 + e[2] * V1;
  y.v[10] += eeE * e[1] * e[1] + R (2) * e[1] * V1;
}

template <typename R>
__device__ __forceinline__ R
warp_sum (R v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync (0xffffffffu, v, o);
  return v;
}

}  // namespace lsg
