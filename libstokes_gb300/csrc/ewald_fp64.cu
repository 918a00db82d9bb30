// ewald_fp64.cu -- FP64 kernels of the Ewald mobility (the plain FP64 path).
//
//  k_real      real-space pair sum  (src/ewald.c:649-789)
//  k_phase     e^{i k.r_j} table    (reciprocal space, both operators)
//  k_sfac      structure factors C(k) = sum_j cos(k.r_j) x_j, S(k) likewise
//  k_backproj  y_i += sum_k cos(k.r_i) P(k) + sin(k.r_i) Q(k)
//              (src/ewald.c:923-1075 refactored through the structure factors)
//  k_combine   self term + partial real-space sums + reciprocal part
//  k_matrix    dense builder via pair moments (src/ewald.c:1092-1677)
//  k_matrix_open  free-space dense builder (src/non-ewald.c:494-666)
//  k_gemv      dense y = M z(x) (src/matrix.c:365-399, :447-478)
//
// The arithmetic is IEEE FP64 throughout; only the summation order differs
// from the reference (pairs in parallel, reciprocal space factorised).
#include "ewald_device.cuh"
#include "engine.h"

namespace lsg {

// ---------------------------------------------------------------------------
// real space
// ---------------------------------------------------------------------------
constexpr int RS_WARPS = 4;            // warps per CTA
constexpr int RS_QCAP = 64;            // per-warp queue of accepted terms
constexpr int RS_IMG_SMEM = 2048;      // images staged in shared memory

// The rmin clamp (src/ewald.c:693-699: r raised to (a_i + a_j) rmin, and
// e = d / r with the raised r) changes only the real-space term of a pair.
// Unclamped, the sum does not depend on the split, so at a split xi other
// than the struct's own xi_ref (clampfix) a clamped pair contributes
//   T(d/rm; s_ref(rm)) + T(d/r; s_xi(r) - s_ref(r)),
// the clamped term of the struct's split plus the change of the unclamped
// term between the splits; the latter is smooth in r and comes from
// split_diff without cancellation, however close the pair.  Equal spheres.
template <int V>
__device__ __noinline__ void
clamp_term (const RealArgs &a, double dx, double dy, double dz, double r, double rm,
            const GenF<V, double> &g, GenU<V, double> &acc)
{
  PairScalars<double> sc, ds;
  real_scalars_mono<V, double> (a.xi_ref, a.xisp_ref, rm, sc);
  split_diff<V, double> (a.xi_ref, a.xi, r, ds);
  const double ec[3] = {dx / rm, dy / rm, dz / rm};
  const double e0[3] = {dx / r, dy / r, dz / r};
  pair_apply<V, double> (ec, sc, g, acc);
  pair_apply<V, double> (e0, ds, g, acc);
}

template <int V, int MODE>
__device__ __forceinline__ void
real_term (const RealArgs &a, int i, int j, double dx, double dy, double dz,
           double ai, GenU<V, double> &acc)
{
  const double rr = dx * dx + dy * dy + dz * dz;
  double r = sqrt (rr);
  double aj = 1.0;
  if (MODE != MODE_MONO) aj = a.rad[j];
  const double rm = (ai + aj) * a.rmin;
  if (r < rm)
    {
      if (MODE == MODE_MONO && a.clampfix && !a.open)
        {
          GenF<V, double> g;
          load_genf<V, double> (a.x + NComp<V>::value * j, g);
          clamp_term<V> (a, dx, dy, dz, r, rm, g, acc);
          return;
        }
      r = rm;
    }
  const double ri = 1.0 / r;
  const double e[3] = {dx * ri, dy * ri, dz * ri};
  PairScalars<double> s;
  if (a.open)
    {
      if (MODE == MODE_MONO) open_scalars<V, double> (r, 1.0, 1.0, 1.0, s);
      else if (MODE == MODE_POLY) open_scalars<V, double> (r, ai, aj, ai, s);
      else open_scalars<V, double> (r, a.slipa[i], a.slipa[j], ai, s);
    }
  else if (MODE == MODE_MONO)
    real_scalars_mono<V, double> (a.xi, a.xisp, r, s);
  else if (MODE == MODE_POLY)
    real_scalars_poly<V, double> (a.xi, a.xisp, r, ai, aj, ai, s);
  else
    real_scalars_poly<V, double> (a.xi, a.xisp, r, a.slipa[i], a.slipa[j], ai, s);
  GenF<V, double> g;
  load_genf<V, double> (a.x + NComp<V>::value * j, g);
  pair_apply<V, double> (e, s, g, acc);
}

// One warp per (target i, source chunk).  Lanes test 32 images at a time;
// accepted (j, image) terms are compacted into a per-warp queue so that every
// evaluation of the (expensive) pair term runs with all 32 lanes busy.
template <int V, int MODE>
__global__ void __launch_bounds__ (RS_WARPS * 32)
k_real (RealArgs a)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ Img4 s_img[];
  __shared__ double s_qd[RS_WARPS][RS_QCAP][3];
  __shared__ int s_qj[RS_WARPS][RS_QCAP];

  const int nimg_s = a.nimg < RS_IMG_SMEM ? a.nimg : 0;
  for (int t = threadIdx.x; t < nimg_s; t += blockDim.x) s_img[t] = a.img[t];
  __syncthreads ();
  const Img4 *img = nimg_s ? s_img : a.img;

  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * RS_WARPS + wib;
  if (w >= (long long) a.np * a.nchunk) return;
  const int i = (int) (w % a.np);
  const int chunk = (int) (w / a.np);
  const int j0 = (int) ((long long) a.np * chunk / a.nchunk);
  const int j1 = (int) ((long long) a.np * (chunk + 1) / a.nchunk);

  const double pix = a.pos[3 * i], piy = a.pos[3 * i + 1], piz = a.pos[3 * i + 2];
  const double ai = (MODE == MODE_MONO) ? 1.0 : a.rad[i];
  GenU<V, double> acc;
  acc.zero ();
  int qn = 0;
  const unsigned lt = (1u << lane) - 1u;

  // free space: every source j != i once, so the lanes stride over the
  // sources directly (no image test, no queue); coincident positions are
  // skipped like the self image of a lattice sum
  if (a.open)
    for (int j = j0 + lane; j < j1; j += 32)
      {
        const double dx = a.pos[3 * j] - pix, dy = a.pos[3 * j + 1] - piy;
        const double dz = a.pos[3 * j + 2] - piz;
        if (j != i && dx * dx + dy * dy + dz * dz != 0.0)
          real_term<V, MODE> (a, i, j, dx, dy, dz, ai, acc);
      }
  else
  for (int j = j0; j < j1; j++)
    {
      const double djx = a.pos[3 * j] - pix;
      const double djy = a.pos[3 * j + 1] - piy;
      const double djz = a.pos[3 * j + 2] - piz;
      for (int m0 = 0; m0 < a.nimg; m0 += 32)
        {
          const int m = m0 + lane;
          bool ok = false;
          double dx = 0.0, dy = 0.0, dz = 0.0;
          if (m < a.nimg)
            {
              const Img4 L = img[m];
              dx = djx + L.x;
              dy = djy + L.y;
              dz = djz + L.z;
              const double rr = dx * dx + dy * dy + dz * dz;
              ok = (rr != 0.0) && (rr <= a.rmax2);
            }
          const unsigned b = __ballot_sync (0xffffffffu, ok);
          if (ok)
            {
              const int slot = qn + __popc (b & lt);
              s_qd[wib][slot][0] = dx;
              s_qd[wib][slot][1] = dy;
              s_qd[wib][slot][2] = dz;
              s_qj[wib][slot] = j;
            }
          qn += __popc (b);
          __syncwarp ();
          if (qn >= 32)
            {
              const int slot = qn - 32 + lane;
              real_term<V, MODE> (a, i, s_qj[wib][slot], s_qd[wib][slot][0],
                                  s_qd[wib][slot][1], s_qd[wib][slot][2], ai, acc);
              qn -= 32;
              __syncwarp ();
            }
        }
    }
  if (lane < qn)
    real_term<V, MODE> (a, i, s_qj[wib][lane], s_qd[wib][lane][0],
                        s_qd[wib][lane][1], s_qd[wib][lane][2], ai, acc);

  double *out = a.partial + ((size_t) chunk * a.np + i) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const double v = warp_sum (acc.v[q]);
      if (lane == 0) out[q] = v;
    }
}

// ---------------------------------------------------------------------------
// reciprocal space
// ---------------------------------------------------------------------------
// ph[k * np + j] = (cos(k.r_j), sin(k.r_j))
__global__ void
k_phase (const double *pos, const double *kt, int nk, int np, double2 *ph)
{
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long) nk * np) return;
  const int k = (int) (t / np), j = (int) (t % np);
  const double *K = kt + KT_STRIDE * k;
  const double th = K[KT_KX] * pos[3 * j] + K[KT_KY] * pos[3 * j + 1] + K[KT_KZ] * pos[3 * j + 2];
  double sn, cs;
  sincos (th, &sn, &cs);
  ph[t] = make_double2 (cs, sn);
}

// One block per k: C(k), S(k) (and the q_j-weighted pair Cq, Sq for
// unequal radii / slip), then, for equal spheres, the per-k operators
// P(k) = Bc C - Bs S and Q(k) = Bc S + Bs C.
template <int V, int MODE>
__global__ void __launch_bounds__ (256)
k_sfac (const double *x, const double2 *ph, const double *kt, const double *qb,
        int np, double *sf)
{
  constexpr int C = NComp<V>::value;
  constexpr int NW = (MODE == MODE_MONO) ? 2 * C : 4 * C;
  const int k = blockIdx.x;
  double acc[NW];
#pragma unroll
  for (int q = 0; q < NW; q++) acc[q] = 0.0;
  for (int j = threadIdx.x; j < np; j += blockDim.x)
    {
      const double2 p = ph[(size_t) k * np + j];
      const double *xj = x + (size_t) C * j;
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          acc[q] += p.x * xj[q];
          acc[C + q] += p.y * xj[q];
        }
      if (MODE != MODE_MONO)
        {
          const double w = qb[j];
#pragma unroll
          for (int q = 0; q < C; q++)
            {
              acc[2 * C + q] += w * p.x * xj[q];
              acc[3 * C + q] += w * p.y * xj[q];
            }
        }
    }
  __shared__ double red[8][NW];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NW; q++)
    {
      const double v = warp_sum (acc[q]);
      if (lane == 0) red[wid][q] = v;
    }
  __syncthreads ();
  if (threadIdx.x < NW)
    {
      double v = 0.0;
      for (int w = 0; w < (int) (blockDim.x >> 5); w++) v += red[w][threadIdx.x];
      red[0][threadIdx.x] = v;
    }
  __syncthreads ();
  double *out = sf + (size_t) SF_STRIDE * k;
  if (MODE != MODE_MONO)
    {
      if (threadIdx.x < NW) out[threadIdx.x] = red[0][threadIdx.x];
      return;
    }
  if (threadIdx.x == 0)
    {
      const double *K = kt + KT_STRIDE * k;
      const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
      GenF<V, double> c, s, ms;
      load_genf<V, double> (red[0], c);
      load_genf<V, double> (red[0] + C, s);
      // -S
      double neg[C];
#pragma unroll
      for (int q = 0; q < C; q++) neg[q] = -red[0][C + q];
      load_genf<V, double> (neg, ms);
      GenU<V, double> P, Q;
      P.zero ();
      Q.zero ();
      recip_apply<V, double> (e, K[KT_YA], K[KT_YB], K[KT_YC], K[KT_YG], K[KT_YH], K[KT_YM],
                              c, ms, P);
      recip_apply<V, double> (e, K[KT_YA], K[KT_YB], K[KT_YC], K[KT_YG], K[KT_YH], K[KT_YM],
                              s, c, Q);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          out[q] = P.v[q];
          out[C + q] = Q.v[q];
        }
    }
}

// One warp per target i, lanes over k.
template <int V, int MODE>
__global__ void __launch_bounds__ (128)
k_backproj (const double2 *ph, const double *kt, const double *sf, int nk, int np,
            const double *arad, const double *qa, double *yrec)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (i >= np) return;
  GenU<V, double> acc;
  acc.zero ();
  double aa = 1.0, qai = 1.0;
  if (MODE != MODE_MONO) { aa = arad[i]; qai = qa[i]; }
  for (int k = lane; k < nk; k += 32)
    {
      const double2 p = ph[(size_t) k * np + i];
      const double *S = sf + (size_t) SF_STRIDE * k;
      if (MODE == MODE_MONO)
        {
#pragma unroll
          for (int q = 0; q < C; q++) acc.v[q] += p.x * S[q] + p.y * S[C + q];
        }
      else
        {
          const double *K = kt + KT_STRIDE * k;
          const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
          const double kk = K[KT_KK], kn = K[KT_K], kexp = K[KT_KEXP];
          const double aa2 = aa * aa, aa3 = aa2 * aa;
          // weights without the source radius, and their q_j coefficients
          // KT_GF, KT_AF: 1 but in the tuned split's G correction
          const double gx = kexp * K[KT_GF], ax = kexp * K[KT_AF];
          const double ya0 = aa * 6.0 * (1.0 - kk * qai / 6.0) * ax;
          const double ya1 = -aa * kk * ax;
          const double yb = aa2 * 3.0 * kn * ax;
          const double yc = aa3 * 1.5 * kk * ax;
          const double yg0 = aa2 * 3.0 * (1.0 - kk * qai / 10.0) * kn * gx;
          const double yg1 = -aa2 * 0.5 * kk * kn * gx;
          const double yh = aa3 * 1.5 * kk * ax;
          const double ym0 = aa3 * 3.0 * (1.0 - kk * qai / 10.0) * kk * ax;
          const double ym1 = -aa3 * 0.3 * kk * kk * ax;
          // v1 = c_i C + s_i S, v2 = s_i C - c_i S; same with the weighted Cq, Sq
          double t1[C], t2[C], u1[C], u2[C];
#pragma unroll
          for (int q = 0; q < C; q++)
            {
              t1[q] = p.x * S[q] + p.y * S[C + q];
              t2[q] = p.y * S[q] - p.x * S[C + q];
              u1[q] = p.x * S[2 * C + q] + p.y * S[3 * C + q];
              u2[q] = p.y * S[2 * C + q] - p.x * S[3 * C + q];
            }
          GenF<V, double> g1, g2, h1, h2;
          load_genf<V, double> (t1, g1);
          load_genf<V, double> (t2, g2);
          load_genf<V, double> (u1, h1);
          load_genf<V, double> (u2, h2);
          recip_apply<V, double> (e, ya0, yb, yc, yg0, yh, ym0, g1, g2, acc);
          recip_apply<V, double> (e, ya1, 0.0, 0.0, yg1, 0.0, ym1, h1, h2, acc);
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const double v = warp_sum (acc.v[q]);
      if (lane == 0) yrec[(size_t) C * i + q] = v;
    }
}

// y_i = self_i . x_i + sum_chunks partial + yrec
template <int V>
__global__ void
k_combine (const double *x, const double *partial, int nchunk, const double *yrec,
           const double *selfc, int np, double *y)
{
  constexpr int C = NComp<V>::value;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  PairScalars<double> s;
  s.xa = s.ya = selfc[3 * i];
  s.xc = s.yc = selfc[3 * i + 1];
  s.xm = s.ym = s.zm = selfc[3 * i + 2];
  s.yb = s.xg = s.yg = s.yh = 0.0;
  const double e[3] = {0.0, 0.0, 0.0};
  GenF<V, double> g;
  load_genf<V, double> (x + (size_t) C * i, g);
  GenU<V, double> acc;
  acc.zero ();
  pair_apply<V, double> (e, s, g, acc);
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      double v = acc.v[q];
      for (int c = 0; c < nchunk; c++) v += partial[((size_t) c * np + i) * C + q];
      if (yrec) v += yrec[(size_t) C * i + q];
      y[(size_t) C * i + q] = v;
    }
}

// ---------------------------------------------------------------------------
// dense builder: pair moments
// ---------------------------------------------------------------------------
// Sums over terms t (real-space images and reciprocal vectors) of
// scalar(t) x monomial(e_t).  The c x c block of a pair is linear in these.
template <int V> struct Moments;
template <> struct Moments<0> { static constexpr int N = 7; };
template <> struct Moments<1> { static constexpr int N = 17; };
template <> struct Moments<2> { static constexpr int N = 68; };
// layout: A0 | A2[6] | B1[3] | C0 | C2[6] | G1[3] | G2[3] | G3[10] | H2[6] |
//         M4[15] | M2[6] | M3 | M4b[6] | M5
enum {
  MO_A0 = 0, MO_A2 = 1, MO_B1 = 7, MO_C0 = 10, MO_C2 = 11,
  MO_G1 = 17, MO_G2 = 20, MO_G3 = 23, MO_H2 = 33, MO_M4 = 39, MO_M2 = 54,
  MO_M3 = 60, MO_M4B = 61, MO_M5 = 67
};

// symmetric index tables: 2nd order (xx xy xz yy yz zz), 3rd, 4th
__device__ __forceinline__ int sym2 (int a, int b)
{
  if (a > b) { int t = a; a = b; b = t; }
  return a == 0 ? b : (a == 1 ? 2 + b : 5);
}
__device__ __forceinline__ int sym3 (int a, int b, int c)
{
  // sort a <= b <= c
  if (a > b) { int t = a; a = b; b = t; }
  if (b > c) { int t = b; b = c; c = t; }
  if (a > b) { int t = a; a = b; b = t; }
  // xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
  const int nx = (a == 0) + (b == 0) + (c == 0);
  const int ny = (a == 1) + (b == 1) + (c == 1);
  // enumerate by (nx, ny)
  if (nx == 3) return 0;
  if (nx == 2) return ny == 1 ? 1 : 2;
  if (nx == 1) return ny == 2 ? 3 : (ny == 1 ? 4 : 5);
  return ny == 3 ? 6 : (ny == 2 ? 7 : (ny == 1 ? 8 : 9));
}
__device__ __forceinline__ int sym4 (int a, int b, int c, int d)
{
  // xxxx xxxy xxxz xxyy xxyz xxzz xyyy xyyz xyzz xzzz yyyy yyyz yyzz yzzz zzzz
  const int nx = (a == 0) + (b == 0) + (c == 0) + (d == 0);
  const int ny = (a == 1) + (b == 1) + (c == 1) + (d == 1);
  switch (nx)
    {
    case 4: return 0;
    case 3: return ny == 1 ? 1 : 2;
    case 2: return ny == 2 ? 3 : (ny == 1 ? 4 : 5);
    case 1: return ny == 3 ? 6 : (ny == 2 ? 7 : (ny == 1 ? 8 : 9));
    default: return ny == 4 ? 10 : (ny == 3 ? 11 : (ny == 2 ? 12 : (ny == 1 ? 13 : 14)));
    }
}

template <int V, typename R = double>
__device__ __forceinline__ void
moments_add (const R e[3], const PairScalars<R> &s, R *mo)
{
  const R e2[6] = {e[0] * e[0], e[0] * e[1], e[0] * e[2], e[1] * e[1], e[1] * e[2], e[2] * e[2]};
  const R a2 = s.xa - s.ya;
  mo[MO_A0] += s.ya;
#pragma unroll
  for (int q = 0; q < 6; q++) mo[MO_A2 + q] += a2 * e2[q];
  if (V == V_F) return;
  const R c2 = s.xc - s.yc;
#pragma unroll
  for (int q = 0; q < 3; q++) mo[MO_B1 + q] += s.yb * e[q];
  mo[MO_C0] += s.yc;
#pragma unroll
  for (int q = 0; q < 6; q++) mo[MO_C2 + q] += c2 * e2[q];
  if (V == V_FT) return;
  const R g1 = -s.xg / R (3.0), g2 = s.yg, g3 = s.xg - R (2.0) * s.yg;
  const R m1 = R (1.5) * s.xm - R (2.0) * s.ym + R (0.5) * s.zm;
  const R m2 = -R (0.5) * s.xm + R (0.5) * s.zm;
  const R m3 = s.xm / R (6.0) - R (0.5) * s.zm;
  const R m4 = R (0.5) * s.ym - R (0.5) * s.zm;
  const R m5 = R (0.5) * s.zm;
#pragma unroll
  for (int q = 0; q < 3; q++)
    {
      mo[MO_G1 + q] += g1 * e[q];
      mo[MO_G2 + q] += g2 * e[q];
    }
  // e3: xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
  const R e3[10] = {e2[0] * e[0], e2[0] * e[1], e2[0] * e[2], e2[1] * e[1], e2[1] * e[2],
                         e2[2] * e[2], e2[3] * e[1], e2[3] * e[2], e2[4] * e[2], e2[5] * e[2]};
#pragma unroll
  for (int q = 0; q < 10; q++) mo[MO_G3 + q] += g3 * e3[q];
#pragma unroll
  for (int q = 0; q < 6; q++)
    {
      mo[MO_H2 + q] += s.yh * e2[q];
      mo[MO_M2 + q] += m2 * e2[q];
      mo[MO_M4B + q] += m4 * e2[q];
    }
  // e4: xxxx xxxy xxxz xxyy xxyz xxzz xyyy xyyz xyzz xzzz yyyy yyyz yyzz yzzz zzzz
  const R e4[15] = {e2[0] * e2[0], e2[0] * e2[1], e2[0] * e2[2], e2[0] * e2[3], e2[0] * e2[4],
                         e2[0] * e2[5], e2[1] * e2[3], e2[1] * e2[4], e2[1] * e2[5], e2[2] * e2[5],
                         e2[3] * e2[3], e2[3] * e2[4], e2[3] * e2[5], e2[4] * e2[5], e2[5] * e2[5]};
#pragma unroll
  for (int q = 0; q < 15; q++) mo[MO_M4 + q] += m1 * e4[q];
  mo[MO_M3] += m3;
  mo[MO_M5] += m5;
}

template <typename R = double>
__device__ __forceinline__ R
levi (int a, int b, int c)
{
  if (a == b || b == c || a == c) return R (0);
  return ((a == 0 && b == 1) || (a == 1 && b == 2) || (a == 2 && b == 0)) ? R (1) : R (-1);
}

// stresslet slots (xx, xy, xz, yz, yy) -> tensor indices
__device__ __forceinline__ void
slot_ab (int q, int &a, int &b)
{
  const int A[5] = {0, 0, 0, 1, 1}, B[5] = {0, 1, 2, 2, 1};
  a = A[q];
  b = B[q];
}

template <typename R = double>
__device__ __forceinline__ R kd (int a, int b) { return a == b ? R (1) : R (0); }

// G_(ab)c from moments
template <typename R>
__device__ __forceinline__ R
g_tensor (const R *mo, int a, int b, int c)
{
  return mo[MO_G1 + c] * kd<R> (a, b) + mo[MO_G2 + a] * kd<R> (b, c) + mo[MO_G2 + b] * kd<R> (a, c)
    + mo[MO_G3 + sym3 (a, b, c)];
}
// H_(ab)c = sum_n eps_bcn H2[an] + eps_acn H2[bn]
template <typename R>
__device__ __forceinline__ R
h_tensor (const R *mo, int a, int b, int c)
{
  R v = R (0);
  for (int n = 0; n < 3; n++)
    v += levi<R> (b, c, n) * mo[MO_H2 + sym2 (a, n)] + levi<R> (a, c, n) * mo[MO_H2 + sym2 (b, n)];
  return v;
}
// M_(ab)(cd)
template <typename R>
__device__ __forceinline__ R
m_tensor (const R *mo, int a, int b, int c, int d)
{
  return mo[MO_M4 + sym4 (a, b, c, d)]
    + mo[MO_M2 + sym2 (c, d)] * kd<R> (a, b) + mo[MO_M2 + sym2 (a, b)] * kd<R> (c, d)
    + mo[MO_M3] * kd<R> (a, b) * kd<R> (c, d)
    + mo[MO_M4B + sym2 (a, d)] * kd<R> (b, c) + mo[MO_M4B + sym2 (a, c)] * kd<R> (b, d)
    + mo[MO_M4B + sym2 (b, d)] * kd<R> (a, c) + mo[MO_M4B + sym2 (b, c)] * kd<R> (a, d)
    + mo[MO_M5] * (kd<R> (a, c) * kd<R> (b, d) + kd<R> (b, c) * kd<R> (a, d));
}

// one block entry (extracted form) from the moments; same = (i == j)
template <int V, typename R = double>
__device__ __forceinline__ R
block_entry (const R *mo, int row, int col, bool same)
{
  const R sgn = same ? R (-1) : R (1);   // src/ft.c:61-75, src/fts.c:72-104
  if (row < 3)
    {
      const int a = row;
      if (col < 3)
        return mo[MO_A0] * kd<R> (a, col) + mo[MO_A2 + sym2 (a, col)];
      if (col < 6)
        {
          const int b = col - 3;
          R v = R (0);
          for (int n = 0; n < 3; n++) v += levi<R> (a, b, n) * mo[MO_B1 + n];
          return sgn * v;
        }
      int p, q;
      slot_ab (col - 6, p, q);
      return -sgn * g_tensor (mo, p, q, a);
    }
  if (row < 6)
    {
      const int a = row - 3;
      if (col < 3)
        {
          R v = R (0);
          for (int n = 0; n < 3; n++) v += levi<R> (a, col, n) * mo[MO_B1 + n];
          return v;
        }
      if (col < 6)
        return mo[MO_C0] * kd<R> (a, col - 3) + mo[MO_C2 + sym2 (a, col - 3)];
      int p, q;
      slot_ab (col - 6, p, q);
      return h_tensor (mo, p, q, a);
    }
  int a, b;
  slot_ab (row - 6, a, b);
  if (col < 3) return g_tensor (mo, a, b, col);
  if (col < 6) return h_tensor (mo, a, b, col - 3);
  int c, d;
  slot_ab (col - 6, c, d);
  return m_tensor (mo, a, b, c, d);
}

// One warp per pair (i, j): lanes share the image candidates (compacted) and
// the reciprocal vectors, accumulate moments, reduce, and write the block.
template <int V, int MODE>
__global__ void __launch_bounds__ (128)
k_matrix (MatArgs a)
{
  constexpr int C = NComp<V>::value;
  constexpr int NM = Moments<V>::N;
  __shared__ double s_qd[4][RS_QCAP][3];
  __shared__ double s_mo[4][NM];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * 4 + wib;
  if (w >= (long long) a.np * a.np) return;
  const int i = (int) (w / a.np), j = (int) (w % a.np);
  const bool same = (i == j);

  double mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0;

  const double ai = (MODE == MODE_MONO) ? 1.0 : a.rad[i];
  const double aj = (MODE == MODE_MONO) ? 1.0 : a.rad[j];
  if (same && lane == 0)
    {
      PairScalars<double> s;
      s.xa = s.ya = a.selfc[3 * i];
      s.xc = s.yc = a.selfc[3 * i + 1];
      s.xm = s.ym = s.zm = a.selfc[3 * i + 2];
      s.yb = s.xg = s.yg = s.yh = 0.0;
      const double e0[3] = {0.0, 0.0, 0.0};
      moments_add<V> (e0, s, mo);
    }

  const double djx = a.pos[3 * j] - a.pos[3 * i];
  const double djy = a.pos[3 * j + 1] - a.pos[3 * i + 1];
  const double djz = a.pos[3 * j + 2] - a.pos[3 * i + 2];
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  auto real_one = [&] (double dx, double dy, double dz) {
    const double rr = dx * dx + dy * dy + dz * dz;
    double r = sqrt (rr);
    const double rm = (ai + aj) * a.rmin;
    if (r < rm) r = rm;
    const double ri = 1.0 / r;
    const double e[3] = {dx * ri, dy * ri, dz * ri};
    PairScalars<double> s;
    if (a.open)
      {
        if (MODE == MODE_MONO) open_scalars<V, double> (r, 1.0, 1.0, 1.0, s);
        else if (MODE == MODE_POLY) open_scalars<V, double> (r, ai, aj, ai, s);
        else open_scalars<V, double> (r, a.slipa[i], a.slipa[j], ai, s);
      }
    else if (MODE == MODE_MONO)
      real_scalars_mono<V, double> (a.xi, a.xisp, r, s);
    else if (MODE == MODE_POLY)
      real_scalars_poly<V, double> (a.xi, a.xisp, r, ai, aj, ai, s);
    else
      real_scalars_poly<V, double> (a.xi, a.xisp, r, a.slipa[i], a.slipa[j], ai, s);
    moments_add<V> (e, s, mo);
  };
  for (int m0 = 0; m0 < a.nimg; m0 += 32)
    {
      const int m = m0 + lane;
      bool ok = false;
      double dx = 0.0, dy = 0.0, dz = 0.0;
      if (m < a.nimg)
        {
          const Img4 L = a.img[m];
          dx = djx + L.x;
          dy = djy + L.y;
          dz = djz + L.z;
          const double rr = dx * dx + dy * dy + dz * dz;
          ok = (rr != 0.0) && (rr <= a.rmax2);
        }
      const unsigned b = __ballot_sync (0xffffffffu, ok);
      if (ok)
        {
          const int slot = qn + __popc (b & lt);
          s_qd[wib][slot][0] = dx;
          s_qd[wib][slot][1] = dy;
          s_qd[wib][slot][2] = dz;
        }
      qn += __popc (b);
      __syncwarp ();
      if (qn >= 32)
        {
          const int slot = qn - 32 + lane;
          real_one (s_qd[wib][slot][0], s_qd[wib][slot][1], s_qd[wib][slot][2]);
          qn -= 32;
          __syncwarp ();
        }
    }
  if (lane < qn) real_one (s_qd[wib][lane][0], s_qd[wib][lane][1], s_qd[wib][lane][2]);

  // reciprocal vectors: cos(k.(r_j - r_i)) from the phase table
  double qai = 1.0, qbj = 1.0;
  if (MODE != MODE_MONO) { qai = a.qa[i]; qbj = a.qa[j]; }
  for (int k = lane; k < a.nk; k += 32)
    {
      const double *K = a.kt + KT_STRIDE * k;
      const double2 pi_ = a.ph[(size_t) k * a.np + i];
      const double2 pj = a.ph[(size_t) k * a.np + j];
      const double cf = pj.x * pi_.x + pj.y * pi_.y;
      const double sf = pj.x * pi_.y - pj.y * pi_.x;
      const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
      double ya = K[KT_YA], yb = K[KT_YB], yc = K[KT_YC], yg = K[KT_YG], yh = K[KT_YH],
             ym = K[KT_YM];
      if (MODE != MODE_MONO)
        {
          const double kk = K[KT_KK], kn = K[KT_K], kexp = K[KT_KEXP];
          const double aa = ai, aa2 = aa * aa, aa3 = aa2 * aa;
          ya = aa * 6.0 * (1.0 - kk * (qai + qbj) / 6.0) * kexp;
          yb = aa2 * 3.0 * kn * kexp;
          yc = aa3 * 1.5 * kk * kexp;
          yg = aa2 * 3.0 * (1.0 - kk * (qai / 10.0 + qbj / 6.0)) * kn * kexp;
          yh = aa3 * 1.5 * kk * kexp;
          ym = aa3 * 3.0 * (1.0 - kk * (qai + qbj) / 10.0) * kk * kexp;
        }
      PairScalars<double> s;
      s.xa = 0.0; s.ya = cf * ya;
      s.yb = sf * yb;
      s.xc = 0.0; s.yc = cf * yc;
      s.xg = 0.0; s.yg = sf * yg;
      s.yh = cf * yh;
      s.xm = 0.0; s.ym = cf * ym; s.zm = 0.0;
      moments_add<V> (e, s, mo);
    }

  // warp reduction, then lanes write the block rows
#pragma unroll
  for (int q = 0; q < NM; q++)
    {
      const double v = warp_sum (mo[q]);
      if (lane == 0) s_mo[wib][q] = v;
    }
  __syncwarp ();
  const size_t n = (size_t) C * a.np;
  double *blk = a.mat + (size_t) C * i * n + (size_t) C * j;
  for (int t = lane; t < C * C; t += 32)
    {
      const int row = t / C, col = t % C;
      blk[row * n + col] = block_entry<V> (s_mo[wib], row, col, same);
    }
}

// Free-space dense matrix: one thread per block (i, j), consecutive j on
// consecutive threads.  A block holds one pair term (or the self term), so
// there is nothing to share between lanes and nothing to reduce; each thread
// writes its block row by row (the C entries of a row are contiguous, and the
// rows of neighbouring threads fill whole sectors in L2).
template <int V, int MODE>
__global__ void __launch_bounds__ (128)
k_matrix_open (MatArgs a)
{
  constexpr int C = NComp<V>::value;
  constexpr int NM = Moments<V>::N;
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long) a.np * a.np) return;
  const int i = (int) (t / a.np), j = (int) (t % a.np);
  const bool same = (i == j);
  double mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0;
  const double ai = (MODE == MODE_MONO) ? 1.0 : a.rad[i];
  const double aj = (MODE == MODE_MONO) ? 1.0 : a.rad[j];
  PairScalars<double> s;
  if (same)
    {
      s.xa = s.ya = a.selfc[3 * i];
      s.xc = s.yc = a.selfc[3 * i + 1];
      s.xm = s.ym = s.zm = a.selfc[3 * i + 2];
      s.yb = s.xg = s.yg = s.yh = 0.0;
      const double e0[3] = {0.0, 0.0, 0.0};
      moments_add<V> (e0, s, mo);
    }
  else
    {
      const double dx = a.pos[3 * j] - a.pos[3 * i];
      const double dy = a.pos[3 * j + 1] - a.pos[3 * i + 1];
      const double dz = a.pos[3 * j + 2] - a.pos[3 * i + 2];
      const double rr = dx * dx + dy * dy + dz * dz;
      if (rr != 0.0)
        {
          double r = sqrt (rr);
          const double rm = (ai + aj) * a.rmin;
          if (r < rm) r = rm;
          const double ri = 1.0 / r;
          const double e[3] = {dx * ri, dy * ri, dz * ri};
          if (MODE == MODE_MONO) open_scalars<V, double> (r, 1.0, 1.0, 1.0, s);
          else if (MODE == MODE_POLY) open_scalars<V, double> (r, ai, aj, ai, s);
          else open_scalars<V, double> (r, a.slipa[i], a.slipa[j], ai, s);
          moments_add<V> (e, s, mo);
        }
    }
  const size_t n = (size_t) C * a.np;
  double *blk = a.mat + (size_t) C * i * n + (size_t) C * j;
#pragma unroll
  for (int row = 0; row < C; row++)
#pragma unroll
    for (int col = 0; col < C; col++)
      blk[row * n + col] = block_entry<V> (mo, row, col, same);
}

// Split-precision dense builder for equal spheres: the structure of
// k_matrix (one warp per pair, compacted image candidates, lanes over the
// reciprocal vectors) with the terms in FP32 and no FP64 work per term (the
// FP64 pipe of this GPU is 1/64 of FP32).  Separations r_j - r_i + image
// are formed from hi + lo float pairs of both (the difference of the hi
// parts is exact where it cancels, so a separation carries one FP32
// rounding); the cutoff test runs on them (a candidate it misclassifies lies at
// the cutoff, where its term is below the split's accuracy).  Reciprocal
// phases and coefficients come from float copies of the FP64 tables.
// Moments accumulate in FP32 per lane (about ten terms each at the
// reference's split), the lanes meet in FP32, and the block entries are
// stored as FP64.  About 1e-7 of the largest entry against the FP64 builder.
// phf[k * np + j] = (cos, sin)(k.r_j) in FP32, from FP64 arguments
__global__ void
k_phase_f32 (const double *pos, const double *kt, int nk, int np, float2 *phf)
{
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long) nk * np) return;
  const int k = (int) (t / np), j = (int) (t % np);
  const double *K = kt + KT_STRIDE * k;
  const double th = K[KT_KX] * pos[3 * j] + K[KT_KY] * pos[3 * j + 1] + K[KT_KZ] * pos[3 * j + 2];
  double sn, cs;
  sincos (th, &sn, &cs);
  phf[t] = make_float2 ((float) cs, (float) sn);
}

cudaError_t
launch_phase_f32 (const double *pos, const double *kt, int nk, int np, float2 *phf,
                  cudaStream_t st)
{
  const long long t = (long long) nk * np;
  k_phase_f32<<<(int) ((t + 255) / 256), 256, 0, st>>> (pos, kt, nk, np, phf);
  return cudaGetLastError ();
}

template <int V>
__global__ void __launch_bounds__ (128)
k_matrix_f32 (MatArgs a)
{
  constexpr int C = NComp<V>::value;
  constexpr int NM = Moments<V>::N;
  __shared__ float s_qd[4][RS_QCAP][3];
  __shared__ float s_mo[4][NM];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * 4 + wib;
  if (w >= (long long) a.np * a.np) return;
  const int i = (int) (w / a.np), j = (int) (w % a.np);
  const bool same = (i == j);
  float mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0f;
  if (same && lane == 0)
    {
      PairScalars<float> s;
      s.xa = s.ya = (float) a.selfc[3 * i];
      s.xc = s.yc = (float) a.selfc[3 * i + 1];
      s.xm = s.ym = s.zm = (float) a.selfc[3 * i + 2];
      s.yb = s.xg = s.yg = s.yh = 0.0f;
      const float e0[3] = {0.0f, 0.0f, 0.0f};
      moments_add<V, float> (e0, s, mo);
    }
  const double djx = a.pos[3 * j] - a.pos[3 * i];
  const double djy = a.pos[3 * j + 1] - a.pos[3 * i + 1];
  const double djz = a.pos[3 * j + 2] - a.pos[3 * i + 2];
  const float fjx = (float) djx, fjy = (float) djy, fjz = (float) djz;
  const float ljx = (float) (djx - (double) fjx), ljy = (float) (djy - (double) fjy),
              ljz = (float) (djz - (double) fjz);
  const float rmax2f = (float) a.rmax2;
  const float xi = (float) a.xi, xisp = (float) a.xisp, rmin2 = (float) (2.0 * a.rmin);
  const unsigned lt = (1u << lane) - 1u;
  int qn = 0;
  auto real_one = [&] (float dx, float dy, float dz) {
    float r = sqrtf (dx * dx + dy * dy + dz * dz);
    if (r < rmin2) r = rmin2;
    const float ri = 1.0f / r;
    const float e[3] = {dx * ri, dy * ri, dz * ri};
    PairScalars<float> s;
    real_scalars_mono<V, float> (xi, xisp, r, s);
    moments_add<V, float> (e, s, mo);
  };
  for (int m0 = 0; m0 < a.nimg; m0 += 32)
    {
      const int m = m0 + lane;
      bool ok = false;
      float dx = 0.0f, dy = 0.0f, dz = 0.0f;
      if (m < a.nimg)
        {
          const float4 Lh = a.imgf[m], Ll = a.imgl[m];
          dx = (fjx + Lh.x) + (ljx + Ll.x);
          dy = (fjy + Lh.y) + (ljy + Ll.y);
          dz = (fjz + Lh.z) + (ljz + Ll.z);
          const float rr = dx * dx + dy * dy + dz * dz;
          // the zero separation (the pair's own image 0, or a distinct pair
          // at identical positions) is skipped, as in k_matrix
          ok = (rr != 0.0f) && (rr <= rmax2f);
        }
      const unsigned b2 = __ballot_sync (0xffffffffu, ok);
      if (ok)
        {
          const int slot = qn + __popc (b2 & lt);
          s_qd[wib][slot][0] = (float) dx;
          s_qd[wib][slot][1] = (float) dy;
          s_qd[wib][slot][2] = (float) dz;
        }
      qn += __popc (b2);
      __syncwarp ();
      if (qn >= 32)
        {
          const int slot = qn - 32 + lane;
          real_one (s_qd[wib][slot][0], s_qd[wib][slot][1], s_qd[wib][slot][2]);
          qn -= 32;
          __syncwarp ();
        }
    }
  if (lane < qn) real_one (s_qd[wib][lane][0], s_qd[wib][lane][1], s_qd[wib][lane][2]);

  // reciprocal vectors: cos(k.(r_j - r_i)) from the float phase table
  for (int k = lane; k < a.nk; k += 32)
    {
      const float *K = a.ktf + KTF_STRIDE * k;
      const float2 pi_ = a.phf[(size_t) k * a.np + i];
      const float2 pj = a.phf[(size_t) k * a.np + j];
      const float cf = pj.x * pi_.x + pj.y * pi_.y;
      const float sf = pj.x * pi_.y - pj.y * pi_.x;
      const float e[3] = {K[0], K[1], K[2]};
      PairScalars<float> s;
      s.xa = 0.0f; s.ya = cf * K[3];
      s.yb = sf * K[4];
      s.xc = 0.0f; s.yc = cf * K[5];
      s.xg = 0.0f; s.yg = sf * K[6];
      s.yh = cf * K[7];
      s.xm = 0.0f; s.ym = cf * K[8]; s.zm = 0.0f;
      moments_add<V, float> (e, s, mo);
    }

#pragma unroll
  for (int q = 0; q < NM; q++)
    {
      const float v = warp_sum (mo[q]);
      if (lane == 0) s_mo[wib][q] = v;
    }
  __syncwarp ();
  const size_t n = (size_t) C * a.np;
  double *blk = a.mat + (size_t) C * i * n + (size_t) C * j;
  for (int t = lane; t < C * C; t += 32)
    {
      const int row = t / C, col = t % C;
      blk[row * n + col] = (double) block_entry<V, float> (s_mo[wib], row, col, same);
    }
}

// Thread-per-pair split-precision dense builder (equal spheres, no shear,
// no clamp) at a split of its own, light in both spaces per pair.  A warp
// holds one target i and 32 consecutive sources j; each thread owns the
// moments of its pair, so there is no reduction.
//  * real space: the minimum-image separation in FP64 becomes hi + lo
//    floats, and the lattice images within rc are enumerated from the box
//    (a slice in y, in z, then the x range), each one a term;
//  * reciprocal space: the half-space table (weights doubled: the terms of k
//    and -k are equal) with the FP32 phase table, (cos, sin)(k.r);
//  * the C x C block goes out row by row through shared memory: each row of
//    the warp's 32 blocks is C * 32 consecutive doubles, stored coalesced
//    with streaming stores (the matrix is far larger than L2; the phase
//    table stays there).
// The diagonal blocks do not depend on the positions: the self term, the
// particle's own lattice images and the reciprocal vectors at phase 1.  One
// warp sums their moments in FP64 (the FP32 sum of about a hundred terms on
// top of the self term loses a few 1e-7 of the entry), once per build.
template <int V>
__global__ void __launch_bounds__ (32)
k_matrix_self (MatPairArgs a, const double *kt, float *selfmo)
{
  constexpr int NM = Moments<V>::N;
  const int lane = threadIdx.x;
  double mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0;
  if (lane == 0)
    {
      PairScalars<double> s;
      s.xa = s.ya = a.self[0];
      s.xc = s.yc = a.self[1];
      s.xm = s.ym = s.zm = a.self[2];
      s.yb = s.xg = s.yg = s.yh = 0.0;
      const double e0[3] = {0.0, 0.0, 0.0};
      moments_add<V, double> (e0, s, mo);
    }
  const double rc2 = (double) a.rc2;
  const double xi = a.xi64, xisp = a.xi64 / sqrt (M_PI);
  const int n1 = (int) ceil (sqrt (rc2) * a.ilx), n2 = (int) ceil (sqrt (rc2) * a.ily),
            n3 = (int) ceil (sqrt (rc2) * a.ilz);
  const int w1 = 2 * n1 + 1, w2 = 2 * n2 + 1, w3 = 2 * n3 + 1;
  for (int t = lane; t < w1 * w2 * w3; t += 32)
    {
      const int b1 = t / (w2 * w3) - n1, b2 = (t / w3) % w2 - n2, b3 = t % w3 - n3;
      const double rx = b1 * a.lx, ry = b2 * a.ly, rz = b3 * a.lz;
      const double rr = rx * rx + ry * ry + rz * rz;
      if (rr == 0.0 || rr > rc2) continue;
      const double r = sqrt (rr), ri = 1.0 / r;
      const double e[3] = {rx * ri, ry * ri, rz * ri};
      PairScalars<double> s;
      real_scalars_mono_ri<V, double> (xi, xisp, r, ri, s);
      moments_add<V, double> (e, s, mo);
    }
  for (int k = lane; k < a.nk; k += 32)
    {
      const double *K = kt + KT_STRIDE * k;
      const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
      PairScalars<double> s;
      s.xa = 0.0; s.ya = K[KT_YA];
      s.yb = 0.0;
      s.xc = 0.0; s.yc = K[KT_YC];
      s.xg = 0.0; s.yg = 0.0;
      s.yh = K[KT_YH];
      s.xm = 0.0; s.ym = K[KT_YM]; s.zm = 0.0;
      moments_add<V, double> (e, s, mo);
    }
#pragma unroll
  for (int q = 0; q < NM; q++)
    {
      const double v = warp_sum (mo[q]);
      if (lane == 0) selfmo[q] = (float) v;
    }
}

// moments that the sine part of a reciprocal term feeds (odd in e); the
// cosine part feeds the others
__host__ __device__ constexpr bool
mo_odd (int q)
{
  return (q >= MO_B1 && q < MO_C0) || (q >= MO_G1 && q < MO_H2);
}
// moments that no reciprocal term reaches (their scalars vanish in k space)
__host__ __device__ constexpr bool
mo_kzero (int q)
{
  return (q >= MO_G1 && q < MO_G2) || (q >= MO_M2 && q < MO_M4B) || q == MO_M5;
}
template <int V> struct MoPad { static constexpr int N = (Moments<V>::N + 3) / 4 * 4; };

// Per reciprocal vector of the half-space table, each moment at unit cosine
// (even moments) or unit sine (odd moments): a pair's term is then
// cf * kco[q] or sf * kco[q], one FMA per moment.
template <int V>
__global__ void
k_matrix_kco (const double *kt, int nk, float *kco)
{
  constexpr int NM = Moments<V>::N, NP = MoPad<V>::N;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const double *K = kt + KT_STRIDE * k;
  const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
  PairScalars<double> s;
  s.xa = 0.0; s.ya = K[KT_YA];
  s.yb = K[KT_YB];
  s.xc = 0.0; s.yc = K[KT_YC];
  s.xg = 0.0; s.yg = K[KT_YG];
  s.yh = K[KT_YH];
  s.xm = 0.0; s.ym = K[KT_YM]; s.zm = 0.0;
  double mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0;
  moments_add<V, double> (e, s, mo);
#pragma unroll
  for (int q = 0; q < NP; q++) kco[(size_t) k * NP + q] = q < NM ? (float) mo[q] : 0.0f;
}

constexpr int MP_TI = 8;     // targets per CTA, one per warp
constexpr int MP_KCH = 64;   // reciprocal vectors per shared-memory chunk

// A CTA holds 8 targets i (one per warp) and 32 consecutive sources j (one
// per lane).  M is built from the pairs j > i only: block (j, i) is block
// (i, j) with the odd moments negated (e -> -e, sin -> -sin), so each thread
// writes both.  Tiles wholly below the diagonal exit at once.
template <int V>
__global__ void __launch_bounds__ (256, 2)
k_matrix_pairs (MatPairArgs a)
{
  constexpr int C = NComp<V>::value;
  constexpr int NM = Moments<V>::N, NP = MoPad<V>::N;
  __shared__ float4 s_k4[MP_KCH * NP / 4];
  __shared__ float s_row[MP_TI][32 * C];
  __shared__ float s_tr[32][MP_TI * C + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int i0 = blockIdx.y * MP_TI, j0 = blockIdx.x * 32;
  if (j0 + 31 < i0) return;   // uniform over the CTA, before any barrier
  const int i = i0 + wib, j = j0 + lane;
  const bool iok = i < a.np, jok = j < a.np;
  const bool same = iok && i == j;
  const bool work = iok && jok && j > i;
  float mo[NM];
#pragma unroll
  for (int q = 0; q < NM; q++) mo[q] = 0.0f;
  if (same)
    {
#pragma unroll
      for (int q = 0; q < NM; q++) mo[q] = __ldg (a.selfmo + q);
    }
  else if (work)
    {
      double dx = a.pos[3 * j] - a.pos[3 * i];
      double dy = a.pos[3 * j + 1] - a.pos[3 * i + 1];
      double dz = a.pos[3 * j + 2] - a.pos[3 * i + 2];
      dx -= a.lx * rint (dx * a.ilx);
      dy -= a.ly * rint (dy * a.ily);
      dz -= a.lz * rint (dz * a.ilz);
      // a separation that is not inside the box after the minimum image
      // (non-finite or huge coordinates) gives NaN blocks and bounded loops
      if (!(fabs (dx) <= a.lx && fabs (dy) <= a.ly && fabs (dz) <= a.lz))
        dx = dy = dz = nan ("");
      const float hx = (float) dx, hy = (float) dy, hz = (float) dz;
      const float lx = (float) (dx - (double) hx), ly = (float) (dy - (double) hy),
                  lz = (float) (dz - (double) hz);
      const float rc = a.rc, rc2 = a.rc2, xi = a.xi, xisp = a.xisp;
      const int b2lo = (int) ceilf ((-rc - hy) * a.ilyf), b2hi = (int) floorf ((rc - hy) * a.ilyf);
      // NaN: the conversions give 0 (one pass, NaN terms)
      for (int b2 = b2lo; b2 <= b2hi; b2++)
        {
          const float fb2 = (float) b2;
          const float ry = fmaf (fb2, a.lyh, hy) + fmaf (fb2, a.lyl, ly);
          const float rem2 = rc2 - ry * ry;
          if (rem2 < 0.0f) continue;
          const float sy = sqrtf (rem2);
          const int b3lo = (int) ceilf ((-sy - hz) * a.ilzf), b3hi = (int) floorf ((sy - hz) * a.ilzf);
          for (int b3 = b3lo; b3 <= b3hi; b3++)
            {
              const float fb3 = (float) b3;
              const float rz = fmaf (fb3, a.lzh, hz) + fmaf (fb3, a.lzl, lz);
              const float rem3 = rem2 - rz * rz;
              if (rem3 < 0.0f) continue;
              const float sz = sqrtf (rem3);
              const int b1lo = (int) ceilf ((-sz - hx) * a.ilxf),
                        b1hi = (int) floorf ((sz - hx) * a.ilxf);
              for (int b1 = b1lo; b1 <= b1hi; b1++)
                {
                  const float fb1 = (float) b1;
                  const float rx = fmaf (fb1, a.lxh, hx) + fmaf (fb1, a.lxl, lx);
                  const float rr = rx * rx + ry * ry + rz * rz;
                  // the zero separation (distinct particles at identical
                  // positions) is skipped
                  if (rr == 0.0f || rr > rc2) continue;
                  const float ri = rsqrtf (rr);
                  const float r = rr * ri;
                  const float e[3] = {rx * ri, ry * ri, rz * ri};
                  PairScalars<float> s;
                  real_scalars_mono_ri<V, float> (xi, xisp, r, ri, s);
                  moments_add<V, float> (e, s, mo);
                }
            }
        }
    }
  // reciprocal space, the coefficient table staged in chunks
  const float2 *phi = a.phf + (iok ? i : 0), *phj = a.phf + (jok ? j : 0);
  for (int kc = 0; kc < a.nk; kc += MP_KCH)
    {
      const int nkc = min (MP_KCH, a.nk - kc);
      __syncthreads ();
      const float4 *src = reinterpret_cast<const float4 *> (a.kco) + (size_t) kc * (NP / 4);
      for (int t = threadIdx.x; t < nkc * (NP / 4); t += blockDim.x) s_k4[t] = __ldg (src + t);
      __syncthreads ();
      if (work)
        for (int k = 0; k < nkc; k++)
          {
            const float2 pi_ = __ldg (phi + (size_t) (kc + k) * a.np);
            const float2 pj = __ldg (phj + (size_t) (kc + k) * a.np);
            const float cf = pj.x * pi_.x + pj.y * pi_.y;
            const float sf = pj.x * pi_.y - pj.y * pi_.x;
            const float4 *c4 = s_k4 + k * (NP / 4);
#pragma unroll
            for (int q4 = 0; q4 < NP / 4; q4++)
              {
                const float4 v = c4[q4];
                const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int u = 0; u < 4; u++)
                  {
                    const int q = 4 * q4 + u;
                    if (q < NM && !mo_kzero (q)) mo[q] = fmaf (mo_odd (q) ? sf : cf, vv[u], mo[q]);
                  }
              }
          }
    }
  const size_t n = (size_t) C * a.np;
  // blocks (i, j), j >= i: this warp's row, lanes l0 .. l1 - 1, C * 32
  // consecutive doubles per matrix row
  {
    const int l0 = max (0, i - j0), l1 = min (32, a.np - j0);
    float *sr = s_row[wib];
    if (iok && l1 > l0)   // uniform over the warp
      {
        double *base = a.mat + (size_t) C * i * n + (size_t) C * j0;
#pragma unroll
        for (int row = 0; row < C; row++)
          {
#pragma unroll
            for (int col = 0; col < C; col++)
              sr[lane * C + col] = block_entry<V, float> (mo, row, col, same);
            __syncwarp ();
            double *dst = base + (size_t) row * n;
            for (int t = C * l0 + lane; t < C * l1; t += 32) __stcs (dst + t, (double) sr[t]);
            __syncwarp ();
          }
      }
  }
  // blocks (j, i), j > i: rows C j + beta hold the CTA's targets side by side
#pragma unroll
  for (int q = 0; q < NM; q++)
    if (mo_odd (q)) mo[q] = -mo[q];
#pragma unroll
  for (int beta = 0; beta < C; beta++)
    {
#pragma unroll
      for (int alpha = 0; alpha < C; alpha++)
        s_tr[lane][wib * C + alpha] = block_entry<V, float> (mo, beta, alpha, false);
      __syncthreads ();
#pragma unroll
      for (int rr = 0; rr < 32 / MP_TI; rr++)
        {
          const int jl = (32 / MP_TI) * wib + rr, jj = j0 + jl;
          const int ni = min (min (MP_TI, jj - i0), a.np - i0);   // targets i < jj
          if (jj < a.np && ni > 0)
            {
              double *dst = a.mat + ((size_t) C * jj + beta) * n + (size_t) C * i0;
              for (int t = lane; t < C * ni; t += 32) __stcs (dst + t, (double) s_tr[jl][t]);
            }
        }
      __syncthreads ();
    }
}

cudaError_t
launch_matrix_self (int version, const MatPairArgs &a, const double *kt, float *selfmo,
                    cudaStream_t st)
{
  if (version == 0) k_matrix_self<0><<<1, 32, 0, st>>> (a, kt, selfmo);
  else if (version == 1) k_matrix_self<1><<<1, 32, 0, st>>> (a, kt, selfmo);
  else k_matrix_self<2><<<1, 32, 0, st>>> (a, kt, selfmo);
  return cudaGetLastError ();
}

int
matrix_kco_stride (int version)
{
  return version == 0 ? MoPad<0>::N : (version == 1 ? MoPad<1>::N : MoPad<2>::N);
}

cudaError_t
launch_matrix_kco (int version, const double *kt, int nk, float *kco, cudaStream_t st)
{
  if (nk <= 0) return cudaSuccess;
  const int g = (nk + 127) / 128;
  if (version == 0) k_matrix_kco<0><<<g, 128, 0, st>>> (kt, nk, kco);
  else if (version == 1) k_matrix_kco<1><<<g, 128, 0, st>>> (kt, nk, kco);
  else k_matrix_kco<2><<<g, 128, 0, st>>> (kt, nk, kco);
  return cudaGetLastError ();
}

cudaError_t
launch_matrix_pairs (int version, const MatPairArgs &a, cudaStream_t st)
{
  const dim3 grid ((a.np + 31) / 32, (a.np + MP_TI - 1) / MP_TI);
  if (version == 0) k_matrix_pairs<0><<<grid, 32 * MP_TI, 0, st>>> (a);
  else if (version == 1) k_matrix_pairs<1><<<grid, 32 * MP_TI, 0, st>>> (a);
  else k_matrix_pairs<2><<<grid, 32 * MP_TI, 0, st>>> (a);
  return cudaGetLastError ();
}

// dense y = M . z(x), one warp per row (z = extracted-form transform for FTS)
__global__ void __launch_bounds__ (256)
k_gemv (const double *mat, const double *z, int n, double *y)
{
  const int lane = threadIdx.x & 31;
  const long long row = (long long) blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row >= n) return;
  const double *mr = mat + (size_t) row * n;
  double acc = 0.0;
  for (int j = lane; j < n; j += 32) acc += mr[j] * z[j];
  acc = warp_sum (acc);
  if (lane == 0) y[row] = acc;
}

// rectangular y[n1] = M[n1 x n2] . x[n2]
__global__ void __launch_bounds__ (256)
k_gemv_rect (const double *mat, const double *x, int n1, int n2, double *y)
{
  const int lane = threadIdx.x & 31;
  const long long row = (long long) blockIdx.x * 8 + (threadIdx.x >> 5);
  if (row >= n1) return;
  const double *mr = mat + (size_t) row * n2;
  double acc = 0.0;
  for (int j = lane; j < n2; j += 32) acc += mr[j] * x[j];
  acc = warp_sum (acc);
  if (lane == 0) y[row] = acc;
}

__global__ void
k_ztransform (const double *x, int np, double *z)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np) return;
  const double *xj = x + 11 * (size_t) j;
  double *zj = z + 11 * (size_t) j;
  for (int q = 0; q < 6; q++) zj[q] = xj[q];
  zj[6] = 2.0 * xj[6] + xj[10];
  zj[7] = 2.0 * xj[7];
  zj[8] = 2.0 * xj[8];
  zj[9] = 2.0 * xj[9];
  zj[10] = 2.0 * xj[10] + xj[6];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <int V, int MODE>
static cudaError_t
launch_real_t (const RealArgs &a, cudaStream_t st)
{
  const long long nw = (long long) a.np * a.nchunk;
  const int grid = (int) ((nw + RS_WARPS - 1) / RS_WARPS);
  const size_t smem = a.nimg < RS_IMG_SMEM ? sizeof (Img4) * a.nimg : 0;
  // static (queue) + dynamic (images) can pass the 48 KB default: opt in
  cudaError_t e = cudaFuncSetAttribute (k_real<V, MODE>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int) (smem > 0 ? smem : 1));
  if (e != cudaSuccess) return e;
  k_real<V, MODE><<<grid, RS_WARPS * 32, smem, st>>> (a);
  return cudaGetLastError ();
}

cudaError_t
launch_real_fp64 (int version, int mode, const RealArgs &a, cudaStream_t st)
{
#define LSG_DISPATCH(V)                                              \
  if (mode == MODE_MONO) return launch_real_t<V, MODE_MONO> (a, st); \
  if (mode == MODE_POLY) return launch_real_t<V, MODE_POLY> (a, st); \
  return launch_real_t<V, MODE_SLIP> (a, st);
  if (version == 0) { LSG_DISPATCH (0) }
  if (version == 1) { LSG_DISPATCH (1) }
  LSG_DISPATCH (2)
#undef LSG_DISPATCH
}

cudaError_t
launch_phase_fp64 (const double *pos, const double *kt, int nk, int np, double2 *ph,
                   cudaStream_t st)
{
  const long long nt = (long long) nk * np;
  if (nt == 0) return cudaSuccess;
  k_phase<<<(int) ((nt + 255) / 256), 256, 0, st>>> (pos, kt, nk, np, ph);
  return cudaGetLastError ();
}

template <int V, int MODE>
static cudaError_t
launch_recip_t (const RecipArgs &a, cudaStream_t st)
{
  if (a.nk > 0)
    {
      k_sfac<V, MODE><<<a.nk, 256, 0, st>>> (a.x, a.ph, a.kt, a.qa, a.np, a.sf);
      k_backproj<V, MODE><<<(a.np + 3) / 4, 128, 0, st>>> (a.ph, a.kt, a.sf, a.nk, a.np,
                                                            a.rad, a.qa, a.yrec);
    }
  else
    cudaMemsetAsync (a.yrec, 0, sizeof (double) * NCOMP (V) * a.np, st);
  return cudaGetLastError ();
}

cudaError_t
launch_recip_fp64 (int version, int mode, const RecipArgs &a, cudaStream_t st)
{
#define LSG_DISPATCH(V)                                               \
  if (mode == MODE_MONO) return launch_recip_t<V, MODE_MONO> (a, st); \
  if (mode == MODE_POLY) return launch_recip_t<V, MODE_POLY> (a, st); \
  return launch_recip_t<V, MODE_SLIP> (a, st);
  if (version == 0) { LSG_DISPATCH (0) }
  if (version == 1) { LSG_DISPATCH (1) }
  LSG_DISPATCH (2)
#undef LSG_DISPATCH
}

cudaError_t
launch_combine_fp64 (int version, const double *x, const double *partial, int nchunk,
                     const double *yrec, const double *selfc, int np, double *y,
                     cudaStream_t st)
{
  const int grid = (np + 127) / 128;
  if (version == 0) k_combine<0><<<grid, 128, 0, st>>> (x, partial, nchunk, yrec, selfc, np, y);
  else if (version == 1) k_combine<1><<<grid, 128, 0, st>>> (x, partial, nchunk, yrec, selfc, np, y);
  else k_combine<2><<<grid, 128, 0, st>>> (x, partial, nchunk, yrec, selfc, np, y);
  return cudaGetLastError ();
}

cudaError_t
launch_matrix_fp64 (int version, int mode, const MatArgs &a, cudaStream_t st)
{
  const long long nw = (long long) a.np * a.np;
  if (a.open)
    {
      const int grid = (int) ((nw + 127) / 128);
#define LSG_DISPATCH(V)                                                               \
  if (mode == MODE_MONO) k_matrix_open<V, MODE_MONO><<<grid, 128, 0, st>>> (a);      \
  else if (mode == MODE_POLY) k_matrix_open<V, MODE_POLY><<<grid, 128, 0, st>>> (a); \
  else k_matrix_open<V, MODE_SLIP><<<grid, 128, 0, st>>> (a);
      if (version == 0) { LSG_DISPATCH (0) }
      else if (version == 1) { LSG_DISPATCH (1) }
      else { LSG_DISPATCH (2) }
#undef LSG_DISPATCH
      return cudaGetLastError ();
    }
  const int grid = (int) ((nw + 3) / 4);
  if (a.f32 && mode == MODE_MONO)
    {
      if (version == 0) k_matrix_f32<0><<<grid, 128, 0, st>>> (a);
      else if (version == 1) k_matrix_f32<1><<<grid, 128, 0, st>>> (a);
      else k_matrix_f32<2><<<grid, 128, 0, st>>> (a);
      return cudaGetLastError ();
    }
#define LSG_DISPATCH(V)                                                        \
  if (mode == MODE_MONO) k_matrix<V, MODE_MONO><<<grid, 128, 0, st>>> (a);      \
  else if (mode == MODE_POLY) k_matrix<V, MODE_POLY><<<grid, 128, 0, st>>> (a); \
  else k_matrix<V, MODE_SLIP><<<grid, 128, 0, st>>> (a);
  if (version == 0) { LSG_DISPATCH (0) }
  else if (version == 1) { LSG_DISPATCH (1) }
  else { LSG_DISPATCH (2) }
#undef LSG_DISPATCH
  return cudaGetLastError ();
}

cudaError_t
launch_gemv_fp64 (int version, const double *mat, const double *x, double *zbuf, int np,
                  double *y, cudaStream_t st)
{
  const int n = NCOMP (version) * np;
  const double *z = x;
  if (version == 2)
    {
      k_ztransform<<<(np + 127) / 128, 128, 0, st>>> (x, np, zbuf);
      z = zbuf;
    }
  k_gemv<<<(n + 7) / 8, 256, 0, st>>> (mat, z, n, y);
  return cudaGetLastError ();
}

cudaError_t
launch_gemv_rect_fp64 (const double *mat, int n1, int n2, const double *x, double *y,
                       cudaStream_t st)
{
  k_gemv_rect<<<(n1 + 7) / 8, 256, 0, st>>> (mat, x, n1, n2, y);
  return cudaGetLastError ();
}

}  // namespace lsg
