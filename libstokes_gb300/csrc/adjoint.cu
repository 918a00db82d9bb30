// adjoint.cu -- vector-Jacobian product of the Ewald mobility product:
// for L(r, box) = g^T M(r, box) f, the gradient dL/dr (3 N) and the box
// derivatives dL/dl_x, dL/dl_y, dL/dl_z, at fixed image and k sets, fixed xi
// and fixed particle positions (the lattice scales, the particles do not).
//
// Real space.  With d = r_j - r_i + t_m (the image convention of the product)
// and phi_ij(d) = g_i^T R(d) f_j,
//   dL/dr_l = - sum_(j,m) grad_d psi(d),  psi(d) = phi_lj(d) + phi_jl(-d),
// because the image set is symmetric; dL/dl_a = sum_(i,j,m) n_(m,a) d_a phi_ij.
// The gradients come from forward-mode dual numbers (value + 3 partials)
// pushed through the same scalar functions and tensor contractions as the
// product, so nothing is stored: every pair term is recomputed.
//
// Reciprocal space.  With S_x(k) = sum_j e^{ik.r_j} x_j and the Hermitian
// operator op_k = Bc + i Bs of the product (F and FT),
//   L_rec = Re sum_k conj(S_g) . op_k S_f,
//   dL/dr_l = sum_k k Im[e^{-ik.r_l} (g_l . W_k + f_l . U_k)],
//   W = op S_f, U = op S_g;
// the box enters through k = 2 pi n / l and pi/V in op_k (dual numbers in
// l_x, l_y, l_z) and through the phases, whose scaling is that of the
// positions: dL_rec/dl_a |phase = -(1/l_a) sum_l r_(l,a) dL_rec/dr_(l,a).
// The self term does not depend on r or the box.
//
// Split.  Once both sums converge L does not depend on xi, so the VJP takes
// its own: a private copy of the system (same particles, box, version and
// tolerance) set up with xi = eta_adj / V^(1/3) (eta_adj = 9 by default,
// LIBSTOKES_GB300_VJP_ETA; 0 keeps the system's own xi), whose real-space
// cutoff is near half the box.  At libstokes' usual xi = sqrt(pi)/L the FP64
// real-space sum runs over hundreds of images per pair; with eta 9 it runs
// over a few, while the k set grows about 30-fold -- the costs of the two
// parts meet.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "ewald_device.cuh"
#include "engine.h"
#include "gpu_engine.h"
#include "stokes_gpu.h"
#include "stokes_abi.h"

namespace lsg {

// value and three partial derivatives
struct D3 {
  double v, d[3];
  __host__ __device__ D3 () : v (0.0), d{0.0, 0.0, 0.0} {}
  __host__ __device__ D3 (double x) : v (x), d{0.0, 0.0, 0.0} {}
};
__host__ __device__ inline D3 operator+ (const D3 &a, const D3 &b)
{ D3 r; r.v = a.v + b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] + b.d[k]; return r; }
__host__ __device__ inline D3 operator- (const D3 &a, const D3 &b)
{ D3 r; r.v = a.v - b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] - b.d[k]; return r; }
__host__ __device__ inline D3 operator- (const D3 &a)
{ D3 r; r.v = -a.v; for (int k = 0; k < 3; k++) r.d[k] = -a.d[k]; return r; }
__host__ __device__ inline D3 operator* (const D3 &a, const D3 &b)
{ D3 r; r.v = a.v * b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
__host__ __device__ inline D3 operator/ (const D3 &a, const D3 &b)
{
  D3 r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
  for (int k = 0; k < 3; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
__host__ __device__ inline D3 &operator+= (D3 &a, const D3 &b) { a = a + b; return a; }
__host__ __device__ inline D3 &operator-= (D3 &a, const D3 &b) { a = a - b; return a; }
// a function of one variable with value fv and derivative dv at a.v
__host__ __device__ inline D3 chain (const D3 &a, double fv, double dv)
{ D3 r; r.v = fv; for (int k = 0; k < 3; k++) r.d[k] = dv * a.d[k]; return r; }

template <> __device__ __forceinline__ D3 dev_erfc<D3> (D3 x)
{
  // d/dx erfc(x) = -2/sqrt(pi) exp(-x^2)
  return chain (x, erfc (x.v), -1.1283791670955126 * exp (-x.v * x.v));
}
template <> __device__ __forceinline__ D3 dev_exp<D3> (D3 x)
{
  const double e = exp (x.v);
  return chain (x, e, e);
}
template <> __device__ __forceinline__ D3 dev_sqrt<D3> (D3 x)
{
  const double s = sqrt (x.v);
  return chain (x, s, 0.5 / s);
}

template <int V>
__device__ __forceinline__ void
genf_const (const double *x, GenF<V, D3> &g)
{
  double t[11];
  for (int q = 0; q < NComp<V>::value; q++) t[q] = x[q];
  GenF<V, double> gd;
  load_genf<V, double> (t, gd);
  for (int a = 0; a < 3; a++) g.F[a] = D3 (gd.F[a]);
  if (V >= V_FT)
    for (int a = 0; a < 3; a++) g.T[a] = D3 (gd.T[a]);
  if (V == V_FTS)
    for (int a = 0; a < 6; a++) g.S[a] = D3 (gd.S[a]);
}

template <int V>
__device__ __forceinline__ D3
dotq (const double *g, const GenU<V, D3> &u)
{
  D3 s;
  for (int q = 0; q < NComp<V>::value; q++) s += D3 (g[q]) * u.v[q];
  return s;
}

// ---------------------------------------------------------------------------
// real space: per (target l, source chunk) the sums of grad psi and of
// n_m (x) grad phi_lj over the accepted (j, image) terms
// ---------------------------------------------------------------------------
struct AdjRealArgs {
  const double *pos, *g, *f;
  const Img4 *img;
  int nimg, np, nchunk;
  double rmax2, rmin, xi, xisp;
  double lx, ly, lz;
  double *partial;      // [nchunk][np][6]: grad psi (3), box (3)
};

constexpr int AR_WARPS = 4;
constexpr int AR_QCAP = 64;

template <int V>
__device__ __forceinline__ void
adj_term (const AdjRealArgs &a, int l, int j, double dx, double dy, double dz, double out[6])
{
  constexpr int C = NComp<V>::value;
  D3 d[3];
  d[0] = D3 (dx); d[0].d[0] = 1.0;
  d[1] = D3 (dy); d[1].d[1] = 1.0;
  d[2] = D3 (dz); d[2].d[2] = 1.0;
  D3 r = dev_sqrt<D3> (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double rm = 2.0 * a.rmin;
  if (r.v < rm) r = D3 (rm);                 // the clamp: no radial dependence
  const D3 e[3] = {d[0] / r, d[1] / r, d[2] / r};
  const D3 me[3] = {-e[0], -e[1], -e[2]};
  PairScalars<D3> s;
  real_scalars_mono<V, D3> (D3 (a.xi), D3 (a.xisp), r, s);
  GenF<V, D3> fj, fl;
  genf_const<V> (a.f + (size_t) C * j, fj);
  genf_const<V> (a.f + (size_t) C * l, fl);
  GenU<V, D3> u1, u2;
  u1.zero ();
  u2.zero ();
  pair_apply<V, D3> (e, s, fj, u1);          // R(d) f_j
  pair_apply<V, D3> (me, s, fl, u2);         // R(-d) f_l
  const D3 p1 = dotq<V> (a.g + (size_t) C * l, u1);   // phi_lj(d)
  const D3 p2 = dotq<V> (a.g + (size_t) C * j, u2);   // phi_jl(-d)
  // grad_d phi_jl(-d) = -(grad phi_jl)(-d): the chain rule is already in me
  for (int k = 0; k < 3; k++) out[k] += p1.d[k] + p2.d[k];
  // box: n_m (x) grad phi_lj, n from the image displacement (no shear)
  out[3] += p1.d[0] * rint ((dx - (a.pos[3 * j] - a.pos[3 * l])) / a.lx);
  out[4] += p1.d[1] * rint ((dy - (a.pos[3 * j + 1] - a.pos[3 * l + 1])) / a.ly);
  out[5] += p1.d[2] * rint ((dz - (a.pos[3 * j + 2] - a.pos[3 * l + 2])) / a.lz);
}

template <int V>
__global__ void __launch_bounds__ (AR_WARPS * 32)
k_adj_real (AdjRealArgs a)
{
  __shared__ double s_qd[AR_WARPS][AR_QCAP][3];
  __shared__ int s_qj[AR_WARPS][AR_QCAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * AR_WARPS + wib;
  if (w >= (long long) a.np * a.nchunk) return;
  const int l = (int) (w % a.np), chunk = (int) (w / a.np);
  const int j0 = (int) ((long long) a.np * chunk / a.nchunk);
  const int j1 = (int) ((long long) a.np * (chunk + 1) / a.nchunk);
  const double plx = a.pos[3 * l], ply = a.pos[3 * l + 1], plz = a.pos[3 * l + 2];
  double out[6] = {0, 0, 0, 0, 0, 0};
  int qn = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (int j = j0; j < j1; j++)
    {
      const double djx = a.pos[3 * j] - plx, djy = a.pos[3 * j + 1] - ply,
                   djz = a.pos[3 * j + 2] - plz;
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
              s_qj[wib][slot] = j;
            }
          qn += __popc (b);
          __syncwarp ();
          if (qn >= 32)
            {
              const int slot = qn - 32 + lane;
              adj_term<V> (a, l, s_qj[wib][slot], s_qd[wib][slot][0], s_qd[wib][slot][1],
                           s_qd[wib][slot][2], out);
              qn -= 32;
              __syncwarp ();
            }
        }
    }
  if (lane < qn)
    adj_term<V> (a, l, s_qj[wib][lane], s_qd[wib][lane][0], s_qd[wib][lane][1],
                 s_qd[wib][lane][2], out);
  double *o = a.partial + ((size_t) chunk * a.np + l) * 6;
#pragma unroll
  for (int k = 0; k < 6; k++)
    {
      const double v = warp_sum (out[k]);
      if (lane == 0) o[k] = v;
    }
}

// ---------------------------------------------------------------------------
// reciprocal space
// ---------------------------------------------------------------------------
// One block per k: S_f, S_g; W = op S_f and U = op S_g (complex, stored as
// [re c][im c]); the op-derivative part of the box gradient,
// Re conj(S_g) . (d op / d l_a) S_f, for a = x, y, z.
template <int V>
__global__ void __launch_bounds__ (256)
k_adj_sfac (const double *g, const double *f, const double2 *ph, const double *kt, int np,
            double xi2, double lx, double ly, double lz, bool box, double *WU, double *dbox)
{
  constexpr int C = NComp<V>::value;
  const int k = blockIdx.x;
  __shared__ double red[8][4 * C];
  double acc[4 * C];
  for (int q = 0; q < 4 * C; q++) acc[q] = 0.0;
  for (int j = threadIdx.x; j < np; j += blockDim.x)
    {
      const double2 p = ph[(size_t) k * np + j];
      for (int q = 0; q < C; q++)
        {
          const double fv = f[(size_t) C * j + q], gv = g[(size_t) C * j + q];
          acc[q] += p.x * fv;
          acc[C + q] += p.y * fv;
          acc[2 * C + q] += p.x * gv;
          acc[3 * C + q] += p.y * gv;
        }
    }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q = 0; q < 4 * C; q++)
    {
      const double v = warp_sum (acc[q]);
      if (lane == 0) red[wid][q] = v;
    }
  __syncthreads ();
  if (threadIdx.x != 0) return;
  double S[4 * C];
  for (int q = 0; q < 4 * C; q++)
    {
      double v = 0.0;
      for (int w = 0; w < (int) (blockDim.x >> 5); w++) v += red[w][q];
      S[q] = v;
    }
  const double *K = kt + (size_t) KT_STRIDE * k;
  const double e[3] = {K[KT_EX], K[KT_EY], K[KT_EZ]};
  // W = (Bc + i Bs)(C + i S): re = Bc C - Bs S, im = Bc S + Bs C
  for (int which = 0; which < 2; which++)
    {
      const double *Cs = S + 2 * C * which, *Ss = Cs + C;
      double ms[11];
      for (int q = 0; q < C; q++) ms[q] = -Ss[q];
      GenF<V, double> gc, gs, gms;
      load_genf<V, double> (Cs, gc);
      load_genf<V, double> (Ss, gs);
      load_genf<V, double> (ms, gms);
      GenU<V, double> P, Q;
      P.zero ();
      Q.zero ();
      recip_apply<V, double> (e, K[KT_YA], K[KT_YB], K[KT_YC], K[KT_YG], K[KT_YH], K[KT_YM], gc,
                              gms, P);
      recip_apply<V, double> (e, K[KT_YA], K[KT_YB], K[KT_YC], K[KT_YG], K[KT_YH], K[KT_YM], gs,
                              gc, Q);
      double *o = WU + ((size_t) k * 2 + which) * 2 * C;
      for (int q = 0; q < C; q++)
        {
          o[q] = P.v[q];
          o[C + q] = Q.v[q];
        }
    }
  if (!box) return;
  // op as a function of the box lengths: k = 2 pi n / l, pi / V
  D3 Lx (lx), Ly (ly), Lz (lz);
  Lx.d[0] = Ly.d[1] = Lz.d[2] = 1.0;
  const double tp = 2.0 * M_PI;
  const D3 kx = D3 (tp * rint (K[KT_KX] * lx / tp)) / Lx;
  const D3 ky = D3 (tp * rint (K[KT_KY] * ly / tp)) / Ly;
  const D3 kz = D3 (tp * rint (K[KT_KZ] * lz / tp)) / Lz;
  const D3 kk = kx * kx + ky * ky + kz * kz;
  const D3 kn = dev_sqrt<D3> (kk);
  const D3 k4z = kk / D3 (4.0 * xi2);
  const D3 pivol = D3 (M_PI) / (Lx * Ly * Lz);
  const D3 kexp = pivol * (D3 (1.0) + k4z * (D3 (1.0) + D3 (2.0) * k4z)) / kk * dev_exp<D3> (-k4z);
  const D3 ya = D3 (6.0) * (D3 (1.0) - kk / D3 (3.0)) * kexp;
  const D3 yb = D3 (3.0) * kn * kexp;
  const D3 yc = D3 (1.5) * kk * kexp;
  const D3 yg = D3 (3.0) * (D3 (1.0) - D3 (4.0 / 15.0) * kk) * kn * kexp;
  const D3 yh = D3 (1.5) * kk * kexp;
  const D3 ym = D3 (3.0) * (D3 (1.0) - kk / D3 (5.0)) * kk * kexp;
  const D3 ed[3] = {kx / kn, ky / kn, kz / kn};
  double cfv[11], sfv[11], msv[11];
  for (int q = 0; q < C; q++)
    {
      cfv[q] = S[q];
      sfv[q] = S[C + q];
      msv[q] = -S[C + q];
    }
  GenF<V, D3> gc, gs, gms;
  genf_const<V> (cfv, gc);
  genf_const<V> (sfv, gs);
  genf_const<V> (msv, gms);
  GenU<V, D3> P, Q;
  P.zero ();
  Q.zero ();
  recip_apply<V, D3> (ed, ya, yb, yc, yg, yh, ym, gc, gms, P);
  recip_apply<V, D3> (ed, ya, yb, yc, yg, yh, ym, gs, gc, Q);
  // Re conj(S_g) . dW = Cg . dP + Sg . dQ
  for (int a = 0; a < 3; a++)
    {
      double s = 0.0;
      for (int q = 0; q < C; q++) s += S[2 * C + q] * P.v[q].d[a] + S[3 * C + q] * Q.v[q].d[a];
      dbox[(size_t) 3 * k + a] = s;
    }
}

// per particle l: sum_k k Im[e^{-ik.r_l} (g_l . W_k + f_l . U_k)]
template <int V>
__global__ void
k_adj_backproj (const double *g, const double *f, const double2 *ph, const double *kt,
                const double *WU, int nk, int np, double *grad)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (l >= np) return;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int k = lane; k < nk; k += 32)
    {
      const double2 p = ph[(size_t) k * np + l];
      const double *W = WU + (size_t) k * 4 * C, *U = W + 2 * C;
      double hr = 0.0, hi = 0.0;     // g_l . W + f_l . U
      for (int q = 0; q < C; q++)
        {
          const double gq = g[(size_t) C * l + q], fq = f[(size_t) C * l + q];
          hr += gq * W[q] + fq * U[q];
          hi += gq * W[C + q] + fq * U[C + q];
        }
      // Im[(cos - i sin)(hr + i hi)] = cos hi - sin hr
      const double im = p.x * hi - p.y * hr;
      const double *K = kt + (size_t) KT_STRIDE * k;
      gx += K[KT_KX] * im;
      gy += K[KT_KY] * im;
      gz += K[KT_KZ] * im;
    }
  gx = warp_sum (gx);
  gy = warp_sum (gy);
  gz = warp_sum (gz);
  if (lane == 0)
    {
      grad[3 * l] = gx;
      grad[3 * l + 1] = gy;
      grad[3 * l + 2] = gz;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct AdjState {
  DevBuf g, f, ph, wu, dbox, partial, grad;
};

// the private copy of a system that carries the VJP's split
struct AdjShadow {
  struct stokes *sv = nullptr;
  double key[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
};

static std::mutex g_shadow_mu;
static std::vector<std::pair<const struct stokes *, AdjShadow>> g_shadow;

static struct stokes *
adj_shadow (struct stokes *sys, double eta)
{
  const double eps = sys->ewald_eps > 0.0 ? sys->ewald_eps : 1e-12;
  const double key[9] = {sys->lx, sys->ly, sys->lz, (double) sys->np, (double) sys->version, eta,
                         eps, (double) sys->shear_mode, sys->shear_shift};
  struct stokes *stale = nullptr, *sv = nullptr;
  {
    std::lock_guard<std::mutex> lk (g_shadow_mu);
    for (auto &e : g_shadow)
      if (e.first == sys)
        {
          if (memcmp (e.second.key, key, sizeof key) == 0) sv = e.second.sv;
          else
            {
              stale = e.second.sv;
              e.second.sv = nullptr;
            }
        }
  }
  // freed outside the lock: stokes_free comes back through release_adjoint
  if (stale) stokes_free (stale);
  if (!sv)
    {
      sv = stokes_init ();
      sv->version = sys->version;
      sv->periodic = 1;
      stokes_set_np (sv, sys->np, sys->nm);
      stokes_set_l (sv, sys->lx, sys->ly, sys->lz);
      sv->shear_mode = sys->shear_mode;
      sv->shear_shift = sys->shear_shift;
      stokes_set_xi (sv, eta / cbrt (sys->lx * sys->ly * sys->lz), eps);
      std::lock_guard<std::mutex> lk (g_shadow_mu);
      bool placed = false;
      for (auto &e : g_shadow)
        if (e.first == sys)
          {
            e.second.sv = sv;
            memcpy (e.second.key, key, sizeof key);
            placed = true;
          }
      if (!placed)
        {
          AdjShadow sh;
          sh.sv = sv;
          memcpy (sh.key, key, sizeof key);
          g_shadow.push_back ({sys, sh});
        }
    }
  stokes_set_pos (sv, sys->pos);
  sv->rmin = sys->rmin;
  return sv;
}

static AdjState *
adj_state (Ctx *c)
{
  static std::mutex mu;
  static std::vector<std::pair<Ctx *, AdjState *>> all;
  std::lock_guard<std::mutex> lk (mu);
  for (auto &e : all)
    if (e.first == c) return e.second;
  AdjState *s = new AdjState ();
  all.push_back ({c, s});
  return s;
}

template <int V>
static cudaError_t
launch_adj (Ctx *c, const struct stokes *sys, AdjState *s, int nchunk, bool box, cudaStream_t st)
{
  const int np = c->np, nk = c->nk;
  AdjRealArgs a;
  a.pos = (const double *) c->pos.p;
  a.g = (const double *) s->g.p;
  a.f = (const double *) s->f.p;
  a.img = (const Img4 *) c->img.p;
  a.nimg = c->nimg;
  a.np = np;
  a.nchunk = nchunk;
  a.rmax2 = c->rmax2;
  a.rmin = c->rmin;
  a.xi = c->xi;
  a.xisp = c->xisp;
  a.lx = sys->lx;
  a.ly = sys->ly;
  a.lz = sys->lz;
  a.partial = (double *) s->partial.p;
  const long long warps = (long long) np * nchunk;
  k_adj_real<V><<<(int) ((warps + AR_WARPS - 1) / AR_WARPS), AR_WARPS * 32, 0, st>>> (a);
  kmark (c, st, "k_adj_real");
  if (nk > 0)
    {
      cudaError_t e = launch_phase_fp64 (a.pos, (const double *) c->kt.p, nk, np,
                                         (double2 *) s->ph.p, st);
      if (e != cudaSuccess) return e;
      kmark (c, st, "k_phase");
      k_adj_sfac<V><<<nk, 256, 0, st>>> (a.g, a.f, (const double2 *) s->ph.p,
                                         (const double *) c->kt.p, np, sys->xi2, sys->lx,
                                         sys->ly, sys->lz, box, (double *) s->wu.p,
                                         (double *) s->dbox.p);
      kmark (c, st, "k_adj_sfac");
      k_adj_backproj<V><<<(np + 3) / 4, 128, 0, st>>> (a.g, a.f, (const double2 *) s->ph.p,
                                                       (const double *) c->kt.p,
                                                       (const double *) s->wu.p, nk, np,
                                                       (double *) s->grad.p);
      kmark (c, st, "k_adj_backproj");
    }
  return cudaGetLastError ();
}

}  // namespace lsg

using namespace lsg;

extern "C" int
stokes_gpu_vjp (struct stokes *sys, const double *g, const double *f, double *dLdr,
                double *dLdbox, double *Lval)
{
  clear_error ();
  if (!sys || !g || !f || !dLdr) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (!sys->periodic) return set_error (STOKES_GPU_ENOTPERIODIC, "the adjoint serves periodic systems");
  if (sys->version > 1)
    return set_error (STOKES_GPU_EINVAL, "the adjoint serves the F and FT versions");
  if (sys->a || sys->slip)
    return set_error (STOKES_GPU_EINVAL, "the adjoint serves equal spheres without slip");
  if (dLdbox && sys->shear_mode != 0)
    return set_error (STOKES_GPU_EINVAL, "box derivatives are defined without shear");
  struct stokes *const usr = sys;
  {
    // mixed precision: the FP32 adjoint (adjoint_f32.cu) unless the system
    // needs the FP64 one (shear, or no minimum-image split)
    Ctx *cu = get_ctx (usr, true);
    if (!cu) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
    if (cu->precision == STOKES_GPU_MIXED)
      {
        const int done = vjp_mixed (cu, usr, g, f, dLdr, dLdbox);
        if (done < 0) return -done;
        if (done == 1)
          {
            if (Lval)
              {
                // L = g . M f with the mixed product
                const size_t n = (size_t) NCOMP (usr->version) * usr->np;
                std::vector<double> y (n);
                const int rc = stokes_gpu_atimes (usr, f, y.data ());
                if (rc) return rc;
                double v = 0.0;
                for (size_t q = 0; q < n; q++) v += g[q] * y[q];
                *Lval = v;
              }
            return STOKES_GPU_OK;
          }
      }
  }
  {
    const char *ev = getenv ("LIBSTOKES_GB300_VJP_ETA");
    const double eta = ev ? atof (ev) : 9.0;
    if (eta > 0.0) sys = adj_shadow (sys, eta);
  }
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  // the adjoint's own split (or, with eta 0, the system's): not the tuned
  // split of the FP64 products
  const bool tune = c->tune;
  c->tune = false;
  int rc = prepare (c, sys, false, 1);
  c->tune = tune;
  if (rc) return rc;
  const int np = sys->np, C = NCOMP (sys->version), nk = c->nk;
  const size_t n = (size_t) C * np;
  AdjState *s = adj_state (c);
  const int nchunk = std::max (1, std::min (64, (152 * 16 + np - 1) / np));
  cudaStream_t st = c->stream;
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair (&s->g, n), std::make_pair (&s->f, n),
                  std::make_pair (&s->ph, (size_t) 2 * std::max (nk, 1) * np),
                  std::make_pair (&s->wu, (size_t) std::max (nk, 1) * 4 * C),
                  std::make_pair (&s->dbox, (size_t) std::max (nk, 1) * 3),
                  std::make_pair (&s->partial, (size_t) nchunk * np * 6),
                  std::make_pair (&s->grad, (size_t) 3 * np)})
    if (e == cudaSuccess) e = pr.first->ensure (sizeof (double) * pr.second);
  if (e == cudaSuccess) e = c->pos.ensure (sizeof (double) * 3 * np);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync (s->g.p, g, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync (s->f.p, f, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail (e, "adjoint buffers");
  const bool box = dLdbox != nullptr;
  e = sys->version == 0 ? launch_adj<0> (c, sys, s, nchunk, box, st)
                        : launch_adj<1> (c, sys, s, nchunk, box, st);
  if (e != cudaSuccess) return cuda_fail (e, "adjoint kernels");
  std::vector<double> part ((size_t) nchunk * np * 6), grec ((size_t) 3 * np, 0.0),
    db ((size_t) 3 * std::max (nk, 1), 0.0);
  e = cudaMemcpyAsync (part.data (), s->partial.p, sizeof (double) * part.size (),
                       cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nk > 0)
    e = cudaMemcpyAsync (grec.data (), s->grad.p, sizeof (double) * grec.size (),
                         cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nk > 0 && box)
    e = cudaMemcpyAsync (db.data (), s->dbox.p, sizeof (double) * 3 * nk, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "adjoint results");
  // dL/dr = - sum grad psi (real) + reciprocal; box sums in FP64 on the host
  double bx[3] = {0, 0, 0}, phase[3] = {0, 0, 0};
  for (int l = 0; l < np; l++)
    {
      double gr[3] = {0, 0, 0};
      for (int ch = 0; ch < nchunk; ch++)
        {
          const double *p = &part[((size_t) ch * np + l) * 6];
          for (int a = 0; a < 3; a++)
            {
              gr[a] += p[a];
              bx[a] += p[3 + a];
            }
        }
      for (int a = 0; a < 3; a++)
        {
          dLdr[3 * l + a] = -gr[a] + grec[3 * l + a];
          phase[a] += sys->pos[3 * l + a] * grec[3 * l + a];
        }
    }
  if (box)
    {
      const double L[3] = {sys->lx, sys->ly, sys->lz};
      for (int a = 0; a < 3; a++)
        {
          double opd = 0.0;
          for (int k = 0; k < nk; k++) opd += db[3 * (size_t) k + a];
          dLdbox[a] = bx[a] + opd - phase[a] / L[a];
        }
    }
  if (Lval)
    {
      // L = g . M f with the FP64 product itself
      std::vector<double> y (n);
      Ctx *cu = get_ctx (usr, true);
      if (!cu) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
      const int prec = cu->precision;
      cu->precision = STOKES_GPU_FP64;
      rc = stokes_gpu_atimes (usr, f, y.data ());
      cu->precision = prec;
      if (rc) return rc;
      double v = 0.0;
      for (size_t q = 0; q < n; q++) v += g[q] * y[q];
      *Lval = v;
    }
  c->launches = 1 + (nk > 0 ? 3 : 0);
  return STOKES_GPU_OK;
}

namespace lsg {
// the VJP's private copy of sys (when sys goes away)
void
release_adjoint (const struct stokes *sys)
{
  struct stokes *sv = nullptr;
  {
    std::lock_guard<std::mutex> lk (g_shadow_mu);
    for (size_t i = 0; i < g_shadow.size (); i++)
      if (g_shadow[i].first == sys)
        {
          sv = g_shadow[i].second.sv;
          g_shadow.erase (g_shadow.begin () + (long) i);
          break;
        }
  }
  if (sv) stokes_free (sv);
}
}  // namespace lsg
