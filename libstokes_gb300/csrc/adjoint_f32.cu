// adjoint_f32.cu -- mixed-precision vector-Jacobian product of the Ewald
// mobility product: for L = g^T M(r, box) f, the gradient dL/dr and the box
// derivatives dL/dl_a, with the arithmetic of the mixed product (FP32 terms,
// fixed-point positions, FP64 final sums).  The mathematics is that of the
// FP64 adjoint (adjoint.cu):
//
//   real space        dL/dr_l = - sum_(j,m) grad_d psi(d),
//                     psi(d) = phi_lj(d) + phi_jl(-d), phi_ij = g_i R(d) f_j,
//                     dL/dl_a = sum n_(m,a) d_a phi_lj  (d = r_j - r_l + n L)
//   reciprocal space  dL/dr_l = sum_k k Im[e^{-ik.r_l} (g_l . W_k + f_l . U_k)],
//                     W = op S_f, U = op S_g, S_x(k) = sum_j e^{ik.r_j} x_j;
//                     box: the op's derivative Re conj(S_g) . (d op / d l_a) S_f
//                     and the phase scaling -(1/l_a) sum_l r_(l,a) dL_rec/dr_(l,a).
//
// With f and g real, the k and -k terms of both reciprocal sums are equal, so
// the sums run over half of k space and count twice.
//
// Split: the VJP's own, chosen like the mixed product's: xi = eta / V^(1/3)
// with eta = 10 or the smallest xi whose real-space cutoff is below half the
// box (one image per pair), whichever is larger; cutoffs from libstokes'
// estimators at tolerance 3e-8.  L does not depend on the split once both
// sums converge.  Systems for which that would need xi a > 0.5 (a few
// spheres in a small box), and sheared systems, take the FP64 adjoint.
//
// Kernels:
//   kva_prep    fixed-point positions (32 bits per axis: exact differences,
//               the periodic wrap is the integer overflow), g and f in FP32,
//               per-axis phase tables e^{2 pi i m u} from the exact phase m q
//   kva_real    one warp per (target, source chunk); candidates compacted
//               into a per-warp queue; FP32 forward-mode duals (value and
//               three partials) through the pair scalars and tensors
//   kva_sfac    one warp per half-space k: S_f, S_g over the particles, then
//               W and U, and the op's box derivative (duals in the box)
//   kva_bp      one thread per particle and a slice of k; W_k, U_k staged in
//               shared memory and read by every thread (broadcast); the phase
//               of consecutive k with the same (m1, m2) reuses its m1 m2 part
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "stokes_gpu.h"

extern "C" void lsg_ewald_cutoffs (double xi, double eps, double lmin, double lmax,
                                   double *rmax_out, double *kmax_out);

namespace lsg {

// FP32 value and three partial derivatives
struct DF {
  float v, d[3];
  __host__ __device__ DF () : v (0.f), d{0.f, 0.f, 0.f} {}
  __host__ __device__ DF (double x) : v ((float) x), d{0.f, 0.f, 0.f} {}
};
__device__ inline DF operator+ (const DF &a, const DF &b)
{ DF r; r.v = a.v + b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] + b.d[k]; return r; }
__device__ inline DF operator- (const DF &a, const DF &b)
{ DF r; r.v = a.v - b.v; for (int k = 0; k < 3; k++) r.d[k] = a.d[k] - b.d[k]; return r; }
__device__ inline DF operator- (const DF &a)
{ DF r; r.v = -a.v; for (int k = 0; k < 3; k++) r.d[k] = -a.d[k]; return r; }
__device__ inline DF operator* (const DF &a, const DF &b)
{
  DF r;
  r.v = a.v * b.v;
  for (int k = 0; k < 3; k++) r.d[k] = fmaf (a.d[k], b.v, a.v * b.d[k]);
  return r;
}
__device__ inline DF operator/ (const DF &a, const DF &b)
{
  DF r;
  const float ib = 1.0f / b.v;
  r.v = a.v * ib;
  for (int k = 0; k < 3; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
__device__ inline DF &operator+= (DF &a, const DF &b) { a = a + b; return a; }
__device__ inline DF &operator-= (DF &a, const DF &b) { a = a - b; return a; }
// a function of one variable with value fv and derivative dv at a.v
__device__ inline DF dchain (const DF &a, float fv, float dv)
{ DF r; r.v = fv; for (int k = 0; k < 3; k++) r.d[k] = dv * a.d[k]; return r; }

template <> __device__ __forceinline__ DF dev_erfc<DF> (DF x)
{
  // d/dx erfc(x) = -2/sqrt(pi) exp(-x^2)
  return dchain (x, erfcf (x.v), -1.1283791670955126f * __expf (-x.v * x.v));
}
template <> __device__ __forceinline__ DF dev_exp<DF> (DF x)
{
  const float e = __expf (x.v);
  return dchain (x, e, e);
}
template <> __device__ __forceinline__ DF dev_sqrt<DF> (DF x)
{
  const float s = sqrtf (x.v);
  return dchain (x, s, 0.5f / s);
}

namespace {

// one half-space reciprocal vector (64 bytes)
struct __align__ (16) VjpK {
  int m1, m2, m3, pad;
  float kx, ky, kz, kn;
  float ex, ey, ez, ya;
  float yb, yc, kk, kexp;
};

__device__ __forceinline__ float2
cmulf (float2 a, float2 b)
{
  return make_float2 (a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// tab[|m| stride + j], conjugated for negative m
__device__ __forceinline__ float2
tabm (const float2 *t, int m, int stride, int j)
{
  const float2 v = t[(size_t) (m < 0 ? -m : m) * stride + j];
  return m < 0 ? make_float2 (v.x, -v.y) : v;
}

constexpr int VJ_CP = 8;   // FP32 g and f per particle, padded (F: 3, FT: 6)

struct VjpArgs {
  const double *pos;        // [np][3] FP64 (as given)
  const double *g, *f;      // FP64 [np c]
  int np;
  double sx, sy, sz;        // 2^32 / L_d
  float scale[3];           // L_d / 2^32
  float L[3];
  float xi, xisp, rc2, rmin;
  uint4 *q;                 // [np] fixed-point x, y, z
  float *gf;                // [np][2][VJ_CP]: g then f (per-pair gathers)
  float *gcm;               // [2][c][np]: g then f, component-major (coalesced sums)
  float3 *p32;              // [np] FP32 positions as given (box derivative)
  float2 *tab;              // [(M0+1) + (M1+1) + (M2+1)][np]
  int M0, M1, M2;
  const float4 *rot;
  const VjpK *kt;
  int nk;
  float *wu;                // [nk][4 c]: W re, W im, U re, U im
  float *dbox;              // [nk][3] or NULL
  float *part;              // [nchunk][np][6]
  int nchunk;
  float *grad;              // [kchunks][np][3]
  int kchunks;
  double *dldr;             // [np][3] the gradient (FP64)
  double *blk;              // [blocks of kva_final][6]: box sums, phase sums
};

__device__ __forceinline__ uint32_t
fixq32 (double v)
{
  return (uint32_t) (unsigned long long) __double2ll_rd (v);
}

template <int V>
__global__ void __launch_bounds__ (128)
kva_prep (VjpArgs a)
{
  constexpr int C = NComp<V>::value;
  const int j = blockIdx.x * 128 + threadIdx.x;
  if (j >= a.np) return;
  const double x = a.pos[3 * j], y = a.pos[3 * j + 1], z = a.pos[3 * j + 2];
  const uint32_t q0 = fixq32 (x * a.sx), q1 = fixq32 (y * a.sy), q2 = fixq32 (z * a.sz);
  a.q[j] = make_uint4 (q0, q1, q2, 0u);
  a.p32[j] = make_float3 ((float) x, (float) y, (float) z);
  for (int c = 0; c < C; c++)
    {
      const float gv = (float) a.g[(size_t) C * j + c], fv = (float) a.f[(size_t) C * j + c];
      a.gf[(size_t) j * 2 * VJ_CP + c] = gv;
      a.gf[(size_t) j * 2 * VJ_CP + VJ_CP + c] = fv;
      a.gcm[(size_t) c * a.np + j] = gv;
      a.gcm[(size_t) (C + c) * a.np + j] = fv;
    }
  // phase tables, m >= 0 per axis
  const int Md[3] = {a.M0, a.M1, a.M2};
  const uint32_t qd[3] = {q0, q1, q2};
  int row = 0;
  for (int d = 0; d < 3; d++)
    for (int m = 0; m <= Md[d]; m++, row++)
      a.tab[(size_t) row * a.np + j] = phase_of (a.rot, (uint32_t) m * qd[d]);
}

// the phase e^{ik.r_j} of half-space vector k from the tables
__device__ __forceinline__ float2
kphase (const VjpArgs &a, const VjpK &K, int j)
{
  const float2 *t0 = a.tab, *t1 = t0 + (size_t) (a.M0 + 1) * a.np,
               *t2 = t1 + (size_t) (a.M1 + 1) * a.np;
  return cmulf (cmulf (t0[(size_t) K.m1 * a.np + j], tabm (t1, K.m2, a.np, j)),
                tabm (t2, K.m3, a.np, j));
}

// e^{2 pi i p / 2^32} from the rotation table in shared memory (phase_of)
__device__ __forceinline__ float2
phase_s (const float4 *srot, uint32_t p)
{
  const uint32_t h = (p + (1u << 21)) >> 22;
  const int32_t r = (int32_t) (p - (h << 22));
  const float th = (float) r * 1.4629180792671596e-09f;
  const float t2 = th * th;
  const float sn = th * (1.0f - t2 * (1.0f / 6.0f));
  const float dc = t2 * (0.5f - t2 * (1.0f / 24.0f));
  const float4 e = srot[h & 1023u];
  const float re = e.x + fmaf (-e.x, dc, fmaf (-e.y, sn, e.z));
  const float im = e.y + fmaf (-e.y, dc, fmaf (e.x, sn, e.w));
  return make_float2 (re, im);
}

// ---------------------------------------------------------------------------
// reciprocal space
// ---------------------------------------------------------------------------
constexpr int SF_T = 256;     // k vectors per CTA of kva_sfac (one per thread)
constexpr int SF_P = 128;     // particles per slice

// partial structure factors of one particle slice: thread = one k; the
// slice's fixed-point positions and g, f sit in shared memory (read by every
// thread alike), the phase e^{ik.r_j} is the exact fixed-point phase
// m1 q_x + m2 q_y + m3 q_z mod 2^32 through the rotation table.
// out: sfp[slice][4 c][nk] = (cos f, sin f, cos g, sin g) sums
template <int V>
__global__ void __launch_bounds__ (SF_T)
kva_sfac (VjpArgs a, float *sfp)
{
  constexpr int C = NComp<V>::value;
  __shared__ float4 s_rot[1024];
  __shared__ uint4 s_q[SF_P];
  __shared__ float s_x[SF_P][2 * C];
  for (int e = threadIdx.x; e < 1024; e += SF_T) s_rot[e] = a.rot[e];
  const int j0 = blockIdx.y * SF_P, nj = min (SF_P, a.np - j0);
  for (int e = threadIdx.x; e < nj; e += SF_T) s_q[e] = a.q[j0 + e];
  for (int e = threadIdx.x; e < nj * 2 * C; e += SF_T)
    {
      const int jl = e / (2 * C), c = e - jl * 2 * C;
      s_x[jl][c] = a.gf[(size_t) (j0 + jl) * 2 * VJ_CP + (c < C ? c : VJ_CP + c - C)];
    }
  __syncthreads ();
  const int k = blockIdx.x * SF_T + threadIdx.x;
  if (k >= a.nk) return;
  const VjpK K = a.kt[k];
  const uint32_t m1 = (uint32_t) K.m1, m2 = (uint32_t) K.m2, m3 = (uint32_t) K.m3;
  float cf[C], sf[C], cg[C], sg[C];
#pragma unroll
  for (int q = 0; q < C; q++) cf[q] = sf[q] = cg[q] = sg[q] = 0.f;
  for (int jl = 0; jl < nj; jl++)
    {
      const uint4 qj = s_q[jl];
      const float2 ph = phase_s (s_rot, m1 * qj.x + m2 * qj.y + m3 * qj.z);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          const float gv = s_x[jl][q], fv = s_x[jl][C + q];
          cg[q] = fmaf (ph.x, gv, cg[q]);
          sg[q] = fmaf (ph.y, gv, sg[q]);
          cf[q] = fmaf (ph.x, fv, cf[q]);
          sf[q] = fmaf (ph.y, fv, sf[q]);
        }
    }
  float *o = sfp + (size_t) blockIdx.y * 4 * C * a.nk + k;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      o[(size_t) q * a.nk] = cf[q];
      o[(size_t) (C + q) * a.nk] = sf[q];
      o[(size_t) (2 * C + q) * a.nk] = cg[q];
      o[(size_t) (3 * C + q) * a.nk] = sg[q];
    }
}

// one thread per k: the slices' sums (fixed order), W = op S_f, U = op S_g,
// and the op's box derivative Re conj(S_g) . (d op / d l_a) S_f
template <int V>
__global__ void __launch_bounds__ (128)
kva_wu (VjpArgs a, const float *sfp, int nslices)
{
  constexpr int C = NComp<V>::value;
  const int k = blockIdx.x * 128 + threadIdx.x;
  if (k >= a.nk) return;
  float cf[C], sf[C], cg[C], sg[C];
#pragma unroll
  for (int q = 0; q < C; q++) cf[q] = sf[q] = cg[q] = sg[q] = 0.f;
  for (int sl = 0; sl < nslices; sl++)
    {
      const float *p = sfp + (size_t) sl * 4 * C * a.nk + k;
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          cf[q] += p[(size_t) q * a.nk];
          sf[q] += p[(size_t) (C + q) * a.nk];
          cg[q] += p[(size_t) (2 * C + q) * a.nk];
          sg[q] += p[(size_t) (3 * C + q) * a.nk];
        }
    }
  const VjpK K = a.kt[k];
  const float e[3] = {K.ex, K.ey, K.ez};
  float *o = a.wu + (size_t) k * 4 * C;
  // W = (Bc + i Bs)(C + i S): re = Bc C - Bs S, im = Bc S + Bs C
  for (int which = 0; which < 2; which++)
    {
      const float *Cs = which ? cg : cf, *Ss = which ? sg : sf;
      float ms[C];
#pragma unroll
      for (int q = 0; q < C; q++) ms[q] = -Ss[q];
      GenF<V, float> gc, gs, gms;
      load_genf<V, float> (Cs, gc);
      load_genf<V, float> (Ss, gs);
      load_genf<V, float> (ms, gms);
      GenU<V, float> P, Q;
      P.zero ();
      Q.zero ();
      recip_apply<V, float> (e, K.ya, K.yb, K.yc, 0.f, 0.f, 0.f, gc, gms, P);
      recip_apply<V, float> (e, K.ya, K.yb, K.yc, 0.f, 0.f, 0.f, gs, gc, Q);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          o[2 * C * which + q] = P.v[q];
          o[2 * C * which + C + q] = Q.v[q];
        }
    }
  if (!a.dbox) return;
  // the op as a function of the box lengths: k = 2 pi m / l, pi / V
  DF Lx (a.L[0]), Ly (a.L[1]), Lz (a.L[2]);
  Lx.d[0] = Ly.d[1] = Lz.d[2] = 1.f;
  const float tp = 6.283185307179586f;
  const DF kx = DF (tp * K.m1) / Lx, ky = DF (tp * K.m2) / Ly, kz = DF (tp * K.m3) / Lz;
  const DF kk = kx * kx + ky * ky + kz * kz;
  const DF kn = dev_sqrt<DF> (kk);
  const DF k4z = kk / DF (4.0 * (double) a.xi * (double) a.xi);
  const DF pivol = DF (M_PI) / (Lx * Ly * Lz);
  const DF kexp = pivol * (DF (1.0) + k4z * (DF (1.0) + DF (2.0) * k4z)) / kk * dev_exp<DF> (-k4z);
  const DF ya = DF (6.0) * (DF (1.0) - kk * DF (1.0 / 3.0)) * kexp;
  const DF yb = DF (3.0) * kn * kexp;
  const DF yc = DF (1.5) * kk * kexp;
  const DF ed[3] = {kx / kn, ky / kn, kz / kn};
  float msv[C];
#pragma unroll
  for (int q = 0; q < C; q++) msv[q] = -sf[q];
  GenF<V, DF> gc, gs, gms;
  {
    GenF<V, float> t1, t2, t3;
    load_genf<V, float> (cf, t1);
    load_genf<V, float> (sf, t2);
    load_genf<V, float> (msv, t3);
    for (int c = 0; c < 3; c++)
      {
        gc.F[c] = DF (t1.F[c]); gs.F[c] = DF (t2.F[c]); gms.F[c] = DF (t3.F[c]);
        if (V >= V_FT) { gc.T[c] = DF (t1.T[c]); gs.T[c] = DF (t2.T[c]); gms.T[c] = DF (t3.T[c]); }
      }
  }
  GenU<V, DF> P, Q;
  P.zero ();
  Q.zero ();
  recip_apply<V, DF> (ed, ya, yb, yc, DF (0.0), DF (0.0), DF (0.0), gc, gms, P);
  recip_apply<V, DF> (ed, ya, yb, yc, DF (0.0), DF (0.0), DF (0.0), gs, gc, Q);
  // Re conj(S_g) . dW = Cg . dP + Sg . dQ
  for (int c = 0; c < 3; c++)
    {
      float sacc = 0.f;
#pragma unroll
      for (int q = 0; q < C; q++) sacc = fmaf (cg[q], P.v[q].d[c], fmaf (sg[q], Q.v[q].d[c], sacc));
      a.dbox[(size_t) 3 * k + c] = sacc;
    }
}

// per particle l and a slice of k: sum_k k Im[e^{-ik.r_l} (g_l . W_k + f_l . U_k)],
// the phase from the fixed-point position through the rotation table
constexpr int BP_T = 128;     // particles per CTA
constexpr int BP_KT = 64;     // k vectors staged per tile

template <int V>
__global__ void __launch_bounds__ (BP_T)
kva_bp (VjpArgs a)
{
  constexpr int C = NComp<V>::value;
  __shared__ float4 s_rot[1024];
  __shared__ float s_wu[BP_KT][4 * C];
  __shared__ int4 s_m[BP_KT];
  __shared__ float4 s_kv[BP_KT];
  for (int e = threadIdx.x; e < 1024; e += BP_T) s_rot[e] = a.rot[e];
  const int l = blockIdx.x * BP_T + threadIdx.x;
  const bool live = l < a.np;
  const int lc = live ? l : 0;
  const int k0 = (int) ((long long) a.nk * blockIdx.y / a.kchunks);
  const int k1 = (int) ((long long) a.nk * (blockIdx.y + 1) / a.kchunks);
  float gl[C], fl[C];
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      gl[q] = a.gf[(size_t) lc * 2 * VJ_CP + q];
      fl[q] = a.gf[(size_t) lc * 2 * VJ_CP + VJ_CP + q];
    }
  const uint4 ql = a.q[lc];
  float gx = 0.f, gy = 0.f, gz = 0.f;
  for (int kb = k0; kb < k1; kb += BP_KT)
    {
      const int nt = min (BP_KT, k1 - kb);
      __syncthreads ();
      for (int e = threadIdx.x; e < nt * 4 * C; e += BP_T)
        s_wu[e / (4 * C)][e % (4 * C)] = a.wu[(size_t) kb * 4 * C + e];
      for (int e = threadIdx.x; e < nt; e += BP_T)
        {
          const VjpK K = a.kt[kb + e];
          s_m[e] = make_int4 (K.m1, K.m2, K.m3, 0);
          s_kv[e] = make_float4 (K.kx, K.ky, K.kz, 0.f);
        }
      __syncthreads ();
#pragma unroll 4
      for (int t = 0; t < nt; t++)
        {
          const int4 m = s_m[t];
          const float2 ph = phase_s (s_rot, (uint32_t) m.x * ql.x + (uint32_t) m.y * ql.y
                                              + (uint32_t) m.z * ql.z);
          float hr = 0.f, hi = 0.f;
#pragma unroll
          for (int q = 0; q < C; q++)
            {
              hr = fmaf (gl[q], s_wu[t][q], fmaf (fl[q], s_wu[t][2 * C + q], hr));
              hi = fmaf (gl[q], s_wu[t][C + q], fmaf (fl[q], s_wu[t][3 * C + q], hi));
            }
          // Im[(cos - i sin)(hr + i hi)] = cos hi - sin hr
          const float im = ph.x * hi - ph.y * hr;
          const float4 kv = s_kv[t];
          gx = fmaf (kv.x, im, gx);
          gy = fmaf (kv.y, im, gy);
          gz = fmaf (kv.z, im, gz);
        }
    }
  if (!live) return;
  float *o = a.grad + ((size_t) blockIdx.y * a.np + l) * 3;
  o[0] = gx;
  o[1] = gy;
  o[2] = gz;
}

// ---------------------------------------------------------------------------
// real space: per (target l, source chunk) the sums of grad psi and of
// n (x) grad phi_lj over the accepted pairs, FP32 duals
// ---------------------------------------------------------------------------
constexpr int AR_W = 4;
constexpr int AR_Q = 64;

template <int V>
__device__ __forceinline__ void
kva_term (const VjpArgs &a, int l, float4 q, float out[6])
{
  constexpr int C = NComp<V>::value;
  const int j = __float_as_int (q.w);
  DF d[3];
  d[0] = DF (q.x); d[0].d[0] = 1.f;
  d[1] = DF (q.y); d[1].d[1] = 1.f;
  d[2] = DF (q.z); d[2].d[2] = 1.f;
  DF r = dev_sqrt<DF> (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const float rm = 2.f * a.rmin;
  if (r.v < rm) r = DF (rm);                 // the clamp: no radial dependence
  const DF e[3] = {d[0] / r, d[1] / r, d[2] / r};
  const DF me[3] = {-e[0], -e[1], -e[2]};
  PairScalars<DF> s;
  real_scalars_mono<V, DF> (DF (a.xi), DF (a.xisp), r, s);
  GenF<V, DF> fj, fl;
  {
    const float *gj = a.gf + (size_t) j * 2 * VJ_CP + VJ_CP;
    const float *gl = a.gf + (size_t) l * 2 * VJ_CP + VJ_CP;
    for (int c = 0; c < 3; c++)
      {
        fj.F[c] = DF (gj[c]);
        fl.F[c] = DF (gl[c]);
        if (V >= V_FT)
          {
            fj.T[c] = DF (gj[3 + c]);
            fl.T[c] = DF (gl[3 + c]);
          }
      }
  }
  GenU<V, DF> u1, u2;
  u1.zero ();
  u2.zero ();
  pair_apply<V, DF> (e, s, fj, u1);          // R(d) f_j
  pair_apply<V, DF> (me, s, fl, u2);         // R(-d) f_l
  DF p1, p2;
  for (int c = 0; c < C; c++)
    {
      p1 += DF (a.gf[(size_t) l * 2 * VJ_CP + c]) * u1.v[c];   // phi_lj(d)
      p2 += DF (a.gf[(size_t) j * 2 * VJ_CP + c]) * u2.v[c];   // phi_jl(-d)
    }
  for (int k = 0; k < 3; k++) out[k] += p1.d[k] + p2.d[k];
  // box: n (x) grad phi_lj, n the lattice vector of the minimum image
  const float3 pj = a.p32[j], pl = a.p32[l];
  out[3] += p1.d[0] * rintf ((q.x - (pj.x - pl.x)) / a.L[0]);
  out[4] += p1.d[1] * rintf ((q.y - (pj.y - pl.y)) / a.L[1]);
  out[5] += p1.d[2] * rintf ((q.z - (pj.z - pl.z)) / a.L[2]);
}

template <int V>
__global__ void __launch_bounds__ (AR_W * 32)
kva_real (VjpArgs a)
{
  __shared__ float4 s_q[AR_W][AR_Q];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * AR_W + wib;
  if (w >= (long long) a.np * a.nchunk) return;
  const int l = (int) (w % a.np), chunk = (int) (w / a.np);
  const int j0 = (int) ((long long) a.np * chunk / a.nchunk);
  const int j1 = (int) ((long long) a.np * (chunk + 1) / a.nchunk);
  const uint4 ql = a.q[l];
  float out[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int qn = 0;
  const unsigned lt = (1u << lane) - 1u;
  float4 *qq = s_q[wib];
  for (int jb = j0; jb < j1; jb += 32)
    {
      const int j = jb + lane;
      bool ok = false;
      float dx = 0.f, dy = 0.f, dz = 0.f;
      if (j < j1)
        {
          const uint4 qj = a.q[j];
          dx = (float) (int32_t) (qj.x - ql.x) * a.scale[0];
          dy = (float) (int32_t) (qj.y - ql.y) * a.scale[1];
          dz = (float) (int32_t) (qj.z - ql.z) * a.scale[2];
          const float rr = dx * dx + dy * dy + dz * dz;
          ok = rr > 0.f && rr < a.rc2;
        }
      const unsigned b = __ballot_sync (0xffffffffu, ok);
      if (ok) qq[qn + __popc (b & lt)] = make_float4 (dx, dy, dz, __int_as_float (j));
      qn += __popc (b);
      __syncwarp ();
      if (qn >= 32)
        {
          kva_term<V> (a, l, qq[qn - 32 + lane], out);
          qn -= 32;
          __syncwarp ();
        }
    }
  if (lane < qn) kva_term<V> (a, l, qq[lane], out);
  float *o = a.part + ((size_t) chunk * a.np + l) * 6;
#pragma unroll
  for (int k = 0; k < 6; k++)
    {
      const float v = warp_sum (out[k]);
      if (lane == 0) o[k] = v;
    }
}

// the gradient per particle in FP64 (real-space chunks, twice the half-space
// reciprocal slices; one warp per particle, lanes over the chunks) and, per
// block, the sums of the real-space box terms and of r_l,a dL_rec/dr_l,a
// (the phase scaling of the box derivative)
constexpr int FIN_T = 256;
constexpr int FIN_P = FIN_T / 32;   // particles per block

__global__ void __launch_bounds__ (FIN_T)
kva_final (VjpArgs a)
{
  __shared__ double s_b[FIN_P][6];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int l = blockIdx.x * FIN_P + w;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};      // grad psi, box, reciprocal
  if (l < a.np)
    {
      for (int ch = lane; ch < a.nchunk; ch += 32)
        {
          const float *p = a.part + ((size_t) ch * a.np + l) * 6;
          for (int k = 0; k < 6; k++) v[k] += p[k];
        }
      if (a.nk > 0)
        for (int kc = lane; kc < a.kchunks; kc += 32)
          for (int k = 0; k < 3; k++) v[6 + k] += a.grad[((size_t) kc * a.np + l) * 3 + k];
    }
  for (int k = 0; k < 9; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync (0xffffffffu, v[k], o);
  if (lane == 0)
    {
      double b[6] = {0, 0, 0, 0, 0, 0};
      if (l < a.np)
        for (int k = 0; k < 3; k++)
          {
            const double rec = 2.0 * v[6 + k];
            a.dldr[3 * l + k] = -v[k] + rec;
            b[k] = v[3 + k];
            b[3 + k] = a.pos[3 * l + k] * rec;
          }
      for (int k = 0; k < 6; k++) s_b[w][k] = b[k];
    }
  __syncthreads ();
  if (threadIdx.x < 6)
    {
      double t = 0.0;
      for (int p = 0; p < FIN_P; p++) t += s_b[p][threadIdx.x];
      a.blk[(size_t) blockIdx.x * 6 + threadIdx.x] = t;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct VjpState {
  uint64_t key = 0;
  double xi = 0.0, rc = 0.0, kc = 0.0;
  int M[3] = {0, 0, 0};
  int nk = 0;
  std::vector<VjpK> hk;
  uint64_t uploaded = 0;        // split whose k table and rotations are on the device
  DevBuf q, gf, gcm, p32, tab, kt, wu, dbox, part, grad, rot, g, f, pos, dldr, blk, sfp;
};

std::mutex g_vjp_mu;
std::vector<std::pair<const Ctx *, VjpState *>> g_vjp;

VjpState *
vjp_state (const Ctx *c)
{
  std::lock_guard<std::mutex> lk (g_vjp_mu);
  for (auto &e : g_vjp)
    if (e.first == c) return e.second;
  VjpState *s = new VjpState ();
  g_vjp.push_back ({c, s});
  return s;
}

double
vjp_eta ()
{
  const char *e = getenv ("LIBSTOKES_GB300_VJP_MIXED_ETA");   // read per call: sweeps
  return e ? atof (e) : 10.0;
}

uint64_t
vjp_key (const struct stokes *sys)
{
  const double v[6] = {sys->lx, sys->ly, sys->lz, (double) sys->np, (double) sys->version,
                       vjp_eta ()};
  uint64_t h = 1469598103934665603ull;
  const unsigned char *b = (const unsigned char *) v;
  for (size_t i = 0; i < sizeof v; i++) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

// the VJP's split and half-space k list; false when no minimum-image split
// with xi a <= 0.5 exists
bool
vjp_split (const struct stokes *sys, VjpState *s)
{
  const uint64_t key = vjp_key (sys);
  if (key == s->key && s->nk >= 0 && s->xi > 0.0) return true;
  const double eps = 3e-8;
  const double lmin = std::min (sys->lx, std::min (sys->ly, sys->lz));
  const double lmax = std::max (sys->lx, std::max (sys->ly, sys->lz));
  const double lv = cbrt (sys->lx * sys->ly * sys->lz);
  // the smallest xi whose cutoff is below half the box, and at least
  // eta / V^(1/3)
  double xi = 6.0 / lv, rc = 0.0, kc = 0.0;
  for (int it = 0; it < 400; it++)
    {
      lsg_ewald_cutoffs (xi, eps, lmin, lmax, &rc, &kc);
      if (rc <= 0.4999 * lmin) break;
      xi *= 1.02;
    }
  if (rc > 0.4999 * lmin || xi > 0.5) return false;
  const double eta = vjp_eta ();
  if (xi < eta / lv && eta / lv <= 0.5)
    {
      xi = eta / lv;
      lsg_ewald_cutoffs (xi, eps, lmin, lmax, &rc, &kc);
    }
  const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly, k0z = 2.0 * M_PI / sys->lz;
  const double pivol = M_PI / (sys->lx * sys->ly * sys->lz), xi2 = xi * xi;
  const int B1 = (int) (kc / k0x) + 1, B2 = (int) (kc / k0y) + 1, B3 = (int) (kc / k0z) + 1;
  s->hk.clear ();
  int M[3] = {0, 0, 0};
  for (int m1 = 0; m1 <= B1; m1++)
    for (int m2 = -B2; m2 <= B2; m2++)
      for (int m3 = -B3; m3 <= B3; m3++)
        {
          if (m1 == 0 && (m2 < 0 || (m2 == 0 && m3 <= 0))) continue;
          const double k1 = k0x * m1, k2 = k0y * m2, k3 = k0z * m3;
          const double kk = k1 * k1 + k2 * k2 + k3 * k3, k = sqrt (kk);
          if (k > kc) continue;
          const double k4z = kk / 4.0 / xi2;
          const double kexp = pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          VjpK r;
          memset (&r, 0, sizeof r);
          r.m1 = m1; r.m2 = m2; r.m3 = m3;
          r.kx = (float) k1; r.ky = (float) k2; r.kz = (float) k3; r.kn = (float) k;
          r.ex = (float) (k1 / k); r.ey = (float) (k2 / k); r.ez = (float) (k3 / k);
          r.ya = (float) (6.0 * (1.0 - kk / 3.0) * kexp);
          r.yb = (float) (3.0 * k * kexp);
          r.yc = (float) (1.5 * kk * kexp);
          r.kk = (float) kk;
          r.kexp = (float) kexp;
          s->hk.push_back (r);
          M[0] = std::max (M[0], m1);
          M[1] = std::max (M[1], abs (m2));
          M[2] = std::max (M[2], abs (m3));
        }
  s->xi = xi;
  s->rc = rc;
  s->kc = kc;
  s->nk = (int) s->hk.size ();
  for (int d = 0; d < 3; d++) s->M[d] = M[d];
  s->key = key;
  return true;
}

template <int V>
int
vjp_mixed_v (Ctx *c, const struct stokes *sys, VjpState *s, const double *g, const double *f,
             double *dLdr, double *dLdbox)
{
  constexpr int C = NComp<V>::value;
  const int np = sys->np, nk = s->nk;
  const size_t n = (size_t) C * np;
  cudaStream_t st = c->stream;
  const int nchunk = std::max (1, std::min (16, (152 * 16 + np - 1) / np));
  const int kchunks = std::max (1, std::min (64, (152 * 8 * BP_T + np - 1) / np));
  const int ntab = (s->M[0] + 1) + (s->M[1] + 1) + (s->M[2] + 1);
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair (&s->q, sizeof (uint4) * np),
                  std::make_pair (&s->gf, sizeof (float) * 2 * VJ_CP * np),
                  std::make_pair (&s->gcm, sizeof (float) * 2 * C * np),
                  std::make_pair (&s->dldr, sizeof (double) * 3 * np),
                  std::make_pair (&s->blk, sizeof (double) * 6 * ((np + FIN_P - 1) / FIN_P)),
                  std::make_pair (&s->sfp, sizeof (float) * 4 * C * (size_t) std::max (nk, 1)
                                             * ((np + SF_P - 1) / SF_P)),
                  std::make_pair (&s->p32, sizeof (float3) * np),
                  std::make_pair (&s->tab, sizeof (float2) * (size_t) ntab * np),
                  std::make_pair (&s->kt, sizeof (VjpK) * std::max (nk, 1)),
                  std::make_pair (&s->wu, sizeof (float) * 4 * C * std::max (nk, 1)),
                  std::make_pair (&s->dbox, sizeof (float) * 3 * std::max (nk, 1)),
                  std::make_pair (&s->part, sizeof (float) * 6 * (size_t) nchunk * np),
                  std::make_pair (&s->grad, sizeof (float) * 3 * (size_t) kchunks * np),
                  std::make_pair (&s->rot, sizeof (float) * 4 * 1024),
                  std::make_pair (&s->g, sizeof (double) * n),
                  std::make_pair (&s->f, sizeof (double) * n),
                  std::make_pair (&s->pos, sizeof (double) * 3 * np)})
    if (e == cudaSuccess) e = pr.first->ensure (pr.second);
  if (e != cudaSuccess) return cuda_fail (e, "mixed VJP buffers");
  // 1024 rotations e^{2 pi i h / 1024} as FP32 pairs hi + lo (phase_of) and
  // the k table, when the split (or the buffers) changed
  if (s->uploaded != (s->key ^ (uint64_t) (uintptr_t) s->kt.p))
  {
    std::vector<float> h (4 * 1024);
    for (int k = 0; k < 1024; k++)
      {
        const double c0 = cos (2.0 * M_PI * k / 1024.0), s0 = sin (2.0 * M_PI * k / 1024.0);
        h[4 * k] = (float) c0;
        h[4 * k + 1] = (float) s0;
        h[4 * k + 2] = (float) (c0 - (double) h[4 * k]);
        h[4 * k + 3] = (float) (s0 - (double) h[4 * k + 1]);
      }
    e = cudaMemcpyAsync (s->rot.p, h.data (), sizeof (float) * h.size (), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nk)
      e = cudaMemcpyAsync (s->kt.p, s->hk.data (), sizeof (VjpK) * nk, cudaMemcpyHostToDevice, st);
    // h is local: the copy must end before it goes away
    if (e == cudaSuccess) e = cudaStreamSynchronize (st);
    if (e != cudaSuccess) return cuda_fail (e, "mixed VJP tables");
    s->uploaded = s->key ^ (uint64_t) (uintptr_t) s->kt.p;
  }
  e = cudaMemcpyAsync (s->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (s->g.p, g, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (s->f.p, f, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail (e, "mixed VJP upload");
  VjpArgs a;
  memset (&a, 0, sizeof a);
  a.pos = (const double *) s->pos.p;
  a.g = (const double *) s->g.p;
  a.f = (const double *) s->f.p;
  a.np = np;
  const double two32 = 4294967296.0;
  a.sx = two32 / sys->lx; a.sy = two32 / sys->ly; a.sz = two32 / sys->lz;
  a.scale[0] = (float) (sys->lx / two32);
  a.scale[1] = (float) (sys->ly / two32);
  a.scale[2] = (float) (sys->lz / two32);
  a.L[0] = (float) sys->lx; a.L[1] = (float) sys->ly; a.L[2] = (float) sys->lz;
  a.xi = (float) s->xi;
  a.xisp = (float) (s->xi / sqrt (M_PI));
  a.rc2 = (float) (s->rc * s->rc);
  a.rmin = (float) sys->rmin;
  a.q = (uint4 *) s->q.p;
  a.gf = (float *) s->gf.p;
  a.gcm = (float *) s->gcm.p;
  a.dldr = (double *) s->dldr.p;
  a.blk = (double *) s->blk.p;
  a.p32 = (float3 *) s->p32.p;
  a.tab = (float2 *) s->tab.p;
  a.M0 = s->M[0]; a.M1 = s->M[1]; a.M2 = s->M[2];
  a.rot = (const float4 *) s->rot.p;
  a.kt = (const VjpK *) s->kt.p;
  a.nk = nk;
  a.wu = (float *) s->wu.p;
  a.dbox = dLdbox ? (float *) s->dbox.p : nullptr;
  a.part = (float *) s->part.p;
  a.nchunk = nchunk;
  a.grad = (float *) s->grad.p;
  a.kchunks = kchunks;
  kmark (c, st, nullptr);
  kva_prep<V><<<(np + 127) / 128, 128, 0, st>>> (a);
  kmark (c, st, "kva_prep");
  const long long warps = (long long) np * nchunk;
  kva_real<V><<<(int) ((warps + AR_W - 1) / AR_W), AR_W * 32, 0, st>>> (a);
  kmark (c, st, "kva_real");
  if (nk > 0)
    {
      const int nsl = (np + SF_P - 1) / SF_P;
      kva_sfac<V><<<dim3 ((nk + SF_T - 1) / SF_T, nsl), SF_T, 0, st>>> (a, (float *) s->sfp.p);
      kmark (c, st, "kva_sfac");
      kva_wu<V><<<(nk + 127) / 128, 128, 0, st>>> (a, (const float *) s->sfp.p, nsl);
      kmark (c, st, "kva_wu");
      kva_bp<V><<<dim3 ((np + BP_T - 1) / BP_T, kchunks), BP_T, 0, st>>> (a);
      kmark (c, st, "kva_bp");
    }
  const int nblk = (np + FIN_P - 1) / FIN_P;
  kva_final<<<nblk, FIN_T, 0, st>>> (a);
  kmark (c, st, "kva_final");
  if ((e = cudaGetLastError ()) != cudaSuccess) return cuda_fail (e, "mixed VJP kernels");
  std::vector<double> blk ((size_t) 6 * nblk);
  std::vector<float> db ((size_t) 3 * std::max (nk, 1), 0.f);
  e = cudaMemcpyAsync (dLdr, s->dldr.p, sizeof (double) * 3 * np, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (blk.data (), s->blk.p, sizeof (double) * blk.size (),
                         cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && nk > 0 && dLdbox)
    e = cudaMemcpyAsync (db.data (), s->dbox.p, sizeof (float) * 3 * nk, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "mixed VJP results");
  if (dLdbox)
    {
      double bx[3] = {0, 0, 0}, phase[3] = {0, 0, 0};
      for (int b = 0; b < nblk; b++)
        for (int k = 0; k < 3; k++)
          {
            bx[k] += blk[(size_t) b * 6 + k];
            phase[k] += blk[(size_t) b * 6 + 3 + k];
          }
      const double L[3] = {sys->lx, sys->ly, sys->lz};
      for (int k = 0; k < 3; k++)
        {
          double opd = 0.0;
          for (int q = 0; q < nk; q++) opd += db[3 * (size_t) q + k];
          dLdbox[k] = bx[k] + 2.0 * opd - phase[k] / L[k];
        }
    }
  c->launches = 3 + (nk > 0 ? 3 : 0);
  return STOKES_GPU_OK;
}

}  // namespace

// 1 when the mixed VJP served the call (result in dLdr, dLdbox), 0 when the
// system needs the FP64 adjoint (shear, no minimum-image split), < 0 on error
// (the status is then -rc)
int
vjp_mixed (Ctx *c, const struct stokes *sys, const double *g, const double *f, double *dLdr,
           double *dLdbox)
{
  if (sys->shear_mode != 0) return 0;
  VjpState *s = vjp_state (c);
  if (!vjp_split (sys, s)) return 0;
  const int rc = sys->version == 0 ? vjp_mixed_v<0> (c, sys, s, g, f, dLdr, dLdbox)
                                   : vjp_mixed_v<1> (c, sys, s, g, f, dLdr, dLdbox);
  return rc ? -rc : 1;
}

void
release_vjp_mixed (const Ctx *c)
{
  VjpState *s = nullptr;
  {
    std::lock_guard<std::mutex> lk (g_vjp_mu);
    for (size_t i = 0; i < g_vjp.size (); i++)
      if (g_vjp[i].first == c)
        {
          s = g_vjp[i].second;
          g_vjp.erase (g_vjp.begin () + (long) i);
          break;
        }
  }
  if (!s) return;
  for (DevBuf *b : {&s->q, &s->gf, &s->gcm, &s->p32, &s->tab, &s->kt, &s->wu, &s->dbox,
                    &s->part, &s->grad, &s->rot, &s->g, &s->f, &s->pos, &s->dldr, &s->blk,
                    &s->sfp})
    b->release ();
  delete s;
}

}  // namespace lsg
