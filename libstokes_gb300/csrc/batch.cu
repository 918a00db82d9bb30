// batch.cu -- many independent periodic systems in one go.
//
// A batch packs the particles of every system (positions, generalised
// forces and velocities in libstokes' own per-particle layout, system after
// system) and runs the product of all systems with a handful of launches
// over the whole batch -- no launch per system.  The launches are captured
// once in a CUDA graph and replayed.
//
// Mixed precision (the ensemble's path): every system gets its own split
// (the re-tuned xi = eta / V^(1/3) of the single-system mixed product, with
// the real-space cutoff below half the box so real space is minimum image),
// its own half-space k list and its own per-axis phase tables.  Launches:
//   mb_prep  (system, particle, axis): fixed-point positions, phase tables
//   mb_real  warp per (system, target, source chunk): FP32 pair sum
//   mb_sfac  warp per (system, k): structure factors and per-k operators
//   mb_bp    warp per (system, particle): back-projection over the system's
//            k list, then the FP64 self term and the final sum
// Work items map to systems by a binary search over per-system cumulative
// counts; a warp never spans two systems, so F and FT systems mix freely.
//
// FP64 (the reference split, parity at 1e-12): each system's FP64 product
// runs on its own branch of the same kind of graph.
//
// An autotuner picks, on the first product, the real-space source chunking
// and the warps per CTA of mb_real from a few timed candidates.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "stokes_gpu.h"

extern "C" void lsg_ewald_cutoffs (double xi, double eps, double lmin, double lmax,
                                   double *rmax_out, double *kmax_out);

namespace lsg {

struct BSys {
  int np, version, c, nchunk;
  int p_off, x_off;          // first particle, first vector element
  int tab_off;               // first float2 of the phase tables
  int M0, M1, M2;
  int k_off, nkh;            // first MixK, count
  int pq_off;                // first float of P | Q  ([2c][nkh])
  int pr_off;                // first float of the real partials ([nchunk][np][c])
  int img_off, nimg;         // lattice images added to the minimum-image difference
  int shear_mode;
  uint32_t shift_q;
  float scale[3];
  float rc2, rmin, xi, xisp;
  double lx, ly, lz, shift;
  double selfc[3];
};

// index of the system whose [cum[s], cum[s+1]) holds t
__device__ __forceinline__ int
find_sys (const int *cum, int nsys, long long t)
{
  int lo = 0, hi = nsys - 1;
  while (lo < hi)
    {
      const int mid = (lo + hi + 1) >> 1;
      if ((long long) cum[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
  return lo;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
struct BatchArgs {
  const BSys *sys;
  int nsys;
  const int *cum_p, *cum_r, *cum_k;     // particles, real warps, k warps
  const double *pos, *x;
  double *y;
  uint32_t *qpos;
  float2 *tab;
  float *xf;
  const MixK *kt;
  float *pq, *pr;
  const float4 *img;                    // per system: image vectors (x, y, z, 0)
};

__global__ void
mb_prep (BatchArgs a, int nptot)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int d = blockIdx.y;
  if (t >= nptot) return;
  const int s = find_sys (a.cum_p, a.nsys, t);
  const BSys S = a.sys[s];
  const int j = t - S.p_off;
  double x = a.pos[3 * t], y = a.pos[3 * t + 1], z = a.pos[3 * t + 2];
  if (S.shear_mode == 1)
    {
      const double w = floor (y / S.ly);
      y -= w * S.ly;
      x -= w * S.shift;
    }
  else if (S.shear_mode == 2)
    {
      const double w = floor (z / S.lz);
      z -= w * S.lz;
      x -= w * S.shift;
    }
  double sv[3] = {x / S.lx, y / S.ly, z / S.lz};
  for (int k = 0; k < 3; k++)
    {
      sv[k] -= floor (sv[k]);
      if (sv[k] >= 1.0) sv[k] = 0.0;
    }
  if (d == 0)
    {
      const double two32 = 4294967296.0;
      for (int k = 0; k < 3; k++)
        {
          double q = floor (sv[k] * two32);
          if (q >= two32) q -= two32;
          a.qpos[4 * t + k] = (uint32_t) q;
        }
      a.qpos[4 * t + 3] = 0u;
      for (int q = 0; q < S.c; q++)
        a.xf[S.x_off + (size_t) j * S.c + q] = (float) a.x[S.x_off + (size_t) j * S.c + q];
    }
  const double sl = S.shift / S.lx;
  double u = sv[d];
  if (d == 0 && S.shear_mode == 1) u = sv[0] - sl * sv[1];
  else if (d == 0 && S.shear_mode == 2) u = sv[0] - sl * sv[2];
  const int Md = d == 0 ? S.M0 : (d == 1 ? S.M1 : S.M2);
  const size_t off = S.tab_off + (d == 0 ? 0 : (d == 1 ? (size_t) (S.M0 + 1) * S.np
                                                       : (size_t) (S.M0 + S.M1 + 2) * S.np));
  double sb, cb;
  sincospi (2.0 * u, &sb, &cb);
  double pr = 1.0, pi = 0.0;
  for (int m = 0; m <= Md; m++)
    {
      a.tab[off + (size_t) m * S.np + j] = make_float2 ((float) pr, (float) pi);
      const double nr = pr * cb - pi * sb;
      pi = pr * sb + pi * cb;
      pr = nr;
    }
}

__device__ __forceinline__ void
bmin_image (const BSys &S, uint4 qi, uint4 qj, float &dx, float &dy, float &dz)
{
  uint32_t ux = qj.x - qi.x;
  const uint32_t uy = qj.y - qi.y;
  const uint32_t uz = qj.z - qi.z;
  if (S.shear_mode == 1)
    {
      const long long raw = (long long) qj.y - (long long) qi.y;
      const long long w = (raw - (long long) (int32_t) uy) >> 32;
      ux -= (uint32_t) w * S.shift_q;
    }
  else if (S.shear_mode == 2)
    {
      const long long raw = (long long) qj.z - (long long) qi.z;
      const long long w = (raw - (long long) (int32_t) uz) >> 32;
      ux -= (uint32_t) w * S.shift_q;
    }
  dx = (float) (int32_t) ux * S.scale[0];
  dy = (float) (int32_t) uy * S.scale[1];
  dz = (float) (int32_t) uz * S.scale[2];
}

template <int V>
__device__ __forceinline__ void
bterm (const BSys &S, const float *xf, int j, float dx, float dy, float dz, GenU<V, float> &acc)
{
  float r = sqrtf (dx * dx + dy * dy + dz * dz);
  const float rm = 2.0f * S.rmin;
  if (r < rm) r = rm;
  const float ri = 1.0f / r;
  const float e[3] = {dx * ri, dy * ri, dz * ri};
  PairScalars<float> sc;
  real_scalars_mono<V, float> (S.xi, S.xisp, r, sc);
  GenF<V, float> g;
  load_genf<V, float> (xf + S.x_off + (size_t) NComp<V>::value * j, g);
  pair_apply<V, float> (e, sc, g, acc);
}

template <int V>
__device__ __forceinline__ void
mb_real_warp (const BatchArgs &a, const BSys &S, int i, int chunk, float (*s_d)[3], int *s_j)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const int j0 = (int) ((long long) S.np * chunk / S.nchunk);
  const int j1 = (int) ((long long) S.np * (chunk + 1) / S.nchunk);
  const uint4 *qp = reinterpret_cast<const uint4 *> (a.qpos) + S.p_off;
  const uint4 qi = qp[i];
  GenU<V, float> acc;
  acc.zero ();
  int qn = 0;
  const unsigned lt = (1u << lane) - 1u;
  for (int jb = j0; jb < j1; jb += 32)
    {
      const int j = jb + lane;
      bool ok = false;
      float dx = 0.f, dy = 0.f, dz = 0.f;
      float d0x = 0.f, d0y = 0.f, d0z = 0.f;
      if (j < j1) bmin_image (S, qi, qp[j], d0x, d0y, d0z);
      // the minimum image and, when the cutoff exceeds half the box, the
      // lattice images around it
      for (int m = 0; m < S.nimg; m++)
        {
          const float4 T = a.img[S.img_off + m];
          bool ok = false;
          float dx = 0.f, dy = 0.f, dz = 0.f;
          if (j < j1)
            {
              dx = d0x + T.x;
              dy = d0y + T.y;
              dz = d0z + T.z;
              const float rr = dx * dx + dy * dy + dz * dz;
              ok = (rr > 0.f) && (rr < S.rc2);
            }
          const unsigned b = __ballot_sync (0xffffffffu, ok);
          if (ok)
            {
              const int slot = qn + __popc (b & lt);
              s_d[slot][0] = dx;
              s_d[slot][1] = dy;
              s_d[slot][2] = dz;
              s_j[slot] = j;
            }
          qn += __popc (b);
          __syncwarp ();
          if (qn >= 32)
            {
              const int slot = qn - 32 + lane;
              bterm<V> (S, a.xf, s_j[slot], s_d[slot][0], s_d[slot][1], s_d[slot][2], acc);
              qn -= 32;
              __syncwarp ();
            }
        }
    }
  if (lane < qn) bterm<V> (S, a.xf, s_j[lane], s_d[lane][0], s_d[lane][1], s_d[lane][2], acc);
  float *out = a.pr + S.pr_off + ((size_t) chunk * S.np + i) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const float v = warp_sum (acc.v[q]);
      if (lane == 0) out[q] = v;
    }
}

constexpr int MB_QCAP = 64;

__global__ void
mb_real (BatchArgs a)
{
  extern __shared__ float s_real[];        // [warps][QCAP][3] floats, then [warps][QCAP] ints
  const int wpb = blockDim.x >> 5, wib = threadIdx.x >> 5;
  float (*s_d)[3] = reinterpret_cast<float (*)[3]> (s_real + (size_t) wib * MB_QCAP * 3);
  int *s_j = reinterpret_cast<int *> (s_real + (size_t) wpb * MB_QCAP * 3) + wib * MB_QCAP;
  const long long w = (long long) blockIdx.x * wpb + wib;
  if (w >= a.cum_r[a.nsys]) return;
  const int s = find_sys (a.cum_r, a.nsys, w);
  const BSys S = a.sys[s];
  const int local = (int) (w - a.cum_r[s]);
  const int i = local % S.np, chunk = local / S.np;
  if (S.version == 0) mb_real_warp<0> (a, S, i, chunk, s_d, s_j);
  else mb_real_warp<1> (a, S, i, chunk, s_d, s_j);
}

// one warp per (system, k): C(k), S(k) over the system's particles, then
// P = Bc C - Bs S, Q = Bc S + Bs C (component-major, [2c][nkh])
template <int V>
__device__ __forceinline__ void
mb_sfac_warp (const BatchArgs &a, const BSys &S, int k)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const MixK K = a.kt[S.k_off + k];
  const float2 *t0 = a.tab + S.tab_off, *t1 = t0 + (size_t) (S.M0 + 1) * S.np,
               *t2 = t1 + (size_t) (S.M1 + 1) * S.np;
  float cs[C], sn[C];
#pragma unroll
  for (int q = 0; q < C; q++) cs[q] = sn[q] = 0.f;
  for (int j = lane; j < S.np; j += 32)
    {
      float2 p0 = t0[(size_t) (K.m1 < 0 ? -K.m1 : K.m1) * S.np + j];
      float2 p1 = t1[(size_t) (K.m2 < 0 ? -K.m2 : K.m2) * S.np + j];
      float2 p2 = t2[(size_t) (K.m3 < 0 ? -K.m3 : K.m3) * S.np + j];
      if (K.m1 < 0) p0.y = -p0.y;
      if (K.m2 < 0) p1.y = -p1.y;
      if (K.m3 < 0) p2.y = -p2.y;
      const float2 p01 = make_float2 (p0.x * p1.x - p0.y * p1.y, p0.x * p1.y + p0.y * p1.x);
      const float2 ph = make_float2 (p01.x * p2.x - p01.y * p2.y, p01.x * p2.y + p01.y * p2.x);
      const float *xj = a.xf + S.x_off + (size_t) C * j;
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          cs[q] = fmaf (ph.x, xj[q], cs[q]);
          sn[q] = fmaf (ph.y, xj[q], sn[q]);
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      cs[q] = warp_sum (cs[q]);
      sn[q] = warp_sum (sn[q]);
    }
  if (lane != 0) return;
  float ns[C];
#pragma unroll
  for (int q = 0; q < C; q++) ns[q] = -sn[q];
  const float e[3] = {K.ex, K.ey, K.ez};
  GenF<V, float> gc, gs, gms;
  load_genf<V, float> (cs, gc);
  load_genf<V, float> (sn, gs);
  load_genf<V, float> (ns, gms);
  GenU<V, float> P, Q;
  P.zero ();
  Q.zero ();
  recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gc, gms, P);
  recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gs, gc, Q);
  float *pq = a.pq + S.pq_off;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      pq[(size_t) q * S.nkh + k] = P.v[q];
      pq[(size_t) (C + q) * S.nkh + k] = Q.v[q];
    }
}

__global__ void
mb_sfac (BatchArgs a)
{
  const long long w = (long long) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= a.cum_k[a.nsys]) return;
  const int s = find_sys (a.cum_k, a.nsys, w);
  const BSys S = a.sys[s];
  const int k = (int) (w - a.cum_k[s]);
  if (S.version == 0) mb_sfac_warp<0> (a, S, k);
  else mb_sfac_warp<1> (a, S, k);
}

// one warp per (system, particle): y_i = self x_i + sum real partials
// + 2 sum_k cos(k.r_i) P + sin(k.r_i) Q
template <int V>
__device__ __forceinline__ void
mb_bp_warp (const BatchArgs &a, const BSys &S, int i)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const float2 *t0 = a.tab + S.tab_off, *t1 = t0 + (size_t) (S.M0 + 1) * S.np,
               *t2 = t1 + (size_t) (S.M1 + 1) * S.np;
  const float *pq = a.pq + S.pq_off;
  float acc[C];
#pragma unroll
  for (int q = 0; q < C; q++) acc[q] = 0.f;
  for (int k = lane; k < S.nkh; k += 32)
    {
      const int4 m = *reinterpret_cast<const int4 *> (&a.kt[S.k_off + k].m1);
      float2 p0 = t0[(size_t) (m.x < 0 ? -m.x : m.x) * S.np + i];
      float2 p1 = t1[(size_t) (m.y < 0 ? -m.y : m.y) * S.np + i];
      float2 p2 = t2[(size_t) (m.z < 0 ? -m.z : m.z) * S.np + i];
      if (m.x < 0) p0.y = -p0.y;
      if (m.y < 0) p1.y = -p1.y;
      if (m.z < 0) p2.y = -p2.y;
      const float2 p01 = make_float2 (p0.x * p1.x - p0.y * p1.y, p0.x * p1.y + p0.y * p1.x);
      const float2 ph = make_float2 (p01.x * p2.x - p01.y * p2.y, p01.x * p2.y + p01.y * p2.x);
#pragma unroll
      for (int q = 0; q < C; q++)
        acc[q] = fmaf (ph.x, pq[(size_t) q * S.nkh + k],
                       fmaf (ph.y, pq[(size_t) (C + q) * S.nkh + k], acc[q]));
    }
#pragma unroll
  for (int q = 0; q < C; q++) acc[q] = warp_sum (acc[q]);
  if (lane != 0) return;
  // self (FP64) + real partials + 2 reciprocal
  PairScalars<double> sc;
  sc.xa = sc.ya = S.selfc[0];
  sc.xc = sc.yc = S.selfc[1];
  sc.xm = sc.ym = sc.zm = S.selfc[2];
  sc.yb = sc.xg = sc.yg = sc.yh = 0.0;
  const double e[3] = {0.0, 0.0, 0.0};
  GenF<V, double> g;
  load_genf<V, double> (a.x + S.x_off + (size_t) C * i, g);
  GenU<V, double> ys;
  ys.zero ();
  pair_apply<V, double> (e, sc, g, ys);
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      double r = 0.0;
      for (int ch = 0; ch < S.nchunk; ch++)
        r += (double) a.pr[S.pr_off + ((size_t) ch * S.np + i) * C + q];
      a.y[S.x_off + (size_t) C * i + q] = ys.v[q] + r + 2.0 * (double) acc[q];
    }
}

__global__ void
mb_bp (BatchArgs a)
{
  const long long w = (long long) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= a.cum_p[a.nsys]) return;
  const int s = find_sys (a.cum_p, a.nsys, w);
  const BSys S = a.sys[s];
  const int i = (int) (w - a.cum_p[s]);
  if (S.version == 0) mb_bp_warp<0> (a, S, i);
  else mb_bp_warp<1> (a, S, i);
}

}  // namespace lsg

// ---------------------------------------------------------------------------
// batch object
// ---------------------------------------------------------------------------
struct stokes_gpu_batch {
  std::vector<struct stokes *> sys;
  int precision = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  int nsys = 0, nptot = 0, nxtot = 0;
  std::vector<int> p_off, x_off;
  // mixed
  std::vector<lsg::BSys> h_sys;
  std::vector<int> h_cum_p, h_cum_r, h_cum_k;
  std::vector<lsg::MixK> h_k;
  std::vector<float4> h_img;
  lsg::DevBuf d_sys, d_cum, d_pos, d_x, d_y, d_qpos, d_tab, d_xf, d_kt, d_pq, d_pr, d_img;
  int tab_tot = 0, k_tot = 0, pq_tot = 0, pr_tot = 0;
  int chunk_mult = 1, real_wpb = 4;     // autotuned
  // split: eta = xi V^(1/3) = eta_scale np^(1/6), the balance of real-space
  // pairs (~ np^2 / eta^3) and k vectors (~ np eta^3); the scale is autotuned
  double eta_scale = 1.6;
  bool tuned = false;
  // FP64: one stream per branch inside the capture
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_ev;
  // graph of one product
  cudaGraphExec_t exec = nullptr;
  double last_ms = 0.0;
};

namespace lsg {

// a fixed eta for every system (measurements of the split), else none
static double
batch_eta_override ()
{
  const char *e = getenv ("LIBSTOKES_GB300_BATCH_ETA");   // read per set-up: sweeps
  return (e && atof (e) > 0.0) ? atof (e) : 0.0;
}

static double
batch_eta (const stokes_gpu_batch *b, int np)
{
  const double o = batch_eta_override ();
  if (o > 0.0) return o;
  return b->eta_scale * pow ((double) np, 1.0 / 6.0);
}

// the mixed split, k list and descriptors of every system
static int
batch_setup_mixed (stokes_gpu_batch *b)
{
  b->h_sys.assign (b->nsys, BSys{});
  b->h_k.clear ();
  b->h_img.clear ();
  b->h_cum_p.assign (b->nsys + 1, 0);
  b->h_cum_k.assign (b->nsys + 1, 0);
  int tab = 0, pq = 0;
  const double eps = 3e-8;  // the single-system mixed split's truncation
  for (int s = 0; s < b->nsys; s++)
    {
      const struct stokes *sys = b->sys[s];
      BSys &S = b->h_sys[s];
      S.np = sys->np;
      S.version = sys->version;
      S.c = NCOMP (sys->version);
      S.p_off = b->p_off[s];
      S.x_off = b->x_off[s];
      const double lmin = fmin (sys->lx, fmin (sys->ly, sys->lz));
      const double lmax = fmax (sys->lx, fmax (sys->ly, sys->lz));
      const double lv = cbrt (sys->lx * sys->ly * sys->lz);
      // xi a <= XI_CAP keeps the self, real and reciprocal parts of the same
      // size (FP32 loses digits to their cancellation when xi a grows);
      // small boxes then take lattice images in real space
      const double XI_CAP = 0.5;
      const double xi = std::min (batch_eta (b, sys->np) / lv, XI_CAP);
      double rc = 0, kc = 0;
      lsg_ewald_cutoffs (xi, eps, lmin, lmax, &rc, &kc);
      (void) lmax;
      const double xisp = xi / sqrt (M_PI), xi2 = xi * xi;
      S.selfc[0] = 1.0 - xisp * (6.0 - 40.0 / 3.0 * xi2);
      S.selfc[1] = 0.75 - xisp * xi2 * 10.0;
      S.selfc[2] = 0.9 - xisp * xi2 * (12.0 - 30.24 * xi2);
      S.xi = (float) xi;
      S.xisp = (float) xisp;
      S.rc2 = (float) (rc * rc);
      // lattice images within the cutoff of a minimum-image difference
      {
        S.img_off = (int) b->h_img.size ();
        const int nx = (int) ceil (rc / sys->lx + 0.5), ny = (int) ceil (rc / sys->ly + 0.5),
                  nz = (int) ceil (rc / sys->lz + 0.5);
        for (int a1 = -nx; a1 <= nx; a1++)
          for (int a2 = -ny; a2 <= ny; a2++)
            for (int a3 = -nz; a3 <= nz; a3++)
              {
                double tx = a1 * sys->lx, ty = a2 * sys->ly, tz = a3 * sys->lz;
                if (sys->shear_mode == 1) tx += a2 * sys->shear_shift;
                else if (sys->shear_mode == 2) tx += a3 * sys->shear_shift;
                // skip images whose nearest point to the half-box cell is out of reach
                const double ex = std::max (0.0, fabs (tx) - 0.5 * sys->lx - (sys->shear_mode ? fabs (sys->shear_shift) : 0.0));
                const double ey = std::max (0.0, fabs (ty) - 0.5 * sys->ly);
                const double ez = std::max (0.0, fabs (tz) - 0.5 * sys->lz);
                if (ex * ex + ey * ey + ez * ez > rc * rc) continue;
                b->h_img.push_back (make_float4 ((float) tx, (float) ty, (float) tz, 0.f));
              }
        S.nimg = (int) b->h_img.size () - S.img_off;
      }
      S.rmin = (float) sys->rmin;
      S.lx = sys->lx; S.ly = sys->ly; S.lz = sys->lz;
      S.shift = sys->shear_shift;
      S.shear_mode = sys->shear_mode;
      const double two32 = 4294967296.0;
      S.scale[0] = (float) (sys->lx / two32);
      S.scale[1] = (float) (sys->ly / two32);
      S.scale[2] = (float) (sys->lz / two32);
      S.shift_q = (uint32_t) (llround (sys->shear_shift / sys->lx * two32) & 0xffffffffll);
      // half-space k list
      const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly,
                   k0z = 2.0 * M_PI / sys->lz;
      const double sl = sys->shear_shift / sys->lx;
      const double pivol = M_PI / (sys->lx * sys->ly * sys->lz);
      const int B1 = (int) (kc / k0x) + 1;
      const int B2 = (int) (kc / k0y) + 1 + (sys->shear_mode == 1 ? (int) ceil (fabs (sl) * B1) : 0);
      const int B3 = (int) (kc / k0z) + 1 + (sys->shear_mode == 2 ? (int) ceil (fabs (sl) * B1) : 0);
      int M[3] = {0, 0, 0};
      S.k_off = (int) b->h_k.size ();
      for (int m1 = 0; m1 <= B1; m1++)
        for (int m2 = -B2; m2 <= B2; m2++)
          for (int m3 = -B3; m3 <= B3; m3++)
            {
              if (m1 == 0 && (m2 < 0 || (m2 == 0 && m3 <= 0))) continue;
              const double k1 = k0x * m1;
              double k2 = k0y * m2, k3 = k0z * m3;
              if (sys->shear_mode == 1) k2 = k0y * ((double) m2 - sl * (double) m1);
              else if (sys->shear_mode == 2) k3 = k0z * ((double) m3 - sl * (double) m1);
              const double kk = k1 * k1 + k2 * k2 + k3 * k3, k = sqrt (kk);
              if (k > kc) continue;
              const double k4z = kk / 4.0 / xi2;
              const double kexp = pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
              MixK r;
              memset (&r, 0, sizeof r);
              r.m1 = m1; r.m2 = m2; r.m3 = m3;
              r.ex = (float) (k1 / k); r.ey = (float) (k2 / k); r.ez = (float) (k3 / k);
              r.ya = (float) (6.0 * (1.0 - kk / 3.0) * kexp);
              r.yb = (float) (3.0 * k * kexp);
              r.yc = (float) (1.5 * kk * kexp);
              b->h_k.push_back (r);
              M[0] = std::max (M[0], m1);
              M[1] = std::max (M[1], abs (m2));
              M[2] = std::max (M[2], abs (m3));
            }
      S.nkh = (int) b->h_k.size () - S.k_off;
      S.M0 = M[0]; S.M1 = M[1]; S.M2 = M[2];
      S.tab_off = tab;
      tab += (M[0] + M[1] + M[2] + 3) * S.np;
      S.pq_off = pq;
      pq += 2 * S.c * std::max (S.nkh, 1);
      b->h_cum_p[s + 1] = b->h_cum_p[s] + S.np;
      b->h_cum_k[s + 1] = b->h_cum_k[s] + S.nkh;
    }
  b->tab_tot = tab;
  b->pq_tot = pq;
  b->k_tot = (int) b->h_k.size ();
  return STOKES_GPU_OK;
}

// real-space chunking (autotuned multiplier): partial offsets, warp counts
static void
batch_chunks (stokes_gpu_batch *b)
{
  b->h_cum_r.assign (b->nsys + 1, 0);
  int pr = 0;
  for (int s = 0; s < b->nsys; s++)
    {
      BSys &S = b->h_sys[s];
      S.nchunk = std::max (1, std::min (b->chunk_mult, S.np / 8));
      S.pr_off = pr;
      pr += S.nchunk * S.np * S.c;
      b->h_cum_r[s + 1] = b->h_cum_r[s] + S.np * S.nchunk;
    }
  b->pr_tot = pr;
}

static int
batch_upload_mixed (stokes_gpu_batch *b)
{
  cudaError_t e = cudaSuccess;
  const int ns = b->nsys;
  std::vector<int> cum ((size_t) 3 * (ns + 1));
  std::copy (b->h_cum_p.begin (), b->h_cum_p.end (), cum.begin ());
  std::copy (b->h_cum_r.begin (), b->h_cum_r.end (), cum.begin () + (ns + 1));
  std::copy (b->h_cum_k.begin (), b->h_cum_k.end (), cum.begin () + 2 * (ns + 1));
  auto up = [&] (DevBuf &d, const void *h, size_t bytes) {
    if (e == cudaSuccess) e = d.ensure (bytes ? bytes : 16);
    if (e == cudaSuccess && bytes)
      e = cudaMemcpyAsync (d.p, h, bytes, cudaMemcpyHostToDevice, b->stream);
  };
  up (b->d_sys, b->h_sys.data (), sizeof (BSys) * ns);
  up (b->d_cum, cum.data (), sizeof (int) * cum.size ());
  up (b->d_kt, b->h_k.data (), sizeof (MixK) * b->h_k.size ());
  up (b->d_img, b->h_img.data (), sizeof (float4) * b->h_img.size ());
  if (e == cudaSuccess) e = b->d_qpos.ensure (sizeof (uint32_t) * 4 * (size_t) b->nptot);
  if (e == cudaSuccess) e = b->d_tab.ensure (sizeof (float2) * (size_t) std::max (b->tab_tot, 1));
  if (e == cudaSuccess) e = b->d_xf.ensure (sizeof (float) * (size_t) b->nxtot);
  if (e == cudaSuccess) e = b->d_pq.ensure (sizeof (float) * (size_t) std::max (b->pq_tot, 1));
  if (e == cudaSuccess) e = b->d_pr.ensure (sizeof (float) * (size_t) std::max (b->pr_tot, 1));
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch tables");
}

static BatchArgs
batch_args (stokes_gpu_batch *b)
{
  BatchArgs a;
  a.sys = (const BSys *) b->d_sys.p;
  a.nsys = b->nsys;
  const int *cum = (const int *) b->d_cum.p;
  a.cum_p = cum;
  a.cum_r = cum + (b->nsys + 1);
  a.cum_k = cum + 2 * (b->nsys + 1);
  a.pos = (const double *) b->d_pos.p;
  a.x = (const double *) b->d_x.p;
  a.y = (double *) b->d_y.p;
  a.qpos = (uint32_t *) b->d_qpos.p;
  a.tab = (float2 *) b->d_tab.p;
  a.xf = (float *) b->d_xf.p;
  a.kt = (const MixK *) b->d_kt.p;
  a.pq = (float *) b->d_pq.p;
  a.pr = (float *) b->d_pr.p;
  a.img = (const float4 *) b->d_img.p;
  return a;
}

// the launches of one mixed product on st
static cudaError_t
batch_launch_mixed (stokes_gpu_batch *b, cudaStream_t st)
{
  BatchArgs a = batch_args (b);
  mb_prep<<<dim3 ((b->nptot + 63) / 64, 3), 64, 0, st>>> (a, b->nptot);
  const int wpb = b->real_wpb;
  const size_t smem = (size_t) wpb * MB_QCAP * (3 * sizeof (float) + sizeof (int));
  const long long rw = b->h_cum_r[b->nsys];
  mb_real<<<(int) ((rw + wpb - 1) / wpb), wpb * 32, smem, st>>> (a);
  const long long kw = b->h_cum_k[b->nsys];
  if (kw > 0) mb_sfac<<<(int) ((kw + 7) / 8), 256, 0, st>>> (a);
  mb_bp<<<(b->nptot + 7) / 8, 256, 0, st>>> (a);
  return cudaGetLastError ();
}

// FP64: every system's product on its own branch
static int
batch_launch_fp64 (stokes_gpu_batch *b, cudaStream_t st)
{
  cudaError_t e = cudaEventRecord (b->side_ev[0], st);
  if (e != cudaSuccess) return cuda_fail (e, "batch fork");
  const int nb = (int) b->side.size ();
  for (int k = 0; k < nb; k++) cudaStreamWaitEvent (b->side[k], b->side_ev[0], 0);
  for (int s = 0; s < b->nsys; s++)
    {
      Ctx *c = get_ctx (b->sys[s], true);
      if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a context");
      const double *pos = (const double *) b->d_pos.p + 3 * (size_t) b->p_off[s];
      const double *x = (const double *) b->d_x.p + b->x_off[s];
      double *y = (double *) b->d_y.p + b->x_off[s];
      int rc = atimes_fp64_dev (c, pos, x, y, b->side[s % nb], false);
      if (rc) return rc;
    }
  for (int k = 0; k < nb; k++)
    {
      cudaEventRecord (b->side_ev[1 + k], b->side[k]);
      cudaStreamWaitEvent (st, b->side_ev[1 + k], 0);
    }
  e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch launches");
}

static int
batch_capture (stokes_gpu_batch *b)
{
  if (b->exec) cudaGraphExecDestroy (b->exec), b->exec = nullptr;
  cudaGraph_t graph;
  cudaError_t e = cudaStreamBeginCapture (b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail (e, "batch capture");
  int rc = STOKES_GPU_OK;
  if (b->precision == STOKES_GPU_MIXED)
    {
      e = batch_launch_mixed (b, b->stream);
      if (e != cudaSuccess) rc = cuda_fail (e, "batch launches");
    }
  else
    rc = batch_launch_fp64 (b, b->stream);
  e = cudaStreamEndCapture (b->stream, &graph);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail (e, "batch capture");
  e = cudaGraphInstantiate (&b->exec, graph, 0);
  cudaGraphDestroy (graph);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch graph");
}

static int
batch_run (stokes_gpu_batch *b, float *ms)
{
  cudaEvent_t e0, e1;
  cudaEventCreate (&e0);
  cudaEventCreate (&e1);
  cudaEventRecord (e0, b->stream);
  cudaError_t e = cudaGraphLaunch (b->exec, b->stream);
  cudaEventRecord (e1, b->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize (e1);
  float t = 0.f;
  cudaEventElapsedTime (&t, e0, e1);
  cudaEventDestroy (e0);
  cudaEventDestroy (e1);
  if (ms) *ms = t;
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch product");
}

// time a few splits, then real-space chunkings and CTA sizes, keep the fastest
static int
batch_autotune (stokes_gpu_batch *b)
{
  auto trial = [&] (bool setup, float *best_ms) -> int {
    int rc = setup ? batch_setup_mixed (b) : STOKES_GPU_OK;
    if (!rc) batch_chunks (b);
    if (!rc) rc = batch_upload_mixed (b);
    if (!rc) rc = batch_capture (b);
    float t = 0.f, tmin = 1e30f;
    for (int rep = 0; rep < 3 && !rc; rep++)
      {
        rc = batch_run (b, &t);
        tmin = std::min (tmin, t);
      }
    *best_ms = tmin;
    return rc;
  };
  int rc = STOKES_GPU_OK;
  float t = 0.f, best = 1e30f;
  b->chunk_mult = 1;
  b->real_wpb = 4;
  if (batch_eta_override () <= 0.0)
    {
      const double scales[4] = {1.2, 1.6, 2.0, 2.4};
      double bs = b->eta_scale;
      for (double sc : scales)
        {
          b->eta_scale = sc;
          if ((rc = trial (true, &t))) return rc;
          if (t < best) { best = t; bs = sc; }
        }
      b->eta_scale = bs;
      if ((rc = batch_setup_mixed (b))) return rc;
    }
  const int mults[3] = {1, 2, 4};
  const int wpbs[2] = {4, 8};
  best = 1e30f;
  int bm = 1, bw = 4;
  for (int m : mults)
    for (int w : wpbs)
      {
        b->chunk_mult = m;
        b->real_wpb = w;
        if ((rc = trial (false, &t))) return rc;
        if (t < best) { best = t; bm = m; bw = w; }
      }
  b->chunk_mult = bm;
  b->real_wpb = bw;
  batch_chunks (b);
  rc = batch_upload_mixed (b);
  if (!rc) rc = batch_capture (b);
  b->tuned = true;
  return rc;
}

}  // namespace lsg

using namespace lsg;

extern "C" {

int
stokes_gpu_batch_create (struct stokes **systems, int nsys, int precision,
                         stokes_gpu_batch **out)
{
  clear_error ();
  if (!systems || nsys <= 0 || !out) return set_error (STOKES_GPU_EINVAL, "bad batch arguments");
  if (precision != STOKES_GPU_FP64 && precision != STOKES_GPU_MIXED)
    return set_error (STOKES_GPU_EINVAL, "unknown precision %d", precision);
  stokes_gpu_batch *b = new stokes_gpu_batch ();
  b->nsys = nsys;
  b->precision = precision;
  b->sys.assign (systems, systems + nsys);
  cudaGetDevice (&b->device);
  for (int s = 0; s < nsys; s++)
    {
      const struct stokes *sys = systems[s];
      int rc = check_sys (sys);
      if (rc) { delete b; return rc; }
      if (precision == STOKES_GPU_MIXED && (sys->version > 1 || sys->a || sys->slip))
        {
          delete b;
          return set_error (STOKES_GPU_EINVAL,
                            "mixed batches serve F and FT equal spheres without slip");
        }
      b->p_off.push_back (b->nptot);
      b->x_off.push_back (b->nxtot);
      b->nptot += sys->np;
      b->nxtot += NCOMP (sys->version) * sys->np;
    }
  cudaError_t e = cudaStreamCreateWithFlags (&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = b->d_pos.ensure (sizeof (double) * 3 * (size_t) b->nptot);
  if (e == cudaSuccess) e = b->d_x.ensure (sizeof (double) * (size_t) b->nxtot);
  if (e == cudaSuccess) e = b->d_y.ensure (sizeof (double) * (size_t) b->nxtot);
  if (e != cudaSuccess) { stokes_gpu_batch_destroy (b); return cuda_fail (e, "batch buffers"); }
  std::vector<double> h ((size_t) 3 * b->nptot);
  for (int s = 0; s < nsys; s++)
    memcpy (&h[3 * (size_t) b->p_off[s]], systems[s]->pos, sizeof (double) * 3 * systems[s]->np);
  e = cudaMemcpy (b->d_pos.p, h.data (), sizeof (double) * h.size (), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { stokes_gpu_batch_destroy (b); return cuda_fail (e, "batch positions"); }
  int rc = STOKES_GPU_OK;
  if (precision == STOKES_GPU_MIXED)
    {
      rc = batch_setup_mixed (b);
      if (!rc)
        {
          batch_chunks (b);
          rc = batch_upload_mixed (b);
        }
    }
  else
    {
      for (int s = 0; s < nsys && !rc; s++)
        {
          Ctx *c = get_ctx (systems[s], true);
          if (!c) rc = set_error (STOKES_GPU_ECUDA, "cannot create a context");
          else
            {
              c->precision = STOKES_GPU_FP64;
              rc = prepare (c, systems[s], false);
            }
        }
      const int nb = std::min (nsys, 16);
      b->side.resize (nb);
      b->side_ev.resize (nb + 1);
      for (int k = 0; k < nb && !rc; k++)
        if (cudaStreamCreateWithFlags (&b->side[k], cudaStreamNonBlocking) != cudaSuccess)
          rc = set_error (STOKES_GPU_ECUDA, "cannot create streams");
      for (int k = 0; k <= nb && !rc; k++)
        if (cudaEventCreateWithFlags (&b->side_ev[k], cudaEventDisableTiming) != cudaSuccess)
          rc = set_error (STOKES_GPU_ECUDA, "cannot create events");
      // one product per system outside the capture sizes every scratch buffer
      if (!rc) rc = batch_launch_fp64 (b, b->stream);
      if (!rc && cudaStreamSynchronize (b->stream) != cudaSuccess)
        rc = set_error (STOKES_GPU_ECUDA, "batch warm-up failed");
    }
  if (!rc) rc = batch_capture (b);
  if (rc) { stokes_gpu_batch_destroy (b); return rc; }
  *out = b;
  return STOKES_GPU_OK;
}

int
stokes_gpu_batch_destroy (stokes_gpu_batch *b)
{
  if (!b) return STOKES_GPU_OK;
  if (b->stream) cudaStreamSynchronize (b->stream);
  if (b->exec) cudaGraphExecDestroy (b->exec);
  for (cudaStream_t s : b->side) cudaStreamDestroy (s);
  for (cudaEvent_t e : b->side_ev) cudaEventDestroy (e);
  for (DevBuf *d : {&b->d_sys, &b->d_cum, &b->d_pos, &b->d_x, &b->d_y, &b->d_qpos, &b->d_tab,
                    &b->d_xf, &b->d_kt, &b->d_pq, &b->d_pr, &b->d_img})
    d->release ();
  if (b->stream) cudaStreamDestroy (b->stream);
  delete b;
  return STOKES_GPU_OK;
}

int
stokes_gpu_batch_size (const stokes_gpu_batch *b, int *np_total, int *n_total)
{
  if (!b) return set_error (STOKES_GPU_EINVAL, "NULL batch");
  if (np_total) *np_total = b->nptot;
  if (n_total) *n_total = b->nxtot;
  return STOKES_GPU_OK;
}

int
stokes_gpu_batch_offsets (const stokes_gpu_batch *b, int *p_off, int *x_off)
{
  if (!b) return set_error (STOKES_GPU_EINVAL, "NULL batch");
  for (int s = 0; s < b->nsys; s++)
    {
      if (p_off) p_off[s] = b->p_off[s];
      if (x_off) x_off[s] = b->x_off[s];
    }
  return STOKES_GPU_OK;
}

int
stokes_gpu_batch_set_positions (stokes_gpu_batch *b, const double *pos_packed)
{
  clear_error ();
  if (!b || !pos_packed) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  cudaError_t e = cudaMemcpyAsync (b->d_pos.p, pos_packed, sizeof (double) * 3 * b->nptot,
                                   cudaMemcpyHostToDevice, b->stream);
  for (int s = 0; s < b->nsys && e == cudaSuccess; s++)
    memcpy (b->sys[s]->pos, pos_packed + 3 * (size_t) b->p_off[s],
            sizeof (double) * 3 * b->sys[s]->np);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch positions");
}

// y = M x for every system; x, y packed host vectors (libstokes layout per
// system, systems in order)
int
stokes_gpu_batch_atimes (stokes_gpu_batch *b, const double *x, double *y)
{
  clear_error ();
  if (!b || !x || !y) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (b->precision == STOKES_GPU_MIXED && !b->tuned)
    {
      cudaError_t e = cudaMemcpy (b->d_x.p, x, sizeof (double) * b->nxtot, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_fail (e, "batch input");
      int rc = batch_autotune (b);
      if (rc) return rc;
    }
  cudaError_t e = cudaMemcpyAsync (b->d_x.p, x, sizeof (double) * b->nxtot,
                                   cudaMemcpyHostToDevice, b->stream);
  if (e != cudaSuccess) return cuda_fail (e, "batch input");
  float ms = 0.f;
  int rc = batch_run (b, &ms);
  if (rc) return rc;
  b->last_ms = ms;
  e = cudaMemcpyAsync (y, b->d_y.p, sizeof (double) * b->nxtot, cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "batch output");
}

// device milliseconds of the last batch product and the autotuned choice
int
stokes_gpu_batch_stats (const stokes_gpu_batch *b, double *out4)
{
  if (!b || !out4) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  out4[0] = b->last_ms;
  out4[1] = b->chunk_mult;
  out4[2] = b->real_wpb;
  out4[3] = b->k_tot;
  return STOKES_GPU_OK;
}

// the mixed batch's split: eta = xi V^(1/3) of system s (the scale times
// np^(1/6), or the fixed override)
int
stokes_gpu_batch_split (const stokes_gpu_batch *b, int s, double *eta, double *xi)
{
  if (!b || s < 0 || s >= b->nsys) return set_error (STOKES_GPU_EINVAL, "bad batch system");
  if (b->precision != STOKES_GPU_MIXED)
    return set_error (STOKES_GPU_EINVAL, "only mixed batches re-split");
  const struct stokes *sys = b->sys[s];
  const double lv = cbrt (sys->lx * sys->ly * sys->lz);
  if (eta) *eta = (double) b->h_sys[s].xi * lv;
  if (xi) *xi = (double) b->h_sys[s].xi;
  return STOKES_GPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Brownian dynamics of every system of a batch (mid-point scheme, Chebyshev
// noise with per-system bounds and coefficients; no repulsion, no flow)
// ---------------------------------------------------------------------------
namespace lsg {

// out = ca_s x + cb_s b1 - b0 + cj_s y per element, the system's constants
// picked through the element-to-system map
__global__ void
kb_clenshaw (int n, const int *esys, const double *ca, const double *cb, const double *cj,
             const double *x, const double *b1, const double *b0, const double *y, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int s = esys[k];
  out[k] = ca[s] * x[k] + cb[s] * b1[k] - (b0 ? b0[k] : 0.0) + cj[s] * y[k];
}

__global__ void
kb_gauss (int n, unsigned long long seed, unsigned long long counter, double *y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  curandStatePhilox4_32_10_t st;
  curand_init (seed, (unsigned long long) i, counter * 4ull, &st);
  y[i] = (double) curand_normal (&st);
}

__global__ void
kb_scale (int n, double s, const double *a, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = s * a[k];
}

// positions: xo = x0 + h u (the first three velocity components of each
// particle; pmap: particle -> first vector element, c per particle)
__global__ void
kb_euler (int np, const int *pxo, const double *x0, const double *u, double h, double *xo)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int o = pxo[p];
  for (int a = 0; a < 3; a++) xo[3 * p + a] = x0[3 * p + a] + h * u[o + a];
}

}  // namespace lsg

extern "C" {

// nsteps mid-point steps of every system: f = fact z, z = M^{-1/2} y by
// Chebyshev (n_cheb terms) on bounds eig[2 s], eig[2 s + 1] (NULL: FP64
// Lanczos on the batch, n_lanczos steps, widened by 0.8 and 1.05); y from
// y_host (n_total per step, NULL: device Philox with seed).  pos_out:
// packed positions after the steps (optional).
int
stokes_gpu_batch_bd (stokes_gpu_batch *b, double peclet, double dt, int n_cheb, int n_lanczos,
                     const double *eig, const double *y_host, unsigned long long seed,
                     int nsteps, double *pos_out)
{
  using namespace lsg;
  clear_error ();
  if (!b || n_cheb < 2 || !(dt > 0.0) || nsteps < 0)
    return set_error (STOKES_GPU_EINVAL, "bad batch BD arguments");
  const int n = b->nxtot, ns = b->nsys, npt = b->nptot;
  cudaStream_t st = b->stream;
  if (b->precision == STOKES_GPU_MIXED && !b->tuned)
    {
      int rc = batch_autotune (b);
      if (rc) return rc;
    }
  // maps and per-system constants
  std::vector<int> esys (n), pxo (npt);
  for (int s = 0; s < ns; s++)
    {
      const int c = NCOMP (b->sys[s]->version), np = b->sys[s]->np;
      for (int k = 0; k < c * np; k++) esys[b->x_off[s] + k] = s;
      for (int i = 0; i < np; i++) pxo[b->p_off[s] + i] = b->x_off[s] + c * i;
    }
  DevBuf d_esys, d_pxo, d_c, d_v, d_pos0;
  cudaError_t e = d_esys.ensure (sizeof (int) * n);
  if (e == cudaSuccess) e = d_pxo.ensure (sizeof (int) * npt);
  if (e == cudaSuccess) e = d_c.ensure (sizeof (double) * 3 * ns);
  if (e == cudaSuccess) e = d_v.ensure (sizeof (double) * 6 * (size_t) n);
  if (e == cudaSuccess) e = d_pos0.ensure (sizeof (double) * 3 * (size_t) npt);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (d_esys.p, esys.data (), sizeof (int) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (d_pxo.p, pxo.data (), sizeof (int) * npt, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail (e, "batch BD buffers");
  double *V = (double *) d_v.p;
  double *yv = V, *zv = V + n, *bb[3] = {V + 2 * (size_t) n, V + 3 * (size_t) n, V + 4 * (size_t) n},
         *fv = V + 5 * (size_t) n;
  double *X = (double *) b->d_x.p, *Y = (double *) b->d_y.p;
  const int gn = (n + 255) / 256;
  auto product = [&] (const double *in, double *out) -> int {
    if (in != X) cudaMemcpyAsync (X, in, sizeof (double) * n, cudaMemcpyDeviceToDevice, st);
    cudaError_t ee = cudaGraphLaunch (b->exec, st);
    if (ee != cudaSuccess) return cuda_fail (ee, "batch product");
    if (out != Y) cudaMemcpyAsync (out, Y, sizeof (double) * n, cudaMemcpyDeviceToDevice, st);
    return STOKES_GPU_OK;
  };
  // bounds
  std::vector<double> bounds ((size_t) 2 * ns);
  if (eig)
    std::copy (eig, eig + 2 * ns, bounds.begin ());
  else
    {
      // FP64 Lanczos per system with full re-orthogonalisation; the matvecs
      // are batch products, the Krylov bases live on the host
      const int m = std::max (2, n_lanczos);
      std::vector<double> Vk ((size_t) (m + 1) * n), w (n), al ((size_t) m * ns, 0.0),
        be ((size_t) (m + 1) * ns, 0.0);
      std::vector<int> steps (ns, m);
      unsigned long long st64 = seed ^ 0x2545F4914F6CDD1Dull;
      for (int k = 0; k < n; k++)
        {
          st64 = st64 * 6364136223846793005ull + 1442695040888963407ull;
          Vk[k] = (double) ((st64 >> 11) & ((1ull << 52) - 1)) / (double) (1ull << 52) - 0.5;
        }
      for (int s = 0; s < ns; s++)
        {
          const int o = b->x_off[s], len = NCOMP (b->sys[s]->version) * b->sys[s]->np;
          double nn = 0.0;
          for (int k = 0; k < len; k++) nn += Vk[o + k] * Vk[o + k];
          nn = 1.0 / sqrt (nn);
          for (int k = 0; k < len; k++) Vk[o + k] *= nn;
        }
      for (int j = 0; j < m; j++)
        {
          e = cudaMemcpyAsync (X, &Vk[(size_t) j * n], sizeof (double) * n, cudaMemcpyHostToDevice, st);
          if (e == cudaSuccess) e = cudaGraphLaunch (b->exec, st);
          if (e == cudaSuccess)
            e = cudaMemcpyAsync (w.data (), Y, sizeof (double) * n, cudaMemcpyDeviceToHost, st);
          if (e == cudaSuccess) e = cudaStreamSynchronize (st);
          if (e != cudaSuccess) return cuda_fail (e, "batch Lanczos");
          for (int s = 0; s < ns; s++)
            {
              if (j >= steps[s]) continue;
              const int o = b->x_off[s], len = NCOMP (b->sys[s]->version) * b->sys[s]->np;
              for (int pass = 0; pass < 2; pass++)
                for (int i = 0; i <= j; i++)
                  {
                    const double *vi = &Vk[(size_t) i * n + o];
                    double d = 0.0;
                    for (int k = 0; k < len; k++) d += vi[k] * w[o + k];
                    if (i == j) al[(size_t) s * m + j] += d;
                    for (int k = 0; k < len; k++) w[o + k] -= d * vi[k];
                  }
              double nb = 0.0;
              for (int k = 0; k < len; k++) nb += w[o + k] * w[o + k];
              nb = sqrt (nb);
              if (j + 1 == m || nb < 1e-12)
                {
                  steps[s] = j + 1;
                  continue;
                }
              be[(size_t) s * (m + 1) + j + 1] = nb;
              for (int k = 0; k < len; k++) Vk[(size_t) (j + 1) * n + o + k] = w[o + k] / nb;
            }
        }
      for (int s = 0; s < ns; s++)
        {
          // extreme eigenvalues of the tridiagonal matrix by bisection
          const int mm = steps[s];
          const double *a = &al[(size_t) s * m], *bt = &be[(size_t) s * (m + 1)];
          double lo = 1e300, hi = -1e300;
          for (int i = 0; i < mm; i++)
            {
              const double r = (i > 0 ? fabs (bt[i]) : 0.0) + (i + 1 < mm ? fabs (bt[i + 1]) : 0.0);
              lo = std::min (lo, a[i] - r);
              hi = std::max (hi, a[i] + r);
            }
          auto below = [&] (double xq) {
            int cnt = 0;
            double d = 1.0;
            for (int i = 0; i < mm; i++)
              {
                d = a[i] - xq - (i > 0 ? bt[i] * bt[i] / d : 0.0);
                if (d == 0.0) d = -1e-300;
                if (d < 0.0) cnt++;
              }
            return cnt;
          };
          double ext[2];
          for (int which = 0; which < 2; which++)
            {
              double l = lo, h = hi;
              const int target = which ? mm - 1 : 0;
              for (int it = 0; it < 200; it++)
                {
                  const double mid = 0.5 * (l + h);
                  if (below (mid) > target) h = mid;
                  else l = mid;
                }
              ext[which] = 0.5 * (l + h);
            }
          if (!(ext[0] > 0.0))
            return set_error (STOKES_GPU_EACCURACY, "batch system %d: mobility not positive definite", s);
          bounds[2 * s] = 0.8 * ext[0];
          bounds[2 * s + 1] = 1.05 * ext[1];
        }
    }
  // coefficients of 1/sqrt on every system's interval
  std::vector<double> coef ((size_t) ns * n_cheb), ca (ns), cb (ns);
  for (int s = 0; s < ns; s++)
    chebyshev_coef (n_cheb, [] (double v) { return 1.0 / sqrt (v); }, bounds[2 * s],
                    bounds[2 * s + 1], &coef[(size_t) s * n_cheb]);
  // per system: 2 da, 2 db (inner steps), da, db (last step), then the
  // coefficients [n_cheb][ns]; uploaded once
  DevBuf d_k;
  e = d_k.ensure (sizeof (double) * (4 + (size_t) n_cheb) * ns);
  if (e != cudaSuccess) return cuda_fail (e, "batch BD constants");
  std::vector<double> hk ((4 + (size_t) n_cheb) * ns);
  for (int s = 0; s < ns; s++)
    {
      const double e0 = bounds[2 * s], e1 = bounds[2 * s + 1];
      const double da = 2.0 / (e1 - e0), db = -(e1 + e0) / (e1 - e0);
      hk[s] = 2.0 * da;
      hk[ns + s] = 2.0 * db;
      hk[2 * ns + s] = da;
      hk[3 * ns + s] = db;
      for (int j = 0; j < n_cheb; j++) hk[(4 + (size_t) j) * ns + s] = coef[(size_t) s * n_cheb + j];
    }
  e = cudaMemcpyAsync (d_k.p, hk.data (), sizeof (double) * hk.size (), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "batch BD constants");
  const double *dk = (const double *) d_k.p;
  auto cj_of = [&] (int j) { return dk + (4 + (size_t) j) * ns; };
  const double fact = peclet > 0.0 ? sqrt (2.0 / (peclet * dt)) : 0.0;
  double *pos = (double *) b->d_pos.p, *pos0 = (double *) d_pos0.p;
  int rc = STOKES_GPU_OK;
  for (int step = 0; step < nsteps && !rc; step++)
    {
      if (y_host)
        e = cudaMemcpyAsync (yv, y_host + (size_t) step * n, sizeof (double) * n,
                             cudaMemcpyHostToDevice, st);
      else
        {
          kb_gauss<<<gn, 256, 0, st>>> (n, seed, (unsigned long long) step, yv);
          e = cudaGetLastError ();
        }
      if (e != cudaSuccess) return cuda_fail (e, "batch noise");
      // Clenshaw (src/chebyshev.c:163-228): b_new = 2 da M b1 + 2 db b1 - b0 + a_j y
      cudaMemsetAsync (bb[0], 0, sizeof (double) * n, st);
      cudaMemsetAsync (bb[1], 0, sizeof (double) * n, st);
      for (int i = 0; i < n_cheb - 1 && !rc; i++)
        {
          double *b2 = bb[(i + 2) % 3], *b1 = bb[(i + 1) % 3], *b0 = bb[i % 3];
          if ((rc = product (b1, fv))) break;
          kb_clenshaw<<<gn, 256, 0, st>>> (n, (const int *) d_esys.p, dk, dk + ns,
                                           cj_of (n_cheb - 1 - i), fv, b1, b0, yv, b2);
        }
      if (rc) break;
      {
        const int i = n_cheb - 1;
        double *b1 = bb[(i + 1) % 3], *b0 = bb[i % 3];
        if ((rc = product (b1, fv))) break;
        kb_clenshaw<<<gn, 256, 0, st>>> (n, (const int *) d_esys.p, dk + 2 * ns, dk + 3 * ns,
                                         cj_of (0), fv, b1, b0, yv, zv);
      }
      // mid-point step with f = fact z
      kb_scale<<<gn, 256, 0, st>>> (n, fact, zv, fv);
      cudaMemcpyAsync (pos0, pos, sizeof (double) * 3 * npt, cudaMemcpyDeviceToDevice, st);
      if ((rc = product (fv, bb[0]))) break;
      kb_euler<<<(npt + 255) / 256, 256, 0, st>>> (npt, (const int *) d_pxo.p, pos0, bb[0],
                                                   0.5 * dt, pos);
      if ((rc = product (fv, bb[0]))) break;
      kb_euler<<<(npt + 255) / 256, 256, 0, st>>> (npt, (const int *) d_pxo.p, pos0, bb[0], dt,
                                                   pos);
      e = cudaGetLastError ();
      if (e != cudaSuccess) rc = cuda_fail (e, "batch BD step");
    }
  if (!rc)
    {
      e = cudaStreamSynchronize (st);
      if (e == cudaSuccess && pos_out)
        e = cudaMemcpy (pos_out, pos, sizeof (double) * 3 * npt, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = cuda_fail (e, "batch BD");
    }
  for (DevBuf *d : {&d_esys, &d_pxo, &d_c, &d_v, &d_pos0, &d_k}) d->release ();
  return rc;
}

}  // extern "C"
