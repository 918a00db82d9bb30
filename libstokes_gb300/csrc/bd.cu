// bd.cu -- device-resident Brownian dynamics with Chebyshev noise.
//
// One mid-point step (src/brownian.c:2352-2560, scheme 0, rmin = 0):
//   y ~ N(0,1); z = M^{-1/2} y by Clenshaw on [l0, l1] (n_cheb products);
//   [every check_every steps: err = |z.Mz - y.y| / z.Mz, one product; above
//    cheb_eps the bounds are re-estimated and z recomputed];
//   f = F + fact z + F_LJ(x);   u = M(x) f + imposed flow(x);
//   x_mid = x + dt/2 u;
//   f = F + fact z + F_LJ(x_mid); u = M(x_mid) f + imposed flow(x_mid);
//   x = x + dt u,                 fact = sqrt(2 / (Pe dt)).
// Positions, noise, forces and velocities never leave the device; the only
// host round trips are the two dot products of the error check.
// Bounds: FP64 Lanczos with full reorthogonalisation (in place of ARPACK's
// Arnoldi in src/dnaupd_c.c), Ritz extremes widened by safety factors.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <vector>

#include "engine.h"
#include "gpu_engine.h"
#include "stokes_bd.h"

namespace lsg {

int cheb_clenshaw_dev (Ctx *c, const double *d_pos, int ncheb, const double *a, int n,
                       const double *d_y, double *d_z, double e0, double e1, cudaStream_t st,
                       DevBuf &work);
int cheb_clenshaw_op (int ncheb, const double *a, int n, const double *d_y, double *d_z,
                      double e0, double e1, cudaStream_t st, DevBuf &work,
                      const std::function<int (const double *, double *)> &op);

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void
k_bd_gauss (int n, unsigned long long seed, unsigned long long counter, double *y)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  curandStatePhilox4_32_10_t s;
  curand_init (seed, (unsigned long long) i, counter * 4ull, &s);
  y[i] = (double) curand_normal (&s);   // float32 deviates
}

// out[0] += a.b, out[1] += c.d   (out zeroed by the caller)
__global__ void
k_bd_dot2 (int n, const double *a, const double *b, const double *c, const double *d,
           double *out)
{
  double s0 = 0.0, s1 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
      s0 += a[i] * b[i];
      s1 += c[i] * d[i];
    }
  for (int o = 16; o > 0; o >>= 1)
    {
      s0 += __shfl_xor_sync (0xffffffffu, s0, o);
      s1 += __shfl_xor_sync (0xffffffffu, s1, o);
    }
  if ((threadIdx.x & 31) == 0)
    {
      atomicAdd (&out[0], s0);
      atomicAdd (&out[1], s1);
    }
}

// dots[i] = V[i] . w for i < m   (one block per i)
__global__ void
k_bd_vdots (int n, const double *V, const double *w, double *dots)
{
  const double *v = V + (size_t) blockIdx.x * n;
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) s += v[k] * w[k];
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync (0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads ();
  if (threadIdx.x == 0)
    {
      double t = 0.0;
      for (int q = 0; q < (int) (blockDim.x >> 5); q++) t += red[q];
      dots[blockIdx.x] = t;
    }
}

// w -= sum_i coef[i] V[i]
__global__ void
k_bd_vaxpy (int n, int m, const double *V, const double *coef, double *w)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double s = w[k];
  for (int i = 0; i < m; i++) s -= coef[i] * V[(size_t) i * n + k];
  w[k] = s;
}

__global__ void
k_bd_scale (int n, const double *w, double s, double *v)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) v[k] = w[k] * s;
}

// generalised force of the mobility problem: F + fact z (and T + fact z_T);
// z is in particle order (F: 3 per particle; FT: U-part then Omega-part of
// each particle, 6 per particle), f has the product's layout (c per particle)
__global__ void
k_bd_force (int nm, int np, int c, double fact, const double *z, const double *fext, double *f)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int zc = (c == 3) ? 3 : 6;
  for (int q = 0; q < c; q++)
    {
      double v = 0.0;
      if (i < nm)
        {
          if (q < zc) v = fact * z[(size_t) i * zc + q];
          if (fext) v += fext[(size_t) i * c + q];
        }
      f[(size_t) i * c + q] = v;
    }
}

// soft repulsion of overlapping pairs (src/ev-LJ.c:105-265): for each of
// the 27 cells of the reference's neighbour table, an image at distance r
// with overlap x = ai + aj - r > 0 pushes i along the primary-cell vector
// (pos_i - pos_j) / r with 12 e (r0/(r0-x))^7 ((r0/(r0-x))^6 - 1), as the
// reference does.  A float minimum-image test skips the pairs that cannot
// overlap; the candidates are redone exactly in FP64.  An open system
// (periodic == 0) has the primary cell only (src/ev-LJ.c:222-233).
__global__ void
k_bd_lj (int nm, int np, int c, const double *pos, double lx, double ly, double lz,
         int shear_mode, double shift, const double *rad, double e_all, double r0_all,
         const double *lje, const double *ljr0, int open, double *f)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm) return;
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const double ai = rad ? rad[i] : 1.0;
  const float flx = (float) lx, fly = (float) ly, flz = (float) lz;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  // the reference's force (src/ev-LJ.c:185-262): the 27 cells around the
  // primary one, the force along the primary-cell vector over the image
  // distance
  for (int j = 0; j < np; j++)
    {
      if (j == i) continue;
      const double aj = rad ? rad[j] : 1.0;
      const double x = xi - pos[3 * j], y = yi - pos[3 * j + 1], z = zi - pos[3 * j + 2];
      if (open)
        {
          const double r = sqrt (x * x + y * y + z * z);
          const double ov = ai + aj - r;
          if (!(ov > 0.0)) continue;
          const double e = lje ? sqrt (lje[i] * lje[j]) : e_all;
          const double r0 = ljr0 ? 0.5 * (ljr0[i] + ljr0[j]) : r0_all;
          double rl = r0 - ov;
          if (rl < 0.0) rl = 1.0e-12;
          const double ri = r0 / rl, ri6 = ri * ri * ri * ri * ri * ri;
          const double fr = 12.0 * e * ri6 * ri * (ri6 - 1.0);
          fx += fr * x / r;
          fy += fr * y / r;
          fz += fr * z / r;
          continue;
        }
      // float pre-test on the wrapped distance (the reference's 27 cells
      // contain the nearest image only when |x| < 1.5 L; keep the exact path
      // whenever that is not clearly the case)
      const float sx = (float) x, sy = (float) y, sz = (float) z;
      float wx = sx - flx * rintf (sx / flx), wy = sy - fly * rintf (sy / fly),
            wz = sz - flz * rintf (sz / flz);
      const float lim = (float) (ai + aj) * 1.001f + 1e-3f;
      const bool far_raw = fabsf (sx) > 1.4f * flx || fabsf (sy) > 1.4f * fly
        || fabsf (sz) > 1.4f * flz || shear_mode != 0;
      if (!far_raw && wx * wx + wy * wy + wz * wz > lim * lim) continue;
      // pair coefficients (src/ev-LJ.c:131-137): geometric mean of e,
      // arithmetic mean of r0
      const double e = lje ? sqrt (lje[i] * lje[j]) : e_all;
      const double r0 = ljr0 ? 0.5 * (ljr0[i] + ljr0[j]) : r0_all;
      for (int kx = -1; kx <= 1; kx++)
        for (int ky = -1; ky <= 1; ky++)
          for (int kz = -1; kz <= 1; kz++)
            {
              double xx = x + kx * lx, yy = y + ky * ly, zz = z + kz * lz;
              if (shear_mode == 1) xx += ky * shift;
              else if (shear_mode == 2) xx += kz * shift;
              const double r = sqrt (xx * xx + yy * yy + zz * zz);
              const double ov = ai + aj - r;
              if (!(ov > 0.0)) continue;
              double rl = r0 - ov;
              if (rl < 0.0) rl = 1.0e-12;
              const double ri = r0 / rl, ri6 = ri * ri * ri * ri * ri * ri;
              const double fr = 12.0 * e * ri6 * ri * (ri6 - 1.0);
              // direction: the primary-cell vector over the image distance
              fx += fr * x / r;
              fy += fr * y / r;
              fz += fr * z / r;
            }
    }
  f[(size_t) i * c] += fx;
  f[(size_t) i * c + 1] += fy;
  f[(size_t) i * c + 2] += fz;
}

// EV_LJ of this library's BD engine: the nearest image (Lees-Edwards aware;
// the overlap range is below half the box) and the force along the image
// vector.  CTA of LJ_T targets; the sources pass through shared memory in
// tiles of LJ_T as FP32 positions for a pre-test on the wrapped distance
// (with a margin); the few pairs that pass it are evaluated in FP64 from
// the global positions.  An open system takes the plain difference.
constexpr int LJ_T = 128;

__global__ void __launch_bounds__ (LJ_T)
k_bd_lj_engine (int nm, int np, int c, const double *pos, double lx, double ly, double lz,
                int shear_mode, double shift, const double *rad, double e_all, double r0_all,
                const double *lje, const double *ljr0, int open, double *f)
{
  __shared__ float s_p[LJ_T][4];
  const int i = blockIdx.x * LJ_T + threadIdx.x;
  const bool live = i < nm;
  const int ii = live ? i : 0;
  const double xi = pos[3 * ii], yi = pos[3 * ii + 1], zi = pos[3 * ii + 2];
  const float fxi = (float) xi, fyi = (float) yi, fzi = (float) zi;
  const double ai = rad ? rad[ii] : 1.0;
  const float flx = (float) lx, fly = (float) ly, flz = (float) lz, fsh = (float) shift;
  const float ilx = 1.0f / flx, ily = 1.0f / fly, ilz = 1.0f / flz;
  const double dlx = 1.0 / lx, dly = 1.0 / ly, dlz = 1.0 / lz;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int j0 = 0; j0 < np; j0 += LJ_T)
    {
      __syncthreads ();
      const int jl = j0 + threadIdx.x;
      if (jl < np)
        {
          s_p[threadIdx.x][0] = (float) pos[3 * jl];
          s_p[threadIdx.x][1] = (float) pos[3 * jl + 1];
          s_p[threadIdx.x][2] = (float) pos[3 * jl + 2];
          s_p[threadIdx.x][3] = rad ? (float) rad[jl] : 1.0f;
        }
      __syncthreads ();
      if (!live) continue;
      const int nt = min (LJ_T, np - j0);
      for (int t = 0; t < nt; t++)
        {
          const int j = j0 + t;
          float sx = fxi - s_p[t][0], sy = fyi - s_p[t][1], sz = fzi - s_p[t][2];
          if (!open)
            {
              if (shear_mode == 1)
                {
                  const float k = rintf (sy * ily);
                  sy -= k * fly;
                  sx -= k * fsh;
                }
              else if (shear_mode == 2)
                {
                  const float k = rintf (sz * ilz);
                  sz -= k * flz;
                  sx -= k * fsh;
                }
              sx -= flx * rintf (sx * ilx);
              sy -= fly * rintf (sy * ily);
              sz -= flz * rintf (sz * ilz);
            }
          const float lim = ((float) ai + s_p[t][3]) * 1.001f + 1e-3f;
          if (sx * sx + sy * sy + sz * sz > lim * lim || j == i) continue;
          const double aj = rad ? rad[j] : 1.0;
          double x = xi - pos[3 * j], y = yi - pos[3 * j + 1], z = zi - pos[3 * j + 2];
          if (!open)
            {
              if (shear_mode == 1)
                {
                  const double k = rint (y * dly);
                  y -= k * ly;
                  x -= k * shift;
                }
              else if (shear_mode == 2)
                {
                  const double k = rint (z * dlz);
                  z -= k * lz;
                  x -= k * shift;
                }
              x -= lx * rint (x * dlx);
              y -= ly * rint (y * dly);
              z -= lz * rint (z * dlz);
            }
          const double r = sqrt (x * x + y * y + z * z);
          const double ov = ai + aj - r;
          if (!(ov > 0.0) || !(r > 0.0)) continue;
          const double e = lje ? sqrt (lje[i] * lje[j]) : e_all;
          const double r0 = ljr0 ? 0.5 * (ljr0[i] + ljr0[j]) : r0_all;
          double rl = r0 - ov;
          if (rl < 0.0) rl = 1.0e-12;
          const double ri = r0 / rl, ri6 = ri * ri * ri * ri * ri * ri;
          const double fr = 12.0 * e * ri6 * ri * (ri6 - 1.0);
          fx += fr * x / r;
          fy += fr * y / r;
          fz += fr * z / r;
        }
    }
  if (!live) return;
  f[(size_t) i * c] += fx;
  f[(size_t) i * c + 1] += fy;
  f[(size_t) i * c + 2] += fz;
}

struct Flow {
  double U[3], O[3], E[5];
};

// x_out = x_base + h (u + Ui + Oi x pos + Ei . pos)   (src/f.c:621-655 and
// src/brownian.c:1889-1930)
__global__ void
k_bd_euler (int nm, int c, const double *x_base, const double *u, const double *pos, Flow fl,
            double h, double *x_out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm) return;
  const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
  const double ezz = -fl.E[0] - fl.E[4];
  const double ux = fl.U[0] + fl.O[1] * pz - fl.O[2] * py + fl.E[0] * px + fl.E[1] * py + fl.E[2] * pz;
  const double uy = fl.U[1] + fl.O[2] * px - fl.O[0] * pz + fl.E[1] * px + fl.E[4] * py + fl.E[3] * pz;
  const double uz = fl.U[2] + fl.O[0] * py - fl.O[1] * px + fl.E[2] * px + fl.E[3] * py + ezz * pz;
  x_out[3 * i] = x_base[3 * i] + h * (u[(size_t) i * c] + ux);
  x_out[3 * i + 1] = x_base[3 * i + 1] + h * (u[(size_t) i * c + 1] + uy);
  x_out[3 * i + 2] = x_base[3 * i + 2] + h * (u[(size_t) i * c + 2] + uz);
}

// fixed particles keep their positions in the position array
__global__ void
k_bd_copy (int n, const double *a, double *b)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) b[k] = a[k];
}

// y += x
__global__ void
k_bd_add (int n, const double *x, double *y)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] += x[k];
}

// z (particle order, zc per particle) -> product input (c per particle)
__global__ void
k_bd_zexpand (int np, int nm, int c, const double *z, double *x)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int zc = (c == 3) ? 3 : 6;
  for (int q = 0; q < c; q++)
    x[(size_t) i * c + q] = (i < nm && q < zc) ? z[(size_t) i * zc + q] : 0.0;
}

// product output (c per particle) -> particle order (zc per particle)
__global__ void
k_bd_zcompress (int nm, int c, const double *x, double *z)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm) return;
  const int zc = (c == 3) ? 3 : 6;
  for (int q = 0; q < zc; q++) z[(size_t) i * zc + q] = x[(size_t) i * c + q];
}

// number of pairs i <= j < nm closer than sqrt(rmin) (a_i + a_j) in the
// primary cell (i != j) or, for a periodic system, in one of the 26
// neighbour cells (src/brownian.c:299-375)
__global__ void
k_bd_overlap (int nm, const double *pos, double lx, double ly, double lz, int shear_mode,
              double shift, const double *rad, double rmin, int open, int *count)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm) return;
  int cnt = 0;
  const double ai = rad ? rad[i] : 1.0;
  for (int j = i; j < nm; j++)
    {
      const double x = pos[3 * i] - pos[3 * j], y = pos[3 * i + 1] - pos[3 * j + 1],
                   z = pos[3 * i + 2] - pos[3 * j + 2];
      const double s = ai + (rad ? rad[j] : 1.0), a2 = s * s;
      const int K = open ? 0 : 1;
      for (int kx = -K; kx <= K; kx++)
        for (int ky = -K; ky <= K; ky++)
          for (int kz = -K; kz <= K; kz++)
            {
              if (kx == 0 && ky == 0 && kz == 0 && i == j) continue;
              double xx = x + kx * lx, yy = y + ky * ly, zz = z + kz * lz;
              if (shear_mode == 1) xx += ky * shift;
              else if (shear_mode == 2) xx += kz * shift;
              if (xx * xx + yy * yy + zz * zz < rmin * a2) cnt++;
            }
    }
  if (cnt) atomicAdd (count, cnt);
}

// ---------------------------------------------------------------------------
// engine
// ---------------------------------------------------------------------------
static inline int gridn (long long n) { return (int) ((n + 255) / 256); }

}  // namespace lsg

struct stokes_gpu_bd {
  struct stokes *sys = nullptr;
  lsg::Ctx *c = nullptr;
  stokes_gpu_bd_params p{};
  int nm = 0, np = 0, C = 3, n = 0;   // n = BD_get_n (noise length)
  lsg::DevBuf x, xmid, y, z, f, u, fext, work, lan, tmp, dots, pos_fixed;
  lsg::DevBuf xnew, lje, ljr0, ovl;    // drop-in BD_evolve_mid
  lsg::DevBuf lubv;                    // drop-in lubrication noise: y, z, L y
  bool lj_arrays = false;              // per-particle EV_LJ coefficients in lje, ljr0
  bool ref_lj = false;                 // drop-in: the reference's EV_LJ pair force
  double eig[2] = {0, 0};
  std::vector<double> coef;
  bool have_bounds = false;
  unsigned long long counter = 0;
  double products = 0, estimates = 0, last_err = -1, steps = 0;
  double *h_dots = nullptr;
};

namespace lsg {

static int
bd_prod (stokes_gpu_bd *b, const double *d_pos, const double *d_in, double *d_out)
{
  b->products += 1;
  return atimes_dev (b->c, d_pos, d_in, d_out, b->c->stream, false);
}

// y . y and z . (M z) on the device, returned on the host
static int
bd_error (stokes_gpu_bd *b, const double *d_pos, double *err)
{
  cudaStream_t st = b->c->stream;
  const int n = b->n, nx = b->C * b->np;
  double *zx = (double *) b->tmp.p, *mz = zx + nx;
  k_bd_zexpand<<<gridn (b->np), 256, 0, st>>> (b->np, b->nm, b->C, (const double *) b->z.p, zx);
  int rc = bd_prod (b, d_pos, zx, mz);
  if (rc) return rc;
  double *d = (double *) b->dots.p;
  cudaMemsetAsync (d, 0, 2 * sizeof (double), st);
  k_bd_dot2<<<64, 256, 0, st>>> (nx, zx, mz, zx, zx, d);   // z.Mz (padded slots are 0)
  cudaMemcpyAsync (b->h_dots, d, 2 * sizeof (double), cudaMemcpyDeviceToHost, st);
  cudaMemsetAsync (d, 0, 2 * sizeof (double), st);
  k_bd_dot2<<<64, 256, 0, st>>> (n, (const double *) b->y.p, (const double *) b->y.p,
                                 (const double *) b->y.p, (const double *) b->y.p, d);
  cudaMemcpyAsync (b->h_dots + 2, d, 2 * sizeof (double), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "Chebyshev error");
  const double zz = b->h_dots[0], yyv = b->h_dots[2];
  // a non-positive z.Mz means the noise left the bounds' interval: infinite
  // error, which makes the caller re-estimate the bounds
  *err = (zz > 0.0) ? fabs (zz - yyv) / zz : HUGE_VAL;
  return STOKES_GPU_OK;
}

// smallest / largest eigenvalue of the symmetric tridiagonal (alpha, beta)
// by Sturm-sequence bisection
static double
tridiag_extreme (const std::vector<double> &al, const std::vector<double> &be, bool want_max)
{
  const int m = (int) al.size ();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; i++)
    {
      const double r = (i > 0 ? fabs (be[i]) : 0.0) + (i + 1 < m ? fabs (be[i + 1]) : 0.0);
      lo = std::min (lo, al[i] - r);
      hi = std::max (hi, al[i] + r);
    }
  auto count_below = [&] (double x) {   // eigenvalues < x
    int cnt = 0;
    double d = 1.0;
    for (int i = 0; i < m; i++)
      {
        const double b2 = i > 0 ? be[i] * be[i] : 0.0;
        d = al[i] - x - (i > 0 ? b2 / d : 0.0);
        if (d == 0.0) d = -1e-300;
        if (d < 0.0) cnt++;
      }
    return cnt;
  };
  const int target = want_max ? m - 1 : 0;   // index of the wanted eigenvalue
  for (int it = 0; it < 200; it++)
    {
      const double mid = 0.5 * (lo + hi);
      if (count_below (mid) > target) hi = mid;
      else lo = mid;
      if (hi - lo <= 1e-15 * std::max (fabs (lo), fabs (hi))) break;
    }
  return 0.5 * (lo + hi);
}

static double f_invsqrt (double x) { return 1.0 / sqrt (x); }

// FP64 Lanczos with full reorthogonalisation, m steps, for a symmetric
// operator op on particle-ordered vectors of length b->n (start vector: a
// device Gaussian of stream `stream`): the extreme Ritz values
static int
lanczos_extremes (stokes_gpu_bd *b, int m, unsigned long long stream,
                  const std::function<int (const double *, double *)> &op, double *lmin,
                  double *lmax)
{
  cudaStream_t st = b->c->stream;
  const int n = b->n;
  cudaError_t e;
  if ((e = b->lan.ensure (sizeof (double) * (size_t) (m + 1) * n)) != cudaSuccess)
    return cuda_fail (e, "Lanczos vectors");
  double *V = (double *) b->lan.p;
  double *w = (double *) b->f.p;            // scratch vector of length >= n
  double *dots = (double *) b->dots.p;
  std::vector<double> al, be (1, 0.0), h (m + 1);
  // start vector: device Gaussian, normalised
  k_bd_gauss<<<gridn (n), 256, 0, st>>> (n, b->p.seed ^ 0x9e3779b97f4a7c15ull, stream, V);
  cudaMemsetAsync (dots, 0, 2 * sizeof (double), st);
  k_bd_dot2<<<64, 256, 0, st>>> (n, V, V, V, V, dots);
  cudaMemcpyAsync (b->h_dots, dots, sizeof (double), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "Lanczos");
  k_bd_scale<<<gridn (n), 256, 0, st>>> (n, V, 1.0 / sqrt (b->h_dots[0]), V);
  for (int j = 0; j < m; j++)
    {
      double *vj = V + (size_t) j * n;
      int rc = op (vj, w);
      if (rc) return rc;
      // two rounds of classical Gram-Schmidt against V[0..j]
      for (int pass = 0; pass < 2; pass++)
        {
          k_bd_vdots<<<j + 1, 256, 0, st>>> (n, V, w, dots);
          cudaMemcpyAsync (h.data (), dots, sizeof (double) * (j + 1), cudaMemcpyDeviceToHost, st);
          if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "Lanczos");
          if (pass == 0) al.push_back (h[j]);
          else al[j] += h[j];
          cudaMemcpyAsync (dots, h.data (), sizeof (double) * (j + 1), cudaMemcpyHostToDevice, st);
          k_bd_vaxpy<<<gridn (n), 256, 0, st>>> (n, j + 1, V, dots, w);
        }
      cudaMemsetAsync (dots, 0, 2 * sizeof (double), st);
      k_bd_dot2<<<64, 256, 0, st>>> (n, w, w, w, w, dots);
      cudaMemcpyAsync (b->h_dots, dots, sizeof (double), cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "Lanczos");
      const double beta = sqrt (b->h_dots[0]);
      if (j + 1 == m || beta < 1e-14) break;
      be.push_back (beta);
      k_bd_scale<<<gridn (n), 256, 0, st>>> (n, w, 1.0 / beta, V + (size_t) (j + 1) * n);
    }
  *lmin = tridiag_extreme (al, be, false);
  *lmax = tridiag_extreme (al, be, true);
  return STOKES_GPU_OK;
}

// bounds of the mobility's spectrum (Ritz extremes widened by lo_fac,
// hi_fac) and the coefficients of 1/sqrt on them
static int
bd_lanczos (stokes_gpu_bd *b, const double *d_pos, int m, double lo_fac, double hi_fac)
{
  cudaStream_t st = b->c->stream;
  const int np = b->np, C = b->C, nx = C * np;
  double *xin = (double *) b->tmp.p, *xout = xin + nx;
  double lmin = 0.0, lmax = 0.0;
  int rc = lanczos_extremes (b, m, 77ull, [&] (const double *v, double *w) {
    k_bd_zexpand<<<gridn (np), 256, 0, st>>> (np, b->nm, C, v, xin);
    const int r = bd_prod (b, d_pos, xin, xout);
    if (r) return r;
    k_bd_zcompress<<<gridn (b->nm), 256, 0, st>>> (b->nm, C, xout, w);
    return (int) STOKES_GPU_OK;
  }, &lmin, &lmax);
  if (rc) return rc;
  if (!(lmin > 0.0))
    return set_error (STOKES_GPU_EACCURACY, "mobility not positive definite (Ritz min %g)", lmin);
  b->eig[0] = lmin * lo_fac;
  b->eig[1] = lmax * hi_fac;
  b->coef.assign (b->p.n_cheb, 0.0);
  chebyshev_coef (b->p.n_cheb, f_invsqrt, b->eig[0], b->eig[1], b->coef.data ());
  b->have_bounds = true;
  b->estimates += 1;
  return STOKES_GPU_OK;
}

// z = M^{-1/2} y at d_pos; y, z particle-ordered (length n)
static int
bd_noise (stokes_gpu_bd *b, const double *d_pos)
{
  cudaStream_t st = b->c->stream;
  const int nx = b->C * b->np;
  double *yx = (double *) b->tmp.p, *zx = yx + nx;
  k_bd_zexpand<<<gridn (b->np), 256, 0, st>>> (b->np, b->nm, b->C, (const double *) b->y.p, yx);
  int rc = cheb_clenshaw_dev (b->c, d_pos, b->p.n_cheb, b->coef.data (), nx, yx, zx, b->eig[0],
                              b->eig[1], st, b->work);
  if (rc) return rc;
  b->products += b->p.n_cheb;
  k_bd_zcompress<<<gridn (b->nm), 256, 0, st>>> (b->nm, b->C, zx, (double *) b->z.p);
  return STOKES_GPU_OK;
}

static Flow
bd_flow (const struct stokes *s)
{
  Flow fl;
  for (int q = 0; q < 3; q++) { fl.U[q] = s->Ui[q]; fl.O[q] = s->Oi[q]; }
  for (int q = 0; q < 5; q++) fl.E[q] = s->Ei[q];
  return fl;
}

static int
bd_forces (stokes_gpu_bd *b, const double *d_pos, double fact)
{
  cudaStream_t st = b->c->stream;
  const struct stokes *s = b->sys;
  k_bd_force<<<gridn (b->np), 256, 0, st>>> (b->nm, b->np, b->C, fact, (const double *) b->z.p,
                                             b->fext.p ? (const double *) b->fext.p : nullptr,
                                             (double *) b->f.p);
  if ((b->p.lj_e != 0.0 || b->lj_arrays) && b->ref_lj)
    k_bd_lj<<<gridn (b->nm), 128, 0, st>>> (b->nm, b->np, b->C, d_pos, s->lx, s->ly, s->lz,
                                            s->shear_mode, s->shear_shift,
                                            s->a ? (const double *) b->c->pp.p : nullptr,
                                            b->p.lj_e, b->p.lj_r0,
                                            b->lj_arrays ? (const double *) b->lje.p : nullptr,
                                            b->lj_arrays ? (const double *) b->ljr0.p : nullptr,
                                            s->periodic == 0, (double *) b->f.p);
  else if (b->p.lj_e != 0.0 || b->lj_arrays)
    k_bd_lj_engine<<<(b->nm + LJ_T - 1) / LJ_T, LJ_T, 0, st>>> (
      b->nm, b->np, b->C, d_pos, s->lx, s->ly, s->lz, s->shear_mode, s->shear_shift,
      s->a ? (const double *) b->c->pp.p : nullptr, b->p.lj_e, b->p.lj_r0,
      b->lj_arrays ? (const double *) b->lje.p : nullptr,
      b->lj_arrays ? (const double *) b->ljr0.p : nullptr, s->periodic == 0,
      (double *) b->f.p);
  cudaError_t e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "BD forces");
}

static void
bd_shift (stokes_gpu_bd *b, double t)
{
  // the shear shift at time t, relative to time 0 and shift 0
  if (b->sys->shear_mode != 0) stokes_set_shear_shift (b->sys, t, 0.0, 0.0);
}

// one mid-point step with the noise already in b->y
static int
bd_step (stokes_gpu_bd *b, double t)
{
  cudaStream_t st = b->c->stream;
  const double dt = b->p.dt;
  const double fact = b->p.peclet > 0.0 ? sqrt (2.0 / (b->p.peclet * dt)) : 0.0;
  double *x = (double *) b->x.p, *xmid = (double *) b->xmid.p;
  bd_shift (b, t);
  int rc = prepare (b->c, b->sys, false);
  if (rc) return rc;
  if (!b->have_bounds && (rc = bd_lanczos (b, x, b->p.n_lanczos, 0.8, 1.05))) return rc;
  if ((rc = bd_noise (b, x))) return rc;
  const bool check = b->p.check_every > 0 && ((long long) b->steps % b->p.check_every) == 0;
  if (check)
    {
      double err = 0.0;
      if ((rc = bd_error (b, x, &err))) return rc;
      b->last_err = err;
      if (b->p.cheb_eps > 0.0 && err > b->p.cheb_eps)
        {
          // re-estimate with a longer Krylov space and wider margins, redo z
          if ((rc = bd_lanczos (b, x, 2 * b->p.n_lanczos, 0.5, 1.1))) return rc;
          if ((rc = bd_noise (b, x))) return rc;
          if ((rc = bd_error (b, x, &err))) return rc;
          b->last_err = err;
          if (!(err < HUGE_VAL))
            return set_error (STOKES_GPU_EACCURACY,
                              "non-positive z.Mz after re-estimating the bounds: the mobility "
                              "is not positive definite (overlapping spheres; set rmin)");
        }
    }
  const Flow fl0 = bd_flow (b->sys);
  // 1: velocity at x, half step
  if ((rc = bd_forces (b, x, fact))) return rc;
  if ((rc = bd_prod (b, x, (const double *) b->f.p, (double *) b->u.p))) return rc;
  k_bd_copy<<<gridn (3 * b->np), 256, 0, st>>> (3 * b->np, x, xmid);
  k_bd_euler<<<gridn (b->nm), 256, 0, st>>> (b->nm, b->C, x, (const double *) b->u.p, x, fl0,
                                             0.5 * dt, xmid);
  // 2: velocity at the mid point
  bd_shift (b, t + 0.5 * dt);
  if ((rc = prepare (b->c, b->sys, false))) return rc;
  const Flow fl1 = bd_flow (b->sys);
  if ((rc = bd_forces (b, xmid, fact))) return rc;
  if ((rc = bd_prod (b, xmid, (const double *) b->f.p, (double *) b->u.p))) return rc;
  // 3: full step from x
  k_bd_euler<<<gridn (b->nm), 256, 0, st>>> (b->nm, b->C, x, (const double *) b->u.p, xmid, fl1,
                                             dt, x);
  cudaError_t e = cudaGetLastError ();
  if (e != cudaSuccess) return cuda_fail (e, "BD step");
  b->steps += 1;
  return STOKES_GPU_OK;
}

static int
bd_sync_pos_to_sys (stokes_gpu_bd *b)
{
  cudaError_t e = cudaMemcpyAsync (b->sys->pos, b->x.p, sizeof (double) * 3 * b->np,
                                   cudaMemcpyDeviceToHost, b->c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "positions");
}

}  // namespace lsg

using namespace lsg;

extern "C" {

int
stokes_gpu_bd_create (struct stokes *sys, const struct stokes_gpu_bd_params *p,
                      stokes_gpu_bd **out)
{
  clear_error ();
  if (!sys || !p || !out) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (sys->version < 0 || sys->version > 1)
    return set_error (STOKES_GPU_EINVAL, "the BD engine serves the F and FT versions");
  if (p->n_cheb < 2 || p->n_lanczos < 2 || !(p->dt > 0.0))
    return set_error (STOKES_GPU_EINVAL, "bad BD parameters");
  if (sys->nm != sys->np)
    return set_error (STOKES_GPU_EINVAL, "the BD engine serves systems without fixed particles");
  if (int rc = check_positions (sys->pos, sys->np)) return rc;
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, false);
  if (rc) return rc;
  c->precision = p->precision;
  stokes_gpu_bd *b = new stokes_gpu_bd ();
  b->sys = sys;
  b->c = c;
  b->p = *p;
  b->np = sys->np;
  b->nm = sys->nm;
  b->C = NCOMP (sys->version);
  b->n = (sys->version == 0 ? 3 : 6) * sys->nm;
  const size_t nx = (size_t) b->C * b->np;
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair (&b->x, 3 * (size_t) b->np), std::make_pair (&b->xmid, 3 * (size_t) b->np),
                  std::make_pair (&b->y, (size_t) b->n), std::make_pair (&b->z, (size_t) b->n),
                  std::make_pair (&b->f, std::max (nx, (size_t) b->n)), std::make_pair (&b->u, nx),
                  std::make_pair (&b->tmp, 2 * nx), std::make_pair (&b->dots, (size_t) 1024)})
    if (e == cudaSuccess) e = pr.first->ensure (sizeof (double) * pr.second);
  if (e == cudaSuccess) e = cudaMallocHost (&b->h_dots, 8 * sizeof (double));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (b->x.p, sys->pos, sizeof (double) * 3 * b->np, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  if (e != cudaSuccess)
    {
      stokes_gpu_bd_destroy (b);
      return cuda_fail (e, "BD engine buffers");
    }
  *out = b;
  return STOKES_GPU_OK;
}

int
stokes_gpu_bd_destroy (stokes_gpu_bd *b)
{
  if (!b) return STOKES_GPU_OK;
  if (b->c) cudaStreamSynchronize (b->c->stream);
  for (DevBuf *d : {&b->x, &b->xmid, &b->y, &b->z, &b->f, &b->u, &b->fext, &b->work, &b->lan,
                    &b->tmp, &b->dots, &b->pos_fixed, &b->xnew, &b->lje, &b->ljr0, &b->ovl,
                    &b->lubv})
    d->release ();
  if (b->h_dots) cudaFreeHost (b->h_dots);
  delete b;
  return STOKES_GPU_OK;
}

int
stokes_gpu_bd_set_positions (stokes_gpu_bd *b, const double *x)
{
  clear_error ();
  if (!b || !x) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (int rc = check_positions (x, b->nm)) return rc;
  memcpy (b->sys->pos, x, sizeof (double) * 3 * b->nm);
  cudaError_t e = cudaMemcpyAsync (b->x.p, b->sys->pos, sizeof (double) * 3 * b->np,
                                   cudaMemcpyHostToDevice, b->c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "positions");
}

int
stokes_gpu_bd_get_positions (stokes_gpu_bd *b, double *x)
{
  clear_error ();
  if (!b || !x) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  int rc = bd_sync_pos_to_sys (b);
  if (rc) return rc;
  memcpy (x, b->sys->pos, sizeof (double) * 3 * b->nm);
  return STOKES_GPU_OK;
}

int
stokes_gpu_bd_set_force (stokes_gpu_bd *b, const double *F, const double *T)
{
  clear_error ();
  if (!b) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (!F && !T)
    {
      b->fext.release ();
      return STOKES_GPU_OK;
    }
  std::vector<double> h ((size_t) b->C * b->np, 0.0);
  for (int i = 0; i < b->nm; i++)
    for (int q = 0; q < 3; q++)
      {
        if (F) h[(size_t) i * b->C + q] = F[3 * i + q];
        if (T && b->C >= 6) h[(size_t) i * b->C + 3 + q] = T[3 * i + q];
      }
  cudaError_t e = b->fext.ensure (sizeof (double) * h.size ());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (b->fext.p, h.data (), sizeof (double) * h.size (), cudaMemcpyHostToDevice,
                         b->c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "external force");
}

int
stokes_gpu_bd_estimate_bounds (stokes_gpu_bd *b, double *eig2)
{
  clear_error ();
  if (!b) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  int rc = prepare (b->c, b->sys, false);
  if (!rc) rc = bd_lanczos (b, (const double *) b->x.p, b->p.n_lanczos, 0.8, 1.05);
  if (rc) return rc;
  if (eig2) { eig2[0] = b->eig[0]; eig2[1] = b->eig[1]; }
  return STOKES_GPU_OK;
}

int
stokes_gpu_bd_set_bounds (stokes_gpu_bd *b, const double *eig2)
{
  clear_error ();
  if (!b || !eig2 || !(eig2[0] > 0.0) || !(eig2[1] > eig2[0]))
    return set_error (STOKES_GPU_EINVAL, "bad bounds");
  b->eig[0] = eig2[0];
  b->eig[1] = eig2[1];
  b->coef.assign (b->p.n_cheb, 0.0);
  chebyshev_coef (b->p.n_cheb, f_invsqrt, b->eig[0], b->eig[1], b->coef.data ());
  b->have_bounds = true;
  return STOKES_GPU_OK;
}

int
stokes_gpu_bd_noise (stokes_gpu_bd *b, const double *y, double *z, double *err)
{
  clear_error ();
  if (!b || !y || !z) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  int rc = prepare (b->c, b->sys, false);
  if (rc) return rc;
  if (!b->have_bounds && (rc = bd_lanczos (b, (const double *) b->x.p, b->p.n_lanczos, 0.8, 1.05)))
    return rc;
  cudaMemcpyAsync (b->y.p, y, sizeof (double) * b->n, cudaMemcpyHostToDevice, b->c->stream);
  if ((rc = bd_noise (b, (const double *) b->x.p))) return rc;
  if (err && (rc = bd_error (b, (const double *) b->x.p, err))) return rc;
  cudaError_t e = cudaMemcpyAsync (z, b->z.p, sizeof (double) * b->n, cudaMemcpyDeviceToHost,
                                   b->c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "noise");
}

int
stokes_gpu_bd_step_noise (stokes_gpu_bd *b, double t, const double *y)
{
  clear_error ();
  if (!b || !y) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  cudaError_t e = cudaMemcpyAsync (b->y.p, y, sizeof (double) * b->n, cudaMemcpyHostToDevice,
                                   b->c->stream);
  if (e != cudaSuccess) return cuda_fail (e, "noise upload");
  int rc = bd_step (b, t);
  if (rc) return rc;
  return bd_sync_pos_to_sys (b);
}

int
stokes_gpu_bd_run (stokes_gpu_bd *b, double t, int nsteps)
{
  clear_error ();
  if (!b || nsteps < 0) return set_error (STOKES_GPU_EINVAL, "bad arguments");
  for (int s = 0; s < nsteps; s++)
    {
      k_bd_gauss<<<gridn (b->n), 256, 0, b->c->stream>>> (b->n, b->p.seed, b->counter++,
                                                          (double *) b->y.p);
      int rc = bd_step (b, t + s * b->p.dt);
      if (rc) return rc;
    }
  cudaError_t e = cudaStreamSynchronize (b->c->stream);
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "BD run");
}

int
stokes_gpu_bd_stats (stokes_gpu_bd *b, double *out4)
{
  if (!b || !out4) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  out4[0] = b->products;
  out4[1] = b->estimates;
  out4[2] = b->last_err;
  out4[3] = b->steps;
  return STOKES_GPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// libstokes' own BD routines on the engine (src/brownian.c)
// ---------------------------------------------------------------------------
namespace lsg {

// one engine per BD_params, re-created when the system behind it changes
struct DropinKey {
  struct BD_params *bd;
  struct stokes *sys;
  int np, version, n_minv, precision;
};

static std::mutex g_dropin_mu;
static std::vector<std::pair<DropinKey, stokes_gpu_bd *>> g_dropin;

[[noreturn]] static void
dropin_die (const char *fn, const char *why)
{
  fprintf (stderr, "libstokes_gb300 %s: %s\n", fn, why);
  exit (1);
}

static int
ctx_precision (struct stokes *sys)
{
  int p = STOKES_GPU_FP64;
  return stokes_gpu_get_precision (sys, &p) == STOKES_GPU_OK ? p : STOKES_GPU_FP64;
}

// the engine of BD (created or refreshed); exits like the reference on
// configurations outside the supported branch
static stokes_gpu_bd *
dropin_engine (struct BD_params *BD, const char *fn)
{
  struct stokes *sys = BD->sys;
  if (!sys) dropin_die (fn, "BD->sys is NULL");
  if (sys->version < 0 || sys->version > 1)
    dropin_die (fn, "the device BD serves the F and FT versions");
  if (sys->np != sys->nm) dropin_die (fn, "the device BD serves systems without fixed particles");
  // flag_lub: the velocities solve the lubricated mobility problem.
  // flag_lub_B adds the lubrication noise (the reference's BD_params_init
  // leaves it 0, its pair check being commented out, src/brownian.c:161-180;
  // a caller sets it): its Chebyshev form runs on the device, the matrix
  // form (n_lub <= 0, LAPACK's Cholesky) does not
  if (BD->flag_mat) dropin_die (fn, "the matrix noise is not on the device path");
  if (BD->flag_lub_B && BD->n_lub <= 0)
    dropin_die (fn, "the matrix form of the lubrication noise (n_lub <= 0) is not on the device path");
  if ((BD->flag_lub || BD->flag_lub_B) && (sys->a || sys->slip))
    dropin_die (fn, "lubrication serves equal spheres without slip");
  if (BD->n_minv <= 0) dropin_die (fn, "n_minv <= 0 (matrix noise) is not on the device path");
  if (BD->br || BD->bonds || BD->ev || BD->ang || BD->ev_dh || BD->cf)
    dropin_die (fn, "only EV_LJ among the interactions is on the device path");
  const DropinKey key{BD, sys, sys->np, sys->version, BD->n_minv, ctx_precision (sys)};
  std::lock_guard<std::mutex> lk (g_dropin_mu);
  for (auto &e : g_dropin)
    if (e.first.bd == BD)
      {
        if (!memcmp (&e.first, &key, sizeof key)) return e.second;
        stokes_gpu_bd_destroy (e.second);
        e = g_dropin.back ();
        g_dropin.pop_back ();
        break;
      }
  stokes_gpu_bd_params p{};
  p.peclet = BD->peclet;
  p.dt = 1.0;                     // per call
  p.n_cheb = BD->n_minv;
  p.n_lanczos = 40;
  p.cheb_eps = BD->eps;
  p.check_every = 1;
  p.precision = key.precision;
  stokes_gpu_bd *b = nullptr;
  if (stokes_gpu_bd_create (sys, &p, &b) != STOKES_GPU_OK)
    dropin_die (fn, stokes_gpu_last_error_message ());
  g_dropin.push_back ({key, b});
  return b;
}

static void
check_rc (int rc, const char *fn)
{
  if (rc != STOKES_GPU_OK) dropin_die (fn, stokes_gpu_last_error_message ());
}

static void
upload (DevBuf &d, const double *h, size_t n, cudaStream_t st, const char *fn)
{
  cudaError_t e = d.ensure (sizeof (double) * (n ? n : 1));
  if (e == cudaSuccess && n)
    e = cudaMemcpyAsync (d.p, h, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
}

// per-particle EV_LJ and the constant force/torque of BD
static void
dropin_interactions (stokes_gpu_bd *b, struct BD_params *BD, const char *fn)
{
  cudaStream_t st = b->c->stream;
  b->lj_arrays = BD->ev_LJ != nullptr;
  b->ref_lj = true;
  if (b->lj_arrays)
    {
      if (BD->ev_LJ->n < b->np) dropin_die (fn, "EV_LJ has fewer entries than particles");
      upload (b->lje, BD->ev_LJ->e, (size_t) b->np, st, fn);
      upload (b->ljr0, BD->ev_LJ->r0, (size_t) b->np, st, fn);
    }
  std::vector<double> h ((size_t) b->C * b->np, 0.0);
  for (int i = 0; i < b->nm; i++)
    for (int q = 0; q < 3; q++)
      {
        if (BD->F) h[(size_t) i * b->C + q] = BD->F[3 * i + q];
        if (BD->T && b->C >= 6) h[(size_t) i * b->C + 3 + q] = BD->T[3 * i + q];
      }
  upload (b->fext, h.data (), h.size (), st, fn);
}

// BD_calc_FB's Chebyshev branch on the device: y from BD->rng, z = M^{-1/2} y
// in b->z (particle order) at positions d_pos; bounds and coefficients are
// BD's own (estimated first when eig_minv[0] == eig_minv[1], re-estimated
// when the error exceeds BD->eps), src/brownian.c:1597-1728
static void
dropin_noise (stokes_gpu_bd *b, struct BD_params *BD, const double *d_pos, const char *fn)
{
  std::vector<double> y ((size_t) b->n);
  for (double &v : y) v = KIrand_Gaussian (BD->rng);
  cudaError_t e = cudaMemcpyAsync (b->y.p, y.data (), sizeof (double) * b->n,
                                   cudaMemcpyHostToDevice, b->c->stream);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  b->p.n_cheb = BD->n_minv;
  auto take_bounds = [&] () {
    BD->eig_minv[0] = b->eig[0];
    BD->eig_minv[1] = b->eig[1];
    for (int k = 0; k < BD->n_minv; k++) BD->a_minv[k] = b->coef[k];
  };
  if (BD->eig_minv[0] == BD->eig_minv[1])
    {
      check_rc (bd_lanczos (b, d_pos, b->p.n_lanczos, 0.8, 1.05), fn);
      take_bounds ();
    }
  b->eig[0] = BD->eig_minv[0];
  b->eig[1] = BD->eig_minv[1];
  b->coef.assign (BD->a_minv, BD->a_minv + BD->n_minv);
  check_rc (bd_noise (b, d_pos), fn);
  double err = 0.0;
  check_rc (bd_error (b, d_pos, &err), fn);
  if (err > BD->eps)
    {
      check_rc (bd_lanczos (b, d_pos, b->p.n_lanczos, 0.8, 1.05), fn);
      take_bounds ();
      check_rc (bd_noise (b, d_pos), fn);
      check_rc (bd_error (b, d_pos, &err), fn);
      if (!(err < HUGE_VAL))
        dropin_die (fn, "non-positive z.Mz after re-estimating the bounds (overlapping spheres?)");
    }
  b->last_err = err;
}

static double f_sqrt (double x) { return sqrt (x); }

// BD_calc_FB's lubrication noise on the device, the Chebyshev form
// (flag_lub_B, n_lub > 0; src/brownian.c:1734-1849): y_lub from BD->rng
// after the mobility noise's draws, z_lub = L^{1/2} y_lub with L the
// lubrication correction of the system (calc_lub_3f / 3ft at d_pos:
// BD_atimes_lub_FU for equal spheres without fixed particles), added to the
// noise in b->z.  The bounds of L are BD's own, estimated first when
// eig_lub[0] == eig_lub[1] and again when |y.Ly - z.z| / y.Ly exceeds
// BD->eps (chebyshev_error_Rsqrt), by FP64 Lanczos in place of ARPACK: the
// Ritz extremes widened by (0.8, 1.05), the lower one at least 0 (L is
// positive semi-definite; sqrt needs the interval in [0, inf)).  A system
// with no pair within lubmax has L = 0 and gets z_lub = 0.
static void
dropin_lub_noise (stokes_gpu_bd *b, struct BD_params *BD, const double *d_pos, const char *fn)
{
  const int n = b->n;
  cudaStream_t st = b->c->stream;
  std::vector<double> y ((size_t) n);
  for (double &v : y) v = KIrand_Gaussian (BD->rng);
  if (BD->n_lub <= 0 || !BD->a_lub) dropin_die (fn, "the lubrication noise needs n_lub > 0");
  cudaError_t e = b->lubv.ensure (sizeof (double) * 3 * (size_t) n);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  double *d_y = (double *) b->lubv.p, *d_z = d_y + n, *d_ly = d_z + n;
  e = cudaMemcpyAsync (d_y, y.data (), sizeof (double) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  const struct stokes *sys = BD->sys;
  const auto op = [&] (const double *in, double *out) {
    return lub_dev (sys, sys->version, d_pos, in, out, st);
  };
  auto estimate = [&] () {
    double lmin = 0.0, lmax = 0.0;
    check_rc (lanczos_extremes (b, b->p.n_lanczos, 78ull, op, &lmin, &lmax), fn);
    BD->eig_lub[0] = std::max (0.0, 0.8 * lmin);
    BD->eig_lub[1] = 1.05 * lmax;
    if (BD->eig_lub[1] > BD->eig_lub[0])
      chebyshev_coef (BD->n_lub, f_sqrt, BD->eig_lub[0], BD->eig_lub[1], BD->a_lub);
  };
  auto error = [&] () {
    check_rc (op (d_y, d_ly), fn);
    double *d = (double *) b->dots.p;
    cudaMemsetAsync (d, 0, 2 * sizeof (double), st);
    k_bd_dot2<<<64, 256, 0, st>>> (n, d_y, d_ly, d_z, d_z, d);
    cudaMemcpyAsync (b->h_dots, d, 2 * sizeof (double), cudaMemcpyDeviceToHost, st);
    cudaError_t e2 = cudaStreamSynchronize (st);
    if (e2 != cudaSuccess) dropin_die (fn, cudaGetErrorString (e2));
    const double yy = b->h_dots[0], zz = b->h_dots[1];
    if (!(yy > 0.0)) dropin_die (fn, "negative norm y.Ly of the lubrication noise");
    return fabs (yy - zz) / yy;
  };
  auto evaluate = [&] () {
    check_rc (cheb_clenshaw_op (BD->n_lub, BD->a_lub, n, d_y, d_z, BD->eig_lub[0],
                                BD->eig_lub[1], st, b->work, op), fn);
  };
  if (BD->eig_lub[0] == BD->eig_lub[1]) estimate ();
  // no positive spectrum: no pair within lubmax, L = 0
  if (!(BD->eig_lub[1] > BD->eig_lub[0])) return;
  evaluate ();
  if (error () > BD->eps)
    {
      estimate ();
      if (!(BD->eig_lub[1] > BD->eig_lub[0])) return;
      evaluate ();
      error ();
    }
  k_bd_add<<<gridn (n), 256, 0, st>>> (n, d_z, (double *) b->z.p);
}

static int
dropin_overlap (stokes_gpu_bd *b, const double *d_pos, double rmin, const char *fn)
{
  const struct stokes *s = b->sys;
  cudaStream_t st = b->c->stream;
  cudaError_t e = b->ovl.ensure (sizeof (int));
  if (e == cudaSuccess) e = cudaMemsetAsync (b->ovl.p, 0, sizeof (int), st);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  k_bd_overlap<<<gridn (b->nm), 128, 0, st>>> (b->nm, d_pos, s->lx, s->ly, s->lz, s->shear_mode,
                                               s->shear_shift,
                                               s->a ? (const double *) b->c->pp.p : nullptr, rmin,
                                               s->periodic == 0, (int *) b->ovl.p);
  int cnt = 0;
  e = cudaMemcpyAsync (&cnt, b->ovl.p, sizeof (int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  return cnt;
}

// q += h dQ/dt(q, o) (src/ode-quaternion.c:60-105 with the inverse of the
// quaternion rate matrix written out)
// the velocities of a drop-in step: u = M f, or with lubrication
// u = (I + M L)^-1 M f (src/brownian.c:2420-2428 through solve_mix_3all)
static int
dropin_velocity (stokes_gpu_bd *b, struct BD_params *BD, const double *d_pos)
{
  if (!BD->flag_lub)
    return bd_prod (b, d_pos, (const double *) b->f.p, (double *) b->u.p);
  int it = 0;
  const int rc = lub_mobility_dev (b->c, BD->sys, d_pos, (const double *) b->f.p,
                                   (double *) b->u.p, b->c->stream, &it);
  b->products += it + 1;
  return rc;
}

static void
quaternion_step (int nm, const double *o, double h, const double *q0, double *q)
{
  for (int i = 0; i < nm; i++)
    {
      const double *Q = q0 + 4 * i, *O = o + 3 * i;
      const double den = Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3];
      const double W[4][3] = {{Q[3], -Q[2], Q[1]},
                              {Q[2], Q[3], -Q[0]},
                              {-Q[1], Q[0], Q[3]},
                              {-Q[0], -Q[1], -Q[2]}};
      for (int r = 0; r < 4; r++)
        {
          double d = 0.0;
          for (int j = 0; j < 3; j++) d += 0.5 * (W[r][j] / den) * O[j];
          q[4 * i + r] = Q[r] + h * d;
        }
    }
}

}  // namespace lsg

extern "C" {

double
BD_params_get_fact (struct BD_params *BD, double dt)
{
  return BD->peclet > 0.0 ? sqrt (2.0 / (BD->peclet * dt)) : 0.0;
}

int
BD_get_n (struct stokes *sys)
{
  if (sys->version == 0) return sys->nm * 3;
  if (sys->version == 1 || sys->version == 2) return sys->nm * 6;
  fprintf (stderr, "invalid version %d\n", sys->version);
  exit (1);
}

void
BD_calc_FB (struct BD_params *BD, double *z)
{
  static const char *fn = "BD_calc_FB";
  struct stokes *sys = BD->sys;
  const int n = BD_get_n (sys);
  if (BD->flag_noHI == 1)
    {
      // free-draining noise (src/brownian.c:1552-1595)
      for (int i = 0; i < sys->nm; i++)
        {
          const double as = sys->a ? sqrt (sys->a[i]) : 1.0;
          if (sys->version == 0)
            for (int q = 0; q < 3; q++) z[3 * i + q] = KIrand_Gaussian (BD->rng) * as;
          else
            {
              const double as3 = as * as * as / sqrt (0.75);
              for (int q = 0; q < 3; q++) z[6 * i + q] = KIrand_Gaussian (BD->rng) * as;
              for (int q = 0; q < 3; q++) z[6 * i + 3 + q] = KIrand_Gaussian (BD->rng) * as3;
            }
        }
      return;
    }
  stokes_gpu_bd *b = dropin_engine (BD, fn);
  check_rc (prepare (b->c, sys, false), fn);
  upload (b->x, sys->pos, 3 * (size_t) sys->np, b->c->stream, fn);
  dropin_noise (b, BD, (const double *) b->x.p, fn);
  if (BD->flag_lub_B) dropin_lub_noise (b, BD, (const double *) b->x.p, fn);
  std::vector<double> zp ((size_t) n);
  cudaError_t e = cudaMemcpyAsync (zp.data (), b->z.p, sizeof (double) * n,
                                   cudaMemcpyDeviceToHost, b->c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (b->c->stream);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  // particle order -> [F part, T part] (src/brownian.c:1851-1871)
  const int nm = sys->nm;
  if (sys->version == 0)
    for (int i = 0; i < n; i++) z[i] = zp[i];
  else
    for (int i = 0; i < nm; i++)
      for (int q = 0; q < 3; q++)
        {
          z[3 * i + q] = zp[6 * i + q];
          z[3 * nm + 3 * i + q] = zp[6 * i + 3 + q];
        }
}

double
BD_evolve_mid (double t, struct BD_params *BD, double *x, double *q, double dt)
{
  static const char *fn = "BD_evolve_mid";
  struct stokes *sys = BD->sys;
  stokes_gpu_bd *b = dropin_engine (BD, fn);
  cudaStream_t st = b->c->stream;
  const int nm = sys->nm, np = sys->np, C = b->C;
  const bool rot = sys->version > 0 && q != nullptr;
  cudaError_t e = b->xnew.ensure (sizeof (double) * 3 * np);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  dropin_interactions (b, BD, fn);
  double *dx = (double *) b->x.p, *dmid = (double *) b->xmid.p, *dnew = (double *) b->xnew.p;
  std::vector<double> o ((size_t) 3 * nm), uh ((size_t) C * np), qmid;
  if (rot) qmid.assign (q, q + 4 * (size_t) nm);

  double dt_local = dt;
  double fact = BD_params_get_fact (BD, dt_local);
  const double *cur = dx;            // the configuration sys->pos holds
  // the overlap checks run only without the real-space clamp
  const bool check = sys->rmin == 0.0 && BD->rmin > 0.0;

redo:
  upload (b->x, x, 3 * (size_t) np, st, fn);
  memcpy (sys->pos, x, sizeof (double) * 3 * nm);
  cur = dx;
  stokes_set_shear_shift (sys, t, BD->t0, BD->s0);
  check_rc (prepare (b->c, sys, false), fn);
redo_fb:
  dropin_noise (b, BD, cur, fn);
  if (BD->flag_lub_B) dropin_lub_noise (b, BD, cur, fn);
redo_scale:
  {
    // 1: velocity at the current configuration, Euler half step from x
    const Flow fl = bd_flow (sys);
    check_rc (bd_forces (b, cur, fact), fn);
    check_rc (dropin_velocity (b, BD, cur), fn);
    k_bd_euler<<<gridn (nm), 256, 0, st>>> (nm, C, dx, (const double *) b->u.p, cur, fl,
                                            0.5 * dt_local, dmid);
    if (check && dropin_overlap (b, dmid, BD->rmin, fn) > 0)
      {
        dt_local *= 0.5;
        if (dt_local < BD->dt_lim)
          {
            fprintf (stderr, "# mid-point: overlap in 1st step. dt = %e < %e => reconstruct FB\n",
                     dt_local, BD->dt_lim);
            dt_local = dt;
            goto redo_fb;
          }
        fact = BD_params_get_fact (BD, dt_local);
        fprintf (stderr, "# mid-point: overlap in 1st step. dt = %e > %e\n", dt_local, BD->dt_lim);
        goto redo_scale;
      }
    // 2: velocity at the mid point, full step from x
    cur = dmid;
    e = cudaMemcpyAsync (sys->pos, dmid, sizeof (double) * 3 * nm, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
    stokes_set_shear_shift (sys, t + 0.5 * dt_local, BD->t0, BD->s0);
    check_rc (prepare (b->c, sys, false), fn);
    const Flow fm = bd_flow (sys);
    check_rc (bd_forces (b, dmid, fact), fn);
    check_rc (dropin_velocity (b, BD, dmid), fn);
    k_bd_euler<<<gridn (nm), 256, 0, st>>> (nm, C, dx, (const double *) b->u.p, dmid, fm,
                                            dt_local, dnew);
    if (check && dropin_overlap (b, dnew, BD->rmin, fn) > 0)
      {
        dt_local *= 0.5;
        if (dt_local < BD->dt_lim)
          {
            fprintf (stderr, "# mid-point: overlap in 2nd step. dt = %e < %e => reconstruct FB\n",
                     dt_local, BD->dt_lim);
            dt_local = dt;
            goto redo;
          }
        fact = BD_params_get_fact (BD, dt_local);
        fprintf (stderr, "# mid-point: overlap in 2nd step. dt = %e > %e\n", dt_local, BD->dt_lim);
        // as in the reference, the redo of the first stage starts from the
        // configuration and shear shift the system holds now (the mid point)
        goto redo_scale;
      }
    if (rot)
      {
        e = cudaMemcpyAsync (uh.data (), b->u.p, sizeof (double) * C * np, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize (st);
        if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
        for (int i = 0; i < nm; i++)
          for (int k = 0; k < 3; k++) o[3 * i + k] = uh[(size_t) i * C + 3 + k] + sys->Oi[k];
        quaternion_step (nm, o.data (), dt_local, q, qmid.data ());
        memcpy (q, qmid.data (), sizeof (double) * 4 * nm);
      }
  }
  e = cudaMemcpyAsync (x, dnew, sizeof (double) * 3 * nm, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) dropin_die (fn, cudaGetErrorString (e));
  b->steps += 1;
  return dt_local;
}

// src/brownian.c:105-260 (no bead-rod, bond-group or lubrication set-up on
// the device path; those pointers are kept for the caller)
struct BD_params *
BD_params_init (struct stokes *sys, unsigned long seed, double *F, double *T, double *E,
                double *uf, double *of, double *ef, int flag_noHI, int flag_lub, int flag_mat,
                double st, struct BeadRod *br, struct BONDS *bonds, double gamma, struct EV *ev,
                struct angles *ang, struct EV_DH *ev_dh, struct EV_LJ *ev_LJ,
                struct confinement *cf, int flag_Q, double peclet, double eps, int n_minv,
                int n_lub, int scheme, double BB_n, double rmin, double dt_lim)
{
  struct BD_params *BD = (struct BD_params *) calloc (1, sizeof (struct BD_params));
  if (!BD) dropin_die ("BD_params_init", "out of memory");
  BD->sys = sys;
  BD->rng = KIrand_init ();
  KIrand_init_genrand (BD->rng, seed);
  BD->F = F; BD->T = T; BD->E = E;
  BD->uf = uf; BD->of = of; BD->ef = ef;
  BD->flag_noHI = flag_noHI;
  BD->flag_mat = flag_mat;
  BD->flag_lub = flag_lub;
  BD->flag_lub_B = 0;
  BD->st = st;
  BD->br = br;
  BD->bonds = bonds;
  BD->groups = nullptr;
  BD->gamma = gamma;
  BD->ev = ev; BD->ang = ang; BD->ev_dh = ev_dh; BD->ev_LJ = ev_LJ; BD->cf = cf;
  BD->flag_Q = flag_Q;
  BD->peclet = peclet;
  BD->eps = eps;
  BD->n_minv = n_minv;
  BD->a_minv = n_minv > 0 ? (double *) calloc ((size_t) n_minv, sizeof (double)) : nullptr;
  BD->n_lub = n_lub;
  BD->a_lub = n_lub > 0 ? (double *) calloc ((size_t) n_lub, sizeof (double)) : nullptr;
  BD->scheme = scheme;
  BD->BB_n = BB_n;
  BD->rmin = rmin;
  BD->dt_lim = dt_lim;
  return BD;
}

// src/brownian.c:262-277; also releases the device engine of BD
void
BD_params_free (struct BD_params *BD)
{
  if (!BD) return;
  {
    std::lock_guard<std::mutex> lk (g_dropin_mu);
    for (size_t k = 0; k < g_dropin.size (); k++)
      if (g_dropin[k].first.bd == BD)
        {
          stokes_gpu_bd_destroy (g_dropin[k].second);
          g_dropin[k] = g_dropin.back ();
          g_dropin.pop_back ();
          break;
        }
  }
  if (BD->rng) KIrand_free (BD->rng);
  free (BD->a_minv);
  free (BD->a_lub);
  free (BD);
}

// src/ev-LJ.c:35-81
struct EV_LJ *
EV_LJ_init (int np)
{
  struct EV_LJ *lj = (struct EV_LJ *) malloc (sizeof (struct EV_LJ));
  if (!lj) dropin_die ("EV_LJ_init", "out of memory");
  lj->n = np;
  lj->flag = (int *) calloc ((size_t) np, sizeof (int));
  lj->e = (double *) calloc ((size_t) np, sizeof (double));
  lj->r0 = (double *) calloc ((size_t) np, sizeof (double));
  if (!lj->flag || !lj->e || !lj->r0) dropin_die ("EV_LJ_init", "out of memory");
  return lj;
}

void
EV_LJ_free (struct EV_LJ *lj)
{
  if (!lj) return;
  free (lj->flag);
  free (lj->e);
  free (lj->r0);
  free (lj);
}

// e -> e / (peclet r0) for the entries not scaled yet
void
EV_LJ_scale (struct EV_LJ *lj, double peclet)
{
  if (!lj) return;
  for (int i = 0; i < lj->n; i++)
    if (lj->flag[i] == 0)
      {
        lj->flag[i] = 1;
        lj->e[i] /= peclet * lj->r0[i];
      }
}

}  // extern "C"
