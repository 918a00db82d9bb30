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
#include <vector>

#include "engine.h"
#include "gpu_engine.h"
#include "stokes_bd.h"

namespace lsg {

int cheb_clenshaw_dev (Ctx *c, const double *d_pos, int ncheb, const double *a, int n,
                       const double *d_y, double *d_z, double e0, double e1, cudaStream_t st,
                       DevBuf &work);

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
// overlap; the candidates are redone exactly in FP64.
__global__ void
k_bd_lj (int nm, int np, int c, const double *pos, double lx, double ly, double lz,
         int shear_mode, double shift, const double *rad, double e, double r0, double *f)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nm) return;
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const double ai = rad ? rad[i] : 1.0;
  const float flx = (float) lx, fly = (float) ly, flz = (float) lz;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int j = 0; j < np; j++)
    {
      if (j == i) continue;
      const double aj = rad ? rad[j] : 1.0;
      const double x = xi - pos[3 * j], y = yi - pos[3 * j + 1], z = zi - pos[3 * j + 2];
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

// FP64 Lanczos with full reorthogonalisation, m steps
static int
bd_lanczos (stokes_gpu_bd *b, const double *d_pos, int m, double lo_fac, double hi_fac)
{
  cudaStream_t st = b->c->stream;
  const int n = b->n, np = b->np, C = b->C, nx = C * np;
  cudaError_t e;
  if ((e = b->lan.ensure (sizeof (double) * (size_t) (m + 1) * n)) != cudaSuccess)
    return cuda_fail (e, "Lanczos vectors");
  double *V = (double *) b->lan.p;
  double *w = (double *) b->f.p;            // scratch vector of length >= n
  double *xin = (double *) b->tmp.p, *xout = xin + nx;
  double *dots = (double *) b->dots.p;
  std::vector<double> al, be (1, 0.0), h (m + 1);
  // start vector: device Gaussian, normalised
  k_bd_gauss<<<gridn (n), 256, 0, st>>> (n, b->p.seed ^ 0x9e3779b97f4a7c15ull, 77ull, V);
  cudaMemsetAsync (dots, 0, 2 * sizeof (double), st);
  k_bd_dot2<<<64, 256, 0, st>>> (n, V, V, V, V, dots);
  cudaMemcpyAsync (b->h_dots, dots, sizeof (double), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "Lanczos");
  k_bd_scale<<<gridn (n), 256, 0, st>>> (n, V, 1.0 / sqrt (b->h_dots[0]), V);
  for (int j = 0; j < m; j++)
    {
      double *vj = V + (size_t) j * n;
      k_bd_zexpand<<<gridn (np), 256, 0, st>>> (np, b->nm, C, vj, xin);
      int rc = bd_prod (b, d_pos, xin, xout);
      if (rc) return rc;
      k_bd_zcompress<<<gridn (b->nm), 256, 0, st>>> (b->nm, C, xout, w);
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
  const double lmin = tridiag_extreme (al, be, false), lmax = tridiag_extreme (al, be, true);
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
  if (b->p.lj_e != 0.0)
    k_bd_lj<<<gridn (b->nm), 128, 0, st>>> (b->nm, b->np, b->C, d_pos, s->lx, s->ly, s->lz,
                                            s->shear_mode, s->shear_shift,
                                            s->a ? (const double *) b->c->pp.p : nullptr,
                                            b->p.lj_e, b->p.lj_r0, (double *) b->f.p);
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
                    &b->tmp, &b->dots, &b->pos_fixed})
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
