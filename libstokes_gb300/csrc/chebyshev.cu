// chebyshev.cu -- Chebyshev routines of libstokes_gb300 (replace
// src/chebyshev.c).  Coefficients and scalar evaluation stay FP64 on the
// host.  chebyshev_eval_atimes keeps the whole Clenshaw recurrence on the
// GPU when the operator is this library's Ewald product: y goes up once,
// ncheb products and vector updates run back to back on the device, z comes
// back once.  Any other operator is driven through its function pointer on
// host vectors, exactly like the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <vector>

#include "stokes_gpu.h"
#include "gpu_engine.h"

namespace lsg {

// out = ca * x + cb * b1 - b0 + cj * y
__global__ void
k_clenshaw (int n, const double *x, const double *b1, const double *b0, const double *y,
            double ca, double cb, double cj, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = ca * x[k] + cb * b1[k] - b0[k] + cj * y[k];
}

// Clenshaw recurrence with every operator application on the device.  op
// maps a device vector of length n to another (stream st).  d_y, d_z:
// device vectors of length n.  Scratch: 4 vectors of n in work.
int
cheb_clenshaw_op (int ncheb, const double *a, int n, const double *d_y, double *d_z, double e0,
                  double e1, cudaStream_t st, DevBuf &work,
                  const std::function<int (const double *, double *)> &op)
{
  cudaError_t e = work.ensure (sizeof (double) * 4 * (size_t) n);
  if (e != cudaSuccess) return cuda_fail (e, "Chebyshev work vectors");
  double *x = (double *) work.p;
  double *b[3] = {x + n, x + 2 * (size_t) n, x + 3 * (size_t) n};
  cudaMemsetAsync (b[0], 0, sizeof (double) * n, st);
  cudaMemsetAsync (b[1], 0, sizeof (double) * n, st);
  const double da = 2.0 / (e1 - e0);
  const double db = -(e1 + e0) / (e1 - e0);
  const int grid = (n + 255) / 256;
  for (int i = 0; i < ncheb - 1; i++)
    {
      double *bi2 = b[(i + 2) % 3], *bi1 = b[(i + 1) % 3], *bi0 = b[i % 3];
      const int j = ncheb - 1 - i;
      int rc = op (bi1, x);
      if (rc) return rc;
      k_clenshaw<<<grid, 256, 0, st>>> (n, x, bi1, bi0, d_y, 2.0 * da, 2.0 * db, a[j], bi2);
    }
  const int i = ncheb - 1;
  double *bi1 = b[(i + 1) % 3], *bi0 = b[i % 3];
  int rc = op (bi1, x);
  if (rc) return rc;
  k_clenshaw<<<grid, 256, 0, st>>> (n, x, bi1, bi0, d_y, da, db, a[0], d_z);
  e = cudaGetLastError ();
  if (e != cudaSuccess) return cuda_fail (e, "Clenshaw kernel");
  return STOKES_GPU_OK;
}

// the same with the context's mobility product at positions d_pos
int
cheb_clenshaw_dev (Ctx *c, const double *d_pos, int ncheb, const double *a, int n,
                   const double *d_y, double *d_z, double e0, double e1, cudaStream_t st,
                   DevBuf &work)
{
  return cheb_clenshaw_op (ncheb, a, n, d_y, d_z, e0, e1, st, work,
                           [&] (const double *in, double *out) {
                             return atimes_dev (c, d_pos, in, out, st, false);
                           });
}

}  // namespace lsg

using namespace lsg;

extern "C" {

// Chebyshev nodes on [x0, x1] (src/chebyshev.c:33-61)
void
chebyshev_coef (int ncheb, double (*func) (double), double x0, double x1, double *a)
{
  const double h = 0.5 * (x1 - x0), m = 0.5 * (x1 + x0);
  std::vector<double> fv (ncheb), th (ncheb);
  for (int k = 1; k <= ncheb; k++)
    {
      th[k - 1] = M_PI * ((double) k - 0.5) / (double) ncheb;
      fv[k - 1] = func (cos (th[k - 1]) * h + m);
    }
  for (int j = 0; j < ncheb; j++)
    {
      double s = 0.0;
      for (int k = 0; k < ncheb; k++) s += fv[k] * cos ((double) j * th[k]);
      a[j] = 2.0 / (double) ncheb * s;
    }
  a[0] *= 0.5;
}

// Clenshaw (src/chebyshev.c:74-105)
double
chebyshev_eval (int ncheb, const double *a, double x0, double x1, double x)
{
  const double t = (x - 0.5 * (x1 + x0)) / (0.5 * (x1 - x0));
  double bk1 = 0.0, bk2 = 0.0;   // b_{k+1}, b_{k+2}
  for (int j = ncheb - 1; j >= 1; j--)
    {
      const double bk = 2.0 * t * bk1 - bk2 + a[j];
      bk2 = bk1;
      bk1 = bk;
    }
  return t * bk1 - bk2 + a[0];
}

// explicit three-term recurrence (src/chebyshev.c:117-148)
double
chebyshev_eval_ (int ncheb, const double *a, double x0, double x1, double x)
{
  const double t = (x - 0.5 * (x1 + x0)) / (0.5 * (x1 - x0));
  double f = a[0];
  if (ncheb < 2) return f;
  double tm = 1.0, tc = t;
  f += a[1] * tc;
  for (int k = 2; k < ncheb; k++)
    {
      const double tn = 2.0 * t * tc - tm;
      tm = tc;
      tc = tn;
      f += a[k] * tc;
    }
  return f;
}

static bool
is_device_operator (void (*atimes) (int, const double *, double *, void *), void *user_data)
{
  // the operator the device evaluates for this system: the Ewald sum of a
  // periodic system, the free-space sum of an open one, or the dispatcher
  const struct stokes *sys = (const struct stokes *) user_data;
  if (sys == nullptr) return false;
  if (atimes == atimes_3all) return true;
  if (atimes == atimes_ewald_3all) return sys->periodic != 0;
  if (atimes == atimes_nonewald_3all) return sys->periodic == 0;
  return false;
}

// z = sum_k a_k T_k(M~) y by Clenshaw (src/chebyshev.c:163-228)
void
chebyshev_eval_atimes (int ncheb, const double *a, int n, const double *y, double *z,
                       double eign0, double eign1,
                       void (*atimes) (int, const double *, double *, void *), void *user_data)
{
  if (is_device_operator (atimes, user_data))
    {
      struct stokes *sys = (struct stokes *) user_data;
      Ctx *c = get_ctx (sys, true);
      int rc = c ? prepare (c, sys, false) : set_error (STOKES_GPU_ECUDA, "no CUDA stream");
      if (!rc && n != NCOMP (sys->version) * sys->np)
        rc = set_error (STOKES_GPU_EINVAL, "n = %d does not match the system", n);
      static thread_local DevBuf dy, work;
      if (!rc)
        {
          cudaError_t e = dy.ensure (sizeof (double) * 2 * (size_t) n);
          if (e == cudaSuccess) e = c->pos.ensure (sizeof (double) * 3 * sys->np);
          if (e != cudaSuccess) rc = cuda_fail (e, "Chebyshev vectors");
        }
      if (!rc)
        {
          double *d_y = (double *) dy.p, *d_z = d_y + n;
          cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * sys->np,
                           cudaMemcpyHostToDevice, c->stream);
          cudaMemcpyAsync (d_y, y, sizeof (double) * n, cudaMemcpyHostToDevice, c->stream);
          rc = cheb_clenshaw_dev (c, (const double *) c->pos.p, ncheb, a, n, d_y, d_z, eign0,
                                  eign1, c->stream, work);
          if (!rc)
            {
              cudaError_t e = cudaMemcpyAsync (z, d_z, sizeof (double) * n,
                                               cudaMemcpyDeviceToHost, c->stream);
              if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
              if (e != cudaSuccess) rc = cuda_fail (e, "Chebyshev");
            }
        }
      if (rc) dropin_failed ("chebyshev_eval_atimes", z, n > 0 ? (size_t) n : 0);
      return;
    }

  // generic operator: host vectors, as in the reference
  std::vector<double> x (n), b (3 * (size_t) n, 0.0);
  const double da = 2.0 / (eign1 - eign0);
  const double db = -(eign1 + eign0) / (eign1 - eign0);
  for (int i = 0; i < ncheb - 1; i++)
    {
      double *bi2 = &b[(size_t) ((i + 2) % 3) * n];
      double *bi1 = &b[(size_t) ((i + 1) % 3) * n];
      double *bi0 = &b[(size_t) (i % 3) * n];
      const int j = ncheb - 1 - i;
      atimes (n, bi1, x.data (), user_data);
      for (int k = 0; k < n; k++)
        bi2[k] = 2.0 * da * x[k] + 2.0 * db * bi1[k] - bi0[k] + a[j] * y[k];
    }
  const int i = ncheb - 1;
  double *bi1 = &b[(size_t) ((i + 1) % 3) * n];
  double *bi0 = &b[(size_t) (i % 3) * n];
  atimes (n, bi1, x.data (), user_data);
  for (int k = 0; k < n; k++) z[k] = da * x[k] + db * bi1[k] - bi0[k] + a[0] * y[k];
}

// |z.Mz - y.y| / z.Mz (src/chebyshev.c:241-269)
double
chebyshev_error_minvsqrt (int n, const double *y, const double *z,
                          void (*atimes) (int, const double *, double *, void *), void *user_data)
{
  std::vector<double> x (n);
  atimes (n, z, x.data (), user_data);
  double yy = 0.0, zz = 0.0;
  for (int k = 0; k < n; k++)
    {
      yy += y[k] * y[k];
      zz += z[k] * x[k];
    }
  if (zz <= 0.0)
    {
      fprintf (stderr, "negative norm! %e\n", zz);
      exit (1);
    }
  return fabs (zz - yy) / zz;
}

// |y.Ry - z.z| / y.Ry (src/chebyshev.c:282-310)
double
chebyshev_error_Rsqrt (int n, const double *y, const double *z,
                       void (*atimes) (int, const double *, double *, void *), void *user_data)
{
  std::vector<double> x (n);
  atimes (n, y, x.data (), user_data);
  double yy = 0.0, zz = 0.0;
  for (int k = 0; k < n; k++)
    {
      yy += y[k] * x[k];
      zz += z[k] * z[k];
    }
  if (yy <= 0.0)
    {
      fprintf (stderr, "negative norm! %e\n", yy);
      exit (1);
    }
  return fabs (yy - zz) / yy;
}

}  // extern "C"
