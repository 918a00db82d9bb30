// krylov.cu -- restarted GMRES on the device: libstokes' iterative solves.
//
// libstokes solves its resistance, mixed and FTS mobility problems with an
// external solver library through iter_init / solve_iter / iter_free
// (src/stokes.c:790-812, src/ewald-3f.c:94, src/ewald-3ft.c:113,
// src/ewald-3fts.c:71 and :286-297).  The replacement here is GMRES(m)
// (Saad and Schultz, 1986) with classical Gram-Schmidt applied twice
// (CGS2), so that each orthogonalisation is two passes of block dot
// products and block updates over the Krylov basis held in HBM:
//
//   k_mdot / k_mdot_fin   h = V^T w in two deterministic stages
//   k_vcombine            w += sign V c   (orthogonalisation, x update)
//   k_vnormalize          v = w / |w| with |w| read on the device
//   k_vaxpby              r = b - A x and the like
//
// The Givens rotations of the (m+1) x m Hessenberg matrix run on the host
// from one small copy per iteration; everything of length n stays on the
// device.  The operator is this library's product (atimes_dev, FP64 or
// mixed per the system's precision) or, for a foreign atimes, the caller's
// function on host copies.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include "gpu_engine.h"
#include "stokes_gpu.h"
#include "stokes_iter.h"

namespace lsg {
namespace {

constexpr int KT = 256;          // threads of the vector kernels
constexpr int MDOT_CHUNK = 8192; // elements per block of a partial dot product

__device__ __forceinline__ double
block_sum (double v)
{
  __shared__ double sh[KT / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync (0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads ();
  v = 0.0;
  if (threadIdx.x < 32)
    {
      v = threadIdx.x < KT / 32 ? sh[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync (0xffffffffu, v, o);
    }
  return v;
}

// part[k * nch + ch] = sum over chunk ch of V_k[i] w[i]
__global__ void __launch_bounds__ (KT)
k_mdot (const double *V, size_t ldv, const double *w, int n, int nch, double *part)
{
  const int k = blockIdx.y, ch = blockIdx.x;
  const int i0 = ch * MDOT_CHUNK, i1 = min (n, i0 + MDOT_CHUNK);
  const double *v = V + (size_t) k * ldv;
  double s = 0.0;
  for (int i = i0 + threadIdx.x; i < i1; i += KT) s += v[i] * w[i];
  s = block_sum (s);
  if (threadIdx.x == 0) part[(size_t) k * nch + ch] = s;
}

// out[k] = sum_ch part[k * nch + ch] (+ out[k] when accumulate)
__global__ void
k_mdot_fin (const double *part, int nch, int J, int accumulate, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= J) return;
  double s = 0.0;
  for (int ch = 0; ch < nch; ch++) s += part[(size_t) k * nch + ch];
  out[k] = accumulate ? out[k] + s : s;
}

// w[i] += sign sum_{k < J} V_k[i] c[k]
__global__ void __launch_bounds__ (KT)
k_vcombine (double *w, const double *V, size_t ldv, const double *c, int J, int n, double sign)
{
  const int i = blockIdx.x * KT + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < J; k++) s += V[(size_t) k * ldv + i] * c[k];
  w[i] += sign * s;
}

// v = w / sqrt(nrm2[0]); hout = sqrt(nrm2[0]) (v = 0 when w = 0)
__global__ void __launch_bounds__ (KT)
k_vnormalize (const double *w, const double *nrm2, double *hout, double *v, int n)
{
  const int i = blockIdx.x * KT + threadIdx.x;
  const double nr = sqrt (nrm2[0]);
  if (i == 0) *hout = nr;
  if (i < n) v[i] = nr > 0.0 ? w[i] / nr : 0.0;
}

// z = a x + b y
__global__ void __launch_bounds__ (KT)
k_vaxpby (int n, double a, const double *x, double b, const double *y, double *z)
{
  const int i = blockIdx.x * KT + threadIdx.x;
  if (i < n) z[i] = a * x[i] + b * y[i];
}

// the FTS mobility operator around the product (src/ewald-3fts.c:200-247):
// mask: t = (0, 0, s) of x = (u, o, s); out: y = (u, o, 0) - z
__global__ void __launch_bounds__ (KT)
k_fts_mask (int np, const double *x, double *t)
{
  const int k = blockIdx.x * KT + threadIdx.x;
  if (k >= 11 * np) return;
  t[k] = (k % 11) < 6 ? 0.0 : x[k];
}

__global__ void __launch_bounds__ (KT)
k_fts_mob_out (int np, const double *x, const double *z, double *y)
{
  const int k = blockIdx.x * KT + threadIdx.x;
  if (k >= 11 * np) return;
  y[k] = ((k % 11) < 6 ? x[k] : 0.0) - z[k];
}

inline int grid_of (long long n) { return (int) ((n + KT - 1) / KT); }

// device workspace of the solver (one per host thread)
struct Krylov {
  DevBuf V, w, t, part, h, h2, s2, cv, b, x;
  double *pin = nullptr;     // pinned host staging: h column or scalars
  size_t pin_cap = 0;
  cudaStream_t own = nullptr;  // stream for foreign operators
  ~Krylov ()
  {
    for (DevBuf *d : {&V, &w, &t, &part, &h, &h2, &s2, &cv, &b, &x}) d->release ();
    if (pin) cudaFreeHost (pin);
    if (own) cudaStreamDestroy (own);
  }
  cudaError_t pinned (size_t count)
  {
    if (count <= pin_cap) return cudaSuccess;
    if (pin) cudaFreeHost (pin);
    pin = nullptr;
    pin_cap = 0;
    cudaError_t e = cudaMallocHost (&pin, sizeof (double) * count);
    if (e == cudaSuccess) pin_cap = count;
    return e;
  }
};
thread_local Krylov t_kry;

using Apply = std::function<int (const double *d_in, double *d_out)>;

struct Gmres {
  Krylov &K;
  int n, m;
  cudaStream_t st;
  int nch;

  // out[0..J) = V[0..J)^T w (device); accumulate adds to out
  void mdot (const double *V, int J, const double *w, double *out, int accumulate)
  {
    k_mdot<<<dim3 (nch, J), KT, 0, st>>> (V, (size_t) n, w, n, nch, (double *) K.part.p);
    k_mdot_fin<<<(J + 31) / 32, 32, 0, st>>> ((const double *) K.part.p, nch, J, accumulate, out);
  }

  // |v|^2 to the host
  int norm2_host (const double *v, double *out)
  {
    mdot (v, 1, v, (double *) K.s2.p, 0);
    cudaMemcpyAsync (K.pin, K.s2.p, sizeof (double), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize (st);
    if (e != cudaSuccess) return cuda_fail (e, "GMRES norm");
    *out = K.pin[0];
    return STOKES_GPU_OK;
  }
};

// restarted GMRES; d_b, d_x device vectors of length n (d_x: start vector in,
// solution out)
int
gmres_dev (int n, const double *d_b, double *d_x, const Apply &A, int m, int maxit, double eps,
           cudaStream_t st, int *iters, double *res, FILE *dbg)
{
  Krylov &K = t_kry;
  if (m > n) m = n;
  if (m < 1) m = 1;
  Gmres G {K, n, m, st, (n + MDOT_CHUNK - 1) / MDOT_CHUNK};
  cudaError_t e;
  if ((e = K.V.ensure (sizeof (double) * (size_t) (m + 1) * n)) != cudaSuccess
      || (e = K.w.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.part.ensure (sizeof (double) * (size_t) (m + 1) * G.nch)) != cudaSuccess
      || (e = K.h.ensure (sizeof (double) * (m + 2))) != cudaSuccess
      || (e = K.h2.ensure (sizeof (double) * (m + 2))) != cudaSuccess
      || (e = K.s2.ensure (sizeof (double) * 2)) != cudaSuccess
      || (e = K.cv.ensure (sizeof (double) * (m + 1))) != cudaSuccess
      || (e = K.pinned ((size_t) m + 2)) != cudaSuccess)
    return cuda_fail (e, "GMRES workspace");
  double *V = (double *) K.V.p, *w = (double *) K.w.p, *h = (double *) K.h.p;
  double *h2 = (double *) K.h2.p;
  const int gn = grid_of (n);

  int rc;
  double bn2;
  if ((rc = G.norm2_host (d_b, &bn2))) return rc;
  const double bnrm = sqrt (bn2);
  *iters = 0;
  if (!(bnrm > 0.0))
    {
      cudaMemsetAsync (d_x, 0, sizeof (double) * n, st);
      *res = 0.0;
      e = cudaStreamSynchronize (st);
      return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "GMRES");
    }

  std::vector<double> H ((size_t) (m + 1) * m), cs (m), sn (m), g (m + 1), y (m);
  int total = 0;
  double rel = HUGE_VAL;
  for (;;)
    {
      // r = b - A x into V_0
      if ((rc = A (d_x, w))) return rc;
      k_vaxpby<<<gn, KT, 0, st>>> (n, 1.0, d_b, -1.0, w, V);
      double beta2;
      if ((rc = G.norm2_host (V, &beta2))) return rc;
      const double beta = sqrt (beta2);
      rel = beta / bnrm;
      if (dbg) fprintf (dbg, "gmres: %d applications, residual %.6e\n", total, rel);
      if (rel <= eps || total >= maxit) break;
      k_vaxpby<<<gn, KT, 0, st>>> (n, 1.0 / beta, V, 0.0, V, V);
      std::fill (g.begin (), g.end (), 0.0);
      g[0] = beta;
      int j = 0;
      bool done = false;
      for (; j < m && total < maxit; j++)
        {
          double *vj = V + (size_t) j * n, *vn = V + (size_t) (j + 1) * n;
          if ((rc = A (vj, w))) return rc;
          total++;
          // CGS2: h = V^T w, w -= V h, twice
          G.mdot (V, j + 1, w, h, 0);
          k_vcombine<<<gn, KT, 0, st>>> (w, V, (size_t) n, h, j + 1, n, -1.0);
          G.mdot (V, j + 1, w, h2, 0);
          k_vcombine<<<gn, KT, 0, st>>> (w, V, (size_t) n, h2, j + 1, n, -1.0);
          k_vaxpby<<<1, KT, 0, st>>> (j + 1, 1.0, h, 1.0, h2, h);
          G.mdot (w, 1, w, (double *) K.s2.p, 0);
          k_vnormalize<<<gn, KT, 0, st>>> (w, (const double *) K.s2.p, h + j + 1, vn, n);
          cudaMemcpyAsync (K.pin, h, sizeof (double) * (j + 2), cudaMemcpyDeviceToHost, st);
          if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "GMRES step");
          // Givens rotations of column j of the Hessenberg matrix
          double *col = &H[(size_t) j * (m + 1)];
          for (int i = 0; i <= j + 1; i++) col[i] = K.pin[i];
          for (int i = 0; i < j; i++)
            {
              const double t0 = cs[i] * col[i] + sn[i] * col[i + 1];
              col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
              col[i] = t0;
            }
          const double r = hypot (col[j], col[j + 1]);
          cs[j] = r > 0.0 ? col[j] / r : 1.0;
          sn[j] = r > 0.0 ? col[j + 1] / r : 0.0;
          col[j] = r;
          col[j + 1] = 0.0;
          g[j + 1] = -sn[j] * g[j];
          g[j] = cs[j] * g[j];
          rel = fabs (g[j + 1]) / bnrm;
          if (dbg) fprintf (dbg, "gmres: %d applications, residual estimate %.6e\n", total, rel);
          if (rel <= eps || K.pin[j + 1] == 0.0)
            {
              j++;
              done = true;
              break;
            }
        }
      // y = R^{-1} g, x += V y
      for (int i = j - 1; i >= 0; i--)
        {
          double s = g[i];
          for (int k = i + 1; k < j; k++) s -= H[(size_t) k * (m + 1) + i] * y[k];
          const double d = H[(size_t) i * (m + 1) + i];
          y[i] = d != 0.0 ? s / d : 0.0;
        }
      if (j > 0)
        {
          for (int i = 0; i < j; i++) K.pin[i] = y[i];
          cudaMemcpyAsync (K.cv.p, K.pin, sizeof (double) * j, cudaMemcpyHostToDevice, st);
          k_vcombine<<<gn, KT, 0, st>>> (d_x, V, (size_t) n, (const double *) K.cv.p, j, n, 1.0);
          // the pinned buffer is reused below: finish the copy first
          if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "GMRES update");
        }
      (void) done;   // the true residual at the top of the loop decides
    }
  *iters = total;
  *res = rel;
  e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "GMRES kernels");
}

// this library's operator for (atimes, user_data), or nullptr
enum OwnOp { OP_NONE, OP_DISPATCH, OP_EWALD, OP_OPEN };

OwnOp
own_operator (void (*atimes) (int, const double *, double *, void *), void *user_data, int n)
{
  const struct stokes *sys = (const struct stokes *) user_data;
  if (sys == nullptr || sys->version < 0 || sys->version > 2) return OP_NONE;
  const int c = sys->version == 0 ? 3 : (sys->version == 1 ? 6 : 11);
  if (n != c * sys->np) return OP_NONE;
  if (atimes == atimes_3all) return OP_DISPATCH;
  if (atimes == atimes_ewald_3all) return sys->periodic ? OP_EWALD : OP_NONE;
  if (atimes == atimes_nonewald_3all) return OP_OPEN;
  return OP_NONE;
}

struct Settings {
  int m = 20, max = 2000;
  double eps = 1e-6;
  FILE *dbg = nullptr;
};

Settings
settings_of (const struct iter *it)
{
  Settings s;
  if (it)
    {
      if (it->restart > 0) s.m = it->restart;
      if (it->max > 0) s.max = it->max;
      if (it->eps > 0.0) s.eps = it->eps;
      if (it->debug && it->out) s.dbg = it->out;
    }
  return s;
}

// solve with the system's own operator: op 0 A = M, op 1 the FTS mobility
// operator.  x: start vector in, solution out (host)
int
solve_own (struct stokes *sys, int op, bool force_open, const double *b, double *x,
           const Settings &S, int *iters, double *res)
{
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  c->force_open = force_open;
  int rc = prepare (c, sys, false);
  if (rc)
    {
      c->force_open = false;
      return rc;
    }
  const int np = sys->np, n = NCOMP (sys->version) * np;
  cudaStream_t st = c->stream;
  Krylov &K = t_kry;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess
      || (e = K.b.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.x.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.t.ensure (sizeof (double) * n)) != cudaSuccess)
    {
      c->force_open = false;
      return cuda_fail (e, "solve buffers");
    }
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync (K.b.p, b, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync (K.x.p, x, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  const double *d_pos = (const double *) c->pos.p;
  double *tmp = (double *) K.t.p;
  Apply A;
  if (op == STOKES_GPU_SOLVE_MOB_FTS)
    A = [&] (const double *in, double *out) -> int {
      k_fts_mask<<<grid_of (n), KT, 0, st>>> (np, in, tmp);
      int r = atimes_dev (c, d_pos, tmp, out, st, false);
      if (r) return r;
      k_fts_mob_out<<<grid_of (n), KT, 0, st>>> (np, in, out, out);
      return STOKES_GPU_OK;
    };
  else
    A = [&] (const double *in, double *out) -> int {
      return atimes_dev (c, d_pos, in, out, st, false);
    };
  rc = gmres_dev (n, (const double *) K.b.p, (double *) K.x.p, A, S.m, S.max, S.eps, st, iters,
                  res, S.dbg);
  if (!rc)
    {
      e = cudaMemcpyAsync (x, K.x.p, sizeof (double) * n, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) rc = cuda_fail (e, "solution");
    }
  c->force_open = false;
  return rc;
}

// solve with a caller's host operator (vectors still on the device)
int
solve_foreign (int n, const double *b, double *x,
               void (*atimes) (int, const double *, double *, void *), void *user_data,
               const Settings &S, int *iters, double *res)
{
  Krylov &K = t_kry;
  cudaError_t e;
  if (!K.own && (e = cudaStreamCreateWithFlags (&K.own, cudaStreamNonBlocking)) != cudaSuccess)
    return cuda_fail (e, "solver stream");
  cudaStream_t st = K.own;
  if ((e = K.b.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.x.ensure (sizeof (double) * n)) != cudaSuccess)
    return cuda_fail (e, "solve buffers");
  cudaMemcpyAsync (K.b.p, b, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync (K.x.p, x, sizeof (double) * n, cudaMemcpyHostToDevice, st);
  std::vector<double> hin (n), hout (n);
  Apply A = [&] (const double *in, double *out) -> int {
    cudaError_t ee = cudaMemcpyAsync (hin.data (), in, sizeof (double) * n,
                                      cudaMemcpyDeviceToHost, st);
    if (ee == cudaSuccess) ee = cudaStreamSynchronize (st);
    if (ee != cudaSuccess) return cuda_fail (ee, "operator input");
    atimes (n, hin.data (), hout.data (), user_data);
    ee = cudaMemcpyAsync (out, hout.data (), sizeof (double) * n, cudaMemcpyHostToDevice, st);
    if (ee == cudaSuccess) ee = cudaStreamSynchronize (st);
    return ee == cudaSuccess ? STOKES_GPU_OK : cuda_fail (ee, "operator output");
  };
  int rc = gmres_dev (n, (const double *) K.b.p, (double *) K.x.p, A, S.m, S.max, S.eps, st,
                      iters, res, S.dbg);
  if (!rc)
    {
      e = cudaMemcpyAsync (x, K.x.p, sizeof (double) * n, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) rc = cuda_fail (e, "solution");
    }
  return rc;
}

}  // namespace
}  // namespace lsg

using namespace lsg;

extern "C" {

struct iter *
iter_init (const char *solver, int max, int restart, double eps, int n, const double *guess,
           int flag_guess, int debug, FILE *out)
{
  struct iter *it = (struct iter *) calloc (1, sizeof (struct iter));
  if (!it) return nullptr;
  const char *name = solver ? solver : "gmres";
  it->solver = (char *) malloc (strlen (name) + 1);
  if (it->solver) strcpy (it->solver, name);
  it->max = max;
  it->restart = restart;
  it->eps = eps;
  it->n = n > 0 ? n : 0;
  it->flag_guess = flag_guess;
  it->debug = debug;
  it->out = out;
  it->res = -1.0;
  if (flag_guess && it->n > 0)
    {
      it->guess = (double *) calloc ((size_t) it->n, sizeof (double));
      if (it->guess && guess) memcpy (it->guess, guess, sizeof (double) * it->n);
    }
  return it;
}

void
iter_free (struct iter *it)
{
  if (!it) return;
  free (it->solver);
  free (it->guess);
  free (it);
}

void
solve_iter (int n, const double *b, double *x,
            void (*atimes) (int, const double *, double *, void *), void *user_data,
            struct iter *it)
{
  clear_error ();
  if (n <= 0 || !b || !x || !atimes)
    {
      set_error (STOKES_GPU_EINVAL, "bad arguments (n = %d)", n);
      dropin_failed ("solve_iter", x, n > 0 && x ? (size_t) n : 0);
      return;
    }
  const Settings S = settings_of (it);
  const bool from_guess = it && it->flag_guess && it->guess && it->n == n;
  if (from_guess)
    memcpy (x, it->guess, sizeof (double) * n);
  else
    memset (x, 0, sizeof (double) * n);
  int iters = 0;
  double res = 0.0;
  int rc;
  const OwnOp op = own_operator (atimes, user_data, n);
  if (op != OP_NONE)
    rc = solve_own ((struct stokes *) user_data, STOKES_GPU_SOLVE_RES, op == OP_OPEN, b, x, S,
                    &iters, &res);
  else
    rc = solve_foreign (n, b, x, atimes, user_data, S, &iters, &res);
  if (rc)
    {
      dropin_failed ("solve_iter", x, (size_t) n);
      return;
    }
  if (it)
    {
      it->niter = iters;
      it->res = res;
      if (it->flag_guess)
        {
          if (it->n != n || !it->guess)
            {
              free (it->guess);
              it->guess = (double *) malloc (sizeof (double) * n);
              it->n = it->guess ? n : 0;
            }
          if (it->guess) memcpy (it->guess, x, sizeof (double) * n);
        }
      if (it->debug && it->out)
        fprintf (it->out, "solve_iter (%s): %d applications, residual %.6e\n",
                 it->solver ? it->solver : "gmres", iters, res);
    }
}

void
solve_mob_3fts_0 (struct stokes *sys, struct iter *iter, const double *f, const double *t,
                  const double *e, double *u, double *o, double *s)
{
  clear_error ();
  if (!sys || !f || !t || !e || !u || !o || !s)
    {
      set_error (STOKES_GPU_EINVAL, "NULL argument");
      dropin_failed ("solve_mob_3fts_0", nullptr, 0);
      return;
    }
  if (sys->version != 2)
    {
      fprintf (stderr, "libstokes solve_mob_3fts_0 : the version is wrong. reset to FTS\n");
      sys->version = 2;
    }
  const int np = sys->np, n = 11 * np;
  std::vector<double> x1 (n), ev (n, 0.0), b (n), x (n, 0.0);
  for (int i = 0; i < np; i++)
    for (int q = 0; q < 3; q++)
      {
        x1[11 * i + q] = f[3 * i + q];
        x1[11 * i + 3 + q] = t[3 * i + q];
      }
  for (int i = 0; i < np; i++)
    for (int q = 0; q < 5; q++)
      {
        x1[11 * i + 6 + q] = 0.0;
        ev[11 * i + 6 + q] = e[5 * i + q];
      }
  // b = M (f, t, 0) - (0, 0, e) (src/ewald-3fts.c:146-190)
  int rc = stokes_gpu_atimes (sys, x1.data (), b.data ());
  if (!rc)
    {
      for (int k = 0; k < n; k++) b[k] -= ev[k];
      struct iter *it = iter ? iter : sys->it;
      const Settings S = settings_of (it);
      if (it && it->flag_guess && it->guess && it->n == n)
        memcpy (x.data (), it->guess, sizeof (double) * n);
      int iters = 0;
      double res = 0.0;
      rc = solve_own (sys, STOKES_GPU_SOLVE_MOB_FTS, false, b.data (), x.data (), S, &iters,
                      &res);
      if (!rc && it)
        {
          it->niter = iters;
          it->res = res;
          if (it->flag_guess && it->guess && it->n == n)
            memcpy (it->guess, x.data (), sizeof (double) * n);
        }
    }
  if (rc)
    {
      // error mode 1: NaN results and the reason in stokes_gpu_last_error ()
      dropin_failed ("solve_mob_3fts_0", x.data (), (size_t) n);
    }
  for (int i = 0; i < np; i++)
    {
      for (int q = 0; q < 3; q++)
        {
          u[3 * i + q] = x[11 * i + q];
          o[3 * i + q] = x[11 * i + 3 + q];
        }
      for (int q = 0; q < 5; q++) s[5 * i + q] = x[11 * i + 6 + q];
    }
}

int
stokes_gpu_solve (struct stokes *sys, int op, const double *b, double *x, int restart, int max,
                  double eps, int *iters, double *res)
{
  clear_error ();
  if (!sys || !b || !x) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  if (op != STOKES_GPU_SOLVE_RES && op != STOKES_GPU_SOLVE_MOB_FTS)
    return set_error (STOKES_GPU_EINVAL, "unknown problem %d", op);
  if (op == STOKES_GPU_SOLVE_MOB_FTS && sys->version != 2)
    return set_error (STOKES_GPU_EINVAL, "the FTS mobility problem needs version 2");
  Settings S;
  if (restart > 0) S.m = restart;
  if (max > 0) S.max = max;
  if (eps > 0.0) S.eps = eps;
  int it = 0;
  double r = 0.0;
  int rc = solve_own (sys, op, false, b, x, S, &it, &r);
  if (iters) *iters = it;
  if (res) *res = r;
  return rc;
}

}  // extern "C"
