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

// the block's sum in thread 0 (callable repeatedly: the first barrier keeps
// a new call from overwriting partials an earlier call is still reading)
__device__ __forceinline__ double
block_sum (double v)
{
  __shared__ double sh[KT / 32];
  __syncthreads ();
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


// One Arnoldi step after the product w = A v_j, in one cooperative launch
// (all blocks resident): both Gram-Schmidt passes, the normalisation of
// v_{j+1}, and -- in block 0 -- the Givens rotation of the new Hessenberg
// column with the residual estimate res[j] = |g_{j+1}| / |b|.  Block b owns
// one contiguous slice of the elements in every pass, so the updates of w
// need no grid barrier; the partial dot products do (three per step), and
// each pass has its own partial buffer so that no block overwrites partials
// another block is still reading.  Within a block, warp q forms the slice's
// dot products with v_q, v_{q+8}, ... (its loads stream along the slice),
// and the update runs one element per thread over all k.  The barrier is a counter and a
// generation word with a bounded wait: a block that gives up sets *status
// and returns.
struct ArnArgs {
  double *V;          // (m + 1) x n basis, v_k at V + k n
  double *w;          // the product A v_j (overwritten)
  double *xin;        // fixed input of the next product: receives v_{j+1}
  int n, j, m;
  double *part;       // [3][G][m + 2] partial sums
  double *H;          // Hessenberg columns, H[col (m + 1) + row]; rotated
                      // once their Givens step ran
  double *cs, *sn, *g;
  int gcol;           // column the extra block rotates (-1: none)
  double *res;        // [m] residual estimates
  double bnrm;
  unsigned *bar;      // arrival count, generation
  int *status;        // nonzero: a barrier wait ran out
  long long spins;    // polls of a barrier wait before it gives up
};

constexpr long long BAR_SPINS = 1ll << 22;   // about 0.1 - 1 s of polling

__device__ bool
grid_barrier (unsigned *bar, int *status, long long max_spins)
{
  __shared__ int s_ok;
  __syncthreads ();
  if (threadIdx.x == 0)
    {
      volatile unsigned *gen = bar + 1;
      const unsigned g0 = *gen;
      __threadfence ();
      int ok = 1;
      if (atomicAdd (bar, 1u) == gridDim.x - 1)
        {
          bar[0] = 0;
          __threadfence ();
          atomicAdd (bar + 1, 1u);
        }
      else
        {
          long long spins = 0;
          while (*gen == g0)
            {
              if (++spins > max_spins || *(volatile int *) status)
                {
                  atomicExch (status, 1);
                  ok = 0;
                  break;
                }
              __nanosleep (32);
            }
        }
      __threadfence ();
      s_ok = ok;
    }
  __syncthreads ();
  return s_ok != 0;
}

__device__ __forceinline__ double
warp_total (double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync (0xffffffffu, v, o);
  return v;
}

// Givens step of Hessenberg column c by one block: the earlier rotations
// and the column come to shared memory in parallel, one thread runs the
// chain there (through global memory it would pay an L2 round trip per
// step); sc: 3 (m + 2) doubles of shared memory
__device__ void
givens_column (const ArnArgs &a, int c, double *sc)
{
  const int ld = a.m + 2;
  double *col = sc, *cs = sc + ld, *sn = sc + 2 * ld;
  double *gcol = a.H + (size_t) c * (a.m + 1);
  for (int i = threadIdx.x; i <= c + 1; i += blockDim.x) col[i] = gcol[i];
  for (int i = threadIdx.x; i < c; i += blockDim.x)
    {
      cs[i] = a.cs[i];
      sn[i] = a.sn[i];
    }
  __syncthreads ();
  if (threadIdx.x == 0)
    {
      for (int i = 0; i < c; i++)
        {
          const double t0 = cs[i] * col[i] + sn[i] * col[i + 1];
          col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
          col[i] = t0;
        }
      const double r = hypot (col[c], col[c + 1]);
      const double ir = r > 0.0 ? 1.0 / r : 0.0;
      const double cc = r > 0.0 ? col[c] * ir : 1.0, ss = col[c + 1] * ir;
      col[c] = r;
      col[c + 1] = 0.0;
      a.cs[c] = cc;
      a.sn[c] = ss;
      const double gc = a.g[c];
      a.g[c + 1] = -ss * gc;
      a.g[c] = cc * gc;
      a.res[c] = fabs (ss * gc) / a.bnrm;
    }
  __syncthreads ();
  for (int i = threadIdx.x; i <= c + 1; i += blockDim.x) gcol[i] = col[i];
}

// the Givens step of column c alone (before the residual history is read)
__global__ void __launch_bounds__ (KT)
k_givens (ArnArgs a, int c)
{
  extern __shared__ double s_g3[];
  givens_column (a, c, s_g3);
}

__global__ void __launch_bounds__ (KT)
k_arnoldi (ArnArgs a)
{
  extern __shared__ double s_h[];   // [m + 2] each: h, this pass, cs, sn
  __shared__ double s_red[KT / 64][64];
  __shared__ double s_w1;
  double *h = s_h, *hp = s_h + (a.m + 2);
  // blocks 0 .. G-1 own slices; block G (the last) rotates column gcol of
  // the previous step meanwhile, off the path of the next product
  const int G = gridDim.x - 1, b = blockIdx.x, J = a.j + 1, ld = a.m + 2;
  const int tid = threadIdx.x, lane = tid & 31, wq = tid >> 5;
  if (b == G)
    {
      if (a.gcol >= 0) givens_column (a, a.gcol, s_h);
      if (!grid_barrier (a.bar, a.status, a.spins)) return;
      grid_barrier (a.bar, a.status, a.spins);
      return;
    }
  // this block's slice [i0, i1), whole warps of elements
  const int per = ((a.n + G - 1) / G + 31) / 32 * 32;
  const int i0 = min (a.n, b * per), i1 = min (a.n, i0 + per);
  double *w = a.w;
  for (int k = tid; k < J; k += KT) h[k] = 0.0;
  for (int pass = 0; pass < 2; pass++)
    {
      double *part = a.part + (size_t) pass * G * ld;
      // slice dot products: warp wq takes k = kb + 8 r, r < 4, four
      // independent sums in flight
      for (int kb = wq; kb < J; kb += 32)
        {
          double d[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 2
          for (int i = i0 + lane; i < i1; i += 32)
            {
              const double wi = w[i];
#pragma unroll
              for (int r = 0; r < 4; r++)
                {
                  const int k = kb + 8 * r;
                  if (k < J) d[r] += a.V[(size_t) k * a.n + i] * wi;
                }
            }
#pragma unroll
          for (int r = 0; r < 4; r++) d[r] = warp_total (d[r]);
          if (lane == 0)
#pragma unroll
            for (int r = 0; r < 4; r++)
              if (kb + 8 * r < J) part[(size_t) b * ld + kb + 8 * r] = d[r];
        }
      if (pass == 1)
        {
          // |w1|^2 of the slice: |w2|^2 = |w1|^2 - |h2|^2 saves a barrier
          double t = 0.0;
          for (int i = i0 + tid; i < i1; i += KT) t += w[i] * w[i];
          t = block_sum (t);
          if (tid == 0) part[(size_t) b * ld + a.m + 1] = t;
        }
      if (!grid_barrier (a.bar, a.status, a.spins)) return;
      // totals over the blocks: eight threads per entry, then three shuffles
      // (other blocks' partials through L2 with __ldcg, not a stale L1 line)
      const int ne = J + pass;
      for (int kb = 0; kb < ne; kb += KT / 8)
        {
          const int k = kb + (tid >> 3), sub = tid & 7;
          const int kk = k < J ? k : a.m + 1;
          // eight loads in flight per thread: the loop is bound by L2
          // latency (across the two dies), not by the adds
          const double *pk = a.part + (size_t) pass * G * ld + kk;
          double t = 0.0;
          if (k < ne)
#pragma unroll 8
            for (int q = sub; q < G; q += 8) t += __ldcg (pk + (size_t) q * ld);
          t += __shfl_xor_sync (0xffffffffu, t, 1);
          t += __shfl_xor_sync (0xffffffffu, t, 2);
          t += __shfl_xor_sync (0xffffffffu, t, 4);
          if (sub == 0 && k < ne)
            {
              if (k < J)
                {
                  hp[k] = t;
                  h[k] += t;
                }
              else
                s_w1 = t;
            }
        }
      __syncthreads ();
      // w -= V hp: four threads per element, each over every fourth k
      for (int base = i0; base < i1; base += 64)
        {
          const int i = base + (tid & 63), kg = tid >> 6;
          double s0 = 0.0, s1 = 0.0;
          if (i < i1)
            for (int k = kg; k < J; k += 8)
              {
                s0 += a.V[(size_t) k * a.n + i] * hp[k];
                if (k + 4 < J) s1 += a.V[(size_t) (k + 4) * a.n + i] * hp[k + 4];
              }
          s_red[kg][tid & 63] = s0 + s1;
          __syncthreads ();
          if (kg == 0 && i < i1)
            w[i] -= (s_red[0][tid] + s_red[1][tid]) + (s_red[2][tid] + s_red[3][tid]);
          __syncthreads ();
        }
    }
  // |w|^2 = |w1|^2 - |h2|^2 and v_{j+1} = w / |w|
  __shared__ double s_nrm, s_inv;
  if (wq == 0)
    {
      double t = 0.0;
      for (int k = lane; k < J; k += 32) t += hp[k] * hp[k];
      t = warp_total (t);
      if (lane == 0)
        {
          const double n2 = s_w1 - t;
          s_nrm = n2 > 0.0 ? sqrt (n2) : 0.0;
          s_inv = s_nrm > 0.0 ? 1.0 / s_nrm : 0.0;
        }
    }
  __syncthreads ();
  const double nrm = s_nrm, inv = s_inv;
  double *vn = a.V + (size_t) (a.j + 1) * a.n;
  for (int i = i0 + tid; i < i1; i += KT)
    {
      const double v = w[i] * inv;
      vn[i] = v;
      a.xin[i] = v;
    }
  if (b != 0) return;
  // column j of the Hessenberg matrix, unrotated: h and |w|
  double *col = a.H + (size_t) a.j * (a.m + 1);
  for (int i = tid; i <= a.j; i += KT) col[i] = h[i];
  if (tid == 0) col[a.j + 1] = nrm;
}

// y = R^{-1} g over the first jj columns (R: the rotated Hessenberg matrix),
// one warp: back substitution with the lanes over the known y_k
__global__ void
k_lsq (const double *H, const double *g, int m, int jj, double *y)
{
  const int lane = threadIdx.x & 31;
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  for (int i = jj - 1; i >= 0; i--)
    {
      double s = 0.0;
      for (int k = i + 1 + lane; k < jj; k += 32) s += H[(size_t) k * (m + 1) + i] * y[k];
      s = warp_total (s);
      if (lane == 0)
        {
          const double d = H[(size_t) i * (m + 1) + i];
          y[i] = d != 0.0 ? (g[i] - s) / d : 0.0;
        }
      __syncwarp ();
    }
}

inline int grid_of (long long n) { return (int) ((n + KT - 1) / KT); }

// device workspace of the solver (one per host thread)
struct Krylov {
  DevBuf V, w, t, part, h, h2, s2, cv, b, x, arn, xin;
  DevBuf rr, dd, t2;           // refinement: FP64 residual, correction, product
  double *pin = nullptr;     // pinned host staging: residual history, scalars
  size_t pin_cap = 0;
  cudaStream_t own = nullptr;  // stream for foreign operators
  int coop_blocks = 0;         // co-resident blocks of k_arnoldi on this device
  ~Krylov ()
  {
    for (DevBuf *d : {&V, &w, &t, &part, &h, &h2, &s2, &cv, &b, &x, &arn, &xin, &rr, &dd, &t2})
      d->release ();
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

// iterations between two reads of the residual history: the products of an
// Arnoldi step are queued without a host round-trip in between
constexpr int CHECK_EVERY = 4;

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
  Gmres Gm {K, n, m, st, (n + MDOT_CHUNK - 1) / MDOT_CHUNK};
  cudaError_t e;
  if (K.coop_blocks == 0)
    {
      int dev = 0, sms = 0, per = 0;
      cudaGetDevice (&dev);
      cudaDeviceGetAttribute (&sms, cudaDevAttrMultiProcessorCount, dev);
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor (&per, k_arnoldi, KT,
                                                         4 * sizeof (double) * 258);
      if (e != cudaSuccess) return cuda_fail (e, "GMRES occupancy");
      K.coop_blocks = sms * (per > 0 ? per : 1);
    }
  if (m > 256) m = 256;   // the shared h arrays of k_arnoldi
  // slices of about 64 elements: the FP64 work of a step spread over many SMs
  int G = (n + 63) / 64;
  if (G > K.coop_blocks - 1) G = K.coop_blocks - 1;
  if (G > 2 * 152) G = 2 * 152;
  if (G < 1) G = 1;
  const size_t ld = (size_t) m + 2;
  // arn: H (m + 1) m | cs m | sn m | g m + 1 | res m | part 3 G ld | bar, status
  const size_t o_cs = (size_t) (m + 1) * m, o_sn = o_cs + m, o_g = o_sn + m, o_res = o_g + m + 1;
  const size_t o_part = o_res + m, o_bar = o_part + 3 * (size_t) G * ld;
  if ((e = K.V.ensure (sizeof (double) * (size_t) (m + 1) * n)) != cudaSuccess
      || (e = K.w.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.xin.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.part.ensure (sizeof (double) * (size_t) (m + 1) * Gm.nch)) != cudaSuccess
      || (e = K.s2.ensure (sizeof (double) * 2)) != cudaSuccess
      || (e = K.cv.ensure (sizeof (double) * (m + 1))) != cudaSuccess
      || (e = K.arn.ensure (sizeof (double) * (o_bar + 2))) != cudaSuccess
      || (e = K.pinned ((size_t) m + 4)) != cudaSuccess)
    return cuda_fail (e, "GMRES workspace");
  double *V = (double *) K.V.p, *w = (double *) K.w.p;
  double *arn = (double *) K.arn.p;
  unsigned *bar = (unsigned *) (arn + o_bar);
  int *status = (int *) (bar + 2);
  cudaMemsetAsync (bar, 0, 2 * sizeof (double), st);
  const int gn = grid_of (n);

  int rc;
  double bn2;
  if ((rc = Gm.norm2_host (d_b, &bn2))) return rc;
  const double bnrm = sqrt (bn2);
  *iters = 0;
  if (!(bnrm > 0.0))
    {
      cudaMemsetAsync (d_x, 0, sizeof (double) * n, st);
      *res = 0.0;
      e = cudaStreamSynchronize (st);
      return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "GMRES");
    }

  ArnArgs aa;
  aa.V = V;
  aa.w = w;
  aa.xin = (double *) K.xin.p;
  aa.n = n;
  aa.m = m;
  aa.part = arn + o_part;
  aa.H = arn;
  aa.cs = arn + o_cs;
  aa.sn = arn + o_sn;
  aa.g = arn + o_g;
  aa.res = arn + o_res;
  aa.bnrm = bnrm;
  aa.bar = bar;
  aa.status = status;
  aa.spins = g_test_bar_spins > 0 ? g_test_bar_spins : BAR_SPINS;
  const size_t smem = 4 * sizeof (double) * ld;

  int total = 0;
  double rel = HUGE_VAL;
  for (;;)
    {
      // r = b - A x into V_0
      if ((rc = A (d_x, w))) return rc;
      k_vaxpby<<<gn, KT, 0, st>>> (n, 1.0, d_b, -1.0, w, V);
      double beta2;
      if ((rc = Gm.norm2_host (V, &beta2))) return rc;
      rel = sqrt (beta2) / bnrm;
      if (dbg) fprintf (dbg, "gmres: %d applications, residual %.6e\n", total, rel);
      if (rel <= eps || total >= maxit) break;
      // v_0 = r / |r|, g = (|r|, 0, ...)
      cudaMemsetAsync (aa.g, 0, sizeof (double) * (m + 1), st);
      k_vnormalize<<<gn, KT, 0, st>>> (V, (const double *) K.s2.p, aa.g, V, n);
      int jj = 0, checked = 0;
      aa.gcol = -1;            // column whose Givens step is still due
      bool conv = false;
      for (int j = 0; j < m && total < maxit; j++)
        {
          // the product reads a fixed buffer: with the same pointers every
          // step, the mixed path replays its recorded graph (k_arnoldi
          // leaves v_{j+1} there; v_0 is copied)
          if (j == 0)
            cudaMemcpyAsync (K.xin.p, V, sizeof (double) * n, cudaMemcpyDeviceToDevice, st);
          if ((rc = A ((const double *) K.xin.p, w))) return rc;
          total++;
          aa.j = j;
          void *args[] = {&aa};
          // G slice blocks and one block for the Givens step of column j - 1
          e = cudaLaunchCooperativeKernel ((const void *) k_arnoldi, G + 1, KT, args, smem, st);
          if (e != cudaSuccess) return cuda_fail (e, "Arnoldi step");
          aa.gcol = j;
          const bool last = j == m - 1 || total >= maxit;
          if ((j + 1 - checked) < CHECK_EVERY && !last) continue;
          // the Givens step of column j itself, then the residual history
          k_givens<<<1, KT, smem, st>>> (aa, j);
          aa.gcol = -1;
          // residual history of the steps since the last read, and the
          // barrier status
          const int cnt = j + 1 - checked;
          cudaMemcpyAsync (K.pin, aa.res + checked, sizeof (double) * cnt,
                           cudaMemcpyDeviceToHost, st);
          cudaMemcpyAsync (K.pin + cnt, status, sizeof (int), cudaMemcpyDeviceToHost, st);
          if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "GMRES step");
          int stat = 0;
          memcpy (&stat, K.pin + cnt, sizeof (int));
          if (stat)
            return set_error (STOKES_GPU_ETIMEOUT, "GMRES: a grid barrier wait ran out");
          for (int q = 0; q < cnt; q++)
            {
              if (dbg)
                fprintf (dbg, "gmres: step %d, residual estimate %.6e\n", checked + q, K.pin[q]);
              if (K.pin[q] <= eps)
                {
                  jj = checked + q + 1;
                  conv = true;
                  break;
                }
            }
          if (conv) break;
          checked = j + 1;
          jj = j + 1;
        }
      // x += V y, y = R^{-1} g over the steps taken (or up to convergence)
      if (jj > 0)
        {
          k_lsq<<<1, 32, 0, st>>> (arn, aa.g, m, jj, (double *) K.cv.p);
          k_vcombine<<<gn, KT, 0, st>>> (d_x, V, (size_t) n, (const double *) K.cv.p, jj, n, 1.0);
        }
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

// Mixed-precision solve with FP64 iterative refinement: the residual
// r = b - A64 x always comes from the FP64 product, and each correction d
// solves A_mixed d = r by GMRES on the mixed product to a relative accuracy
// eps |b| / |r| (not below 1e-5: the mixed product carries about 3e-7, so
// GMRES stalls near 1e-6); x += d in FP64.  A correction reduces the error by
// about cond(A) times the mixed product's error, so eps = 1e-10 takes two to
// four FP64 products.  Convergence: |b - A64 x| <= eps |b|.  *iters counts
// every operator application (mixed and FP64).
int
refine_dev (int n, const double *d_b, double *d_x, const Apply &A, const Apply &A64, int m,
            int maxit, double eps, cudaStream_t st, int *iters, double *res, FILE *dbg)
{
  Krylov &K = t_kry;
  cudaError_t e;
  if ((e = K.rr.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.dd.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.t2.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.part.ensure (sizeof (double) * (size_t) ((n + MDOT_CHUNK - 1) / MDOT_CHUNK)))
           != cudaSuccess
      || (e = K.s2.ensure (sizeof (double) * 2)) != cudaSuccess
      || (e = K.pinned (4)) != cudaSuccess)
    return cuda_fail (e, "refinement workspace");
  double *r = (double *) K.rr.p, *d = (double *) K.dd.p, *t = (double *) K.t2.p;
  Gmres Gm {K, n, 1, st, (n + MDOT_CHUNK - 1) / MDOT_CHUNK};
  const int gn = grid_of (n);
  int rc;
  double bn2;
  if ((rc = Gm.norm2_host (d_b, &bn2))) return rc;
  const double bnrm = sqrt (bn2);
  if (!(bnrm > 0.0))
    {
      cudaMemsetAsync (d_x, 0, sizeof (double) * n, st);
      *iters = 0;
      *res = 0.0;
      e = cudaStreamSynchronize (st);
      return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "refinement");
    }
  int total = 0;
  double rel = HUGE_VAL;
  for (int outer = 0; outer < 16; outer++)
    {
      // r = b - A64 x
      if ((rc = A64 (d_x, t))) return rc;
      total++;
      k_vaxpby<<<gn, KT, 0, st>>> (n, 1.0, d_b, -1.0, t, r);
      double r2;
      if ((rc = Gm.norm2_host (r, &r2))) return rc;
      const double rel_new = sqrt (r2) / bnrm;
      if (dbg) fprintf (dbg, "refinement: %d applications, FP64 residual %.6e\n", total, rel_new);
      // stop when converged, out of applications, or no longer improving
      if (rel_new <= eps || total >= maxit || !(rel_new < 0.5 * rel))
        {
          rel = std::min (rel, rel_new);
          break;
        }
      rel = rel_new;
      const double ein = std::max (eps / rel, 1e-5);
      cudaMemsetAsync (d, 0, sizeof (double) * n, st);
      int it = 0;
      double ir = 0.0;
      if ((rc = gmres_dev (n, r, d, A, m, maxit - total, ein, st, &it, &ir, dbg))) return rc;
      total += it + 1;       // its iterations and its start residual
      k_vaxpby<<<gn, KT, 0, st>>> (n, 1.0, d_x, 1.0, d, d_x);
    }
  *iters = total;
  *res = rel;
  e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "refinement kernels");
}

// solve with the system's own operator: op 0 A = M, op 1 the FTS mobility
// operator.  x: start vector in, solution out (host).  Mixed precision:
// GMRES on the mixed product inside FP64 iterative refinement (refine_dev).
int
solve_own (struct stokes *sys, int op, bool force_open, const double *b, double *x,
           const Settings &S, int *iters, double *res)
{
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  c->force_open = force_open;
  const bool refine = c->precision == STOKES_GPU_MIXED;
  // the FP64 tables as well when the FP64 product computes the residuals
  int rc = prepare (c, sys, false, refine ? 1 : -1);
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
  else if (op == STOKES_GPU_SOLVE_MOB_LUB)
    // (I + M L) u: the lubricated mobility problem of src/ewald-3f.c:411-445
    A = [&] (const double *in, double *out) -> int {
      int r = lub_dev (sys, sys->version, d_pos, in, tmp, st);
      if (!r) r = atimes_dev (c, d_pos, tmp, out, st, false);
      if (r) return r;
      k_vaxpby<<<grid_of (n), KT, 0, st>>> (n, 1.0, in, 1.0, out, out);
      return STOKES_GPU_OK;
    };
  else
    A = [&] (const double *in, double *out) -> int {
      return atimes_dev (c, d_pos, in, out, st, false);
    };
  if (refine)
    {
      double *tmp64 = nullptr;
      if ((e = K.h2.ensure (sizeof (double) * n)) != cudaSuccess)
        {
          c->force_open = false;
          return cuda_fail (e, "solve buffers");
        }
      tmp64 = (double *) K.h2.p;
      Apply A64;
      if (op == STOKES_GPU_SOLVE_MOB_FTS)
        A64 = [&] (const double *in, double *out) -> int {
          k_fts_mask<<<grid_of (n), KT, 0, st>>> (np, in, tmp64);
          int r = atimes_fp64_dev (c, d_pos, tmp64, out, st, false);
          if (r) return r;
          k_fts_mob_out<<<grid_of (n), KT, 0, st>>> (np, in, out, out);
          return STOKES_GPU_OK;
        };
      else if (op == STOKES_GPU_SOLVE_MOB_LUB)
        A64 = [&] (const double *in, double *out) -> int {
          int r = lub_dev (sys, sys->version, d_pos, in, tmp64, st);
          if (!r) r = atimes_fp64_dev (c, d_pos, tmp64, out, st, false);
          if (r) return r;
          k_vaxpby<<<grid_of (n), KT, 0, st>>> (n, 1.0, in, 1.0, out, out);
          return STOKES_GPU_OK;
        };
      else
        A64 = [&] (const double *in, double *out) -> int {
          return atimes_fp64_dev (c, d_pos, in, out, st, false);
        };
      rc = refine_dev (n, (const double *) K.b.p, (double *) K.x.p, A, A64, S.m, S.max, S.eps,
                       st, iters, res, S.dbg);
    }
  else
    rc = gmres_dev (n, (const double *) K.b.p, (double *) K.x.p, A, S.m, S.max, S.eps, st,
                    iters, res, S.dbg);
  if (!rc)
    {
      e = cudaMemcpyAsync (x, K.x.p, sizeof (double) * n, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) rc = cuda_fail (e, "solution");
    }
  c->force_open = false;
  return rc;
}

// the lubricated mobility problem of a Brownian step, on device vectors in
// the particle layout: d_u = (I + M L)^-1 M d_f at positions d_pos, the
// product of the context as prepared, GMRES settings from sys->it, start 0
// (src/ewald-3f.c:447-490, src/ewald-3ft.c)
int
lub_mobility_dev_impl (Ctx *c, struct stokes *sys, const double *d_pos, const double *d_f,
                       double *d_u, cudaStream_t st, int *iters)
{
  const int n = NCOMP (sys->version) * sys->np;
  Krylov &K = t_kry;
  cudaError_t e;
  if ((e = K.b.ensure (sizeof (double) * n)) != cudaSuccess
      || (e = K.t.ensure (sizeof (double) * n)) != cudaSuccess)
    return cuda_fail (e, "solve buffers");
  double *b = (double *) K.b.p, *tmp = (double *) K.t.p;
  int rc = atimes_dev (c, d_pos, d_f, b, st, false);
  if (rc) return rc;
  if ((e = cudaMemsetAsync (d_u, 0, sizeof (double) * n, st)) != cudaSuccess)
    return cuda_fail (e, "solve start");
  Apply A = [&] (const double *in, double *out) -> int {
    int r = lub_dev (sys, sys->version, d_pos, in, tmp, st);
    if (!r) r = atimes_dev (c, d_pos, tmp, out, st, false);
    if (r) return r;
    k_vaxpby<<<grid_of (n), KT, 0, st>>> (n, 1.0, in, 1.0, out, out);
    return STOKES_GPU_OK;
  };
  const Settings S = settings_of (sys->it);
  double res = 0.0;
  return gmres_dev (n, b, d_u, A, S.m, S.max, S.eps, st, iters, &res, S.dbg);
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

namespace lsg {
int
lub_mobility_dev (Ctx *c, struct stokes *sys, const double *d_pos, const double *d_f,
                  double *d_u, cudaStream_t st, int *iters)
{
  return lub_mobility_dev_impl (c, sys, d_pos, d_f, d_u, st, iters);
}
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
  if (op != STOKES_GPU_SOLVE_RES && op != STOKES_GPU_SOLVE_MOB_FTS
      && op != STOKES_GPU_SOLVE_MOB_LUB)
    return set_error (STOKES_GPU_EINVAL, "unknown problem %d", op);
  if (op == STOKES_GPU_SOLVE_MOB_FTS && sys->version != 2)
    return set_error (STOKES_GPU_EINVAL, "the FTS mobility problem needs version 2");
  if (op == STOKES_GPU_SOLVE_MOB_LUB && sys->version > 1)
    return set_error (STOKES_GPU_EINVAL, "the lubricated mobility problem serves F and FT");
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
