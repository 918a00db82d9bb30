// open_f32.cu -- the free-space product in mixed precision.
//
// The same operator as the FP64 free-space path (src/non-ewald.c:330-481):
// self terms plus every ordered pair i != j once.  The pair terms run in FP32:
// the positions enter as hi + lo float pairs, so a separation carries one
// FP32 rounding, not that of the absolute coordinates.  Each lane keeps a
// compensated sum (TwoSum cascade) of its terms, the lanes of a warp meet
// through the same compensated addition, and a chunk's (sum, error) pair is
// stored as two floats.  The combine kernel adds chunks and the self term in
// FP64.
//
//   k_open_prep     FP64 positions, radii and x -> hi/lo floats, FP32 x
//   k_open_f32      one warp per (target, source chunk), lanes over sources
//   k_open_combine  y = self . x + sum of the chunks, FP64
#include "ewald_device.cuh"
#include "engine.h"
#include "gpu_engine.h"
#include "stokes_gpu.h"

namespace lsg {

struct OpenF32Args {
  const float4 *ph;     // hi parts of the positions; radius in w
  const float4 *pl;     // lo parts; slip-effective radius in w
  const float *xf;      // x in FP32 [np c]
  int np, nchunk;
  float rmin;
  float2 *partial;      // [nchunk][np][c] (sum, error)
};

__global__ void
k_open_prep (const double *pos, const double *x, const double *rad, const double *slipa, int np,
             int n, float4 *ph, float4 *pl, float *xf)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) xf[t] = (float) x[t];
  if (t >= np) return;
  float h[3], l[3];
#pragma unroll
  for (int d = 0; d < 3; d++)
    {
      const double p = pos[3 * t + d];
      h[d] = (float) p;
      l[d] = (float) (p - (double) h[d]);
    }
  ph[t] = make_float4 (h[0], h[1], h[2], rad ? (float) rad[t] : 1.0f);
  pl[t] = make_float4 (l[0], l[1], l[2], slipa ? (float) slipa[t] : 1.0f);
}

// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void
two_sum (float a, float b, float &s, float &e)
{
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

template <int V, int MODE>
__global__ void __launch_bounds__ (128)
k_open_f32 (OpenF32Args a)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const long long w = ((long long) blockIdx.x * 128 + threadIdx.x) >> 5;
  if (w >= (long long) a.np * a.nchunk) return;
  const int i = (int) (w % a.np);
  const int chunk = (int) (w / a.np);
  const int j0 = (int) ((long long) a.np * chunk / a.nchunk);
  const int j1 = (int) ((long long) a.np * (chunk + 1) / a.nchunk);
  const float4 hi = a.ph[i], li = a.pl[i];
  const float ai = (MODE == MODE_MONO) ? 1.0f : hi.w;
  float s[C], c[C];
#pragma unroll
  for (int q = 0; q < C; q++) s[q] = c[q] = 0.0f;
  for (int j = j0 + lane; j < j1; j += 32)
    {
      const float4 hj = a.ph[j], lj = a.pl[j];
      const float dx = (hj.x - hi.x) + (lj.x - li.x);
      const float dy = (hj.y - hi.y) + (lj.y - li.y);
      const float dz = (hj.z - hi.z) + (lj.z - li.z);
      const float rr = dx * dx + dy * dy + dz * dz;
      if (j == i || rr == 0.0f) continue;
      const float aj = (MODE == MODE_MONO) ? 1.0f : hj.w;
      float r = sqrtf (rr);
      const float rm = (ai + aj) * a.rmin;
      if (r < rm) r = rm;
      const float ri = 1.0f / r;
      const float e[3] = {dx * ri, dy * ri, dz * ri};
      PairScalars<float> sc;
      if (MODE == MODE_MONO) open_scalars<V, float> (r, 1.0f, 1.0f, 1.0f, sc);
      else if (MODE == MODE_POLY) open_scalars<V, float> (r, ai, aj, ai, sc);
      else open_scalars<V, float> (r, li.w, lj.w, ai, sc);
      GenF<V, float> g;
      load_genf<V, float> (a.xf + (size_t) C * j, g);
      GenU<V, float> t;
      t.zero ();
      pair_apply<V, float> (e, sc, g, t);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          float err;
          two_sum (s[q], t.v[q], s[q], err);
          c[q] += err;
        }
    }
  float2 *out = a.partial + ((size_t) chunk * a.np + i) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      float sq = s[q], cq = c[q];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        {
          const float so = __shfl_xor_sync (0xffffffffu, sq, o);
          const float co = __shfl_xor_sync (0xffffffffu, cq, o);
          float err;
          two_sum (sq, so, sq, err);
          cq += co + err;
        }
      if (lane == 0) out[q] = make_float2 (sq, cq);
    }
}

// y_i = self_i . x_i + sum over chunks of (sum + error), in FP64
template <int V>
__global__ void
k_open_combine (const double *x, const float2 *partial, int nchunk, const double *selfc, int np,
                double *y)
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
      for (int k = 0; k < nchunk; k++)
        {
          const float2 p = partial[((size_t) k * np + i) * C + q];
          v += (double) p.x + (double) p.y;
        }
      y[(size_t) C * i + q] = v;
    }
}

// chunks of sources per target: about 32 warps per SM in all
static int
open_nchunk (int np)
{
  int nc = (152 * 32 + np - 1) / np;
  if (nc < 1) nc = 1;
  if (nc > np) nc = np;
  if (nc > 64) nc = 64;
  return nc;
}

int
atimes_open_f32_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                     cudaStream_t st, bool timed)
{
  const int np = c->np, C = NCOMP (c->version), n = C * np;
  const int nchunk = open_nchunk (np);
  // layout of the scratch: ph, pl [np] float4; xf [n] float; partial float2
  const size_t o_pl = (size_t) np * sizeof (float4);
  const size_t o_xf = o_pl + (size_t) np * sizeof (float4);
  const size_t o_pt = (o_xf + (size_t) n * sizeof (float) + 15) / 16 * 16;
  const size_t bytes = o_pt + (size_t) nchunk * n * sizeof (float2);
  cudaError_t e = c->openf.ensure (bytes);
  if (e != cudaSuccess) return cuda_fail (e, "free-space scratch");
  char *base = (char *) c->openf.p;
  float4 *ph = (float4 *) base, *pl = (float4 *) (base + o_pl);
  float *xf = (float *) (base + o_xf);
  float2 *part = (float2 *) (base + o_pt);
  const double *pp = (const double *) c->pp.p;
  const double *rad = c->mode == MODE_MONO ? nullptr : pp;
  const double *slipa = c->mode == MODE_SLIP ? pp + np : nullptr;
  const double *selfc = pp + 3 * np;

  // phase events as the other paths: start, (no reciprocal part), end of the
  // pair sum, end
  cudaEvent_t *E = phase_events (c, timed);
  if (E) cudaEventRecord (E[0], st);
  kmark (c, st, nullptr);
  const int pn = n > np ? n : np;
  k_open_prep<<<(pn + 255) / 256, 256, 0, st>>> (d_pos, d_x, rad, slipa, np, n, ph, pl, xf);
  kmark (c, st, "k_open_prep");
  if (E) cudaEventRecord (E[1], st);
  OpenF32Args a;
  a.ph = ph;
  a.pl = pl;
  a.xf = xf;
  a.np = np;
  a.nchunk = nchunk;
  a.rmin = (float) c->rmin;
  a.partial = part;
  const long long nw = (long long) np * nchunk;
  const int grid = (int) ((nw * 32 + 127) / 128);
#define LSG_OPEN(V)                                                                   \
  if (c->mode == MODE_MONO) k_open_f32<V, MODE_MONO><<<grid, 128, 0, st>>> (a);      \
  else if (c->mode == MODE_POLY) k_open_f32<V, MODE_POLY><<<grid, 128, 0, st>>> (a); \
  else k_open_f32<V, MODE_SLIP><<<grid, 128, 0, st>>> (a);
  if (c->version == 0) { LSG_OPEN (0) }
  else if (c->version == 1) { LSG_OPEN (1) }
  else { LSG_OPEN (2) }
#undef LSG_OPEN
  kmark (c, st, "k_open_f32");
  if (E) cudaEventRecord (E[2], st);
  const int gc = (np + 127) / 128;
  if (c->version == 0) k_open_combine<0><<<gc, 128, 0, st>>> (d_x, part, nchunk, selfc, np, d_y);
  else if (c->version == 1) k_open_combine<1><<<gc, 128, 0, st>>> (d_x, part, nchunk, selfc, np, d_y);
  else k_open_combine<2><<<gc, 128, 0, st>>> (d_x, part, nchunk, selfc, np, d_y);
  kmark (c, st, "k_open_combine");
  if (E) cudaEventRecord (E[3], st);
  c->launches = 3;
  c->timed = timed;
  e = cudaGetLastError ();
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, "free-space kernels");
}

}  // namespace lsg
