// kspace_tc.cu -- reciprocal space of the mixed product on the tensor cores.
//
// Both halves of the reciprocal sum are GEMMs with a thin N = 16 (the c <= 11
// components of a particle, zero-padded):
//
//   forward        D[(cos|sin, k), q] = sum_j {cos, sin}(k.r_j) x_j[q]
//                  M = 128 rows = 64 k vectors x (cos, sin), K = particles
//   back-projection D[i, q] = sum_k cos(k.r_i) P_k[q] + sin(k.r_i) Q_k[q]
//                  M = 128 particles, K = (k, cos|sin) pairs, split over CTAs
//
// The A operand (the phase tile) is built on the fly in shared memory from
// per-axis phase tables, e^{ik.r} = t0[m1] t1[m2] t2[m3]; B comes from x or
// from P, Q.  Every operand is split into TF32 hi + lo parts and each
// product is accumulated as hi*hi + hi*lo + lo*hi (3xTF32), FP32 accumulation
// in TMEM, rotating over four accumulators to shorten each FP32 sum.  Shared
// memory tiles are double buffered: the CTA builds tile t + 1 while the
// tensor core works on tile t; an mbarrier per buffer (tcgen05.commit) says
// when a buffer may be overwritten.  Every wait is bounded; a wait that runs
// out sets *status and the CTA drains and frees its TMEM.
#include <cuda_runtime.h>

#include "ewald_device.cuh"
#include "mixed.h"
#include "tc_umma.cuh"

namespace lsg {
namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_ROWS = 128;                   // MMA M
constexpr int TC_N = 16;                       // MMA N (components, padded)
constexpr int TC_KTILE = 32;                   // K per shared-memory tile
constexpr uint32_t A_BYTES = TC_ROWS * TC_KTILE * 4;   // one precision of A
constexpr uint32_t B_BYTES = TC_N * TC_KTILE * 4;      // one precision of B
constexpr uint32_t SM_A = 0;                            // [stage][hi|lo]
constexpr uint32_t SM_B = SM_A + 4 * A_BYTES;           // [stage][hi|lo]
constexpr uint32_t SM_VAR = SM_B + 4 * B_BYTES;         // kernel-specific
constexpr int NACC = 4;                                 // rotating accumulators
constexpr uint32_t TMEM_COLS = 64;                      // NACC * TC_N
constexpr uint32_t WAIT_LIMIT = 1u << 26;

__device__ __forceinline__ float2
cmulf (float2 a, float2 b)
{
  return make_float2 (a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ void
put_split (unsigned char *hi, unsigned char *lo, uint32_t o, float v)
{
  uint32_t h, l;
  umma::split_tf32 (v, h, l);
  *reinterpret_cast<uint32_t *> (hi + o) = h;
  *reinterpret_cast<uint32_t *> (lo + o) = l;
}

// issue the 4 K-steps x 3 products of one tile into accumulator `acc`
__device__ __forceinline__ void
issue_tile (unsigned char *smem, int stage, uint32_t tmem, int acc, bool first)
{
  const uint32_t idesc = umma::idesc_tf32 (TC_ROWS, TC_N);
  const uint32_t base = umma::smem_u32 (smem);
  const uint32_t a_hi = base + SM_A + (2 * stage) * A_BYTES, a_lo = a_hi + A_BYTES;
  const uint32_t b_hi = base + SM_B + (2 * stage) * B_BYTES, b_lo = b_hi + B_BYTES;
  const uint32_t d = tmem + (uint32_t) (acc * TC_N);
#pragma unroll
  for (int s = 0; s < TC_KTILE / 8; s++)
    {
      const uint64_t ah = umma::smem_desc (a_hi + s * TC_ROWS * 32, 128, 256);
      const uint64_t al = umma::smem_desc (a_lo + s * TC_ROWS * 32, 128, 256);
      const uint64_t bh = umma::smem_desc (b_hi + s * TC_N * 32, 128, 256);
      const uint64_t bl = umma::smem_desc (b_lo + s * TC_N * 32, 128, 256);
      umma::mma_tf32 (d, ah, bh, idesc, (first && s == 0) ? 0u : 1u);
      umma::mma_tf32 (d, ah, bl, idesc, 1u);
      umma::mma_tf32 (d, al, bh, idesc, 1u);
    }
}

// sum of the used accumulators of this thread's TMEM lane (16 columns)
__device__ __forceinline__ void
read_acc (uint32_t tmem, int nacc, float out[16])
{
  const int warp = threadIdx.x >> 5;
  for (int q = 0; q < 16; q++) out[q] = 0.f;
  for (int a = 0; a < nacc; a++)
    {
      float v[16];
      umma::tmem_ld16 (tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) (a * TC_N), v);
#pragma unroll
      for (int q = 0; q < 16; q++) out[q] += v[q];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// forward: C(k), S(k), then P = Bc C - Bs S, Q = Bc S + Bs C
// ---------------------------------------------------------------------------
struct SfacTcArgs {
  const MixK *kt;
  int nkh;
  PhaseTables t;
  const float *xf;
  float *pq;
  int *status;
};

template <int V>
__global__ void __launch_bounds__ (TC_THREADS)
mk_sfac_tc (SfacTcArgs a)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ __align__ (1024) unsigned char smem[];
  __shared__ __align__ (8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ MixK krow[64];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int k0 = blockIdx.x * 64;
  const int np = a.t.np;
  const int nt0 = a.t.M0 + 1, nt1 = a.t.M1 + 1, nt2 = a.t.M2 + 1;
  float2 *tabs = reinterpret_cast<float2 *> (smem + SM_VAR);   // [row][32]
  const int ntab = nt0 + nt1 + nt2;

  if (tid < 64)
    {
      MixK z = {};
      krow[tid] = (k0 + tid < a.nkh) ? a.kt[k0 + tid] : z;
    }
  if (warp == 0) umma::tmem_alloc (&tslot, TMEM_COLS);
  if (tid == 0)
    {
      umma::mbar_init (&mbar[0], 1);
      umma::mbar_init (&mbar[1], 1);
      umma::fence_mbar_init ();
    }
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
  const uint32_t tmem = tslot;

  const int ntiles = (np + TC_KTILE - 1) / TC_KTILE;
  const int kk = tid & 63;                 // this thread's k vector
  const int jh = (tid >> 6) * 16;          // and half of the particle tile
  const MixK K = krow[kk];
  const int am1 = K.m1 < 0 ? -K.m1 : K.m1, am2 = K.m2 < 0 ? -K.m2 : K.m2,
            am3 = K.m3 < 0 ? -K.m3 : K.m3;
  const bool live = (k0 + kk) < a.nkh;
  bool ok = true;
  int done = 0;
  for (int t = 0; t < ntiles; t++)
    {
      const int s = t & 1;
      if (t >= 2)
        {
          ok = __syncthreads_and (umma::mbar_wait (&mbar[s], ((t >> 1) - 1) & 1, WAIT_LIMIT)) != 0;
          if (!ok) break;
        }
      __syncthreads ();   // the previous tile's generation is done with `tabs`
      const int j0 = t * TC_KTILE;
      for (int e = tid; e < ntab * TC_KTILE; e += TC_THREADS)
        {
          const int row = e / TC_KTILE, jj = e % TC_KTILE, j = j0 + jj;
          size_t src;
          if (row < nt0) src = (size_t) row * np;
          else if (row < nt0 + nt1) src = a.t.off1 + (size_t) (row - nt0) * np;
          else src = a.t.off2 + (size_t) (row - nt0 - nt1) * np;
          tabs[e] = (j < np) ? a.t.tab[src + j] : make_float2 (0.f, 0.f);
        }
      __syncthreads ();
      unsigned char *Ahi = smem + SM_A + (2 * s) * A_BYTES, *Alo = Ahi + A_BYTES;
      unsigned char *Bhi = smem + SM_B + (2 * s) * B_BYTES, *Blo = Bhi + B_BYTES;
      // B: x, 16 rows (components) by 32 particles
      for (int e = tid; e < TC_N * TC_KTILE; e += TC_THREADS)
        {
          const int q = e / TC_KTILE, jj = e % TC_KTILE, j = j0 + jj;
          const float v = (q < C && j < np) ? a.xf[(size_t) j * C + q] : 0.f;
          put_split (Bhi, Blo, umma::off (q, jj, TC_N), v);
        }
      // A: row kk = cos(k.r_j), row 64 + kk = sin(k.r_j)
#pragma unroll 4
      for (int jj = jh; jj < jh + 16; jj++)
        {
          float2 p0 = tabs[am1 * TC_KTILE + jj];
          float2 p1 = tabs[(nt0 + am2) * TC_KTILE + jj];
          float2 p2 = tabs[(nt0 + nt1 + am3) * TC_KTILE + jj];
          if (K.m1 < 0) p0.y = -p0.y;
          if (K.m2 < 0) p1.y = -p1.y;
          if (K.m3 < 0) p2.y = -p2.y;
          float2 ph = cmulf (cmulf (p0, p1), p2);
          if (!live) ph = make_float2 (0.f, 0.f);
          put_split (Ahi, Alo, umma::off (kk, jj, TC_ROWS), ph.x);
          put_split (Ahi, Alo, umma::off (64 + kk, jj, TC_ROWS), ph.y);
        }
      umma::fence_async_smem ();
      __syncthreads ();
      if (tid == 0)
        {
          umma::fence_after_sync ();
          issue_tile (smem, s, tmem, t & (NACC - 1), t < NACC);
          umma::mma_commit (&mbar[s]);
        }
      done = t + 1;
    }
  // drain: the last commit covers every MMA issued before it
  if (done > 0)
    {
      const int last = done - 1;
      const bool fin = __syncthreads_and (
        umma::mbar_wait (&mbar[last & 1], (last >> 1) & 1, WAIT_LIMIT)) != 0;
      ok = ok && fin;
    }
  umma::fence_after_sync ();
  float *cs = reinterpret_cast<float *> (smem + SM_A);   // [128][16], A tiles are free now
  if (ok)
    {
      float v[16];
      read_acc (tmem, done < NACC ? done : NACC, v);
#pragma unroll
      for (int q = 0; q < 16; q++) cs[tid * 16 + q] = v[q];
    }
  else if (tid == 0)
    atomicExch (a.status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
  if (!ok || tid >= 64 || !live) return;
  // per-k operators
  float csum[C], ssum[C], nsum[C];
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      csum[q] = cs[kk * 16 + q];
      ssum[q] = cs[(64 + kk) * 16 + q];
      nsum[q] = -ssum[q];
    }
  const float e[3] = {K.ex, K.ey, K.ez};
  GenF<V, float> gc, gs, gms;
  load_genf<V, float> (csum, gc);
  load_genf<V, float> (ssum, gs);
  load_genf<V, float> (nsum, gms);
  GenU<V, float> P, Q;
  P.zero ();
  Q.zero ();
  recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gc, gms, P);
  recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gs, gc, Q);
  const int k = k0 + kk;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      a.pq[(size_t) q * a.nkh + k] = P.v[q];
      a.pq[(size_t) (C + q) * a.nkh + k] = Q.v[q];
    }
}

// ---------------------------------------------------------------------------
// back-projection over one slice of k space
// ---------------------------------------------------------------------------
struct BpTcArgs {
  const MixK *kt;
  int nkh, nsplit;
  PhaseTables t;
  const float *pq;
  float *partial;
  int *status;
};

template <int V>
__global__ void __launch_bounds__ (TC_THREADS)
mk_bp_tc (BpTcArgs a)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ __align__ (1024) unsigned char smem[];
  __shared__ __align__ (8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ int4 kms[2][16];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int np = a.t.np;
  const int i0 = blockIdx.x * TC_ROWS;
  const int split = blockIdx.y;
  const int nt0 = a.t.M0 + 1, nt1 = a.t.M1 + 1, nt2 = a.t.M2 + 1;
  const int ntab = nt0 + nt1 + nt2;
  float2 *ptab = reinterpret_cast<float2 *> (smem + SM_VAR);   // [row][128 particles]
  // this CTA's particles: their phase-table columns
  for (int e = tid; e < ntab * TC_ROWS; e += TC_THREADS)
    {
      const int row = e / TC_ROWS, ii = e % TC_ROWS, i = i0 + ii;
      size_t src;
      if (row < nt0) src = (size_t) row * np;
      else if (row < nt0 + nt1) src = a.t.off1 + (size_t) (row - nt0) * np;
      else src = a.t.off2 + (size_t) (row - nt0 - nt1) * np;
      ptab[e] = (i < np) ? a.t.tab[src + i] : make_float2 (0.f, 0.f);
    }
  if (warp == 0) umma::tmem_alloc (&tslot, TMEM_COLS);
  if (tid == 0)
    {
      umma::mbar_init (&mbar[0], 1);
      umma::mbar_init (&mbar[1], 1);
      umma::fence_mbar_init ();
    }
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
  const uint32_t tmem = tslot;

  // k slice of this CTA, in whole tiles of 16 vectors
  const int ntile_all = (a.nkh + 15) / 16;
  const int tb = (int) ((long long) ntile_all * split / a.nsplit);
  const int te = (int) ((long long) ntile_all * (split + 1) / a.nsplit);
  bool ok = true;
  int done = 0;
  for (int t = tb; t < te; t++)
    {
      const int u = t - tb, s = u & 1;
      if (u >= 2)
        {
          ok = __syncthreads_and (umma::mbar_wait (&mbar[s], ((u >> 1) - 1) & 1, WAIT_LIMIT)) != 0;
          if (!ok) break;
        }
      const int kb = t * 16;
      if (tid < 16)
        {
          const int k = kb + tid;
          kms[s][tid] = (k < a.nkh) ? *reinterpret_cast<const int4 *> (&a.kt[k].m1)
                                    : make_int4 (0, 0, 0, -1);
        }
      __syncthreads ();
      unsigned char *Ahi = smem + SM_A + (2 * s) * A_BYTES, *Alo = Ahi + A_BYTES;
      unsigned char *Bhi = smem + SM_B + (2 * s) * B_BYTES, *Blo = Bhi + B_BYTES;
      // B: 16 rows (components) by 32 = 16 k x (P, Q)
      for (int e = tid; e < TC_N * TC_KTILE; e += TC_THREADS)
        {
          const int q = e / TC_KTILE, col = e % TC_KTILE, k = kb + (col >> 1);
          float v = 0.f;
          if (q < C && k < a.nkh)
            v = a.pq[(size_t) ((col & 1) ? C + q : q) * a.nkh + k];
          put_split (Bhi, Blo, umma::off (q, col, TC_N), v);
        }
      // A: row = particle tid, columns (cos, sin) of the 16 k vectors
#pragma unroll 4
      for (int c16 = 0; c16 < 16; c16++)
        {
          const int4 m = kms[s][c16];
          float2 ph = make_float2 (0.f, 0.f);
          if (m.w == 0)
            {
              float2 p0 = ptab[(m.x < 0 ? -m.x : m.x) * TC_ROWS + tid];
              float2 p1 = ptab[(nt0 + (m.y < 0 ? -m.y : m.y)) * TC_ROWS + tid];
              float2 p2 = ptab[(nt0 + nt1 + (m.z < 0 ? -m.z : m.z)) * TC_ROWS + tid];
              if (m.x < 0) p0.y = -p0.y;
              if (m.y < 0) p1.y = -p1.y;
              if (m.z < 0) p2.y = -p2.y;
              ph = cmulf (cmulf (p0, p1), p2);
            }
          put_split (Ahi, Alo, umma::off (tid, 2 * c16, TC_ROWS), ph.x);
          put_split (Ahi, Alo, umma::off (tid, 2 * c16 + 1, TC_ROWS), ph.y);
        }
      umma::fence_async_smem ();
      __syncthreads ();
      if (tid == 0)
        {
          umma::fence_after_sync ();
          issue_tile (smem, s, tmem, u & (NACC - 1), u < NACC);
          umma::mma_commit (&mbar[s]);
        }
      done = u + 1;
    }
  if (done > 0)
    {
      const int last = done - 1;
      const bool fin = __syncthreads_and (
        umma::mbar_wait (&mbar[last & 1], (last >> 1) & 1, WAIT_LIMIT)) != 0;
      ok = ok && fin;
    }
  umma::fence_after_sync ();
  const int i = i0 + tid;
  if (ok)
    {
      float v[16];
      read_acc (tmem, done < NACC ? done : NACC, v);
      if (i < np)
        {
          float *out = a.partial + ((size_t) split * np + i) * C;
#pragma unroll
          for (int q = 0; q < C; q++) out[q] = (done > 0) ? v[q] : 0.f;
        }
    }
  else if (tid == 0)
    atomicExch (a.status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename K>
static cudaError_t
set_smem (K kernel, size_t bytes)
{
  return cudaFuncSetAttribute (kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
}

cudaError_t
launch_sfac_tc (int version, const MixK *kt, int nkh, PhaseTables t, const float *xf, float *pq,
                int *status, cudaStream_t st)
{
  if (nkh <= 0) return cudaSuccess;
  SfacTcArgs a{kt, nkh, t, xf, pq, status};
  const size_t smem = SM_VAR + sizeof (float2) * (size_t) (t.M0 + t.M1 + t.M2 + 3) * TC_KTILE;
  const int grid = (nkh + 63) / 64;
  cudaError_t e;
  if (version == 0)
    {
      if ((e = set_smem (mk_sfac_tc<0>, smem)) != cudaSuccess) return e;
      mk_sfac_tc<0><<<grid, TC_THREADS, smem, st>>> (a);
    }
  else if (version == 1)
    {
      if ((e = set_smem (mk_sfac_tc<1>, smem)) != cudaSuccess) return e;
      mk_sfac_tc<1><<<grid, TC_THREADS, smem, st>>> (a);
    }
  else
    {
      if ((e = set_smem (mk_sfac_tc<2>, smem)) != cudaSuccess) return e;
      mk_sfac_tc<2><<<grid, TC_THREADS, smem, st>>> (a);
    }
  return cudaGetLastError ();
}

int
backproj_splits (int np, int nkh)
{
  const int mtiles = (np + TC_ROWS - 1) / TC_ROWS;
  const int ktiles = (nkh + 15) / 16;
  int ns = (2 * 152 + mtiles - 1) / mtiles;        // about two CTAs per SM
  if (ns > ktiles / 4) ns = ktiles / 4;            // at least four tiles each
  return ns < 1 ? 1 : ns;
}

cudaError_t
launch_backproj_tc (int version, const MixK *kt, int nkh, PhaseTables t, const float *pq,
                    int nsplit, float *partial, int *status, cudaStream_t st)
{
  BpTcArgs a{kt, nkh, nsplit, t, pq, partial, status};
  const size_t smem = SM_VAR + sizeof (float2) * (size_t) (t.M0 + t.M1 + t.M2 + 3) * TC_ROWS;
  dim3 grid ((t.np + TC_ROWS - 1) / TC_ROWS, nsplit);
  cudaError_t e;
  if (version == 0)
    {
      if ((e = set_smem (mk_bp_tc<0>, smem)) != cudaSuccess) return e;
      mk_bp_tc<0><<<grid, TC_THREADS, smem, st>>> (a);
    }
  else if (version == 1)
    {
      if ((e = set_smem (mk_bp_tc<1>, smem)) != cudaSuccess) return e;
      mk_bp_tc<1><<<grid, TC_THREADS, smem, st>>> (a);
    }
  else
    {
      if ((e = set_smem (mk_bp_tc<2>, smem)) != cudaSuccess) return e;
      mk_bp_tc<2><<<grid, TC_THREADS, smem, st>>> (a);
    }
  return cudaGetLastError ();
}

}  // namespace lsg
