// kspace_tc.cu -- reciprocal space of the mixed product as tensor-core GEMMs.
//
// With the fixed-point fractional coordinates u_d(j) of the particles, the
// phase of k = (m1, m2, m3) factorises, e^{ik.r_j} = t0[m1](j) T_r(j) with
// t0[m1] = e^{2 pi i m1 u_x} and T_r = e^{2 pi i (m2 u_y + m3 u_z)} for the
// row r = (m2, m3).  So the structure factors of every k vector of the list
// come out of ONE complex GEMM over the particles and the back-projection
// out of another:
//
//   forward   S[r, (m1, q)] = sum_j T_r(j) Z_(m1,q)(j),   Z = t0[m1] x_q
//             real rows r; columns (m1, re|im, q); K = (j, a|b) with
//             (a, b) = (Re, Im) T_r(j):  A[r][(j, a|b)];
//             B row (m1, re, q) = (u, -v), row (m1, im, q) = (v, u) with
//             (u, v) = Z  (image ZF)
//   operator  W_k = P_k + i Q_k for every k of the half-space list (k_kop)
//   backward  H[i, (m1, re|im, q)] = sum_r conj(T_r)(i) W[r, (m1, q)]:
//             A'[i][(r, a|b)]; B' row (m1, re, q) = (U, V), row
//             (m1, im, q) = (V, -U) with (U, V) = W  (image WB);
//             y_i[q] += Re(conj(t0[m1])(i) H) over m1 in the epilogue.
//
// The B operands are written once per product as IMAGES: FP32 arrays
// [2][rows][K] (plane 0 the TF32-rounded value, plane 1 the TF32-rounded
// remainder, x = hi + lo), K contiguous and already in the sign pattern
// above, loaded per tile by TMA (32 K values = 128 bytes per row, 128-byte
// swizzle).  The A operands -- the row phases T_r -- are not stored: the
// worker warps build each tile straight into shared memory, in the same
// swizzled layout: the forward's as products t_y[m2](j) t_z[m3](j) of the
// per-axis phases (a particle-major table written by mk_prep), the
// backward's by phase_of from the exact fixed-point phase m2 q_y + m3 q_z
// mod 2^32.  The products are tcgen05 kind::tf32 MMAs (M = 128, N <= 256, K = 8 per instruction) in
// 3xTF32: hi*hi + hi*lo + lo*hi.  The tensor core's FP32 accumulation
// truncates at the accumulator's magnitude, so every 32-wide K tile starts a
// fresh accumulator that is drained into FP32 registers (round to nearest);
// within a tile the two small correction products go in first and the
// hi*hi products last, so the corrections are summed at their own magnitude
// and each later add truncates no more than a hi*hi-only chain would.
//
// Warp roles (320 threads, one CTA per SM):
//   warps 0-7   workers: build the A operand of each stage, and drain the
//               double-buffered TMEM accumulators (2 x 256 columns = 512
//               columns); warp w reads TMEM lanes 32 (w % 4) and columns
//               128 (w / 4) of each buffer
//   warp 8      one lane issues the B-operand TMA loads of a 2-stage ring
//   warp 9      one lane issues the MMAs of a tile when its stage is full
//               and its accumulator buffer has been drained
// The roles meet only at mbarriers; every wait is bounded and watches a CTA
// error flag, so a wait that runs out ends every role and raises *status;
// the TMA lane waits for its loads in flight and the MMA lane for its MMAs
// before the CTA frees its TMEM and exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "tc_umma.cuh"
#include "tma_host.h"

namespace lsg {
namespace {

constexpr int NT = 320;                 // threads per CTA (10 warps)
constexpr int NDRAIN = 8;               // drain warps 0..7
constexpr int NWORK = NDRAIN * 32;      // they also build the A operand
constexpr int TMA_WARP = 8;
constexpr int MMA_WARP = 9;
constexpr int TM = 128;                 // MMA M
constexpr int TN = 256;                 // largest MMA N (columns per tile)
constexpr int KT = 32;                  // K values per tile (128 bytes per row)
constexpr int PT = KT / 2;              // complex entries per K tile
constexpr int STAGES = 2;
constexpr int CPT = TN / 2;             // accumulator columns per drain thread (128)
constexpr uint32_t A_BYTES = TM * KT * 4;
constexpr uint32_t B_BYTES = TN * KT * 4;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // 96 KB: hi + lo of A and B
constexpr uint32_t SMEM_DYN = STAGES * STAGE_BYTES + 1024;    // + room to align to 1 KB
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t WAIT_LIMIT = 1u << 18;   // polls of up to ~20 us each

struct Sync {
  uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], done;
  uint64_t never;       // nothing arrives here: the wait of the failure-injection test
  uint32_t tslot;
  int err;
};

__device__ __forceinline__ unsigned char *
align1k (unsigned char *p)
{
  return p + ((1024u - (umma::smem_u32 (p) & 1023u)) & 1023u);
}

__device__ __forceinline__ void
cta_setup (Sync &s)
{
  const int warp = threadIdx.x >> 5;
  if (warp == 0) umma::tmem_alloc (&s.tslot, TMEM_COLS);
  if (threadIdx.x == 32)
    {
      for (int k = 0; k < STAGES; k++)
        {
          umma::mbar_init (&s.full[k], 1 + NWORK);   // TMA lane + A builders
          umma::mbar_init (&s.empty[k], 1);
        }
      for (int b = 0; b < 2; b++)
        {
          umma::mbar_init (&s.acc_full[b], 1);
          umma::mbar_init (&s.acc_empty[b], NDRAIN * 32);
        }
      umma::mbar_init (&s.done, 1);
      umma::mbar_init (&s.never, 1);
      s.err = 0;
      umma::fence_mbar_init ();
    }
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
}

// the TMA lane: the B operand (hi and lo planes, rows from brow) of tile t
// (K values k0 + 32 t ..) into stage t % STAGES
__device__ __forceinline__ void
tma_role (Sync &s, unsigned char *smem, const CUtensorMap *tb, int brow, int k0, int ntiles,
          uint32_t b_bytes)
{
  volatile int *err = &s.err;
  const uint32_t tx = 2 * b_bytes;
  umma::tma_prefetch_desc (tb);
  int issued = 0;
  for (int t = 0; t < ntiles; t++)
    {
      const int st = t % STAGES;
      if (t >= STAGES
          && !umma::mbar_wait_or_abort (&s.empty[st], ((t / STAGES) - 1) & 1, WAIT_LIMIT, err))
        break;
      unsigned char *sb = smem + (size_t) st * STAGE_BYTES;
      const int kx = k0 + KT * t;
      umma::mbar_expect_tx (&s.full[st], tx);
      umma::tma_load_3d (sb + 2 * A_BYTES, tb, kx, brow, 0, &s.full[st]);
      umma::tma_load_3d (sb + 2 * A_BYTES + B_BYTES, tb, kx, brow, 1, &s.full[st]);
      issued = t + 1;
    }
  // the last load of each stage must land before the shared memory goes away
  volatile int never = 0;
  for (int t = issued > STAGES ? issued - STAGES : 0; t < issued; t++)
    umma::mbar_wait_or_abort (&s.full[t % STAGES], (t / STAGES) & 1, WAIT_LIMIT, &never);
}

// the MMA lane: tile t in stage t % STAGES, accumulator buffer t & 1
__device__ __forceinline__ void
mma_role (Sync &s, const unsigned char *smem, uint32_t tmem, uint32_t idesc, int ntiles,
          int stall)
{
  volatile int *err = &s.err;
  // failure injection (tests): a wait that cannot complete runs out, raises
  // the CTA error flag and ends every role before any MMA is issued
  if (stall > 0 && !umma::mbar_wait_or_abort (&s.never, 0, (uint32_t) stall, err)) ntiles = 0;
  for (int t = 0; t < ntiles; t++)
    {
      const int st = t % STAGES, b = t & 1;
      if (!umma::mbar_wait_or_abort (&s.full[st], (t / STAGES) & 1, WAIT_LIMIT, err)) break;
      if (t >= 2 && !umma::mbar_wait_or_abort (&s.acc_empty[b], ((t >> 1) - 1) & 1, WAIT_LIMIT, err))
        break;
      umma::fence_after_sync ();
      const uint32_t base = umma::smem_u32 (smem) + (uint32_t) st * STAGE_BYTES;
      const uint32_t ahi = base, alo = base + A_BYTES, bhi = base + 2 * A_BYTES,
                     blo = bhi + B_BYTES;
      const uint32_t d = tmem + (uint32_t) (b * TN);
      // corrections first (summed at their own magnitude), then hi*hi
#pragma unroll
      for (int k = 0; k < KT / 8; k++)
        {
          const uint64_t dah = umma::smem_desc_sw128 (ahi + 32 * k);
          const uint64_t dal = umma::smem_desc_sw128 (alo + 32 * k);
          const uint64_t dbh = umma::smem_desc_sw128 (bhi + 32 * k);
          const uint64_t dbl = umma::smem_desc_sw128 (blo + 32 * k);
          umma::mma_tf32 (d, dah, dbl, idesc, k ? 1u : 0u);
          umma::mma_tf32 (d, dal, dbh, idesc, 1u);
        }
#pragma unroll
      for (int k = 0; k < KT / 8; k++)
        umma::mma_tf32 (d, umma::smem_desc_sw128 (ahi + 32 * k),
                        umma::smem_desc_sw128 (bhi + 32 * k), idesc, 1u);
      umma::mma_commit (&s.empty[st]);
      umma::mma_commit (&s.acc_full[b]);
    }
  // every MMA issued so far has completed once `done` flips
  umma::mma_commit (&s.done);
  volatile int never = 0;
  umma::mbar_wait_or_abort (&s.done, 0, WAIT_LIMIT, &never);
}

// a complex value as TF32 hi and lo parts (FP32 bit patterns)
__device__ __forceinline__ void
split2 (float2 v, float2 &hi, float2 &lo)
{
  uint32_t hx, lx, hy, ly;
  umma::split_tf32 (v.x, hx, lx);
  umma::split_tf32 (v.y, hy, ly);
  hi = make_float2 (__uint_as_float (hx), __uint_as_float (hy));
  lo = make_float2 (__uint_as_float (lx), __uint_as_float (ly));
}

// the A hi/lo planes of one stage: chunk c (16 bytes, two complex values) of
// row `row` in the 128-byte swizzled layout the MMA descriptors expect
__device__ __forceinline__ void
put_a (unsigned char *stage, int row, int c, float2 v0, float2 v1)
{
  float2 h0, l0, h1, l1;
  split2 (v0, h0, l0);
  split2 (v1, h1, l1);
  const uint32_t o = (uint32_t) row * 128u + ((uint32_t) (c ^ (row & 7)) << 4);
  *reinterpret_cast<float4 *> (stage + o) = make_float4 (h0.x, h0.y, h1.x, h1.y);
  *reinterpret_cast<float4 *> (stage + A_BYTES + o) = make_float4 (l0.x, l0.y, l1.x, l1.y);
}

// worker warps 0-7: build the A operand of every stage and drain the
// accumulators.  Thread (row = tid % 128, half = tid / 128) builds complex
// values 8 half .. 8 half + 7 of its A row in each tile (prod (t, k): value k
// of the row in tile t).  Tiles 0 and 1 are built up front; once tile t's
// accumulator is full its MMAs are done, so its stage takes tile t + 2,
// built before tile t is drained (the MMA of tile t + 1 runs meanwhile).
template <class Prod>
__device__ __forceinline__ bool
worker_role (Sync &s, unsigned char *smem, uint32_t tmem, int ntiles, float acc[CPT],
             const Prod &prod)
{
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = tid & 127, half = tid >> 7;
  volatile int *err = &s.err;
  auto build = [&] (int t) {
    unsigned char *stage = smem + (size_t) (t % STAGES) * STAGE_BYTES;
    float2 v[8];
    prod.values (t, 8 * half, v);
    // the inputs of this stage's next tile, into L1 ahead of its build
    if (t + STAGES < ntiles) prod.prefetch (t + STAGES, 8 * half + (threadIdx.x & 7));
#pragma unroll
    for (int c = 0; c < 4; c++) put_a (stage, row, 4 * half + c, v[2 * c], v[2 * c + 1]);
    umma::fence_async_smem ();      // generic writes -> the MMA's async reads
    umma::mbar_arrive (&s.full[t % STAGES]);
  };
  for (int t = 0; t < STAGES && t < ntiles; t++) build (t);
  const uint32_t lane_base = (uint32_t) ((warp & 3) * 32) << 16;
  const uint32_t col = (uint32_t) ((warp >> 2) * CPT);
  for (int t = 0; t < ntiles; t++)
    {
      const int b = t & 1;
      if (!umma::mbar_wait_or_abort (&s.acc_full[b], (t >> 1) & 1, WAIT_LIMIT, err)) return false;
      umma::fence_after_sync ();
      if (t + STAGES < ntiles) build (t + STAGES);
      const uint32_t dm = tmem + lane_base + (uint32_t) (b * TN) + col;
#pragma unroll
      for (int cc = 0; cc < CPT; cc += 32)
        {
          float m[16], c[16];
          umma::tmem_ld16 (dm + cc, m);
          umma::tmem_ld16 (dm + cc + 16, c);
#pragma unroll
          for (int u = 0; u < 16; u++)
            {
              acc[cc + u] += m[u];
              acc[cc + 16 + u] += c[u];
            }
        }
      umma::fence_before_sync ();
      umma::mbar_arrive (&s.acc_empty[b]);
    }
  return true;
}

// A of the forward GEMM: row r = (m2, m3), K = particles from j0.  values():
// entries k0 .. k0 + 7 of tile t, T_r(j) = t_y[m2](j) t_z[m3](j) from the
// particle-major phase table (the 16 particles of a tile are shared by every
// row, so these loads mostly hit L1; indices are clamped so every load is in
// bounds, entries past the particles are zero).  The sixteen loads issue
// back to back, then the products.
struct ProdF {
  const float2 *tyz;
  int wyz, np, j0;
  int iy, iz;               // this row's entries in a particle's table row
  bool live;
  __device__ __forceinline__ void values (int t, int k0, float2 v[8]) const
  {
    float2 a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      {
        const float2 *row = tyz + (size_t) min (j0 + PT * t + k0 + k, np - 1) * wyz;
        a[k] = __ldg (row + iy);
        b[k] = __ldg (row + iz);
      }
#pragma unroll
    for (int k = 0; k < 8; k++)
      {
        const bool ok = live && j0 + PT * t + k0 + k < np;
        v[k] = ok ? make_float2 (a[k].x * b[k].x - a[k].y * b[k].y, a[k].x * b[k].y + a[k].y * b[k].x)
                  : make_float2 (0.f, 0.f);
      }
  }
  __device__ __forceinline__ void prefetch (int t, int k) const
  {
    const float2 *row = tyz + (size_t) min (j0 + PT * t + k, np - 1) * wyz;
    umma::prefetch_l1 (row + iy);
    umma::prefetch_l1 (row + iz);
  }
};

// A of the backward GEMM: row = particle (fixed-point qy, qz), K = rows from
// r0: T_r(i) from the exact fixed-point phase m2 q_y + m3 q_z mod 2^32 by the
// table-driven phase_of (the eight rows' (m2, m3) load first, back to back)
struct ProdB {
  const int2 *rowm;
  const float4 *rot;
  int R, r0;
  uint32_t qy, qz;
  bool live;
  __device__ __forceinline__ void values (int t, int k0, float2 v[8]) const
  {
    int2 mm[8];
#pragma unroll
    for (int k = 0; k < 8; k++) mm[k] = __ldg (rowm + min (r0 + PT * t + k0 + k, R - 1));
#pragma unroll
    for (int k = 0; k < 8; k++)
      {
        const bool ok = live && r0 + PT * t + k0 + k < R;
        const float2 p = phase_of (rot, (uint32_t) mm[k].x * qy + (uint32_t) mm[k].y * qz);
        v[k] = ok ? p : make_float2 (0.f, 0.f);
      }
  }
  __device__ __forceinline__ void prefetch (int t, int k) const
  {
    umma::prefetch_l1 (rowm + min (r0 + PT * t + k, R - 1));
  }
};

// Once every tile is drained no load or MMA touches the stages any more, so
// the drain threads park their accumulator rows there: H[row][column], row
// stride HLD floats (odd, so a warp's 32 rows fall in distinct banks).
constexpr int HLD = TN + 1;
static_assert (TM * HLD * 4 <= (int) (STAGES * STAGE_BYTES), "parked tile exceeds the stages");

__device__ __forceinline__ void
park (unsigned char *smem, const float acc[CPT])
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = (warp & 3) * 32 + lane, cb = (warp >> 2) * CPT;
  float *H = reinterpret_cast<float *> (smem) + row * HLD + cb;
#pragma unroll
  for (int u = 0; u < CPT; u++) H[u] = acc[u];
}

// forward worker threads: build and drain every tile, then column
// n = (m, re|im, q) of row r goes to
// Hs[((m C + q) 2 + re|im) TM + r], the order of the partial structure
// factors sf[split][m1][q][re|im][r], so that each m1's block of rows is one
// TMA store.  CB: the thread's first column (compile time, so the index
// arithmetic folds away).
template <int C, int CB>
__device__ __forceinline__ void
drain_park_sf (Sync &s, uint32_t tmem, int ntiles, unsigned char *smem, int ncol,
               const ProdF &prod)
{
  float acc[CPT];
#pragma unroll
  for (int u = 0; u < CPT; u++) acc[u] = 0.f;
  if (!worker_role (s, smem, tmem, ntiles, acc, prod)) return;
  const int row = ((threadIdx.x >> 5) & 3) * 32 + (threadIdx.x & 31);
  float *Hs = reinterpret_cast<float *> (smem) + row;
#pragma unroll
  for (int u = 0; u < CPT; u++)
    {
      constexpr int P = 2 * C;
      const int n = CB + u;
      const int m = n / P, rem = n - m * P, part = rem >= C ? 1 : 0, q = rem - part * C;
      if (n < ncol) Hs[((m * C + q) * 2 + part) * TM] = acc[u];
    }
  // these writes are read by the TMA unit (async proxy) after the barrier
  umma::fence_async_smem ();
}


}  // namespace

// ---------------------------------------------------------------------------
// forward: partial structure factors of one (row tile, m1 tile, particle slice)
// ---------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__ (NT, 1)
k_sfac_gemm (const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmS,
             KGemm g, int *status)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ unsigned char dsm[];
  __shared__ Sync s;
  unsigned char *smem = align1k (dsm);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r0 = blockIdx.x * TM;
  const int m1b = blockIdx.y * g.gf, nm1 = min (g.gf, g.n1 - m1b);
  const int split = blockIdx.z;
  const int jb = split * g.jper, je = min (g.t.np, jb + g.jper);
  const int ntiles = (je > jb) ? (je - jb + PT - 1) / PT : 0;
  const int ncol = nm1 * 2 * C;

  cta_setup (s);
  const uint32_t tmem = s.tslot;

  if (warp == TMA_WARP)
    {
      if (lane == 0)
        tma_role (s, smem, &tmB, m1b * 2 * C, 2 * jb, ntiles, (uint32_t) g.nf * KT * 4);
      __syncwarp ();
    }
  else if (warp == MMA_WARP)
    {
      if (lane == 0) mma_role (s, smem, tmem, umma::idesc_tf32 (TM, g.nf), ntiles, g.stall);
      __syncwarp ();
    }
  else
    {
      // A rows: r = (m2, m3), values T_r(j) over the slice's particles
      ProdF prod;
      const int r = r0 + (tid & 127);
      prod.tyz = g.t.tyz;
      prod.wyz = g.t.wyz;
      prod.np = g.t.np;
      prod.j0 = jb;
      prod.live = r < g.R;
      const int2 mm = prod.live ? g.rowm[r] : make_int2 (0, 0);
      prod.iy = g.t.M1 + mm.x;
      prod.iz = (2 * g.t.M1 + 1) + g.t.M2 + mm.y;
      if (warp >> 2) drain_park_sf<C, CPT> (s, tmem, ntiles, smem, ncol, prod);
      else drain_park_sf<C, 0> (s, tmem, ntiles, smem, ncol, prod);
    }
  __syncthreads ();
  if (!s.err && tid == 0)
    {
      // one TMA store per m1: 2C rows (q, re|im) of 128 r each; rows past
      // the end of sf are dropped by the TMA unit
      const float *Hs = reinterpret_cast<const float *> (smem);
      for (int m = 0; m < nm1; m++)
        umma::tma_store_2d (&tmS, Hs + (size_t) m * 2 * C * TM, r0,
                            (split * g.n1 + m1b + m) * 2 * C);
      umma::bulk_commit ();
      umma::bulk_wait_read ();
    }
  __syncthreads ();
  if (tid == 0 && s.err) atomicExch (status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// per-k operators: W_k = P_k + i Q_k from the summed structure factors,
// written into the image WB (each (row, m1) belongs to at most one k)
// ---------------------------------------------------------------------------
constexpr int KOP_K = 32;    // k vectors per CTA
constexpr int KOP_G = 8;     // particle-slice groups per k (one slice each up to 8 slices)
static_assert (KOP_G == 8, "k_kop's image writes assume eight groups");

// CTA of KOP_K x KOP_G threads: thread (kk, sg) sums the slices sg, sg + 8,
// ... of the forward partials of k = blockIdx.x * KOP_K + kk (one slice per
// thread up to eight slices, so its loads are all independent; loads of
// neighbouring k are neighbouring rows, so they coalesce); the eight sums
// meet in shared memory; group 0 forms P_k and group 1 Q_k; then the groups
// write the (re | im row) x (hi | lo plane) entries of the image, each pair
// of groups half of the components.
template <int V>
__global__ void __launch_bounds__ (KOP_K * KOP_G)
k_kop (KGemm g, const MixK *kt, int nk, const float *sf)
{
  constexpr int C = NComp<V>::value;
  __shared__ float s_v[KOP_G][2 * C][KOP_K];
  const int kk = threadIdx.x % KOP_K, sg = threadIdx.x / KOP_K;
  const int k = blockIdx.x * KOP_K + kk;
  const size_t Rp = (size_t) g.Rp;
  MixK K;
  float cs[C], sn[C];
#pragma unroll
  for (int q = 0; q < C; q++) cs[q] = sn[q] = 0.f;
  if (k < nk)
    {
      K = kt[k];
      for (int s = sg; s < g.nsplit; s += KOP_G)
        {
          const float *base = sf + (((size_t) s * g.n1 + K.m1) * C * 2) * Rp + K.r;
#pragma unroll
          for (int q = 0; q < C; q++)
            {
              cs[q] += base[(size_t) (2 * q) * Rp];
              sn[q] += base[(size_t) (2 * q + 1) * Rp];
            }
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      s_v[sg][2 * q][kk] = cs[q];
      s_v[sg][2 * q + 1][kk] = sn[q];
    }
  __syncthreads ();
  GenU<V, float> P;
  P.zero ();
  if (k < nk && sg < 2)
    {
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          float a = 0.f, b = 0.f;
#pragma unroll
          for (int h = 0; h < KOP_G; h++)
            {
              a += s_v[h][2 * q][kk];
              b += s_v[h][2 * q + 1][kk];
            }
          cs[q] = a;
          sn[q] = b;
        }
      const float e[3] = {K.ex, K.ey, K.ez};
      GenF<V, float> ga, gb;
      if (sg == 0)
        {
          // P = A(k) C - B(k) S with the sine part entering negated
#pragma unroll
          for (int q = 0; q < C; q++) sn[q] = -sn[q];
          load_genf<V, float> (cs, ga);
          load_genf<V, float> (sn, gb);
        }
      else
        {
          load_genf<V, float> (sn, ga);
          load_genf<V, float> (cs, gb);
        }
      recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, ga, gb, P);
    }
  __syncthreads ();
  if (sg < 2)
#pragma unroll
    for (int q = 0; q < C; q++) s_v[sg][q][kk] = P.v[q];
  __syncthreads ();
  if (k >= nk) return;
  // group sg: image row (m1, re) for sg even, (m1, im) for odd; plane
  // (sg / 2) % 2; groups 0-3 write the components q < C / 2, groups 4-7 the
  // others
  const int part = sg & 1, plane = (sg >> 1) & 1;
  const int qa = (sg < 4) ? 0 : C / 2, qb = (sg < 4) ? C / 2 : C;
  float *img = g.WB + (size_t) plane * g.pWB;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      if (q < qa || q >= qb) continue;
      const float U = s_v[0][q][kk], Vv = s_v[1][q][kk];
      float2 hi, lo;
      split2 (part ? make_float2 (Vv, -U) : make_float2 (U, Vv), hi, lo);
      const size_t row = ((size_t) K.m1 * 2 + part) * C + q;
      reinterpret_cast<float2 *> (img + row * g.KB)[K.r] = plane ? lo : hi;
    }
}

// ---------------------------------------------------------------------------
// back-projection: y_i partial over one (m1 tile, row slice)
// ---------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__ (NT, 1)
k_bp_gemm (const __grid_constant__ CUtensorMap tmB, KGemm g, float *ypart, int *status)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ unsigned char dsm[];
  __shared__ Sync s;
  unsigned char *smem = align1k (dsm);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int np = g.t.np;
  const int i0 = blockIdx.x * TM;
  const int m1b = blockIdx.y * g.gb, nm1 = min (g.gb, g.n1 - m1b);
  const int ks = blockIdx.z;
  const int rb = ks * g.rper, re_ = min (g.R, rb + g.rper);
  const int ntiles = (re_ > rb) ? (re_ - rb + PT - 1) / PT : 0;
  const int ncol = nm1 * 2 * C;
  const float2 *t0 = g.t.tab;

  cta_setup (s);
  const uint32_t tmem = s.tslot;

  if (warp == TMA_WARP)
    {
      if (lane == 0)
        tma_role (s, smem, &tmB, m1b * 2 * C, 2 * rb, ntiles, (uint32_t) g.nb * KT * 4);
      __syncwarp ();
    }
  else if (warp == MMA_WARP)
    {
      if (lane == 0) mma_role (s, smem, tmem, umma::idesc_tf32 (TM, g.nb), ntiles, g.stall);
      __syncwarp ();
    }
  else
    {
      // A rows: particle i, values T_r(i) over the slice's rows r
      ProdB prod;
      const int i = i0 + (tid & 127);
      prod.rowm = g.rowm;
      prod.rot = g.t.rot;
      prod.R = g.R;
      prod.r0 = rb;
      prod.live = i < np;
      const uint4 q = prod.live ? g.t.qpos[i] : make_uint4 (0u, 0u, 0u, 0u);
      prod.qy = q.y;
      prod.qz = q.z;
      float acc[CPT];
#pragma unroll
      for (int u = 0; u < CPT; u++) acc[u] = 0.f;
      if (worker_role (s, smem, tmem, ntiles, acc, prod)) park (smem, acc);
    }
  __syncthreads ();
  if (tid == 0 && s.err) atomicExch (status, 1);
  if (!s.err)
    {
      // y_i[q] = sum over m1 of Re(conj(t0[m1])(i) H[i, (m1, q)]), one
      // (particle, component) per thread
      const float *H = reinterpret_cast<const float *> (smem);
      const size_t chunk = (size_t) ks * gridDim.y + blockIdx.y;
      for (int e = tid; e < TM * C; e += NT)
        {
          const int r = e / C, q = e - r * C, i = i0 + r;
          if (i >= np) continue;
          float y = 0.f;
          for (int m = 0; m < nm1; m++)
            {
              const float2 ph = t0[(size_t) (m1b + m) * np + i];
              y = fmaf (ph.x, H[r * HLD + m * 2 * C + q], y);
              y = fmaf (ph.y, H[r * HLD + m * 2 * C + C + q], y);
            }
          ypart[(chunk * np + i) * C + q] = y;
        }
    }
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int round_up (int n, int m) { return (n + m - 1) / m * m; }

KGemm
kgemm_plan (int version, PhaseTables t, const int2 *rowm, int R)
{
  KGemm g{};
  g.t = t;
  g.rowm = rowm;
  g.R = R;
  g.Rk = round_up (R > 0 ? R : 1, 16);
  g.Rp = round_up (R > 0 ? R : 1, 32);
  g.c = NCOMP (version);
  g.n1 = t.M0 + 1;
  g.ldT = round_up (t.np, 16);
  g.KF = 2 * g.ldT;
  g.KB = 2 * g.Rk;
  g.NZ = g.n1 * 2 * g.c;
  g.nrt = (R + TM - 1) / TM;
  // columns (m1, re|im, q), at most TN per tile, balanced over the tiles;
  // both GEMMs use the same column tiling
  const int per = 2 * g.c;
  const int g0 = TN / per;
  g.ntile_f = (g.n1 + g0 - 1) / g0;
  g.gf = (g.n1 + g.ntile_f - 1) / g.ntile_f;
  g.nf = round_up (g.gf * per, 16);
  g.gb = g.gf;
  g.ntile_b = g.ntile_f;
  g.nb = g.nf;
  // particle slices: about one wave of CTAs
  const int base = g.nrt * g.ntile_f;
  int ns = base > 0 ? 152 / base : 1;        // never a second, partial wave
  const int maxns = (t.np + PT - 1) / PT;
  if (ns > maxns) ns = maxns;
  if (ns < 1) ns = 1;
  g.jper = ((t.np + ns - 1) / ns + PT - 1) / PT * PT;
  g.nsplit = (t.np + g.jper - 1) / g.jper;
  g.mtiles = (t.np + TM - 1) / TM;
  // row slices of the backward K: about one wave of CTAs
  const int bb = g.mtiles * g.ntile_b;
  int kss = bb > 0 ? 152 / bb : 1;
  const int maxk = (R + PT - 1) / PT;
  if (kss > maxk) kss = maxk;
  if (kss < 1) kss = 1;
  g.rper = ((R + kss - 1) / kss + PT - 1) / PT * PT;
  g.ksplit = R > 0 ? (R + g.rper - 1) / g.rper : 1;
  g.pZF = (size_t) g.NZ * g.KF;
  g.pWB = (size_t) g.NZ * g.KB;
  return g;
}

bool
kgemm_fits (const KGemm &g)
{
  return g.R > 0 && g.t.np > 0 && g.c <= 11 && g.gf >= 1 && g.nf <= TN && g.nf >= 16;
}

size_t
kgemm_sf_floats (const KGemm &g)
{
  return (size_t) g.nsplit * g.n1 * g.c * 2 * (size_t) g.Rp;
}
size_t kgemm_zf_floats (const KGemm &g) { return 2 * g.pZF; }
size_t kgemm_wb_floats (const KGemm &g) { return 2 * g.pWB; }
int kgemm_ypart_chunks (const KGemm &g) { return g.ksplit * g.ntile_b; }
size_t kgemm_ypart_floats (const KGemm &g) { return (size_t) kgemm_ypart_chunks (g) * g.t.np * g.c; }

int
kgemm_maps (const KGemm &g, float *sf, KMaps *m)
{
  int e = encode_planes_sw128 (&m->zf, g.ZF, 2, (unsigned long long) g.NZ, g.KF, g.nf);
  if (!e) e = encode_planes_sw128 (&m->wb, g.WB, 2, (unsigned long long) g.NZ, g.KB, g.nb);
  if (!e)
    e = encode_rows_plain (&m->sf, sf, (unsigned long long) g.nsplit * g.n1 * g.c * 2, g.Rp, TM,
                           2 * g.c);
  return e;
}

// the shared-memory opt-in is a per-device function attribute; set once
// per device
template <int V>
static cudaError_t
gemm_attrs ()
{
  static int attr_dev = -1;
  int dev = 0;
  cudaError_t e = cudaGetDevice (&dev);
  if (e != cudaSuccess) return e;
  if (attr_dev != dev)
    {
      if ((e = cudaFuncSetAttribute (k_sfac_gemm<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int) SMEM_DYN)) != cudaSuccess)
        return e;
      if ((e = cudaFuncSetAttribute (k_bp_gemm<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int) SMEM_DYN)) != cudaSuccess)
        return e;
      attr_dev = dev;
    }
  return cudaSuccess;
}

template <int V>
static cudaError_t
forward_v (const KGemm &g, const KMaps &mp, const MixK *kt, int nk, int *status, cudaStream_t st,
           Ctx *prof)
{
  cudaError_t e = gemm_attrs<V> ();
  if (e != cudaSuccess) return e;
  k_sfac_gemm<V><<<dim3 (g.nrt, g.ntile_f, g.nsplit), NT, SMEM_DYN, st>>> (mp.zf, mp.sf, g, status);
  kmark (prof, st, "k_sfac_gemm");
  k_kop<V><<<(nk + KOP_K - 1) / KOP_K, KOP_K * KOP_G, 0, st>>> (g, kt, nk, g.sf);
  kmark (prof, st, "k_kop");
  return cudaGetLastError ();
}

template <int V>
static cudaError_t
backward_v (const KGemm &g, const KMaps &mp, float *ypart, int *status, cudaStream_t st,
            Ctx *prof)
{
  cudaError_t e = gemm_attrs<V> ();
  if (e != cudaSuccess) return e;
  k_bp_gemm<V><<<dim3 (g.mtiles, g.ntile_b, g.ksplit), NT, SMEM_DYN, st>>> (mp.wb, g, ypart,
                                                                            status);
  kmark (prof, st, "k_bp_gemm");
  return cudaGetLastError ();
}

cudaError_t
launch_kspace_forward (int version, const KGemm &g, const KMaps &maps, const MixK *kt, int nk,
                       int *status, cudaStream_t st, Ctx *prof)
{
  if (version == 0) return forward_v<0> (g, maps, kt, nk, status, st, prof);
  if (version == 1) return forward_v<1> (g, maps, kt, nk, status, st, prof);
  return forward_v<2> (g, maps, kt, nk, status, st, prof);
}

cudaError_t
launch_kspace_backward (int version, const KGemm &g, const KMaps &maps, float *ypart, int *status,
                        cudaStream_t st, Ctx *prof)
{
  if (version == 0) return backward_v<0> (g, maps, ypart, status, st, prof);
  if (version == 1) return backward_v<1> (g, maps, ypart, status, st, prof);
  return backward_v<2> (g, maps, ypart, status, st, prof);
}

}  // namespace lsg
