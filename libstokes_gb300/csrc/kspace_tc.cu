// kspace_tc.cu -- reciprocal space of the mixed product as tensor-core GEMMs.
//
// With per-axis phase tables t_d[m](j) = e^{2 pi i m u_d(j)}, the phase of a
// k vector factorises, e^{ik.r_j} = t0[m1](j) T_r(j) with T_r = t1[m2] t2[m3]
// for the row r = (m2, m3).  So the structure factors of every k vector of the
// list come out of ONE complex GEMM over the particles,
//
//   forward   S[r, (m1, q)] = sum_j T_r(j) Z_(m1,q)(j),  Z = t0[m1] x_q
//             real rows (r, re|im), K = (j, u|v) with a, b = Re, Im T and
//             u, v = Re, Im Z:  A[(r,re),(j,u|v)] = (a, -b), A[(r,im),.] = (b, a)
//   operator  W_k = P_k + i Q_k from S(k) for every k of the half-space list
//   backward  H[i, (m1, re|im, q)] = sum_(r, u|v) conj(T_r)(i) W[r, (m1, q)]
//             A'[i,(r,u|v)] = (a, b), B' columns Re H <- (Re W, Im W),
//             Im H <- (Im W, -Re W);  y_i[q] += Re(conj(t0[m1])(i) H) summed
//             over m1 in the epilogue.
//
// The rows r are the (m2, m3) combinations that occur in the k list; T_r(j)
// is tabulated once per product (k_tprep) for both GEMMs.  Both are tcgen05
// kind::tf32 MMAs (M = 128, N <= 128, K = 8 per instruction) in 3xTF32:
// x = hi + lo, products hi*hi + hi*lo + lo*hi.  The tensor core's FP32
// accumulation truncates at the accumulator's magnitude, so the chains are
// kept short: every 32-wide K tile starts fresh accumulators (hi*hi in one,
// the two corrections in another) that are drained into FP32 registers
// (round to nearest).
//
// Warp roles (512 threads, one CTA per SM):
//   warps 0-7   drain: double-buffered TMEM accumulators (2 x (main +
//               correction) x 128 columns = 512 columns); warp w reads TMEM
//               lanes 32 (w % 4) and columns 64 (w / 4) of each buffer
//   warps 8-14  builders: fill a 3-stage ring of shared-memory operand tiles
//               (K-major, no swizzle, hi and lo), whole 8-row core matrices
//               per warp with 8-byte stores
//   warp 15     one lane issues the MMAs of a tile when its stage is full
//               and its accumulator buffer has been drained
// The roles meet only at mbarriers; every wait is bounded and watches a CTA
// error flag, so a wait that runs out ends every role, raises *status, and
// the MMA lane waits for its MMAs in flight before the TMEM is freed.
#include <cuda_runtime.h>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "tc_umma.cuh"

namespace lsg {
namespace {

constexpr int NT = 512;                 // threads per CTA (16 warps)
constexpr int NDRAIN = 8;               // drain warps 0..7
constexpr int BW0 = 8, NBW = 7;         // builder warps 8..14
constexpr int MMA_WARP = 15;
constexpr int TM = 128;                 // MMA M
constexpr int TN = 128;                 // largest MMA N (columns per tile)
constexpr int KT = 32;                  // K per shared-memory tile
constexpr int STAGES = 3;
constexpr int CPT = TN / 2;             // accumulator columns per drain thread (64)
constexpr int PT = 16;                  // particles (forward) or rows (backward) per K tile
constexpr uint32_t A_BYTES = TM * KT * 4;
constexpr uint32_t B_BYTES = TN * KT * 4;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // 64 KB: hi + lo of A and B
constexpr uint32_t SMEM_DYN = STAGES * STAGE_BYTES;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t WAIT_LIMIT = 1u << 18;   // polls of up to ~20 us each
constexpr int UF = (32 + 64 + NBW - 1) / NBW;    // forward units per builder warp per tile
constexpr int UB = (64 + 64 + NBW - 1) / NBW;    // backward units per builder warp per tile

__device__ __forceinline__ float2
cmulf (float2 a, float2 b)
{
  return make_float2 (a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// the two K-adjacent values (v0, v1) at an even k, split into hi and lo
__device__ __forceinline__ void
put2 (unsigned char *hi, unsigned char *lo, uint32_t o, float v0, float v1)
{
  uint32_t h0, l0, h1, l1;
  umma::split_tf32 (v0, h0, l0);
  umma::split_tf32 (v1, h1, l1);
  *reinterpret_cast<uint2 *> (hi + o) = make_uint2 (h0, h1);
  *reinterpret_cast<uint2 *> (lo + o) = make_uint2 (l0, l1);
}

// a warp fills one 8-row group x one K step (8 values) of a 128-row tile:
// lane -> row 8 g + (lane & 7), K pair lane >> 3 (k = 8 step + 2 (lane >> 3))
__device__ __forceinline__ uint32_t
pair_off (int g, int step, int lane)
{
  return umma::off ((uint32_t) (8 * g + (lane & 7)), (uint32_t) (8 * step + 2 * (lane >> 3)),
                    (uint32_t) TM);
}

// phase-table value t_d[m](j) for any sign of m (rows m = 0..M_d stored)
__device__ __forceinline__ float2
tval (const float2 *row0, int m, size_t stride, size_t j)
{
  const float2 v = row0[(size_t) (m < 0 ? -m : m) * stride + j];
  return m < 0 ? make_float2 (v.x, -v.y) : v;
}

struct Sync {
  uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], done;
  uint32_t tslot;
  int err;
};

__device__ __forceinline__ void
cta_setup (Sync &s)
{
  const int warp = threadIdx.x >> 5;
  if (warp == 0) umma::tmem_alloc (&s.tslot, TMEM_COLS);
  if (threadIdx.x == 32)
    {
      for (int k = 0; k < STAGES; k++)
        {
          umma::mbar_init (&s.full[k], NBW * 32);
          umma::mbar_init (&s.empty[k], 1);
        }
      for (int b = 0; b < 2; b++)
        {
          umma::mbar_init (&s.acc_full[b], 1);
          umma::mbar_init (&s.acc_empty[b], NDRAIN * 32);
        }
      umma::mbar_init (&s.done, 1);
      s.err = 0;
      umma::fence_mbar_init ();
    }
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
}

// the MMA lane: tile t in stage t % STAGES, accumulator buffer t & 1
__device__ __forceinline__ void
mma_role (Sync &s, const unsigned char *smem, uint32_t tmem, uint32_t idesc, int ntiles)
{
  volatile int *err = &s.err;
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
      const uint32_t dm = tmem + (uint32_t) (b * 2 * TN), dc = dm + TN;
#pragma unroll
      for (int k = 0; k < KT / 8; k++)
        {
          const uint64_t dah = umma::smem_desc (ahi + k * TM * 32, 128, 256);
          const uint64_t dal = umma::smem_desc (alo + k * TM * 32, 128, 256);
          const uint64_t dbh = umma::smem_desc (bhi + k * TN * 32, 128, 256);
          const uint64_t dbl = umma::smem_desc (blo + k * TN * 32, 128, 256);
          umma::mma_tf32 (dm, dah, dbh, idesc, k ? 1u : 0u);
          umma::mma_tf32 (dc, dah, dbl, idesc, k ? 1u : 0u);
          umma::mma_tf32 (dc, dal, dbh, idesc, 1u);
        }
      umma::mma_commit (&s.empty[st]);
      umma::mma_commit (&s.acc_full[b]);
    }
  // every MMA issued so far has completed once `done` flips
  umma::mma_commit (&s.done);
  volatile int never = 0;
  umma::mbar_wait_or_abort (&s.done, 0, WAIT_LIMIT, &never);
}

// drain warps: acc += both accumulators of each tile
__device__ __forceinline__ bool
drain_role (Sync &s, uint32_t tmem, int ntiles, float acc[CPT])
{
  const int warp = threadIdx.x >> 5;
  volatile int *err = &s.err;
  const uint32_t lane_base = (uint32_t) ((warp & 3) * 32) << 16;
  const uint32_t col = (uint32_t) ((warp >> 2) * CPT);
  for (int t = 0; t < ntiles; t++)
    {
      const int b = t & 1;
      if (!umma::mbar_wait_or_abort (&s.acc_full[b], (t >> 1) & 1, WAIT_LIMIT, err)) return false;
      umma::fence_after_sync ();
      const uint32_t dm = tmem + lane_base + (uint32_t) (b * 2 * TN) + col;
#pragma unroll
      for (int cc = 0; cc < CPT; cc += 16)
        {
          float m[16], c[16];
          umma::tmem_ld16 (dm + cc, m);
          umma::tmem_ld16 (dm + TN + cc, c);
#pragma unroll
          for (int u = 0; u < 16; u++) acc[cc + u] += m[u] + c[u];
        }
      umma::fence_before_sync ();
      umma::mbar_arrive (&s.acc_empty[b]);
    }
  return true;
}

// builders: a ring of tiles; the loads of tile t + 1 are issued right after
// tile t is stored, before waiting for tile t + 1's stage to come free
template <typename Load, typename Store>
__device__ __forceinline__ void
build_role (Sync &s, unsigned char *smem, int ntiles, Load load, Store store)
{
  volatile int *err = &s.err;
  if (ntiles > 0) load (0);
  for (int t = 0; t < ntiles; t++)
    {
      const int st = t % STAGES;
      if (t >= STAGES
          && !umma::mbar_wait_or_abort (&s.empty[st], ((t / STAGES) - 1) & 1, WAIT_LIMIT, err))
        return;
      unsigned char *sb = smem + (size_t) st * STAGE_BYTES;
      store (t, sb, sb + A_BYTES, sb + 2 * A_BYTES, sb + 2 * A_BYTES + B_BYTES);
      umma::fence_async_smem ();
      umma::mbar_arrive (&s.full[st]);
      if (t + 1 < ntiles) load (t + 1);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// T_r(j) = t1[m2](j) t2[m3](j) for every row r and particle j
// ---------------------------------------------------------------------------
__global__ void
k_tprep (KGemm g)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (j >= g.ldT) return;
  float2 v = make_float2 (0.f, 0.f);
  if (j < g.t.np)
    {
      const int2 mm = g.rowm[r];
      v = cmulf (tval (g.t.tab + g.t.off1, mm.x, g.t.np, j), tval (g.t.tab + g.t.off2, mm.y, g.t.np, j));
    }
  g.T[(size_t) r * g.ldT + j] = v;
}

// ---------------------------------------------------------------------------
// forward: partial structure factors of one (row tile, m1 tile, particle slice)
// ---------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__ (NT, 1)
k_sfac_gemm (KGemm g, const float *xf, float *sf, int *status)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ __align__ (1024) unsigned char smem[];
  __shared__ Sync s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int np = g.t.np;
  const int r0 = blockIdx.x * 64;
  const int m1b = blockIdx.y * g.gf, nm1 = min (g.gf, g.n1 - m1b);
  const int split = blockIdx.z;
  const int jb = split * g.jper, je = min (np, jb + g.jper);
  const int ntiles = (je > jb) ? (je - jb + PT - 1) / PT : 0;
  const int ncol = nm1 * C;
  const float2 *t0 = g.t.tab;

  cta_setup (s);
  const uint32_t tmem = s.tslot;

  if (warp >= BW0 && warp < BW0 + NBW)
    {
      const int bw = warp - BW0;
      const int ngb = (ncol + 7) >> 3;           // B row groups in use
      // unit u < 32: A, 8 groups of complex rows x 4 K steps, (a, -b) to row
      // rl and (b, a) to row 64 + rl; unit u >= 32: B, rows n = (m1, q),
      // pair (u, v) = Z = t0[m1] x_q.  Per unit, fixed over the tiles: the
      // shared-memory offset with the unit's particle offset jj in bits
      // 20-23 (sof), the element offsets of its inputs for tile 0 (e0, e1;
      // -1: no input).  va/vx: the tile's loaded inputs.
      uint32_t sof[UF];
      int e0[UF], e1[UF];
#pragma unroll
      for (int k = 0; k < UF; k++)
        {
          const int u = bw + k * NBW;
          e0[k] = e1[k] = -1;
          sof[k] = 0;
          if (u < 32)
            {
              const int gg = u >> 2, step = u & 3, rl = 8 * gg + (lane & 7);
              const int jj = 4 * step + (lane >> 3);
              sof[k] = pair_off (gg, step, lane) | ((uint32_t) jj << 20);
              if (r0 + rl < g.R) e0[k] = (r0 + rl) * g.ldT + jb + jj;
            }
          else if (u - 32 < ngb * 4)
            {
              const int v = u - 32, gg = v >> 2, step = v & 3, n = 8 * gg + (lane & 7);
              const int jj = 4 * step + (lane >> 3);
              sof[k] = pair_off (gg, step, lane) | ((uint32_t) jj << 20);
              if (n < ncol)
                {
                  const int m = n / C, q = n - m * C;
                  e0[k] = (m1b + m) * np + jb + jj;
                  e1[k] = (jb + jj) * C + q;
                }
            }
        }
      float2 va[UF];
      float vx[UF];
      auto load = [&] (int t) {
        const int lim = je - jb - PT * t;          // particles left in the slice
#pragma unroll
        for (int k = 0; k < UF; k++)
          {
            const int u = bw + k * NBW;
            const bool in = e0[k] >= 0 && (int) (sof[k] >> 20) < lim;
            va[k] = make_float2 (0.f, 0.f);
            vx[k] = 0.f;
            if (u < 32)
              {
                if (in) va[k] = g.T[e0[k] + PT * t];
              }
            else if (in)
              {
                va[k] = t0[e0[k] + PT * t];
                vx[k] = xf[e1[k] + PT * C * t];
              }
          }
      };
      auto store = [&] (int, unsigned char *Ahi, unsigned char *Alo, unsigned char *Bhi,
                        unsigned char *Blo) {
#pragma unroll
        for (int k = 0; k < UF; k++)
          {
            const int u = bw + k * NBW;
            const uint32_t o = sof[k] & 0xFFFFFu;
            if (u < 32)
              {
                put2 (Ahi, Alo, o, va[k].x, -va[k].y);
                put2 (Ahi, Alo, o + 2048u, va[k].y, va[k].x);   // row + 64
              }
            else if (u - 32 < ngb * 4)
              put2 (Bhi, Blo, o, va[k].x * vx[k], va[k].y * vx[k]);
          }
      };
      build_role (s, smem, ntiles, load, store);
    }
  else if (warp == MMA_WARP)
    {
      if (lane == 0) mma_role (s, smem, tmem, umma::idesc_tf32 (TM, g.nf), ntiles);
      __syncwarp ();
    }
  else
    {
      float acc[CPT];
#pragma unroll
      for (int u = 0; u < CPT; u++) acc[u] = 0.f;
      if (drain_role (s, tmem, ntiles, acc) && !s.err)
    {
      // this thread: TMEM lane = D row, 64 columns from (warp >> 2) * 64;
      // sf[split][m1][q][re|im][row], rows padded to nrt * 64
      const int row = (warp & 3) * 32 + lane;
      const int rl = row & 63, part = row >> 6;
      const int cb = (warp >> 2) * CPT;
      const size_t Rp = (size_t) g.nrt * 64;
#pragma unroll
      for (int u = 0; u < CPT; u++)
        {
          const int n = cb + u;
          if (n >= ncol) break;
          const int m = n / C, q = n - m * C;
          sf[((((size_t) split * g.n1 + m1b + m) * C + q) * 2 + part) * Rp + r0 + rl] = acc[u];
        }
    }
    }
  __syncthreads ();
  if (tid == 0 && s.err) atomicExch (status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// per-k operators: W[r][m1][q] += P_k + i Q_k from the summed structure factors
// ---------------------------------------------------------------------------
template <int V>
__global__ void
k_kop (KGemm g, const MixK *kt, int nk, const float *sf, float2 *W)
{
  constexpr int C = NComp<V>::value;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const MixK K = kt[k];
  const size_t Rp = (size_t) g.nrt * 64;
  float cs[C], sn[C], ns[C];
#pragma unroll
  for (int q = 0; q < C; q++) cs[q] = sn[q] = 0.f;
  // one slice at a time, its 2C loads issued together
  for (int s = 0; s < g.nsplit; s++)
    {
      const float *base = sf + (((size_t) s * g.n1 + K.m1) * C * 2) * Rp + K.r;
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          cs[q] += base[(size_t) (2 * q) * Rp];
          sn[q] += base[(size_t) (2 * q + 1) * Rp];
        }
    }
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
  float2 *w = W + ((size_t) K.r * g.n1 + K.m1) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      atomicAdd (&w[q].x, P.v[q]);
      atomicAdd (&w[q].y, Q.v[q]);
    }
}

// ---------------------------------------------------------------------------
// back-projection: y_i partial over one (m1 tile, row slice)
// ---------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__ (NT, 1)
k_bp_gemm (KGemm g, const float2 *W, float *ypart, int *status)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ __align__ (1024) unsigned char smem[];
  __shared__ Sync s;
  __shared__ float s_y[TM][C];
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
  for (int e = tid; e < TM * C; e += NT) s_y[e / C][e % C] = 0.f;
  __syncthreads ();

  if (warp >= BW0 && warp < BW0 + NBW)
    {
      const int bw = warp - BW0;
      const int ngb = (ncol + 7) >> 3;
      // unit u < 64: A', rows = particles, K pair = (a, b) of T_r(i); unit
      // u >= 64: B', rows n = (m1, re|im, q), K pair from W[r][m1][q].  Per
      // unit, fixed over the tiles: the shared-memory offset with the unit's
      // row offset rr in bits 20-23 and the im flag in bit 24 (sof), the
      // element offset of its input for tile 0 (e0; -1: no input).
      uint32_t sof[UB];
      int e0[UB];
#pragma unroll
      for (int k = 0; k < UB; k++)
        {
          const int u = bw + k * NBW;
          e0[k] = -1;
          sof[k] = 0;
          if (u < 64)
            {
              const int gg = u >> 2, step = u & 3, i = i0 + 8 * gg + (lane & 7);
              const int rr = 4 * step + (lane >> 3);
              sof[k] = pair_off (gg, step, lane) | ((uint32_t) rr << 20);
              if (i < np) e0[k] = (rb + rr) * g.ldT + i;
            }
          else if (u - 64 < ngb * 4)
            {
              const int v = u - 64, gg = v >> 2, step = v & 3, n = 8 * gg + (lane & 7);
              const int rr = 4 * step + (lane >> 3);
              const int m = n / (2 * C), rem = n - m * 2 * C, im = rem >= C, q = rem - im * C;
              sof[k] = pair_off (gg, step, lane) | ((uint32_t) rr << 20) | ((uint32_t) im << 24);
              if (n < ncol) e0[k] = ((rb + rr) * g.n1 + m1b + m) * C + q;
            }
        }
      float2 va[UB];
      auto load = [&] (int t) {
        const int lim = re_ - rb - PT * t;          // rows left in the slice
#pragma unroll
        for (int k = 0; k < UB; k++)
          {
            const int u = bw + k * NBW;
            const bool in = e0[k] >= 0 && (int) ((sof[k] >> 20) & 15u) < lim;
            va[k] = make_float2 (0.f, 0.f);
            if (u < 64)
              {
                if (in) va[k] = g.T[e0[k] + PT * g.ldT * t];
              }
            else if (in)
              va[k] = W[e0[k] + PT * g.n1 * C * t];
          }
      };
      auto store = [&] (int, unsigned char *Ahi, unsigned char *Alo, unsigned char *Bhi,
                        unsigned char *Blo) {
#pragma unroll
        for (int k = 0; k < UB; k++)
          {
            const int u = bw + k * NBW;
            const uint32_t o = sof[k] & 0xFFFFFu;
            if (u < 64)
              put2 (Ahi, Alo, o, va[k].x, va[k].y);
            else if (u - 64 < ngb * 4)
              {
                const bool im = (sof[k] >> 24) & 1u;
                put2 (Bhi, Blo, o, im ? va[k].y : va[k].x, im ? -va[k].x : va[k].y);
              }
          }
      };
      build_role (s, smem, ntiles, load, store);
    }
  else if (warp == MMA_WARP)
    {
      if (lane == 0) mma_role (s, smem, tmem, umma::idesc_tf32 (TM, g.nb), ntiles);
      __syncwarp ();
    }
  else
    {
      float acc[CPT];
#pragma unroll
      for (int u = 0; u < CPT; u++) acc[u] = 0.f;
      if (drain_role (s, tmem, ntiles, acc) && !s.err)
    {
      const int row = (warp & 3) * 32 + lane;
      const int i = i0 + row;
      if (i < np)
        {
          // y_i[q] += Re(conj(t0[m1])(i) H) over this thread's columns
          float yq[C];
#pragma unroll
          for (int q = 0; q < C; q++) yq[q] = 0.f;
          const int cb = (warp >> 2) * CPT;
          int cur = -1;
          float2 ph = make_float2 (0.f, 0.f);
#pragma unroll
          for (int u = 0; u < CPT; u++)
            {
              const int n = cb + u;
              if (n >= ncol) break;
              const int m = n / (2 * C), rem = n - m * 2 * C, im = rem >= C, q = rem - im * C;
              if (m != cur)
                {
                  ph = t0[(size_t) (m1b + m) * np + i];
                  cur = m;
                }
              const float c = (im ? ph.y : ph.x) * acc[u];
#pragma unroll
              for (int qq = 0; qq < C; qq++)
                if (qq == q) yq[qq] += c;
            }
#pragma unroll
          for (int q = 0; q < C; q++) atomicAdd (&s_y[row][q], yq[q]);
        }
    }
    }
  __syncthreads ();
  if (tid == 0 && s.err) atomicExch (status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  const size_t chunk = (size_t) ks * gridDim.y + blockIdx.y;
  for (int e = tid; e < TM * C; e += NT)
    {
      const int r = e / C, q = e % C;
      if (i0 + r < np) ypart[(chunk * np + i0 + r) * C + q] = s_y[r][q];
    }
  if (warp == 0) umma::tmem_dealloc (tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int round16 (int n) { return (n + 15) / 16 * 16; }

KGemm
kgemm_plan (int version, PhaseTables t, const int2 *rowm, int R)
{
  KGemm g{};
  g.t = t;
  g.rowm = rowm;
  g.R = R;
  g.c = NCOMP (version);
  g.n1 = t.M0 + 1;
  g.nrt = (R + 63) / 64;
  g.ldT = round16 (t.np);
  // forward columns (m1, q), at most TN per tile, balanced over the tiles
  g.ntile_f = (g.n1 * g.c + TN - 1) / TN;
  g.gf = (g.n1 + g.ntile_f - 1) / g.ntile_f;
  while (g.gf * g.c > TN) g.gf--;
  g.ntile_f = (g.n1 + g.gf - 1) / g.gf;
  g.nf = round16 (g.gf * g.c);
  // particle slices: about one wave of CTAs
  const int base = g.nrt * g.ntile_f;
  int ns = 152 / base;            // never a second, partial wave
  const int maxns = (t.np + PT - 1) / PT;
  if (ns > maxns) ns = maxns;
  if (ns < 1) ns = 1;
  g.jper = ((t.np + ns - 1) / ns + PT - 1) / PT * PT;
  g.nsplit = (t.np + g.jper - 1) / g.jper;
  // backward columns (m1, re|im, q), at most TN per tile
  g.ntile_b = (g.n1 * 2 * g.c + TN - 1) / TN;
  g.gb = (g.n1 + g.ntile_b - 1) / g.ntile_b;
  while (g.gb * 2 * g.c > TN) g.gb--;
  g.ntile_b = (g.n1 + g.gb - 1) / g.gb;
  g.nb = round16 (g.gb * 2 * g.c);
  g.mtiles = (t.np + TM - 1) / TM;
  // row slices of the backward K: about one wave of CTAs
  const int bb = g.mtiles * g.ntile_b;
  int kss = 152 / bb;
  const int maxk = (R + PT - 1) / PT;
  if (kss > maxk) kss = maxk;
  if (kss < 1) kss = 1;
  g.rper = ((R + kss - 1) / kss + PT - 1) / PT * PT;
  g.ksplit = R > 0 ? (R + g.rper - 1) / g.rper : 1;
  return g;
}

bool
kgemm_fits (const KGemm &g)
{
  return g.R > 0 && g.t.np > 0 && g.c <= 11 && g.gf >= 1 && g.gb >= 1 && g.nf <= TN
         && g.nb <= TN;
}

size_t
kgemm_sf_floats (const KGemm &g)
{
  return (size_t) g.nsplit * g.n1 * g.c * 2 * ((size_t) g.nrt * 64);
}
size_t kgemm_w_elems (const KGemm &g) { return (size_t) g.R * g.n1 * g.c; }
size_t kgemm_t_elems (const KGemm &g) { return (size_t) g.R * g.ldT; }
int kgemm_ypart_chunks (const KGemm &g) { return g.ksplit * g.ntile_b; }
size_t kgemm_ypart_floats (const KGemm &g) { return (size_t) kgemm_ypart_chunks (g) * g.t.np * g.c; }

template <int V>
static cudaError_t
launch_v (const KGemm &g, const MixK *kt, int nk, const float *xf, float *sf, float2 *W,
          float *ypart, int *status, cudaStream_t st, Ctx *prof)
{
  cudaError_t e;
  if ((e = cudaFuncSetAttribute (k_sfac_gemm<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) SMEM_DYN)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute (k_bp_gemm<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) SMEM_DYN)) != cudaSuccess)
    return e;
  k_tprep<<<dim3 ((g.ldT + 127) / 128, g.R), 128, 0, st>>> (g);
  kmark (prof, st, "k_tprep");
  k_sfac_gemm<V><<<dim3 (g.nrt, g.ntile_f, g.nsplit), NT, SMEM_DYN, st>>> (g, xf, sf, status);
  kmark (prof, st, "k_sfac_gemm");
  if ((e = cudaMemsetAsync (W, 0, sizeof (float2) * kgemm_w_elems (g), st)) != cudaSuccess)
    return e;
  k_kop<V><<<(nk + 127) / 128, 128, 0, st>>> (g, kt, nk, sf, W);
  kmark (prof, st, "k_kop");
  k_bp_gemm<V><<<dim3 (g.mtiles, g.ntile_b, g.ksplit), NT, SMEM_DYN, st>>> (g, W, ypart, status);
  kmark (prof, st, "k_bp_gemm");
  return cudaGetLastError ();
}

cudaError_t
launch_kspace_gemm (int version, const KGemm &g, const MixK *kt, int nk, const float *xf,
                    float *sf, float2 *W, float *ypart, int *status, cudaStream_t st, Ctx *prof)
{
  if (version == 0) return launch_v<0> (g, kt, nk, xf, sf, W, ypart, status, st, prof);
  if (version == 1) return launch_v<1> (g, kt, nk, xf, sf, W, ypart, status, st, prof);
  return launch_v<2> (g, kt, nk, xf, sf, W, ypart, status, st, prof);
}

}  // namespace lsg
