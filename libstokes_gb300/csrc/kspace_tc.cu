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
// The rows r are the (m2, m3) combinations that occur in the k list, so the
// only padding is along m1.  Both GEMMs are tcgen05 kind::tf32 MMAs (M = 128,
// N <= 256, K = 8 per instruction) in 3xTF32: x = hi + lo, products hi*hi +
// hi*lo + lo*hi.  The tensor core's FP32 accumulation truncates at the
// accumulator's magnitude, so accumulation chains are kept short: hi*hi goes
// to one TMEM accumulator and the two correction products to a second one
// (columns 256..511), each restarted every K tile of 32; after each tile the
// 16 warps drain both into FP32 registers (round to nearest) while the next
// tile is being built.  Operands are built in shared memory (K-major, no
// swizzle; each warp writes whole 8-row core matrices, 8 bytes per lane) in
// two stages; every wait is bounded (a wait that runs out raises *status and
// the CTA frees its TMEM).
#include <cuda_runtime.h>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "tc_umma.cuh"

namespace lsg {
namespace {

constexpr int NT = 512;                 // threads per CTA (16 warps)
constexpr int TM = 128;                 // MMA M
constexpr int TN = 256;                 // MMA N
constexpr int KT = 32;                  // K per shared-memory tile
constexpr int CPT = TN / 4;             // accumulator columns per thread (64)
constexpr uint32_t A_BYTES = TM * KT * 4;
constexpr uint32_t B_BYTES = TN * KT * 4;
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // hi + lo of A and B
constexpr uint32_t SMEM_DYN = 2 * STAGE_BYTES;
constexpr uint32_t TMEM_COLS = 512;     // main accumulator + correction accumulator
constexpr uint32_t WAIT_LIMIT = 1u << 26;
constexpr int PT = 16;                  // particles (forward) or rows (backward) per K tile
constexpr int GF_MAX = TN / 3;          // m1 values per forward column tile (F version)

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

// a warp fills one 8-row group x one K step (8 values) of a tile: lane ->
// row 8 g + (lane & 7), K pair kp = lane >> 3 (k = 8 step + 2 kp); the byte
// offset of that pair in a tile of `rows` rows
__device__ __forceinline__ uint32_t
pair_off (int g, int step, int lane, int rows)
{
  return umma::off ((uint32_t) (8 * g + (lane & 7)), (uint32_t) (8 * step + 2 * (lane >> 3)),
                    (uint32_t) rows);
}

// phase-table value t_d[m](j) for any sign of m (rows m = 0..M_d stored)
__device__ __forceinline__ float2
tval (const float2 *row0, int m, size_t stride, size_t j)
{
  const float2 v = row0[(size_t) (m < 0 ? -m : m) * stride + j];
  return m < 0 ? make_float2 (v.x, -v.y) : v;
}

// the MMAs of one K tile: hi*hi into the main accumulator, hi*lo + lo*hi into
// the correction accumulator, both restarted at the tile's first K step
__device__ __forceinline__ void
issue_stage (const unsigned char *smem, int s, uint32_t tmem, uint32_t idesc)
{
  const uint32_t base = umma::smem_u32 (smem) + (uint32_t) s * STAGE_BYTES;
  const uint32_t ahi = base, alo = base + A_BYTES;
  const uint32_t bhi = base + 2 * A_BYTES, blo = bhi + B_BYTES;
#pragma unroll
  for (int st = 0; st < KT / 8; st++)
    {
      const uint64_t dah = umma::smem_desc (ahi + st * TM * 32, 128, 256);
      const uint64_t dal = umma::smem_desc (alo + st * TM * 32, 128, 256);
      const uint64_t dbh = umma::smem_desc (bhi + st * TN * 32, 128, 256);
      const uint64_t dbl = umma::smem_desc (blo + st * TN * 32, 128, 256);
      umma::mma_tf32 (tmem, dah, dbh, idesc, st ? 1u : 0u);
      umma::mma_tf32 (tmem + TN, dah, dbl, idesc, st ? 1u : 0u);
      umma::mma_tf32 (tmem + TN, dal, dbh, idesc, 1u);
    }
}

// add this thread's 64 columns of both accumulators into acc (FP32, RN)
__device__ __forceinline__ void
drain (uint32_t tmem, int warp, float acc[CPT])
{
  const uint32_t lane_base = (uint32_t) ((warp & 3) * 32) << 16;
  const uint32_t col = (uint32_t) ((warp >> 2) * CPT);
#pragma unroll
  for (int cc = 0; cc < CPT; cc += 16)
    {
      float m[16], c[16];
      umma::tmem_ld16 (tmem + lane_base + col + cc, m);
      umma::tmem_ld16 (tmem + lane_base + TN + col + cc, c);
#pragma unroll
      for (int u = 0; u < 16; u++) acc[cc + u] += m[u] + c[u];
    }
}

// K-tile pipeline shared by both GEMMs: build tile t into stage t & 1 while
// the MMAs of tile t - 1 run, then drain tile t - 1 and issue tile t.
// Returns false when a wait ran out (acc then holds a partial sum).
template <typename Build>
__device__ __forceinline__ bool
run_pipeline (unsigned char *smem, uint64_t *mbar, uint32_t tmem, uint32_t idesc, int ntiles,
              Build build, float acc[CPT])
{
  const int tid = threadIdx.x, warp = tid >> 5;
  bool ok = true;
  for (int t = 0; t < ntiles && ok; t++)
    {
      const int s = t & 1;
      unsigned char *st = smem + (size_t) s * STAGE_BYTES;
      build (t, st, st + A_BYTES, st + 2 * A_BYTES, st + 2 * A_BYTES + B_BYTES);
      umma::fence_async_smem ();
      if (t > 0)
        {
          const int p = t - 1;
          ok = __syncthreads_and (umma::mbar_wait (&mbar[p & 1], (p >> 1) & 1, WAIT_LIMIT)) != 0;
          if (!ok) break;
          umma::fence_after_sync ();
          drain (tmem, warp, acc);
        }
      umma::fence_before_sync ();
      __syncthreads ();
      if (tid == 0)
        {
          umma::fence_after_sync ();
          issue_stage (smem, s, tmem, idesc);
          umma::mma_commit (&mbar[s]);
        }
    }
  if (ok && ntiles > 0)
    {
      const int p = ntiles - 1;
      ok = __syncthreads_and (umma::mbar_wait (&mbar[p & 1], (p >> 1) & 1, WAIT_LIMIT)) != 0;
      if (ok)
        {
          umma::fence_after_sync ();
          drain (tmem, warp, acc);
        }
    }
  umma::fence_before_sync ();
  __syncthreads ();
  return ok;
}

__device__ __forceinline__ void
cta_setup (uint32_t *tslot, uint64_t *mbar)
{
  if ((threadIdx.x >> 5) == 0) umma::tmem_alloc (tslot, TMEM_COLS);
  if (threadIdx.x == 0)
    {
      umma::mbar_init (&mbar[0], 1);
      umma::mbar_init (&mbar[1], 1);
      umma::fence_mbar_init ();
    }
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
}

}  // namespace

// ---------------------------------------------------------------------------
// forward: partial structure factors of one (row tile, m1 tile, particle slice)
// ---------------------------------------------------------------------------
template <int V>
__global__ void __launch_bounds__ (NT, 1)
k_sfac_gemm (KGemm g, const float *xf, float *sf, int *status)
{
  constexpr int C = NComp<V>::value;
  extern __shared__ __align__ (1024) unsigned char smem[];
  __shared__ __align__ (8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ int2 s_rows[64];             // (m2, m3) of the tile's rows
  __shared__ float2 s_t0[GF_MAX][PT];     // t0[m1](j) of the tile's m1 values
  __shared__ float s_x[PT][C];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int np = g.t.np;
  const int r0 = blockIdx.x * 64;
  const int m1b = blockIdx.y * g.gf, nm1 = min (g.gf, g.n1 - m1b);
  const int split = blockIdx.z;
  const int jb = split * g.jper, je = min (np, jb + g.jper);
  const int ntiles = (je > jb) ? (je - jb + PT - 1) / PT : 0;
  const float2 *t0 = g.t.tab, *t1 = g.t.tab + g.t.off1, *t2 = g.t.tab + g.t.off2;
  const int ncol = nm1 * C;

  cta_setup (&tslot, mbar);
  const uint32_t tmem = tslot;
  for (int e = tid; e < 64; e += NT)
    s_rows[e] = (r0 + e < g.R) ? g.rowm[r0 + e] : make_int2 (0, 0);

  auto build = [&] (int t, unsigned char *Ahi, unsigned char *Alo, unsigned char *Bhi,
                    unsigned char *Blo) {
    const int j0 = jb + PT * t;
    for (int e = tid; e < nm1 * PT; e += NT)
      {
        const int jj = e % PT, m = e / PT, j = j0 + jj;
        s_t0[m][jj] = j < je ? t0[(size_t) (m1b + m) * np + j] : make_float2 (0.f, 0.f);
      }
    for (int e = tid; e < PT * C; e += NT)
      {
        const int jj = e / C, q = e % C, j = j0 + jj;
        s_x[jj][q] = (j < je) ? xf[(size_t) j * C + q] : 0.f;
      }
    __syncthreads ();
    // A: 8 row groups of complex rows x 4 K steps; each lane fills the pair
    // (a, -b) of row rl and (b, a) of row 64 + rl
    for (int u = warp; u < 8 * (KT / 8); u += NT / 32)
      {
        const int gg = u >> 2, step = u & 3;
        const int rl = 8 * gg + (lane & 7), jj = 4 * step + (lane >> 3), j = j0 + jj;
        float a = 0.f, b = 0.f;
        if (r0 + rl < g.R && j < je)
          {
            const int2 mm = s_rows[rl];
            const float2 T = cmulf (tval (t1, mm.x, np, j), tval (t2, mm.y, np, j));
            a = T.x;
            b = T.y;
          }
        put2 (Ahi, Alo, pair_off (gg, step, lane, TM), a, -b);
        put2 (Ahi, Alo, pair_off (gg + 8, step, lane, TM), b, a);
      }
    // B: rows n = (m1, q); pair (u, v) = Z = t0[m1] x_q
    const int ng = (ncol + 7) >> 3;
    for (int u = warp; u < ng * (KT / 8); u += NT / 32)
      {
        const int gg = u >> 2, step = u & 3;
        const int n = 8 * gg + (lane & 7), jj = 4 * step + (lane >> 3);
        float zu = 0.f, zv = 0.f;
        if (n < ncol)
          {
            const int m = n / C, q = n - m * C;
            const float2 ph = s_t0[m][jj];
            const float xv = s_x[jj][q];
            zu = ph.x * xv;
            zv = ph.y * xv;
          }
        put2 (Bhi, Blo, pair_off (gg, step, lane, TN), zu, zv);
      }
  };
  float acc[CPT];
#pragma unroll
  for (int u = 0; u < CPT; u++) acc[u] = 0.f;
  const bool ok = run_pipeline (smem, mbar, tmem, umma::idesc_tf32 (TM, g.nf), ntiles, build, acc);

  if (ok)
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
  else if (tid == 0)
    atomicExch (status, 1);
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
  __shared__ __align__ (8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ float s_y[TM][C];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int np = g.t.np;
  const int i0 = blockIdx.x * TM;
  const int m1b = blockIdx.y * g.gb, nm1 = min (g.gb, g.n1 - m1b);
  const int ks = blockIdx.z;
  const int rb = ks * g.rper, re_ = min (g.R, rb + g.rper);
  const int ntiles = (re_ > rb) ? (re_ - rb + PT - 1) / PT : 0;
  const float2 *t0 = g.t.tab, *t1 = g.t.tab + g.t.off1, *t2 = g.t.tab + g.t.off2;
  const int ncol = nm1 * 2 * C;

  cta_setup (&tslot, mbar);
  const uint32_t tmem = tslot;
  for (int e = tid; e < TM * C; e += NT) s_y[e / C][e % C] = 0.f;

  auto build = [&] (int t, unsigned char *Ahi, unsigned char *Alo, unsigned char *Bhi,
                    unsigned char *Blo) {
    const int rt = rb + PT * t;
    // A': rows = particles, K pair = (a, b) of T_r(i)
    for (int u = warp; u < (TM / 8) * (KT / 8); u += NT / 32)
      {
        const int gg = u >> 2, step = u & 3;
        const int i = i0 + 8 * gg + (lane & 7), r = rt + 4 * step + (lane >> 3);
        float a = 0.f, b = 0.f;
        if (i < np && r < re_)
          {
            const int2 mm = g.rowm[r];
            const float2 T = cmulf (tval (t1, mm.x, np, i), tval (t2, mm.y, np, i));
            a = T.x;
            b = T.y;
          }
        put2 (Ahi, Alo, pair_off (gg, step, lane, TM), a, b);
      }
    // B': rows n = (m1, re|im, q); K pair from W[r][m1][q]
    const int ng = (ncol + 7) >> 3;
    for (int u = warp; u < ng * (KT / 8); u += NT / 32)
      {
        const int gg = u >> 2, step = u & 3;
        const int n = 8 * gg + (lane & 7), r = rt + 4 * step + (lane >> 3);
        float v0 = 0.f, v1 = 0.f;
        if (n < ncol && r < re_)
          {
            const int m = n / (2 * C), rem = n - m * 2 * C, im = rem >= C, q = rem - im * C;
            const float2 w = W[((size_t) r * g.n1 + m1b + m) * C + q];
            v0 = im ? w.y : w.x;
            v1 = im ? -w.x : w.y;
          }
        put2 (Bhi, Blo, pair_off (gg, step, lane, TN), v0, v1);
      }
  };
  float acc[CPT];
#pragma unroll
  for (int u = 0; u < CPT; u++) acc[u] = 0.f;
  const bool ok = run_pipeline (smem, mbar, tmem, umma::idesc_tf32 (TM, g.nb), ntiles, build, acc);

  const int row = (warp & 3) * 32 + lane;
  const int i = i0 + row;
  if (ok && i < np)
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
  else if (!ok && tid == 0)
    atomicExch (status, 1);
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
  KGemm g;
  g.t = t;
  g.rowm = rowm;
  g.R = R;
  g.c = NCOMP (version);
  g.n1 = t.M0 + 1;
  g.nrt = (R + 63) / 64;
  // forward columns (m1, q), at most 256 per tile
  g.ntile_f = (g.n1 * g.c + TN - 1) / TN;
  g.gf = (g.n1 + g.ntile_f - 1) / g.ntile_f;
  while (g.gf * g.c > TN) g.gf--;
  g.ntile_f = (g.n1 + g.gf - 1) / g.gf;
  g.nf = round16 (g.gf * g.c);
  // particle slices: about one wave of CTAs
  const int base = g.nrt * g.ntile_f;
  int ns = (152 + base / 2) / base;
  const int maxns = (t.np + PT - 1) / PT;
  if (ns > maxns) ns = maxns;
  if (ns < 1) ns = 1;
  g.jper = ((t.np + ns - 1) / ns + PT - 1) / PT * PT;
  g.nsplit = (t.np + g.jper - 1) / g.jper;
  // backward columns (m1, re|im, q), at most 256 per tile
  g.ntile_b = (g.n1 * 2 * g.c + TN - 1) / TN;
  g.gb = (g.n1 + g.ntile_b - 1) / g.ntile_b;
  while (g.gb * 2 * g.c > TN) g.gb--;
  g.ntile_b = (g.n1 + g.gb - 1) / g.gb;
  g.nb = round16 (g.gb * 2 * g.c);
  g.mtiles = (t.np + TM - 1) / TM;
  // row slices of the backward K: about one wave of CTAs
  const int bb = g.mtiles * g.ntile_b;
  int kss = (152 + bb / 2) / bb;
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
  return g.R > 0 && g.t.np > 0 && g.c <= 11 && g.gf >= 1 && g.gf <= GF_MAX && g.gb >= 1;
}

size_t
kgemm_sf_floats (const KGemm &g)
{
  return (size_t) g.nsplit * g.n1 * g.c * 2 * ((size_t) g.nrt * 64);
}
size_t kgemm_w_elems (const KGemm &g) { return (size_t) g.R * g.n1 * g.c; }
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
