// mixed.cu -- mixed-precision Ewald mobility product (relative L2 error
// <= 1e-6 against the FP64 path).
//
// The sum is re-split so that most of the work moves to where GB300 is fast:
//  * split: xi = eta / V^(1/3) with eta ~ 10 (libstokes uses xi = sqrt(pi)/L),
//    cutoffs from libstokes' own error estimators at tolerance eps_m; the
//    real-space cutoff stays below half the box, so the real-space sum is a
//    minimum-image all-pairs sum;
//  * positions: 32-bit fixed point per axis (L <-> 2^32).  Differences are
//    exact integer subtractions and the periodic wrap is the integer
//    overflow, so pair geometry costs no FP64 and loses no digits;
//  * real space: FP32 pair terms (erfcf/expf), compacted per warp;
//  * reciprocal space: structure factors C(k), S(k) over half of k space with
//    e^{ik.r} built from per-particle FP64-accurate phase tables (stored FP32),
//    FP32 accumulation; back-projection y_i = 2 sum_k cos P + sin Q;
//  * FP64: the self term, the split constants and the final combination.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "ewald_device.cuh"
#include "gpu_engine.h"
#include "mixed.h"
#include "stokes_gpu.h"
#include "tc_umma.cuh"

extern "C" void lsg_ewald_cutoffs (double xi, double eps, double lmin, double lmax,
                                   double *rmax_out, double *kmax_out);

namespace lsg {

static int
cuda_ok (cudaError_t e, const char *what)
{
  return e == cudaSuccess ? STOKES_GPU_OK : cuda_fail (e, what);
}

struct MixedState {
  uint64_t fp = 0;
  double xi = 0, rc = 0, kc = 0, eta = 0, eps = 0;
  int M[3] = {0, 0, 0};
  int nkh = 0;
  int nk_split = 0;      // rows of the re-tuned split; the rest: reference G term
  double selfc[3] = {0, 0, 0};
  std::vector<MixK> h_k;
  DevBuf kt, qpos, tab, xf, pq, part_real, part_rec, selfbuf, status, sf, rowm, rot;
  DevBuf img_zf, img_wb;        // GEMM B-operand images (kspace_tc.cu)
  DevBuf tyz;                   // particle-major y, z phases (the GEMMs' A operands)
  DevBuf img;                   // real-space lattice offsets (float4)
  int nimg = 1;
  KMaps maps;
  uint64_t img_key = 0;         // buffers and plan the maps and zeroed pads belong to
  // the real-space kernel runs on this side stream, concurrently with the
  // reciprocal chain (low priority: it fills the SMs the chain leaves idle)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // the recorded launch sequence (run_mixed_sequence)
  cudaGraphExec_t gexec = nullptr;
  uint64_t gkey = 0, gcand = 0;
  int nrow = 0;          // (m2, m3) rows of the tensor-core contraction
  int *h_status = nullptr;      // pinned copy of the kernels' status word
  bool tensor = true;           // reciprocal space on the tensor cores
  KGemm plan;
  uint64_t self_fp = 0;
  int self_np = 0;
  int nchunk_r = 1, nchunk_k = 1;
  int real_g = 1;               // warps per target of mk_real
  int nc[3] = {0, 0, 0};        // cell list of mk_real (nc[0] == 0: no cells)
  DevBuf sq, cstart;
  // unequal radii: radii and their squares (FP32), the per-particle self
  // terms at the split (FP64, [np][3]), for the split they were made at
  bool poly = false;
  double amax = 1.0;
  DevBuf prad, pqa, pself;
  uint64_t poly_fp = 0;
};

constexpr int MX_WARPS = 8;      // warps per CTA in the mixed kernels
constexpr int MX_QCAP = 64;      // per-warp queue of accepted pairs
constexpr int MX_MTAB = 64;      // largest |m| per axis kept in shared memory

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------
struct PrepArgs {
  const double *pos;
  const double *x;
  int np, c;
  double sx, sy, sz;    // 2^32 / L_d
  double shift;         // Lees-Edwards shift (flow axis x)
  double sl;            // shift / lx
  int shear_mode;
  int ntab;             // (M0 + 1) + (M1 + 1) + (M2 + 1) table rows
  int m0end, m1end;     // first row of the y and z tables
  const float4 *rot;    // e^{2 pi i h / 1024}, h = 0..1023: (hi.re, hi.im, lo.re, lo.im)
  uint32_t *qpos;       // [np][4] fixed-point x, y, z (+ pad)
  float2 *tab;          // [ntab][np]
  float *xf;            // [np][cpad(c)]
  float *zf;            // forward GEMM image ZF (tensor-core path) or NULL
  size_t zplane;        // floats per ZF plane
  int kf;               // floats per ZF row
  float2 *tyz;          // particle-major y, z phases for both signs of m (or NULL)
  int wyz, M1, M2;
};

constexpr int PREP_P = 32;       // particles per mk_prep CTA
constexpr int PREP_ROWS = 4;     // table rows per mk_prep CTA (one entry per thread)
constexpr int PREP_CMAX = 11;    // components per particle at most

// floor(v) mod 2^32 for |v| < 2^62: the 32-bit fixed-point coordinate, the
// periodic wrap being the modulo
__device__ __forceinline__ uint32_t
fixq (double v)
{
  return (uint32_t) (unsigned long long) __double2ll_rd (v);
}

// Fixed-point positions (wrapped to the primary cell, Lees-Edwards aware),
// x in FP32 and the per-axis phase tables tab[m][j] = e^{2 pi i m u_d(j)}.
// u_d is the particle's fractional coordinate on axis d as a 32-bit fixed
// point q_d, so m u_d mod 1 is the exact integer product m q_d mod 2^32; on
// a sheared lattice the flow-axis phase coordinate is u_x - (shift/lx) u_g.
// With a ZF image (the tensor-core path) the CTA also writes, for its
// flow-axis rows m1, Z = t0[m1] x_q as TF32 hi/lo pairs in the forward
// GEMM's sign pattern: image row (m1, re, q) = (Re Z, -Im Z), (m1, im, q) =
// (Im Z, Re Z) at column pair j.
// CTA (blockIdx.x, blockIdx.y): PREP_P particles x PREP_ROWS table rows, one
// entry per thread; the few FP64 operations per particle are repeated by
// each row group.
__global__ void __launch_bounds__ (128)
mk_prep (PrepArgs a)
{
  __shared__ uint32_t s_q[4][PREP_P];
  __shared__ float s_x[PREP_P * PREP_CMAX];
  const int t = threadIdx.x;
  const int jb = blockIdx.x * PREP_P;
  {
    const size_t e0 = (size_t) jb * a.c;
    const int nx = PREP_P * a.c;
    const int cp = (a.c + 3) & ~3;
    for (int e = t; e < nx; e += blockDim.x)
      {
        const float v = (e0 + e < (size_t) a.np * a.c) ? (float) a.x[e0 + e] : 0.f;
        s_x[e] = v;
        if (blockIdx.y == 0 && e0 + e < (size_t) a.np * a.c)
          a.xf[(size_t) (jb + e / a.c) * cp + e % a.c] = v;
      }
  }
  if (t < PREP_P)
    {
      const int j = jb + t;
      uint32_t q0 = 0, q1 = 0, q2 = 0, qu = 0;
      if (j < a.np)
        {
          double x = a.pos[3 * j];
          const double y = a.pos[3 * j + 1], z = a.pos[3 * j + 2];
          if (a.shear_mode == 1 || a.shear_mode == 2)
            {
              // wraps along the gradient axis shift the flow coordinate
              const long long G = __double2ll_rd ((a.shear_mode == 1 ? y * a.sy : z * a.sz));
              const double w = (double) (G >> 32);
              x = fma (-w, a.shift, x);
            }
          q0 = fixq (x * a.sx);
          q1 = fixq (y * a.sy);
          q2 = fixq (z * a.sz);
          qu = q0;
          if (a.shear_mode == 1) qu = q0 - fixq (a.sl * (double) q1);
          else if (a.shear_mode == 2) qu = q0 - fixq (a.sl * (double) q2);
          if (blockIdx.y == 0)
            reinterpret_cast<uint4 *> (a.qpos)[j] = make_uint4 (q0, q1, q2, 0u);
        }
      s_q[0][t] = qu; s_q[1][t] = q1; s_q[2][t] = q2;
    }
  __syncthreads ();
  // row group y takes rows y, y + G, y + 2 G, y + 3 G (G = gridDim.y), so the
  // flow-axis rows, which also write ZF, spread over the groups; thread
  // (rr, jl) computes entry (row rr of the group, particle jl)
  __shared__ float2 s_ph[PREP_ROWS][PREP_P];
  const int G = gridDim.y;
  {
    const int rr = t / PREP_P, jl = t % PREP_P, j = jb + jl;
    const int row = (int) blockIdx.y + rr * G;
    if (row < a.ntab && j < a.np)
      {
        const int d = row < a.m0end ? 0 : (row < a.m1end ? 1 : 2);
        const uint32_t m = (uint32_t) (row - (d == 0 ? 0 : (d == 1 ? a.m0end : a.m1end)));
        const float2 ph = phase_of (a.rot, m * s_q[d][jl]);
        a.tab[(size_t) row * a.np + j] = ph;
        if (d != 0 && a.tyz)
          {
            float2 *ty = a.tyz + (size_t) j * a.wyz + (d == 1 ? a.M1 : 2 * a.M1 + 1 + a.M2);
            ty[(int) m] = ph;
            ty[-(int) m] = make_float2 (ph.x, -ph.y);
          }
        s_ph[rr][jl] = ph;
      }
  }
  if (!a.zf) return;
  __syncthreads ();
  // Z = t0[m1] x_q as TF32 hi / lo pairs for the flow-axis rows of this
  // group, one (row, component, particle) entry per thread at a time (the
  // particle fastest: neighbouring threads store neighbouring columns)
  int nz = 0;                                  // flow-axis rows of the group
  while (nz < PREP_ROWS && (int) blockIdx.y + nz * G < a.m0end) nz++;
  for (int e = t; e < nz * PREP_P * a.c; e += blockDim.x)
    {
      const int rr = e / (PREP_P * a.c), rem = e - rr * PREP_P * a.c;
      const int q = rem / PREP_P, jl = rem - q * PREP_P, j = jb + jl;
      if (j >= a.np) continue;
      const int m = (int) blockIdx.y + rr * G;
      const float2 ph = s_ph[rr][jl];
      const float xq = s_x[jl * a.c + q];
      const float u = ph.x * xq, v = ph.y * xq;
      for (int part = 0; part < 2; part++)
        {
          const float p0 = part ? v : u, p1 = part ? u : -v;
          uint32_t h0, l0, h1, l1;
          umma::split_tf32 (p0, h0, l0);
          umma::split_tf32 (p1, h1, l1);
          float2 *o = reinterpret_cast<float2 *> (
                        a.zf + (((size_t) m * 2 + part) * a.c + q) * a.kf) + j;
          o[0] = make_float2 (__uint_as_float (h0), __uint_as_float (h1));
          o[a.zplane / 2] = make_float2 (__uint_as_float (l0), __uint_as_float (l1));
        }
    }
}

__device__ __forceinline__ float2
cmul (float2 a, float2 b)
{
  return make_float2 (a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2
tab_get (const float2 *t, int m, size_t stride, size_t j)
{
  // t[|m| * stride + j], conjugated for negative m
  const float2 v = t[(size_t) (m < 0 ? -m : m) * stride + j];
  return m < 0 ? make_float2 (v.x, -v.y) : v;
}

// components of x per particle in the padded FP32 copy xf (float4 loads)
__host__ __device__ constexpr int
cpad (int c)
{
  return (c + 3) & ~3;
}

struct RealMixArgs {
  const uint32_t *qpos;  // [np][4] fixed-point positions
  const float *xf;       // [np][cpad(c)] FP32 x
  int np;
  int G;                 // warps per target (their sums meet in shared memory)
  float scale[3];        // L_d / 2^32
  int shear_mode;
  uint32_t shift_q;      // shift / lx * 2^32 (two's complement)
  float rc2, rmin;
  float xi, xisp;
  const float *rad, *slipa;
  float *out;            // [2][np][c]: the compensated sum of each target as hi + lo
  const float4 *img;     // lattice offsets added to the minimum-image difference
  int nimg;              // 1 (the zero offset) while the cutoff is below half the box
  // cell list (NULL cstart: every particle is a candidate source)
  const uint4 *sq;       // particles in cell order: (q_x, q_y, q_z, particle index)
  const int *cstart;     // [ncell + 1] first slot of each cell in sq
  int nc[3];             // cells per axis (cell side >= rc / 2)
  // rmin clamp (rm2 = (2 rmin)^2): with clampfix the clamped pairs are left
  // to mk_clamp, which evaluates them at the struct's own split xi_ref
  int clampfix;
  float rm2;
  float xi_ref, xisp_ref;
  float *out_clamp;      // [np][c]: mk_clamp's sums (a third combine chunk)
};

// minimum-image displacement r_j - r_i from fixed-point positions
__device__ __forceinline__ void
min_image (const RealMixArgs &a, uint4 qi, uint4 qj, float &dx, float &dy, float &dz)
{
  uint32_t ux = qj.x - qi.x;
  const uint32_t uy = qj.y - qi.y;
  const uint32_t uz = qj.z - qi.z;
  if (a.shear_mode == 1)
    {
      // number of gradient-axis wraps taken by the 32-bit subtraction
      const long long raw = (long long) qj.y - (long long) qi.y;
      const long long w = (raw - (long long) (int32_t) uy) >> 32;
      ux -= (uint32_t) w * a.shift_q;
    }
  else if (a.shear_mode == 2)
    {
      const long long raw = (long long) qj.z - (long long) qi.z;
      const long long w = (raw - (long long) (int32_t) uz) >> 32;
      ux -= (uint32_t) w * a.shift_q;
    }
  dx = (float) (int32_t) ux * a.scale[0];
  dy = (float) (int32_t) uy * a.scale[1];
  dz = (float) (int32_t) uz * a.scale[2];
}

// one pair term (source j at displacement d from the target) added to t;
// pairs under the rmin clamp arrive here only when the clamp is applied in
// place (clampfix = 0); otherwise mk_clamp takes them
template <int V, bool POLY>
__device__ __forceinline__ void
mix_term (const RealMixArgs &a, float4 d, float ai, GenU<V, float> &t)
{
  const int j = __float_as_int (d.w);
  const float rr = d.x * d.x + d.y * d.y + d.z * d.z;
  // 1 / r from the reciprocal square root with one Newton step (1 ulp)
  float ri = rsqrtf (rr);
  ri = ri * fmaf (-0.5f * rr, ri * ri, 1.5f);
  float r = rr * ri;
  const float rm = 2.0f * a.rmin;          // (a_i + a_j) rmin for unit spheres
  if (r < rm)
    {
      r = rm;
      ri = 1.0f / rm;
    }
  constexpr int C = NComp<V>::value, CP = cpad (C);
  // x_j as float4 loads of the padded copy
  float xj[CP];
  const float4 *src = reinterpret_cast<const float4 *> (a.xf + (size_t) CP * j);
#pragma unroll
  for (int k = 0; k < CP / 4; k++)
    {
      const float4 v = __ldg (src + k);
      xj[4 * k] = v.x; xj[4 * k + 1] = v.y; xj[4 * k + 2] = v.z; xj[4 * k + 3] = v.w;
    }
  GenF<V, float> g;
  load_genf<V, float> (xj, g);
  const float e[3] = {d.x * ri, d.y * ri, d.z * ri};
  PairScalars<float> s;
  if (POLY)
    // unequal radii (rmin = 0): the SD-form scalars of the pair's radii,
    // scaled by the target's (src/ewald.c:204-359, :383-420)
    real_scalars_poly<V, float> (a.xi, a.xisp, r, ai, __ldg (a.rad + j), ai, s);
  else
    real_scalars_mono_ri<V, float> (a.xi, a.xisp, r, ri, s);
  pair_apply<V, float> (e, s, g, t);
}

// error-free sum of two values: a + b = s + e exactly
__device__ __forceinline__ void
two_sum (float a, float b, float &s, float &e)
{
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

constexpr int RG_WARPS = 8;      // warps per CTA of mk_real
constexpr int RG_QCAP = 192;     // queue entries per warp (the reduction reuses them)
constexpr int RG_MAXIMG = 4;     // lattice offsets tested per candidate in one pass
// a pass adds at most 32 RG_MAXIMG entries to at most 31 left over
static_assert (31 + 32 * RG_MAXIMG <= RG_QCAP, "mk_real queue too small");

// The real-space sum of the mixed split: G warps per target particle.  Each
// warp takes a share of the candidate sources (a slice of all particles, or
// rows of neighbouring cells of the cell list), tests 32 at a time against
// the cutoff (the minimum image and, for cutoffs beyond half the box, the
// split's lattice offsets) and queues the accepted pairs (displacement and
// source index, one float4 each) in shared memory; every 32 queued pairs the
// lanes evaluate one term each, so the FP32 pipe only sees accepted terms.
// With lattice offsets (cutoff beyond half the box) each lane tests all
// offsets of its source into a bit mask and one warp prefix sum places the
// accepted ones.  Each lane sums its terms per component (a few tens at
// most), the 32 lane sums meet in a shuffle tree (pairwise summation), the
// G warps of the target meet with TwoSum (error-free, the rounding errors
// carried along), and the result is written as the FP32 pair hi + lo,
// which the combine adds in FP64.
template <int V, bool POLY>
__global__ void __launch_bounds__ (RG_WARPS * 32, 3)
mk_real (RealMixArgs a)
{
  constexpr int C = NComp<V>::value;
  __shared__ float4 s_q[RG_WARPS][RG_QCAP];
  __shared__ float s_red[RG_WARPS][2][C];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int tpc = RG_WARPS / a.G;                       // targets per CTA
  const int tl = wib / a.G, part = wib - tl * a.G;
  const int slot = blockIdx.x * tpc + tl;
  const bool live = slot < a.np;
  const bool cells = a.cstart != nullptr;
  uint4 qi = make_uint4 (0u, 0u, 0u, 0u);
  int i = 0;
  if (live)
    {
      if (cells)
        {
          qi = a.sq[slot];
          i = (int) qi.w;
        }
      else
        {
          qi = reinterpret_cast<const uint4 *> (a.qpos)[slot];
          i = slot;
        }
    }
  GenU<V, float> sum;
  sum.zero ();
  const float ai = (POLY && live) ? __ldg (a.rad + i) : 1.0f;
  float4 *q = s_q[wib];
  int qn = 0;
  const unsigned lt = (1u << lane) - 1u;

  // test the candidate sources s0 .. s1 - 1 (slots of the source array)
  auto scan = [&] (int s0, int s1) {
    for (int sb = s0; sb < s1; sb += 32)
      {
        const int sj = sb + lane;
        float d0x = 0.f, d0y = 0.f, d0z = 0.f;
        int j = 0;
        if (sj < s1)
          {
            const uint4 qj = cells ? a.sq[sj] : reinterpret_cast<const uint4 *> (a.qpos)[sj];
            j = cells ? (int) qj.w : sj;
            min_image (a, qi, qj, d0x, d0y, d0z);
          }
        if (a.nimg == 1)
          {
            // minimum image only: one ballot places the accepted pairs
            const float rr = d0x * d0x + d0y * d0y + d0z * d0z;
            const bool ok = sj < s1 && rr > 0.f && rr < a.rc2 && !(a.clampfix && rr < a.rm2);
            const unsigned b = __ballot_sync (0xffffffffu, ok);
            if (ok) q[qn + __popc (b & lt)] = make_float4 (d0x, d0y, d0z, __int_as_float (j));
            qn += __popc (b);
          }
        else
          for (int m0 = 0; m0 < a.nimg; m0 += RG_MAXIMG)
            {
              // this lane's accepted offsets m0 .. m0 + 3 as a bit mask, then
              // a warp prefix sum of the counts places them
              unsigned mask = 0u;
              if (sj < s1)
#pragma unroll
                for (int k = 0; k < RG_MAXIMG; k++)
                  {
                    if (m0 + k >= a.nimg) break;
                    const float4 T = a.img[m0 + k];
                    const float dx = d0x + T.x, dy = d0y + T.y, dz = d0z + T.z;
                    const float rr = dx * dx + dy * dy + dz * dz;
                    if (rr > 0.f && rr < a.rc2 && !(a.clampfix && rr < a.rm2)) mask |= 1u << k;
                  }
              const int cnt = __popc (mask);
              int pre = cnt;
#pragma unroll
              for (int o = 1; o < 32; o <<= 1)
                {
                  const int v = __shfl_up_sync (0xffffffffu, pre, o);
                  if (lane >= o) pre += v;
                }
              int slot = qn + pre - cnt;
              while (mask)
                {
                  const int k = __ffs (mask) - 1;
                  mask &= mask - 1u;
                  const float4 T = a.img[m0 + k];
                  q[slot++] = make_float4 (d0x + T.x, d0y + T.y, d0z + T.z, __int_as_float (j));
                }
              qn += __shfl_sync (0xffffffffu, pre, 31);
              __syncwarp ();
              while (qn >= 32)
                {
                  mix_term<V, POLY> (a, q[qn - 32 + lane], ai, sum);
                  qn -= 32;
                  __syncwarp ();
                }
            }
        __syncwarp ();
        if (qn >= 32)
          {
            mix_term<V, POLY> (a, q[qn - 32 + lane], ai, sum);
            qn -= 32;
            __syncwarp ();
          }
      }
  };

  if (live)
    {
      if (!cells)
        scan ((int) ((long long) a.np * part / a.G), (int) ((long long) a.np * (part + 1) / a.G));
      else
        {
          // rows (dx, dy) of the 5 x 5 x 5 neighbouring cells (cell side >=
          // rc / 2); the 5 cells of a row along z are one or two contiguous
          // runs of slots; the rows are dealt round-robin to the G warps
          const int cx = (int) (((unsigned long long) qi.x * (unsigned) a.nc[0]) >> 32);
          const int cy = (int) (((unsigned long long) qi.y * (unsigned) a.nc[1]) >> 32);
          const int cz = (int) (((unsigned long long) qi.z * (unsigned) a.nc[2]) >> 32);
          const int nz = a.nc[2];
          for (int row = part; row < 25; row += a.G)
            {
              const int ox = row / 5 - 2, oy = row % 5 - 2;
              const int x = (cx + ox + a.nc[0]) % a.nc[0], y = (cy + oy + a.nc[1]) % a.nc[1];
              const int base = (x * a.nc[1] + y) * nz;
              const int z0 = cz - 2, z1 = cz + 2;          // inclusive, may wrap
              if (z0 >= 0 && z1 < nz)
                scan (a.cstart[base + z0], a.cstart[base + z1 + 1]);
              else if (z0 < 0)
                {
                  scan (a.cstart[base], a.cstart[base + z1 + 1]);
                  scan (a.cstart[base + z0 + nz], a.cstart[base + nz]);
                }
              else
                {
                  scan (a.cstart[base + z0], a.cstart[base + nz]);
                  scan (a.cstart[base], a.cstart[base + z1 - nz + 1]);
                }
            }
        }
      if (lane < qn) mix_term<V, POLY> (a, q[lane], ai, sum);
    }
  // the 32 lane sums of this warp by a shuffle tree (pairwise summation)
#pragma unroll
  for (int k = 0; k < C; k++)
    {
      const float v = warp_sum (sum.v[k]);
      if (lane == 0)
        {
          s_red[wib][0][k] = v;
          s_red[wib][1][k] = 0.f;
        }
    }
  __syncthreads ();
  // the G warps of the target: part 0 adds them and writes hi, lo
  if (live && part == 0 && lane < C)
    {
      float S0 = s_red[wib][0][lane], E0 = s_red[wib][1][lane];
      for (int p = 1; p < a.G; p++)
        {
          float s2, e2;
          two_sum (S0, s_red[wib + p][0][lane], s2, e2);
          S0 = s2;
          E0 += e2 + s_red[wib + p][1][lane];
        }
      const float hi = S0 + E0;
      const float lo = E0 - (hi - S0);
      a.out[(size_t) i * C + lane] = hi;
      a.out[((size_t) a.np + i) * C + lane] = lo;
    }
}

// The rmin clamp of libstokes (src/ewald.c:693-699: r raised to (a_i + a_j)
// rmin = rm, e = d / r with the raised r) changes the real-space term of a
// clamped pair only; unclamped, the sum does not depend on the split.  At
// the mixed split a clamped pair therefore contributes
//   T(d/rm; s_ref(rm)) + T(d/r; s_xi(r) - s_ref(r)):
// the clamped term of the struct's split xi_ref, plus the change of the
// unclamped term between the splits, which split_diff gives without
// cancellation however close the pair.  mk_real skips these pairs; one warp
// per target here tests the candidates (minimum image and the split's
// lattice offsets) and sums the few clamped terms.
template <int V>
__global__ void __launch_bounds__ (256)
mk_clamp (RealMixArgs a)
{
  constexpr int C = NComp<V>::value, CP = cpad (C);
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= a.np) return;
  const uint4 qi = reinterpret_cast<const uint4 *> (a.qpos)[i];
  float acc[C];
#pragma unroll
  for (int q = 0; q < C; q++) acc[q] = 0.f;
  const float rm = sqrtf (a.rm2);
  for (int j = lane; j < a.np; j += 32)
    {
      const uint4 qj = reinterpret_cast<const uint4 *> (a.qpos)[j];
      float d0x, d0y, d0z;
      min_image (a, qi, qj, d0x, d0y, d0z);
      for (int m = 0; m < a.nimg; m++)
        {
          const float4 T = a.img[m];
          const float dx = d0x + T.x, dy = d0y + T.y, dz = d0z + T.z;
          const float rr = dx * dx + dy * dy + dz * dz;
          if (!(rr > 0.f && rr < a.rm2)) continue;
          const float r = sqrtf (rr);
          float xj[CP];
#pragma unroll
          for (int k = 0; k < C; k++) xj[k] = a.xf[(size_t) CP * j + k];
          GenF<V, float> g;
          load_genf<V, float> (xj, g);
          PairScalars<float> sc, ds;
          real_scalars_mono<V, float> (a.xi_ref, a.xisp_ref, rm, sc);
          split_diff<V, float> (a.xi_ref, a.xi, r, ds);
          const float ec[3] = {dx / rm, dy / rm, dz / rm};
          const float e0[3] = {dx / r, dy / r, dz / r};
          GenU<V, float> t;
          t.zero ();
          pair_apply<V, float> (ec, sc, g, t);
          pair_apply<V, float> (e0, ds, g, t);
#pragma unroll
          for (int q = 0; q < C; q++) acc[q] += t.v[q];
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const float v = warp_sum (acc[q]);
      if (lane == 0) a.out_clamp[(size_t) i * C + q] = v;
    }
}

// The cell list of mk_real: particles sorted by cell, stably (in particle
// order within a cell, so the sums are reproducible).  One CTA of 1024
// threads; warp w owns particles [w N / 32, (w + 1) N / 32): it counts them
// per cell (its own row of counts); thread c turns column c (cell c) into
// the warps' offsets within the cell, a block scan of the cell totals gives
// the cell starts, and each warp places its particles in order, 32 at a
// time, lanes of one cell ranked by __match_any_sync.
constexpr int CELL_THREADS = 1024;
constexpr int CELL_MAX = 1000;           // cells (<= CELL_THREADS: one per thread)

__global__ void __launch_bounds__ (CELL_THREADS)
mk_cells (const uint4 *qpos, int np, int nc0, int nc1, int nc2, int *cstart, uint4 *sq)
{
  extern __shared__ int s_cnt[];          // [32][ncell]: counts, then slots
  __shared__ int s_part[32];
  const int ncell = nc0 * nc1 * nc2;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int k = threadIdx.x; k < 32 * ncell; k += blockDim.x) s_cnt[k] = 0;
  __syncthreads ();
  const int p0 = (int) ((long long) np * w / 32), p1 = (int) ((long long) np * (w + 1) / 32);
  auto cell_of = [&] (uint4 q) {
    const int x = (int) (((unsigned long long) q.x * (unsigned) nc0) >> 32);
    const int y = (int) (((unsigned long long) q.y * (unsigned) nc1) >> 32);
    const int z = (int) (((unsigned long long) q.z * (unsigned) nc2) >> 32);
    return (x * nc1 + y) * nc2 + z;
  };
  for (int p = p0 + lane; p < p1; p += 32) atomicAdd (&s_cnt[w * ncell + cell_of (qpos[p])], 1);
  __syncthreads ();
  const int c = threadIdx.x;
  int tot = 0;
  if (c < ncell)
    for (int ww = 0; ww < 32; ww++)
      {
        const int v = s_cnt[ww * ncell + c];
        s_cnt[ww * ncell + c] = tot;
        tot += v;
      }
  // block-wide exclusive scan of the cell totals
  int v = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
    {
      const int n = __shfl_up_sync (0xffffffffu, v, o);
      if (lane >= o) v += n;
    }
  if (lane == 31) s_part[w] = v;
  __syncthreads ();
  if (w == 0)
    {
      int pv = s_part[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
        {
          const int n = __shfl_up_sync (0xffffffffu, pv, o);
          if (lane >= o) pv += n;
        }
      s_part[lane] = pv;
    }
  __syncthreads ();
  const int start = v - tot + (w > 0 ? s_part[w - 1] : 0);
  if (c < ncell)
    {
      for (int ww = 0; ww < 32; ww++) s_cnt[ww * ncell + c] += start;
      cstart[c] = start;
      if (c == ncell - 1) cstart[ncell] = start + tot;
    }
  __syncthreads ();
  for (int pb = p0; pb < p1; pb += 32)
    {
      const int p = pb + lane;
      const bool ok = p < p1;
      const uint4 qv = ok ? qpos[p] : make_uint4 (0u, 0u, 0u, 0u);
      const int cc = ok ? cell_of (qv) : -1;
      const unsigned peers = __match_any_sync (0xffffffffu, cc);
      const int rank = __popc (peers & ((1u << lane) - 1u));
      if (ok) sq[s_cnt[w * ncell + cc] + rank] = make_uint4 (qv.x, qv.y, qv.z, (unsigned) p);
      __syncwarp ();
      if (ok && rank == 0) s_cnt[w * ncell + cc] += __popc (peers);
      __syncwarp ();
    }
}

struct KMixArgs {
  const MixK *kt;
  const float2 *tab;
  const float *xf;
  int np, nkh;
  size_t off1, off2;     // offsets of the y and z tables in tab
  float *pq;             // [2c][nkh] P then Q, component-major
};

// one warp per half-space k: C(k) = sum_j cos(k.r_j) x_j, S(k) likewise,
// then P = Bc C - Bs S and Q = Bc S + Bs C
template <int V>
__global__ void __launch_bounds__ (MX_WARPS * 32)
mk_sfac (KMixArgs a)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * MX_WARPS + (threadIdx.x >> 5);
  if (k >= a.nkh) return;
  const MixK K = a.kt[k];
  const float2 *t0 = a.tab, *t1 = a.tab + a.off1, *t2 = a.tab + a.off2;
  float cs[C], sn[C];
#pragma unroll
  for (int q = 0; q < C; q++) cs[q] = sn[q] = 0.f;
  for (int j = lane; j < a.np; j += 32)
    {
      const float2 ph = cmul (cmul (tab_get (t0, K.m1, a.np, j), tab_get (t1, K.m2, a.np, j)),
                              tab_get (t2, K.m3, a.np, j));
      const float *xj = a.xf + (size_t) cpad (C) * j;
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          const float v = xj[q];
          cs[q] = fmaf (ph.x, v, cs[q]);
          sn[q] = fmaf (ph.y, v, sn[q]);
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      cs[q] = warp_sum (cs[q]);
      sn[q] = warp_sum (sn[q]);
    }
  if (lane == 0)
    {
      const float e[3] = {K.ex, K.ey, K.ez};
      float nsn[C];
#pragma unroll
      for (int q = 0; q < C; q++) nsn[q] = -sn[q];
      GenF<V, float> gc, gs, gms;
      load_genf<V, float> (cs, gc);
      load_genf<V, float> (sn, gs);
      load_genf<V, float> (nsn, gms);
      GenU<V, float> P, Q;
      P.zero ();
      Q.zero ();
      recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gc, gms, P);
      recip_apply<V, float> (e, K.ya, K.yb, K.yc, K.yg, K.yh, K.ym, gs, gc, Q);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          a.pq[(size_t) q * a.nkh + k] = P.v[q];
          a.pq[(size_t) (C + q) * a.nkh + k] = Q.v[q];
        }
    }
}

struct BpMixArgs {
  const MixK *kt;
  const float2 *tab;
  const float *pq;
  int np, nkh, nchunk;
  int M0, M1, M2;
  size_t off1, off2;
  float *partial;        // [nchunk][np][c]
};

// one warp per (target i, k chunk): y_i += cos(k.r_i) P(k) + sin(k.r_i) Q(k)
template <int V>
__global__ void __launch_bounds__ (MX_WARPS * 32)
mk_backproj (BpMixArgs a)
{
  constexpr int C = NComp<V>::value;
  __shared__ float2 s_t[MX_WARPS][3][MX_MTAB + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * MX_WARPS + wib;
  if (w >= (long long) a.np * a.nchunk) return;
  const int i = (int) (w % a.np);
  const int chunk = (int) (w / a.np);
  const int Md[3] = {a.M0, a.M1, a.M2};
  const size_t off[3] = {0, a.off1, a.off2};
  for (int d = 0; d < 3; d++)
    for (int m = lane; m <= Md[d]; m += 32)
      s_t[wib][d][m] = a.tab[off[d] + (size_t) m * a.np + i];
  __syncwarp ();
  const int k0 = (int) ((long long) a.nkh * chunk / a.nchunk);
  const int k1 = (int) ((long long) a.nkh * (chunk + 1) / a.nchunk);
  float acc[C];
#pragma unroll
  for (int q = 0; q < C; q++) acc[q] = 0.f;
  for (int k = k0 + lane; k < k1; k += 32)
    {
      const int4 m = *reinterpret_cast<const int4 *> (&a.kt[k].m1);
      float2 p0 = s_t[wib][0][m.x < 0 ? -m.x : m.x];
      float2 p1 = s_t[wib][1][m.y < 0 ? -m.y : m.y];
      float2 p2 = s_t[wib][2][m.z < 0 ? -m.z : m.z];
      if (m.x < 0) p0.y = -p0.y;
      if (m.y < 0) p1.y = -p1.y;
      if (m.z < 0) p2.y = -p2.y;
      const float2 ph = cmul (cmul (p0, p1), p2);
#pragma unroll
      for (int q = 0; q < C; q++)
        acc[q] = fmaf (ph.x, a.pq[(size_t) q * a.nkh + k],
                       fmaf (ph.y, a.pq[(size_t) (C + q) * a.nkh + k], acc[q]));
    }
  float *out = a.partial + ((size_t) chunk * a.np + i) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const float v = warp_sum (acc[q]);
      if (lane == 0) out[q] = v;
    }
}

// Unequal radii (SIMT).  The reciprocal weights of a pair depend on both
// radii, linearly in the source's squared radius q_j (src/ewald.c:985-1025),
// so each half-space k keeps four raw sums: C = sum_j cos(k.r_j) x_j, S with
// sin, and Cq, Sq weighted by q_j.  The k table holds, for unequal radii,
// ya = kexp (the A, B, C, H, M factor), yb = |k|, yc = |k|^2 and yg = the G
// factor (-kexp on the split's own vectors, +2 kexp_ref of the reference's
// split for its G term).
template <int V>
__global__ void __launch_bounds__ (MX_WARPS * 32)
mk_sfac_poly (KMixArgs a, const float *qa)
{
  constexpr int C = NComp<V>::value;
  const int lane = threadIdx.x & 31;
  const int k = blockIdx.x * MX_WARPS + (threadIdx.x >> 5);
  if (k >= a.nkh) return;
  const MixK K = a.kt[k];
  const float2 *t0 = a.tab, *t1 = a.tab + a.off1, *t2 = a.tab + a.off2;
  float cs[C], sn[C], cq[C], sq[C];
#pragma unroll
  for (int q = 0; q < C; q++) cs[q] = sn[q] = cq[q] = sq[q] = 0.f;
  for (int j = lane; j < a.np; j += 32)
    {
      const float2 ph = cmul (cmul (tab_get (t0, K.m1, a.np, j), tab_get (t1, K.m2, a.np, j)),
                              tab_get (t2, K.m3, a.np, j));
      const float *xj = a.xf + (size_t) cpad (C) * j;
      const float w = __ldg (qa + j);
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          const float v = xj[q], vq = w * v;
          cs[q] = fmaf (ph.x, v, cs[q]);
          sn[q] = fmaf (ph.y, v, sn[q]);
          cq[q] = fmaf (ph.x, vq, cq[q]);
          sq[q] = fmaf (ph.y, vq, sq[q]);
        }
    }
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      cs[q] = warp_sum (cs[q]);
      sn[q] = warp_sum (sn[q]);
      cq[q] = warp_sum (cq[q]);
      sq[q] = warp_sum (sq[q]);
    }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < C; q++)
      {
        a.pq[(size_t) q * a.nkh + k] = cs[q];
        a.pq[(size_t) (C + q) * a.nkh + k] = sn[q];
        a.pq[(size_t) (2 * C + q) * a.nkh + k] = cq[q];
        a.pq[(size_t) (3 * C + q) * a.nkh + k] = sq[q];
      }
}

// one warp per (target i, k chunk): the target's weights (its radius a_i
// scales the SD form, q_i = a_i^2 enters the Laplacian terms) applied to
// v1 = c_i C + s_i S, v2 = s_i C - c_i S and to the q-weighted sums
template <int V>
__global__ void __launch_bounds__ (MX_WARPS * 32)
mk_backproj_poly (BpMixArgs a, const float *rad)
{
  constexpr int C = NComp<V>::value;
  __shared__ float2 s_t[MX_WARPS][3][MX_MTAB + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const long long w = (long long) blockIdx.x * MX_WARPS + wib;
  if (w >= (long long) a.np * a.nchunk) return;
  const int i = (int) (w % a.np);
  const int chunk = (int) (w / a.np);
  const int Md[3] = {a.M0, a.M1, a.M2};
  const size_t off[3] = {0, a.off1, a.off2};
  for (int d = 0; d < 3; d++)
    for (int m = lane; m <= Md[d]; m += 32)
      s_t[wib][d][m] = a.tab[off[d] + (size_t) m * a.np + i];
  __syncwarp ();
  const float aa = __ldg (rad + i), qai = aa * aa, aa2 = aa * aa, aa3 = aa2 * aa;
  const int k0 = (int) ((long long) a.nkh * chunk / a.nchunk);
  const int k1 = (int) ((long long) a.nkh * (chunk + 1) / a.nchunk);
  GenU<V, float> acc;
  acc.zero ();
  for (int k = k0 + lane; k < k1; k += 32)
    {
      const MixK K = a.kt[k];
      float2 p0 = s_t[wib][0][K.m1 < 0 ? -K.m1 : K.m1];
      float2 p1 = s_t[wib][1][K.m2 < 0 ? -K.m2 : K.m2];
      float2 p2 = s_t[wib][2][K.m3 < 0 ? -K.m3 : K.m3];
      if (K.m1 < 0) p0.y = -p0.y;
      if (K.m2 < 0) p1.y = -p1.y;
      if (K.m3 < 0) p2.y = -p2.y;
      const float2 p = cmul (cmul (p0, p1), p2);
      float t1[C], t2[C], u1[C], u2[C];
#pragma unroll
      for (int q = 0; q < C; q++)
        {
          const float Cc = a.pq[(size_t) q * a.nkh + k], Ss = a.pq[(size_t) (C + q) * a.nkh + k];
          const float Cq = a.pq[(size_t) (2 * C + q) * a.nkh + k];
          const float Sq = a.pq[(size_t) (3 * C + q) * a.nkh + k];
          t1[q] = p.x * Cc + p.y * Ss;
          t2[q] = p.y * Cc - p.x * Ss;
          u1[q] = p.x * Cq + p.y * Sq;
          u2[q] = p.y * Cq - p.x * Sq;
        }
      const float e[3] = {K.ex, K.ey, K.ez};
      const float ax = K.ya, kn = K.yb, kk = K.yc, gx = K.yg;
      const float ya0 = aa * 6.0f * (1.0f - kk * qai * (1.0f / 6.0f)) * ax;
      const float ya1 = -aa * kk * ax;
      const float yb = aa2 * 3.0f * kn * ax;
      const float yc = aa3 * 1.5f * kk * ax;
      const float yg0 = aa2 * 3.0f * (1.0f - kk * qai * 0.1f) * kn * gx;
      const float yg1 = -aa2 * 0.5f * kk * kn * gx;
      const float yh = aa3 * 1.5f * kk * ax;
      const float ym0 = aa3 * 3.0f * (1.0f - kk * qai * 0.1f) * kk * ax;
      const float ym1 = -aa3 * 0.3f * kk * kk * ax;
      GenF<V, float> g1, g2, h1, h2;
      load_genf<V, float> (t1, g1);
      load_genf<V, float> (t2, g2);
      load_genf<V, float> (u1, h1);
      load_genf<V, float> (u2, h2);
      recip_apply<V, float> (e, ya0, yb, yc, yg0, yh, ym0, g1, g2, acc);
      recip_apply<V, float> (e, ya1, 0.0f, 0.0f, yg1, 0.0f, ym1, h1, h2, acc);
    }
  float *out = a.partial + ((size_t) chunk * a.np + i) * C;
#pragma unroll
  for (int q = 0; q < C; q++)
    {
      const float v = warp_sum (acc.v[q]);
      if (lane == 0) out[q] = v;
    }
}

// The self term of equal spheres as a C x C matrix: column q is the self
// block applied to the unit vector of component q (one thread per column,
// run once per split).
template <int V>
__global__ void
mk_selfmat (double xa, double xc, double xm, double *S)
{
  constexpr int C = NComp<V>::value;
  const int q = threadIdx.x;
  if (q >= C) return;
  PairScalars<double> s;
  s.xa = s.ya = xa;
  s.xc = s.yc = xc;
  s.xm = s.ym = s.zm = xm;
  s.yb = s.xg = s.yg = s.yh = 0.0;
  const double e[3] = {0.0, 0.0, 0.0};
  double u[C];
#pragma unroll
  for (int k = 0; k < C; k++) u[k] = (k == q) ? 1.0 : 0.0;
  GenF<V, double> g;
  load_genf<V, double> (u, g);
  GenU<V, double> acc;
  acc.zero ();
  pair_apply<V, double> (e, s, g, acc);
#pragma unroll
  for (int k = 0; k < C; k++) S[k * C + q] = acc.v[k];
}

// the final sum of a mixed product, y = S x + sum of the real-space partials
// + 2 sum of the reciprocal partials (half k space)
struct CombineArgs {
  const double *x;      // input vector, FP64 [np c]
  const float *pr;      // real-space partials [ncr][np c]
  int ncr;
  const float *pk;      // reciprocal partials [nck][np c]
  int nck;
  const double *S;      // self block of equal spheres, c x c
  const double *selfp;  // unequal radii: [np][3] factors of S's F, T, S parts (S unit)
  int np, c;
  double *y;            // output [np c]
};

constexpr int CMB_OUT = 32;      // elements per CTA (one per lane)
constexpr int CMB_WARPS = 8;     // chunk groups per element (one per warp)
constexpr int CMB_BATCH = 4;     // loads in flight per thread

// CTA of eight warps over the 32 consecutive elements t = i c + q of its
// lanes: warp w sums the chunks w, w + 8, ... of the real-space partials
// and, doubled (half k space; exact in FP32), of the reciprocal ones, so
// each load instruction reads 32 consecutive elements of one chunk and up
// to four loads per thread are in flight at once (TwoSum-compensated FP32).
// The warps' (sum, compensation) pairs meet in shared memory; warp 0 adds
// them in FP64 with the FP64 self term (at most five FMAs: the self block
// is diagonal for F and T and couples the five stresslet components) and
// writes 32 consecutive elements of y.
__global__ void __launch_bounds__ (CMB_OUT * CMB_WARPS)
mk_combine (CombineArgs a)
{
  __shared__ float2 s_p[CMB_WARPS][CMB_OUT];
  const int n = a.np * a.c;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = blockIdx.x * CMB_OUT + lane;
  const int tt = t < n ? t : n - 1;
  const int ntot = a.ncr + a.nck;
  float sum = 0.f, comp = 0.f;
  for (int k0 = w; k0 < ntot; k0 += CMB_BATCH * CMB_WARPS)
    {
      float v[CMB_BATCH];
#pragma unroll
      for (int u = 0; u < CMB_BATCH; u++)
        {
          const int k = k0 + u * CMB_WARPS;
          v[u] = k < a.ncr ? a.pr[(size_t) k * n + tt]
                 : (k < ntot ? 2.f * a.pk[(size_t) (k - a.ncr) * n + tt] : 0.f);
        }
#pragma unroll
      for (int u = 0; u < CMB_BATCH; u++)
        {
          // TwoSum: sum + v = sn + e exactly
          const float sn = sum + v[u];
          const float bp = sn - sum;
          comp += (sum - (sn - bp)) + (v[u] - bp);
          sum = sn;
        }
    }
  s_p[w][lane] = make_float2 (sum, comp);
  __syncthreads ();
  if (w != 0 || t >= n) return;
  double r = 0.0;
#pragma unroll
  for (int g = 0; g < CMB_WARPS; g++) r += (double) s_p[g][lane].x + (double) s_p[g][lane].y;
  const int i = t / a.c, q = t - i * a.c;
  const int q0 = (q < 6) ? q : 6, nq = (q < 6) ? 1 : 5;
  const double *xi = a.x + (size_t) a.c * i;
  double self = 0.0;
  for (int k = 0; k < nq; k++) self = fma (a.S[q * a.c + q0 + k], xi[q0 + k], self);
  if (a.selfp) self *= a.selfp[3 * i + (q < 3 ? 0 : (q < 6 ? 1 : 2))];
  a.y[t] = self + r;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static uint64_t
mix_fingerprint (const struct stokes *sys, double eta, double eps)
{
  double v[17] = {sys->lx, sys->ly, sys->lz, (double) sys->version, (double) sys->np,
                  (double) sys->shear_mode, sys->shear_shift, eta, eps, sys->rmin,
                  sys->a ? 1.0 : 0.0, sys->slip ? 1.0 : 0.0, sys->xi, sys->kmax,
                  (double) sys->kmaxx, (double) sys->kmaxy, (double) sys->kmaxz};
  uint64_t h = 1469598103934665603ull;
  const unsigned char *b = (const unsigned char *) v;
  for (size_t q = 0; q < sizeof v; q++) { h ^= b[q]; h *= 1099511628211ull; }
  return h;
}

static double
env_double (const char *name, double dflt)
{
  const char *s = getenv (name);
  return s ? atof (s) : dflt;
}

// default split parameter eta = xi V^(1/3), minimum image, by version and
// system size.  Measured on one GB300 (FTS at phi 0.3, FT 0.25, F 0.2) with
// the real space recorded after the forward GEMM; an eta below the smallest
// minimum-image split is raised to it, so small values all time the same:
//   FTS  N <= 512: 8 (N = 512 49.0 us against 52.5 with images at 10);
//        N <= 4096: 10 (N = 4096 273 us against 283 with images at 11);
//        above: 11 (N = 8192 726 us against 936 with images at 13)
//   FT   N = 1025-8192: 9 (N = 4096 171 us against 233 at 12; N = 8192
//        444 against 614 at 14)
//   F    N = 1025-4096: 9 (N = 2048 69.6 us against 75.2 at 12); above 12
//        (N = 16384 1131 us against 1189 at 9)
//   N <= 1024: the time is flat over eta 7-11 for all three
static double
default_eta (int version, int np)
{
  if (np <= 256) return 8.0;
  if (version == 2) return np <= 512 ? 8.0 : (np <= 4096 ? 10.0 : 11.0);
  if (np <= 1024) return 10.0;
  if (version == 1) return np <= 8192 ? 9.0 : 10.0;
  return np <= 4096 ? 9.0 : 12.0;
}

// eta when lattice images are asked for (LIBSTOKES_GB300_MIXED_IMAGES=1)
// or the box is too small for a minimum-image cutoff (measured before the
// real space moved behind the forward GEMM: FTS N = 256 53 us at eta 7
// against 61 us at the minimum-image split of then)
static double
default_eta_images (int np)
{
  if (np <= 256) return 7.0;
  if (np <= 1024) return 10.0;
  if (np <= 4096) return 11.0;
  return 13.0;
}

// choose xi, cutoffs and the half-space k list of the mixed split
static int
mixed_setup (Ctx *c, const struct stokes *sys, MixedState *m)
{
  // truncation of the sums: 3e-8 (measured at FTS N = 1000: the error
  // against FP64 is 2.92e-7 at 1e-8, 2.99e-7 at 3e-8, 3.03e-7 at 1e-7 --
  // FP32 rounding, not truncation, sets it -- and the cutoffs shrink)
  const double eps = env_double ("LIBSTOKES_GB300_MIXED_EPS", 3e-8);
  // minimum image unless asked otherwise: with the real space overlapping
  // the back-projection, lattice images were faster at no measured size
  // (FTS N = 256-512 level at eta 8; N = 4096 283 against 273 us; N = 8192
  // and 16384 level at eta 11, where the cutoff is below half the box)
  bool images = env_double ("LIBSTOKES_GB300_MIXED_IMAGES", 0.0) != 0.0;
  double eta = env_double ("LIBSTOKES_GB300_MIXED_ETA",
                           images ? default_eta_images (sys->np)
                                  : default_eta (sys->version, sys->np));
  uint64_t fp = mix_fingerprint (sys, eta + (images ? 1000.0 : 0.0), eps);
  const bool poly = c->mode == MODE_POLY;
  double amax = 1.0;
  if (poly)
    {
      // the radii enter the split (xi a_max <= 0.5) and every table
      amax = 0.0;
      for (int q = 0; q < sys->np; q++)
        {
          amax = std::max (amax, sys->a[q]);
          uint64_t b;
          memcpy (&b, &sys->a[q], sizeof b);
          fp = (fp ^ b) * 1099511628211ull;
        }
    }
  if (fp == m->fp && m->kt.p) return STOKES_GPU_OK;
  m->poly = poly;
  m->amax = amax;

  const double lmin = fmin (sys->lx, fmin (sys->ly, sys->lz));
  const double lmax = fmax (sys->lx, fmax (sys->ly, sys->lz));
  const double lv = cbrt (sys->lx * sys->ly * sys->lz);
  // xi a <= 0.5 keeps the self, real and reciprocal parts of comparable size
  // (FP32 loses digits to their cancellation when xi a grows)
  const double XI_CAP = 0.5 / amax;
  double xi = std::min (eta / lv, XI_CAP), rc = 0, kc = 0;
  if (!images)
    {
      for (int it = 0; it < 200; it++)
        {
          lsg_ewald_cutoffs (xi, eps, lmin, lmax, &rc, &kc);
          if (rc <= 0.4999 * lmin) break;
          xi *= 1.03;   // the cutoff must stay below half the box (minimum image)
        }
      // a small box would need xi above the cap for a minimum-image cutoff:
      // take lattice images in real space instead (measured: F and FT at
      // L = 6 reached 1e-5 against FP64 at the forced xi, 1e-7 with images)
      if (rc > 0.4999 * lmin || xi > XI_CAP)
        {
          images = true;
          xi = std::min (eta / lv, XI_CAP);
        }
    }
  if (images) lsg_ewald_cutoffs (xi, eps, lmin, lmax, &rc, &kc);
  // lattice offsets within the cutoff of a minimum-image difference (just
  // the zero offset while the cutoff is below half the box)
  {
    std::vector<float4> hi;
    const int nx = (int) ceil (rc / sys->lx + 0.5), ny = (int) ceil (rc / sys->ly + 0.5),
              nz = (int) ceil (rc / sys->lz + 0.5);
    for (int a1 = -nx; a1 <= nx; a1++)
      for (int a2 = -ny; a2 <= ny; a2++)
        for (int a3 = -nz; a3 <= nz; a3++)
          {
            double tx = a1 * sys->lx, ty = a2 * sys->ly, tz = a3 * sys->lz;
            if (sys->shear_mode == 1) tx += a2 * sys->shear_shift;
            else if (sys->shear_mode == 2) tx += a3 * sys->shear_shift;
            // the nearest point of the offset half-box cell must be within reach
            const double ex = std::max (0.0, fabs (tx) - 0.5 * sys->lx
                                               - (sys->shear_mode ? fabs (sys->shear_shift) : 0.0));
            const double ey = std::max (0.0, fabs (ty) - 0.5 * sys->ly);
            const double ez = std::max (0.0, fabs (tz) - 0.5 * sys->lz);
            if (ex * ex + ey * ey + ez * ez > rc * rc) continue;
            hi.push_back (make_float4 ((float) tx, (float) ty, (float) tz, 0.f));
          }
    cudaError_t e = m->img.ensure (sizeof (float4) * hi.size ());
    if (e == cudaSuccess)
      e = cudaMemcpyAsync (m->img.p, hi.data (), sizeof (float4) * hi.size (),
                           cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
    if (e != cudaSuccess) return cuda_fail (e, "mixed real-space images");
    m->nimg = (int) hi.size ();
  }
  m->xi = xi;
  m->rc = rc;
  m->kc = kc;
  m->eta = xi * lv;
  m->eps = eps;
  const double xisp = xi / sqrt (M_PI), xi2 = xi * xi;
  m->selfc[0] = 1.0 - xisp * (6.0 - 40.0 / 3.0 * xi2);
  m->selfc[1] = 0.75 - xisp * xi2 * 10.0;
  m->selfc[2] = 0.9 - xisp * xi2 * (12.0 - 30.24 * xi2);

  // half-space reciprocal vectors inside |k| <= kc (shear-shifted lattice)
  const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly, k0z = 2.0 * M_PI / sys->lz;
  const double sl = sys->shear_shift / sys->lx;
  const double pivol = M_PI / (sys->lx * sys->ly * sys->lz);
  const int B1 = (int) (kc / k0x) + 1;
  const int B2 = (int) (kc / k0y) + 1 + (sys->shear_mode == 1 ? (int) ceil (fabs (sl) * B1) : 0);
  const int B3 = (int) (kc / k0z) + 1 + (sys->shear_mode == 2 ? (int) ceil (fabs (sl) * B1) : 0);
  m->h_k.clear ();
  int M[3] = {0, 0, 0};
  for (int m1 = 0; m1 <= B1; m1++)
    for (int m2 = -B2; m2 <= B2; m2++)
      for (int m3 = -B3; m3 <= B3; m3++)
        {
          // half space: m1 > 0, or m1 == 0 and (m2 > 0 or (m2 == 0 and m3 > 0))
          if (m1 == 0 && (m2 < 0 || (m2 == 0 && m3 <= 0))) continue;
          const double k1 = k0x * m1;
          double k2 = k0y * m2, k3 = k0z * m3;
          if (sys->shear_mode == 1) k2 = k0y * ((double) m2 - sl * (double) m1);
          else if (sys->shear_mode == 2) k3 = k0z * ((double) m3 - sl * (double) m1);
          const double kk = k1 * k1 + k2 * k2 + k3 * k3;
          const double k = sqrt (kk);
          if (k > kc) continue;
          const double k4z = kk / 4.0 / xi2;
          const double kexp = pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          MixK r;
          memset (&r, 0, sizeof r);
          r.m1 = m1; r.m2 = m2; r.m3 = m3;
          r.ex = (float) (k1 / k); r.ey = (float) (k2 / k); r.ez = (float) (k3 / k);
          if (poly)
            {
              // the per-k factors of the unequal-radius weights
              // (mk_backproj_poly); G with the xi-independent sign
              r.ya = (float) kexp;
              r.yb = (float) k;
              r.yc = (float) kk;
              r.yg = (float) -kexp;
              r.yh = r.ym = 0.f;
            }
          else
            {
              r.ya = (float) (6.0 * (1.0 - kk / 3.0) * kexp);
              r.yb = (float) (3.0 * k * kexp);
              r.yc = (float) (1.5 * kk * kexp);
              // G coupling with the sign that makes real + reciprocal
              // independent of xi (the opposite of libstokes'
              // src/ewald.c:1060-1066)
              r.yg = (float) (-3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp);
              r.yh = (float) (1.5 * kk * kexp);
              r.ym = (float) (3.0 * (1.0 - kk / 5.0) * kk * kexp);
            }
          m->h_k.push_back (r);
          M[0] = std::max (M[0], abs (m1));
          M[1] = std::max (M[1], abs (m2));
          M[2] = std::max (M[2], abs (m3));
        }
  m->nk_split = (int) m->h_k.size ();
  // libstokes' FTS result depends on its own xi through the sign of its
  // reciprocal G term: y_ref = y_xi_invariant + 2 G_ref(xi_ref), where G_ref is
  // the reciprocal G part as libstokes evaluates it.  Add that term on the
  // reference's own k set (half space; the combine doubles it again).
  if (sys->version == 2)
    {
      const double rxi2 = sys->xi2;
      auto kkey = [] (int a, int b, int c) {
        return ((int64_t) a << 42) ^ ((int64_t) (b + (1 << 20)) << 21) ^ (int64_t) (c + (1 << 20));
      };
      std::unordered_map<int64_t, int> own;
      for (int k = 0; k < m->nk_split; k++)
        own.emplace (kkey (m->h_k[k].m1, m->h_k[k].m2, m->h_k[k].m3), k);
      for (int m1 = 0; m1 <= sys->kmaxx; m1++)
        for (int m2 = -sys->kmaxy; m2 <= sys->kmaxy; m2++)
          for (int m3 = -sys->kmaxz; m3 <= sys->kmaxz; m3++)
            {
              if (m1 == 0 && (m2 < 0 || (m2 == 0 && m3 <= 0))) continue;
              const double k1 = k0x * m1;
              double k2 = k0y * m2, k3 = k0z * m3;
              if (sys->shear_mode == 1) k2 = k0y * ((double) m2 - sl * (double) m1);
              else if (sys->shear_mode == 2) k3 = k0z * ((double) m3 - sl * (double) m1);
              const double kk = k1 * k1 + k2 * k2 + k3 * k3;
              const double k = sqrt (kk);
              if (sys->kmax != 0.0 && k > sys->kmax) continue;
              const double k4z = kk / 4.0 / rxi2;
              const double kexp = sys->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
              MixK r;
              memset (&r, 0, sizeof r);
              r.m1 = m1; r.m2 = m2; r.m3 = m3;
              r.ex = (float) (k1 / k); r.ey = (float) (k2 / k); r.ez = (float) (k3 / k);
              if (poly)
                {
                  // the G factor alone (no A, B, C, H, M part)
                  r.ya = 0.f;
                  r.yb = (float) k;
                  r.yc = (float) kk;
                  r.yg = (float) (2.0 * kexp);
                }
              else
                r.yg = (float) (2.0 * 3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp);
              // the operator is linear in its coefficients, so a k vector of
              // the split's own list takes the term into its yg; each (m1,
              // m2, m3) then appears once, which the GEMM path relies on
              const auto hit = own.find (kkey (m1, m2, m3));
              if (hit != own.end ())
                {
                  m->h_k[(size_t) hit->second].yg += r.yg;
                  continue;
                }
              m->h_k.push_back (r);
              M[0] = std::max (M[0], abs (m1));
              M[1] = std::max (M[1], abs (m2));
              M[2] = std::max (M[2], abs (m3));
            }
    }
  if (M[0] > MX_MTAB || M[1] > MX_MTAB || M[2] > MX_MTAB)
    return set_error (STOKES_GPU_ETOOBIG, "mixed split: |m| above %d", MX_MTAB);
  m->M[0] = M[0]; m->M[1] = M[1]; m->M[2] = M[2];
  m->nkh = (int) m->h_k.size ();
  // rows of the tensor-core contraction: the (m2, m3) combinations in use,
  // in (m2, m3) order
  std::vector<int> rowid ((size_t) (2 * M[1] + 1) * (2 * M[2] + 1), -1);
  for (const MixK &k : m->h_k) rowid[(size_t) (k.m2 + M[1]) * (2 * M[2] + 1) + (k.m3 + M[2])] = 0;
  std::vector<int2> rows;
  for (int a = -M[1]; a <= M[1]; a++)
    for (int b = -M[2]; b <= M[2]; b++)
      {
        int &id = rowid[(size_t) (a + M[1]) * (2 * M[2] + 1) + (b + M[2])];
        if (id < 0) continue;
        id = (int) rows.size ();
        rows.push_back (make_int2 (a, b));
      }
  for (MixK &k : m->h_k) k.r = rowid[(size_t) (k.m2 + M[1]) * (2 * M[2] + 1) + (k.m3 + M[2])];
  m->nrow = (int) rows.size ();
  cudaError_t e = m->rowm.ensure (sizeof (int2) * (rows.empty () ? 1 : rows.size ()));
  if (e == cudaSuccess && !rows.empty ())
    e = cudaMemcpyAsync (m->rowm.p, rows.data (), sizeof (int2) * rows.size (),
                         cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  if (e != cudaSuccess) return cuda_fail (e, "mixed row table");
  e = m->kt.ensure (sizeof (MixK) * (m->nkh > 0 ? m->nkh : 1));
  if (e != cudaSuccess) return cuda_fail (e, "mixed k table");
  if (m->nkh)
    {
      e = cudaMemcpyAsync (m->kt.p, m->h_k.data (), sizeof (MixK) * m->nkh,
                           cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
      if (e != cudaSuccess) return cuda_fail (e, "mixed k table");
    }
  m->fp = fp;
  return STOKES_GPU_OK;
}

// Runs `sequence` (the launches of one mixed product on st) directly, or as
// a CUDA graph: the first call with a new configuration launches directly,
// the second records the sequence into a graph (stream capture), later calls
// replay it with one launch.  The configuration key covers the split, every
// buffer, the caller's pointers and the phase events, which the recorded
// nodes hold.  Products inside a profiling window, products issued while
// the caller's stream is itself being captured, and
// LIBSTOKES_GB300_GRAPHS=0 launch directly.
template <class Seq>
static int
run_mixed_sequence (Ctx *c, MixedState *m, const double *d_pos, const double *d_x, double *d_y,
                    cudaStream_t st, cudaEvent_t *E, Seq &sequence)
{
  static const bool enabled = [] {
    const char *g = getenv ("LIBSTOKES_GB300_GRAPHS");
    return !(g && strcmp (g, "0") == 0);
  }();
  // the context's own phase events record from inside the graph (event
  // record nodes); a profiling window's ring of events changes per product
  bool use = enabled && !c->kprof_on && (E == nullptr || E == c->ev) && m->plan.stall == 0;
  if (use)
    {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing (st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        use = false;
    }
  if (!use) return sequence ();
  uint64_t key = 1469598103934665603ull;
  auto mix = [&] (uint64_t v) { key = (key ^ v) * 1099511628211ull; };
  mix (m->fp);
  mix (m->img_key);
  mix ((uint64_t) m->tensor);
  mix ((uint64_t) m->nchunk_r);
  mix ((uint64_t) m->real_g);
  mix ((uint64_t) m->nc[0] * 1000003ull + (uint64_t) m->nc[1] * 1009ull + (uint64_t) m->nc[2]);
  mix ((uint64_t) m->nchunk_k);
  const void *ptrs[] = {d_pos, d_x, d_y, m->kt.p, m->qpos.p, m->tab.p, m->xf.p, m->pq.p,
                        m->part_real.p, m->part_rec.p, m->selfbuf.p, m->status.p, m->sf.p,
                        m->rowm.p, m->rot.p, m->img_zf.p, m->img_wb.p, m->h_status, m->tyz.p,
                        m->img.p, m->sq.p, m->cstart.p, m->prad.p, m->pqa.p, m->pself.p};
  for (const void *p : ptrs) mix ((uint64_t) (uintptr_t) p);
  mix ((uint64_t) (uintptr_t) E);
  // a captured cudaEventRecord is only a dependency, not a record: around a
  // replay the start and end events are recorded on the stream itself, and
  // the real-space span is the one of the configuration's last direct launch
  auto replay = [&] () -> int {
    if (E) cudaEventRecord (E[0], st);
    const cudaError_t le = cudaGraphLaunch (m->gexec, st);
    if (E) cudaEventRecord (E[3], st);
    return cuda_ok (le, "mixed product graph");
  };
  if (m->gexec && key == m->gkey) return replay ();
  if (key != m->gcand)
    {
      m->gcand = key;
      return sequence ();
    }
  // second call with this configuration: record it
  if (m->gexec)
    {
      cudaGraphExecDestroy (m->gexec);
      m->gexec = nullptr;
    }
  cudaError_t e = cudaStreamBeginCapture (st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return sequence ();
  const int rc = sequence ();
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture (st, &g);
  if (rc)
    {
      if (g) cudaGraphDestroy (g);
      return rc;
    }
  if (e != cudaSuccess || !g)
    {
      if (g) cudaGraphDestroy (g);
      cudaGetLastError ();
      return sequence ();           // not recorded: launch directly
    }
  e = cudaGraphInstantiate (&m->gexec, g, 0);
  cudaGraphDestroy (g);
  if (e != cudaSuccess)
    {
      m->gexec = nullptr;
      cudaGetLastError ();
      return sequence ();
    }
  m->gkey = key;
  return replay ();
}

int
atimes_mixed_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                  cudaStream_t st, bool timed)
{
  if (c->mode == MODE_SLIP)
    return set_error (STOKES_GPU_EINVAL,
                      "mixed precision serves spheres without slip (libstokes' slip sum depends on "
                      "its own xi); use STOKES_GPU_FP64");
  if (c->mode == MODE_POLY && c->sys->rmin > 0.0)
    return set_error (STOKES_GPU_EINVAL,
                      "mixed precision with unequal radii needs rmin = 0; use STOKES_GPU_FP64");
  if (c->open)
    return set_error (STOKES_GPU_EINVAL,
                      "mixed precision serves periodic systems; the free-space operator runs in FP64");
  if (!c->mixed) c->mixed = new MixedState ();
  MixedState *m = c->mixed;
  const struct stokes *sys = c->sys;
  int rc = mixed_setup (c, sys, m);
  if (rc) return rc;
  const int np = c->np, C = NCOMP (c->version);
  const int ntab = (m->M[0] + 1) + (m->M[1] + 1) + (m->M[2] + 1);
  // the real-space sum: G warps per target; its hi + lo output is two
  // combine chunks.  Measured on one GB300 (FTS, phi 0.3, G = 1, 2, 4, 8):
  // best G 4 at N = 1000 (minimum-image split) and 4096, 2 at 16384, 1 at
  // 32768 -- about 4K to 32K warps in all, enough to balance the SMs
  // without many per-warp reductions
  m->nchunk_r = sys->rmin > 0.0 ? 3 : 2;       // + the clamp kernel's sums
  {
    int g = np <= 512 ? 8 : (np <= 4096 ? 4 : (np <= 16384 ? 2 : 1));
    const int ge = (int) env_double ("LIBSTOKES_GB300_REAL_G", 0.0);
    if (ge == 1 || ge == 2 || ge == 4 || ge == 8) g = ge;
    m->real_g = g;
  }
  // cell list when the box holds at least 6 cells of side >= rc / 2 per axis
  // (5 x 5 x 5 neighbouring cells then prune the candidates) on an
  // unsheared lattice with the minimum image alone
  {
    int nc[3];
    const double L[3] = {sys->lx, sys->ly, sys->lz};
    bool ok = sys->shear_mode == 0 && m->nimg == 1
              && env_double ("LIBSTOKES_GB300_CELLS", 1.0) != 0.0;
    for (int d = 0; d < 3; d++)
      {
        nc[d] = std::min (10, (int) floor (2.0 * L[d] / m->rc));
        ok = ok && nc[d] >= 6;
      }
    if (ok && nc[0] * nc[1] * nc[2] > CELL_MAX) ok = false;
    for (int d = 0; d < 3; d++) m->nc[d] = ok ? nc[d] : 0;
  }
  const size_t off1 = (size_t) (m->M[0] + 1) * np;
  const size_t off2 = off1 + (size_t) (m->M[1] + 1) * np;
  PhaseTables pt{(const float2 *) m->tab.p, off1, off2, m->M[0], m->M[1], m->M[2], np,
                 (const uint4 *) m->qpos.p, (const float4 *) m->rot.p};
  {
    // reciprocal space on the tensor cores unless LIBSTOKES_GB300_KSPACE=simt
    const char *ks = getenv ("LIBSTOKES_GB300_KSPACE");   // read per call: tests switch it
    m->plan = kgemm_plan (c->version, pt, (const int2 *) m->rowm.p, m->nrow);
    m->plan.stall = g_test_gemm_stall;
    m->tensor = !(ks && strcmp (ks, "simt") == 0) && !m->poly && m->nkh > 0
                && kgemm_fits (m->plan);
  }
  if (m->tensor)
    m->nchunk_k = kgemm_ypart_chunks (m->plan);
  else
    {
      m->nchunk_k = std::max (1, std::min (64, (152 * 48 + np - 1) / np));
      if (m->nchunk_k * 32 > m->nkh) m->nchunk_k = std::max (1, m->nkh / 32);
    }
  // a status word raised by a bounded device wait of the previous product
  if (m->h_status && *m->h_status)
    {
      *m->h_status = 0;
      cudaMemsetAsync (m->status.p, 0, sizeof (int), st);
      return set_error (STOKES_GPU_ETIMEOUT,
                        "a tensor-core wait of the previous mixed product ran out");
    }
  cudaError_t e;
  if (!m->h_status)
    {
      if ((e = cudaMallocHost (&m->h_status, sizeof (int))) != cudaSuccess) return cuda_fail (e, "status");
      *m->h_status = 0;
      if ((e = m->status.ensure (sizeof (int))) != cudaSuccess) return cuda_fail (e, "status");
      cudaMemsetAsync (m->status.p, 0, sizeof (int), st);
    }
  if (!m->side)
    {
      int lo = 0, hi = 0;
      cudaDeviceGetStreamPriorityRange (&lo, &hi);
      if (cudaStreamCreateWithPriority (&m->side, cudaStreamNonBlocking, lo) != cudaSuccess
          || cudaEventCreateWithFlags (&m->ev_fork, cudaEventDisableTiming) != cudaSuccess
          || cudaEventCreateWithFlags (&m->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return set_error (STOKES_GPU_ECUDA, "mixed product: side stream");
    }
  if ((e = m->qpos.ensure (sizeof (uint32_t) * 4 * np)) != cudaSuccess) return cuda_fail (e, "qpos");
  if ((e = m->tab.ensure (sizeof (float2) * (size_t) ntab * np)) != cudaSuccess) return cuda_fail (e, "phase tables");
  m->plan.t.tab = (const float2 *) m->tab.p;
  if ((e = m->xf.ensure (sizeof (float) * (size_t) cpad (C) * np)) != cudaSuccess) return cuda_fail (e, "xf");
  if (m->nc[0])
    {
      const int ncell = m->nc[0] * m->nc[1] * m->nc[2];
      if ((e = m->sq.ensure (sizeof (uint4) * np)) != cudaSuccess) return cuda_fail (e, "cell order");
      if ((e = m->cstart.ensure (sizeof (int) * (ncell + 1))) != cudaSuccess) return cuda_fail (e, "cell starts");
      if ((e = cudaFuncSetAttribute (mk_cells, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int) sizeof (int) * 32 * CELL_MAX)) != cudaSuccess)
        return cuda_fail (e, "cell kernel attribute");
    }
  if (m->tensor)
    {
      if ((e = m->sf.ensure (sizeof (float) * kgemm_sf_floats (m->plan))) != cudaSuccess) return cuda_fail (e, "structure factors");
      if ((e = m->img_zf.ensure (sizeof (float) * kgemm_zf_floats (m->plan))) != cudaSuccess) return cuda_fail (e, "image ZF");
      if ((e = m->img_wb.ensure (sizeof (float) * kgemm_wb_floats (m->plan))) != cudaSuccess) return cuda_fail (e, "image WB");
      m->plan.ZF = (float *) m->img_zf.p;
      m->plan.WB = (float *) m->img_wb.p;
      m->plan.sf = (float *) m->sf.p;
      const int wyz = (2 * m->M[1] + 1) + (2 * m->M[2] + 1);
      if ((e = m->tyz.ensure (sizeof (float2) * (size_t) wyz * np)) != cudaSuccess)
        return cuda_fail (e, "phase table (particle-major)");
      m->plan.t.tyz = (const float2 *) m->tyz.p;
      m->plan.t.wyz = wyz;
    }
  else if ((e = m->pq.ensure (sizeof (float) * (m->poly ? 4 : 2) * C
                               * (size_t) (m->nkh > 0 ? m->nkh : 1))) != cudaSuccess)
    return cuda_fail (e, "pq");
  if ((e = m->part_real.ensure (sizeof (float) * (size_t) m->nchunk_r * np * C)) != cudaSuccess) return cuda_fail (e, "real partials");
  if ((e = m->part_rec.ensure (sizeof (float) * (size_t) m->nchunk_k * np * C)) != cudaSuccess) return cuda_fail (e, "k partials");
  // the self block as a C x C matrix, rebuilt when the split changes; with
  // unequal radii the unit block, scaled per particle by its self terms
  if (m->fp != m->self_fp || !m->selfbuf.p)
    {
      if ((e = m->selfbuf.ensure (sizeof (double) * C * C)) != cudaSuccess) return cuda_fail (e, "self");
      double *S = (double *) m->selfbuf.p;
      const double s0 = m->poly ? 1.0 : m->selfc[0], s1 = m->poly ? 1.0 : m->selfc[1],
                   s2 = m->poly ? 1.0 : m->selfc[2];
      if (c->version == 0) mk_selfmat<0><<<1, 32, 0, st>>> (s0, s1, s2, S);
      else if (c->version == 1) mk_selfmat<1><<<1, 32, 0, st>>> (s0, s1, s2, S);
      else mk_selfmat<2><<<1, 32, 0, st>>> (s0, s1, s2, S);
      if ((e = cudaStreamSynchronize (st)) != cudaSuccess) return cuda_fail (e, "mixed self matrix");
      m->self_fp = m->fp;
    }
  if (m->poly && m->poly_fp != m->fp)
    {
      // radii, squared radii and the self terms at the split
      // (src/ewald.c:579-642 with this split's xi)
      std::vector<float> r ((size_t) np), q ((size_t) np);
      std::vector<double> sf ((size_t) 3 * np);
      const double xisp = m->xi / sqrt (M_PI), xi2 = m->xi * m->xi;
      for (int i = 0; i < np; i++)
        {
          const double a = sys->a[i], a2 = a * a, a3 = a2 * a;
          r[i] = (float) a;
          q[i] = (float) a2;
          sf[3 * i] = 1.0 - a * xisp * (6.0 - 40.0 / 3.0 * xi2 * a2);
          sf[3 * i + 1] = 0.75 - a3 * xisp * xi2 * 10.0;
          sf[3 * i + 2] = 0.9 - a3 * xisp * xi2 * (12.0 - 30.24 * xi2 * a2);
        }
      if ((e = m->prad.ensure (sizeof (float) * np)) != cudaSuccess
          || (e = m->pqa.ensure (sizeof (float) * np)) != cudaSuccess
          || (e = m->pself.ensure (sizeof (double) * 3 * np)) != cudaSuccess)
        return cuda_fail (e, "particle tables");
      e = cudaMemcpyAsync (m->prad.p, r.data (), sizeof (float) * np, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync (m->pqa.p, q.data (), sizeof (float) * np, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync (m->pself.p, sf.data (), sizeof (double) * 3 * np,
                             cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) return cuda_fail (e, "particle tables");
      m->poly_fp = m->fp;
    }
  // 1024 rotations e^{2 pi i h / 1024} as FP32 pairs hi + lo, made once
  if (!m->rot.p)
    {
      std::vector<float> h (4 * 1024);
      for (int k = 0; k < 1024; k++)
        {
          const double c0 = cos (2.0 * M_PI * k / 1024.0), s0 = sin (2.0 * M_PI * k / 1024.0);
          h[4 * k] = (float) c0;
          h[4 * k + 1] = (float) s0;
          h[4 * k + 2] = (float) (c0 - (double) h[4 * k]);
          h[4 * k + 3] = (float) (s0 - (double) h[4 * k + 1]);
        }
      if ((e = m->rot.ensure (sizeof (float) * 4 * 1024)) != cudaSuccess) return cuda_fail (e, "rotations");
      e = cudaMemcpyAsync (m->rot.p, h.data (), sizeof (float) * 4 * 1024, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) return cuda_fail (e, "rotations");
    }

  m->plan.t.qpos = (const uint4 *) m->qpos.p;
  m->plan.t.rot = (const float4 *) m->rot.p;
  if (m->tensor)
    {
      // the pads of ZF and the (row, m1) slots of WB that no k vector owns
      // stay zero; zeroed, and the TMA maps encoded, when the split or the
      // buffers change
      uint64_t key = m->fp * 1000003ull;
      for (const void *p : {(const void *) m->img_zf.p, (const void *) m->img_wb.p,
                            (const void *) m->sf.p})
        key = (key ^ (uint64_t) (uintptr_t) p) * 1099511628211ull;
      if (key != m->img_key)
        {
          e = cudaMemsetAsync (m->img_zf.p, 0, sizeof (float) * kgemm_zf_floats (m->plan), st);
          if (e == cudaSuccess)
            e = cudaMemsetAsync (m->img_wb.p, 0, sizeof (float) * kgemm_wb_floats (m->plan), st);
          if (e != cudaSuccess) return cuda_fail (e, "GEMM images");
          const int me = kgemm_maps (m->plan, (float *) m->sf.p, &m->maps);
          if (me) return set_error (STOKES_GPU_ECUDA, "TMA tensor maps of the GEMM images (%d)", me);
          m->img_key = key;
        }
    }

  cudaEvent_t *E = phase_events (c, timed);
  // the launch sequence of one product (kernels, copies and stream events);
  // recorded into a CUDA graph once the same configuration repeats
  auto sequence = [&] () -> int {
    if (E) cudaEventRecord (E[0], st);
    kmark (c, st, nullptr);
    PrepArgs pa;
    pa.pos = d_pos; pa.x = d_x; pa.np = np; pa.c = C;
    {
      const double two32 = 4294967296.0;
      pa.sx = two32 / sys->lx; pa.sy = two32 / sys->ly; pa.sz = two32 / sys->lz;
    }
    pa.shift = sys->shear_shift;
    pa.sl = sys->shear_shift / sys->lx;
    pa.shear_mode = sys->shear_mode;
    pa.ntab = ntab;
    pa.m0end = m->M[0] + 1;
    pa.m1end = m->M[0] + m->M[1] + 2;
    pa.rot = (const float4 *) m->rot.p;
    pa.qpos = (uint32_t *) m->qpos.p; pa.tab = (float2 *) m->tab.p; pa.xf = (float *) m->xf.p;
    pa.zf = m->tensor ? m->plan.ZF : nullptr;
    pa.zplane = m->plan.pZF;
    pa.kf = m->plan.KF;
    pa.tyz = m->tensor ? (float2 *) m->tyz.p : nullptr;
    pa.wyz = (2 * m->M[1] + 1) + (2 * m->M[2] + 1);
    pa.M1 = m->M[1];
    pa.M2 = m->M[2];
    mk_prep<<<dim3 ((np + PREP_P - 1) / PREP_P, (ntab + PREP_ROWS - 1) / PREP_ROWS), 128, 0, st>>> (pa);
    kmark (c, st, "mk_prep");

    RealMixArgs ra;
    memset (&ra, 0, sizeof ra);
    ra.qpos = (const uint32_t *) m->qpos.p; ra.xf = (const float *) m->xf.p;
    ra.np = np; ra.G = m->real_g;
    const double two32 = 4294967296.0;
    ra.scale[0] = (float) (sys->lx / two32);
    ra.scale[1] = (float) (sys->ly / two32);
    ra.scale[2] = (float) (sys->lz / two32);
    ra.shear_mode = sys->shear_mode;
    {
      double sq = sys->shear_shift / sys->lx * two32;
      long long iq = llround (sq);
      ra.shift_q = (uint32_t) (iq & 0xffffffffll);
    }
    ra.rc2 = (float) (m->rc * m->rc);
    ra.rmin = (float) sys->rmin;
    ra.xi = (float) m->xi;
    ra.xisp = (float) (m->xi / sqrt (M_PI));
    ra.rad = m->poly ? (const float *) m->prad.p : nullptr;
    ra.slipa = nullptr;
    ra.clampfix = sys->rmin > 0.0 ? 1 : 0;
    ra.rm2 = (float) (4.0 * sys->rmin * sys->rmin);
    ra.out_clamp = (float *) m->part_real.p + (size_t) 2 * np * C;
    ra.xi_ref = (float) sys->xi;
    ra.xisp_ref = (float) (sys->xi / sqrt (M_PI));
    ra.out = (float *) m->part_real.p;
    ra.img = (const float4 *) m->img.p;
    ra.nimg = m->nimg;
    if (m->nc[0])
      {
        ra.sq = (const uint4 *) m->sq.p;
        ra.cstart = (const int *) m->cstart.p;
        for (int d = 0; d < 3; d++) ra.nc[d] = m->nc[d];
      }
    const int tpc = RG_WARPS / m->real_g;
    const int gr = (np + tpc - 1) / tpc;
    // concurrent with the reciprocal chain unless a profiling window times
    // the launches one by one (then in order: reciprocal, real, combine).
    // The host call's own timing (E == c->ev) keeps the overlap and times
    // the real space on the side stream
    const bool overlap = (!E || E == c->ev) && !c->kprof_on && m->side;
    auto launch_real = [&] (cudaStream_t rs) {
      if (m->nc[0])
        {
          const int ncell = m->nc[0] * m->nc[1] * m->nc[2];
          mk_cells<<<1, CELL_THREADS, sizeof (int) * 32 * ncell, rs>>> (
            (const uint4 *) m->qpos.p, np, m->nc[0], m->nc[1], m->nc[2], (int *) m->cstart.p,
            (uint4 *) m->sq.p);
          kmark (c, rs, "mk_cells");
        }
      if (m->poly)
        {
          if (c->version == 0) mk_real<0, true><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
          else if (c->version == 1) mk_real<1, true><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
          else mk_real<2, true><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
        }
      else if (c->version == 0) mk_real<0, false><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
      else if (c->version == 1) mk_real<1, false><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
      else mk_real<2, false><<<gr, RG_WARPS * 32, 0, rs>>> (ra);
      if (ra.clampfix)
        {
          const int gc = (np + 7) / 8;
          if (c->version == 0) mk_clamp<0><<<gc, 256, 0, rs>>> (ra);
          else if (c->version == 1) mk_clamp<1><<<gc, 256, 0, rs>>> (ra);
          else mk_clamp<2><<<gc, 256, 0, rs>>> (ra);
        }
    };
    // the real space depends on mk_prep only and joins before the combine;
    // on the tensor-core path its launch is recorded after the forward
    // GEMM's, so the GEMM takes the SMs first and the real-space CTAs fill
    // what the chain leaves idle up to the back-projection (measured, one
    // GB300: FTS N = 256 49 -> 39 us, FT N = 2048 123 -> 112 us, FTS
    // N = 4096 295 -> 283 us, N = 1000 unchanged)
    auto fork_real = [&] () {
      cudaStreamWaitEvent (m->side, m->ev_fork, 0);
      if (E) cudaEventRecord (E[1], m->side);
      launch_real (m->side);
      if (E) cudaEventRecord (E[2], m->side);
      cudaEventRecord (m->ev_join, m->side);
    };
    const bool fused = m->nkh > 0 && m->tensor;
    if (overlap)
      {
        cudaEventRecord (m->ev_fork, st);
        if (!fused) fork_real ();
      }

    KMixArgs ka;
    ka.kt = (const MixK *) m->kt.p; ka.tab = (const float2 *) m->tab.p;
    ka.xf = (const float *) m->xf.p; ka.np = np; ka.nkh = m->nkh;
    ka.off1 = off1; ka.off2 = off2; ka.pq = (float *) m->pq.p;
    BpMixArgs ba;
    ba.kt = ka.kt; ba.tab = ka.tab; ba.pq = ka.pq; ba.np = np; ba.nkh = m->nkh;
    ba.nchunk = m->nchunk_k; ba.M0 = m->M[0]; ba.M1 = m->M[1]; ba.M2 = m->M[2];
    ba.off1 = off1; ba.off2 = off2; ba.partial = (float *) m->part_rec.p;
    const int gk = (m->nkh + MX_WARPS - 1) / MX_WARPS;
    const int gb = (int) (((long long) np * m->nchunk_k + MX_WARPS - 1) / MX_WARPS);
    CombineArgs cb;
    cb.x = d_x;
    cb.pr = (const float *) m->part_real.p;
    cb.ncr = m->nchunk_r;
    cb.pk = (const float *) m->part_rec.p;
    cb.nck = m->nchunk_k;
    cb.S = (const double *) m->selfbuf.p;
    cb.selfp = m->poly ? (const double *) m->pself.p : nullptr;
    cb.np = np;
    cb.c = C;
    cb.y = d_y;
    // reciprocal space up to the k operators (tensor cores) or the SIMT sums;
    // then the real-space partials, the back-projection and the final sum
    if (fused)
      {
        if ((e = launch_kspace_forward (c->version, m->plan, m->maps, ka.kt, m->nkh,
                                        (int *) m->status.p, st, c)) != cudaSuccess)
          return cuda_fail (e, "reciprocal space (tensor cores)");
        if (overlap) fork_real ();
      }
    else if (m->nkh > 0 && m->poly)
      {
        const float *qa = (const float *) m->pqa.p, *rad = (const float *) m->prad.p;
        if (c->version == 0) mk_sfac_poly<0><<<gk, MX_WARPS * 32, 0, st>>> (ka, qa);
        else if (c->version == 1) mk_sfac_poly<1><<<gk, MX_WARPS * 32, 0, st>>> (ka, qa);
        else mk_sfac_poly<2><<<gk, MX_WARPS * 32, 0, st>>> (ka, qa);
        kmark (c, st, "mk_sfac_poly");
        if (c->version == 0) mk_backproj_poly<0><<<gb, MX_WARPS * 32, 0, st>>> (ba, rad);
        else if (c->version == 1) mk_backproj_poly<1><<<gb, MX_WARPS * 32, 0, st>>> (ba, rad);
        else mk_backproj_poly<2><<<gb, MX_WARPS * 32, 0, st>>> (ba, rad);
        kmark (c, st, "mk_backproj_poly");
      }
    else if (m->nkh > 0)
      {
        if (c->version == 0) mk_sfac<0><<<gk, MX_WARPS * 32, 0, st>>> (ka);
        else if (c->version == 1) mk_sfac<1><<<gk, MX_WARPS * 32, 0, st>>> (ka);
        else mk_sfac<2><<<gk, MX_WARPS * 32, 0, st>>> (ka);
        kmark (c, st, "mk_sfac");
        if (c->version == 0) mk_backproj<0><<<gb, MX_WARPS * 32, 0, st>>> (ba);
        else if (c->version == 1) mk_backproj<1><<<gb, MX_WARPS * 32, 0, st>>> (ba);
        else mk_backproj<2><<<gb, MX_WARPS * 32, 0, st>>> (ba);
        kmark (c, st, "mk_backproj");
      }
    else
      cudaMemsetAsync (m->part_rec.p, 0, sizeof (float) * (size_t) m->nchunk_k * np * C, st);
    if (!overlap)
      {
        if (E) cudaEventRecord (E[1], st);
        launch_real (st);
        kmark (c, st, "mk_real");
        if (E) cudaEventRecord (E[2], st);
      }
    if (fused
        && (e = launch_kspace_backward (c->version, m->plan, m->maps, (float *) m->part_rec.p,
                                        (int *) m->status.p, st, c)) != cudaSuccess)
      return cuda_fail (e, "reciprocal space (tensor cores)");
    // the real-space partials must be complete before the combine
    if (overlap) cudaStreamWaitEvent (st, m->ev_join, 0);
    mk_combine<<<(np * C + CMB_OUT - 1) / CMB_OUT, CMB_OUT * CMB_WARPS, 0, st>>> (cb);
    kmark (c, st, "mk_combine");
    if (E) cudaEventRecord (E[3], st);
    if (m->tensor)
      cudaMemcpyAsync (m->h_status, m->status.p, sizeof (int), cudaMemcpyDeviceToHost, st);
    e = cudaGetLastError ();
    if (e != cudaSuccess) return cuda_fail (e, "mixed kernels");
    return STOKES_GPU_OK;
  };
  int rs = run_mixed_sequence (c, m, d_pos, d_x, d_y, st, E, sequence);
  if (rs) return rs;
  c->launches = (m->nkh == 0 ? 3 : (m->tensor ? 6 : 5)) + (m->nc[0] ? 1 : 0)
                + (sys->rmin > 0.0 ? 1 : 0);
  c->timed = timed;
  return STOKES_GPU_OK;
}

int
mixed_check_status (Ctx *c)
{
  MixedState *m = c->mixed;
  if (!m || !m->h_status || !*m->h_status) return STOKES_GPU_OK;
  *m->h_status = 0;
  cudaMemsetAsync (m->status.p, 0, sizeof (int), c->stream);
  cudaStreamSynchronize (c->stream);
  return set_error (STOKES_GPU_ETIMEOUT, "a tensor-core wait of the mixed product ran out");
}

void
release_mixed (Ctx *c)
{
  if (!c->mixed) return;
  MixedState *m = c->mixed;
  for (DevBuf *b : {&m->kt, &m->qpos, &m->tab, &m->xf, &m->pq, &m->part_real, &m->part_rec,
                    &m->selfbuf, &m->status, &m->sf, &m->rowm, &m->rot, &m->img_zf,
                    &m->img_wb, &m->tyz, &m->img, &m->sq, &m->cstart})
    b->release ();
  if (m->h_status) cudaFreeHost (m->h_status);
  if (m->gexec) cudaGraphExecDestroy (m->gexec);
  if (m->side) cudaStreamDestroy (m->side);
  if (m->ev_fork) cudaEventDestroy (m->ev_fork);
  if (m->ev_join) cudaEventDestroy (m->ev_join);
  delete m;
  c->mixed = nullptr;
}

// (i, j, image) terms with 0 < r^2 < rc^2 under the test mk_real applies
// (fixed-point minimum image plus the split's lattice offsets, FP32
// distances): the unit count of the mixed real-space roofline
__global__ void
mk_count_real (RealMixArgs a, unsigned long long *count)
{
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long cnt = 0;
  if (t < (long long) a.np * a.np)
    {
      const int i = (int) (t / a.np), j = (int) (t % a.np);
      const uint4 qi = reinterpret_cast<const uint4 *> (a.qpos)[i];
      const uint4 qj = reinterpret_cast<const uint4 *> (a.qpos)[j];
      float d0x, d0y, d0z;
      min_image (a, qi, qj, d0x, d0y, d0z);
      for (int m = 0; m < a.nimg; m++)
        {
          const float4 T = a.img[m];
          const float dx = d0x + T.x, dy = d0y + T.y, dz = d0z + T.z;
          const float rr = dx * dx + dy * dy + dz * dz;
          cnt += (rr > 0.f && rr < a.rc2) ? 1ull : 0ull;
        }
    }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync (0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd (count, cnt);
}

int
mixed_count_real (Ctx *c, long long *out)
{
  if (!c->mixed || !c->mixed->qpos.p)
    return set_error (STOKES_GPU_EINVAL, "no mixed product run yet");
  MixedState *m = c->mixed;
  const struct stokes *sys = c->sys;
  RealMixArgs ra;
  memset (&ra, 0, sizeof ra);
  ra.qpos = (const uint32_t *) m->qpos.p;
  ra.np = c->np;
  const double two32 = 4294967296.0;
  ra.scale[0] = (float) (sys->lx / two32);
  ra.scale[1] = (float) (sys->ly / two32);
  ra.scale[2] = (float) (sys->lz / two32);
  ra.shear_mode = sys->shear_mode;
  ra.shift_q = (uint32_t) (llround (sys->shear_shift / sys->lx * two32) & 0xffffffffll);
  ra.rc2 = (float) (m->rc * m->rc);
  ra.img = (const float4 *) m->img.p;
  ra.nimg = m->nimg;
  DevBuf cnt;
  cudaError_t e = cnt.ensure (sizeof (unsigned long long));
  if (e != cudaSuccess) return cuda_fail (e, "count");
  cudaMemsetAsync (cnt.p, 0, sizeof (unsigned long long), c->stream);
  const long long nt = (long long) c->np * c->np;
  mk_count_real<<<(int) ((nt + 255) / 256), 256, 0, c->stream>>> (ra, (unsigned long long *) cnt.p);
  unsigned long long h = 0;
  e = cudaMemcpyAsync (&h, cnt.p, sizeof h, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  cnt.release ();
  if (e != cudaSuccess) return cuda_fail (e, "count");
  *out = (long long) h;
  return STOKES_GPU_OK;
}

int
mixed_split_info (Ctx *c, double *out)
{
  if (!c->mixed) return set_error (STOKES_GPU_EINVAL, "no mixed product run yet");
  MixedState *m = c->mixed;
  out[0] = m->xi; out[1] = m->rc; out[2] = m->kc; out[3] = m->eta; out[4] = m->eps;
  out[5] = m->nkh; out[6] = m->M[0]; out[7] = m->M[1]; out[8] = m->M[2];
  return STOKES_GPU_OK;
}

}  // namespace lsg

extern "C" int
stokes_gpu_count_mixed_real_terms (struct stokes *sys, long long *count)
{
  using namespace lsg;
  if (!sys || !count) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c) return set_error (STOKES_GPU_EINVAL, "no product run for this system yet");
  return mixed_count_real (c, count);
}

extern "C" int
stokes_gpu_mixed_split (struct stokes *sys, double *info9)
{
  using namespace lsg;
  if (!sys || !info9) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c) return set_error (STOKES_GPU_EINVAL, "no product run for this system yet");
  return mixed_split_info (c, info9);
}
