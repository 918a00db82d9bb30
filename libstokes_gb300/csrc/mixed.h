// mixed.h -- data shared by the mixed-precision host code (mixed.cu) and its
// reciprocal-space tensor-core kernels (kspace_tc.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace lsg {

// one half-space reciprocal vector (64 bytes); r: its (m2, m3) row of the
// tensor-core contraction
struct __align__ (16) MixK {
  int m1, m2, m3, r;
  float ex, ey, ez;
  float ya, yb, yc, yg, yh, ym;
  float f0, f1, f2;
};

// per-axis phase tables e^{2 pi i m u_j}: tab[off_d + m * np + j], m = 0..M_d;
// qpos: the 32-bit fixed-point fractional coordinates the tables come from
// (x, y, z, pad per particle); rot: the 1024 rotations of phase_of
struct PhaseTables {
  const float2 *tab;
  size_t off1, off2;
  int M0, M1, M2;
  int np;
  const uint4 *qpos;
  const float4 *rot;
  // particle-major y and z phases for both signs of m: tyz[j wyz + M1 + m2]
  // = e^{2 pi i m2 u_y(j)}, tyz[j wyz + (2 M1 + 1) + M2 + m3] = e^{2 pi i m3
  // u_z(j)}, wyz = (2 M1 + 1) + (2 M2 + 1)
  const float2 *tyz;
  int wyz;
};

// e^{2 pi i p / 2^32} to FP32 accuracy from a fixed-point phase p (turns x
// 2^32): the nearest of 1024 tabulated rotations e^{2 pi i h / 1024} (rot[h]
// = (hi.re, hi.im, lo.re, lo.im), each a float pair hi + lo) times a short
// Taylor series of the remaining angle |theta| <= pi / 1024 (table-driven
// argument reduction).  Truncation errors are below 1e-14; the result
// carries one FP32 rounding (3e-8 measured over 2e6 random phases).
__device__ __forceinline__ float2
phase_of (const float4 *rot, uint32_t p)
{
  const uint32_t h = (p + (1u << 21)) >> 22;             // nearest table entry
  const int32_t r = (int32_t) (p - (h << 22));           // |r| <= 2^21
  const float th = (float) r * 1.4629180792671596e-09f;  // 2 pi / 2^32
  const float t2 = th * th;
  const float sn = th * (1.0f - t2 * (1.0f / 6.0f));     // sin th
  const float dc = t2 * (0.5f - t2 * (1.0f / 24.0f));    // 1 - cos th
  const float4 e = __ldg (rot + (h & 1023u));
  // (e.x + e.z + i (e.y + e.w)) (1 - dc + i sn), small terms first
  const float re = e.x + fmaf (-e.x, dc, fmaf (-e.y, sn, e.z));
  const float im = e.y + fmaf (-e.y, dc, fmaf (e.x, sn, e.w));
  return make_float2 (re, im);
}

// e^{2 pi i p / 2^32} without a table: the nearest quarter turn q (exact:
// a swap and sign change) and sin, cos of the remaining angle |x| <= pi / 4
// by their Taylor series to x^11 and x^12 in nested (Horner) form; x is
// formed from the exact integer remainder with a two-part 2 pi / 2^32.  The
// truncation errors are below 1e-11; FP32 rounding leaves about 1e-7 at most
// (8.5e-8 measured over 3e6 random phases, 2e-8 on average).  No memory
// access, so it suits kernels whose lanes would otherwise gather from a table.
__device__ __forceinline__ float2
phase_poly (uint32_t p)
{
  const uint32_t q = (p + (1u << 29)) >> 30;             // nearest quarter turn
  const int32_t r = (int32_t) (p - (q << 30));           // |r| <= 2^29
  const float ch = 1.4629180792671596e-09f;               // 2 pi / 2^32 = ch + cl
  const float cl = -4.0709404e-17f;
  const float rh = (float) (r & ~0xFF), rl = (float) (r & 0xFF);
  const float x = fmaf (rh, ch, fmaf (rl, ch, rh * cl));
  const float x2 = x * x;
  float sn = fmaf (-x2, 1.0f / 110.0f, 1.0f);
  sn = fmaf (-x2 * (1.0f / 72.0f), sn, 1.0f);
  sn = fmaf (-x2 * (1.0f / 42.0f), sn, 1.0f);
  sn = fmaf (-x2 * (1.0f / 20.0f), sn, 1.0f);
  sn = fmaf (-x2 * (1.0f / 6.0f), sn, 1.0f);
  sn *= x;
  float cs = fmaf (-x2, 1.0f / 132.0f, 1.0f);
  cs = fmaf (-x2 * (1.0f / 90.0f), cs, 1.0f);
  cs = fmaf (-x2 * (1.0f / 56.0f), cs, 1.0f);
  cs = fmaf (-x2 * (1.0f / 30.0f), cs, 1.0f);
  cs = fmaf (-x2 * (1.0f / 12.0f), cs, 1.0f);
  cs = fmaf (-x2 * 0.5f, cs, 1.0f);
  switch (q & 3u)
    {
    case 0: return make_float2 (cs, sn);
    case 1: return make_float2 (-sn, cs);
    case 2: return make_float2 (-cs, -sn);
    default: return make_float2 (sn, -cs);
    }
}

// plan of the separable tensor-core reciprocal sum (kspace_tc.cu).  The k
// vectors of the list are (m1, row) with row = one (m2, m3) combination that
// occurs in it; R rows, n1 = M0 + 1 values of m1.  The B operands of the
// GEMMs are images [2 planes: TF32 hi, lo][rows][K] in FP32 (K contiguous):
//   ZF [NZ][KF]  rows (m1, re|im, q): t0[m1](j) x_q(j) in the forward sign pattern
//   WB [NZ][KB]  rows (m1, re|im, q): the k operators W in the backward pattern
// The A operands (the row phases T_r(j)) are built in shared memory by the
// GEMM kernels themselves.
struct KGemm {
  PhaseTables t;
  const int2 *rowm;       // (m2, m3) of each row, R entries
  int R, Rk, Rp;          // rows; padded to 16 (backward K) and 32 (partials)
  int c;                  // components per particle (3, 6, 11)
  int n1;                 // M0 + 1
  int nrt;                // forward row tiles of 128 rows
  int gf, ntile_f, nf;    // m1 per forward column tile, tiles, MMA N
  int jper, nsplit;       // particles per forward K slice, number of slices
  int gb, ntile_b, nb;    // m1 per backward column tile, tiles, MMA N
  int mtiles;             // 128-particle row tiles of the backward GEMM
  int rper, ksplit;       // rows per backward K slice, number of slices
  int ldT;                // particles padded to a multiple of 16
  int KF, KB, NZ;         // K extents (floats) of the images, rows of ZF and WB
  float *ZF, *WB;
  size_t pZF, pWB;        // plane strides (floats)
  float *sf;              // forward partials [nsplit][n1][c][re|im][Rp]
  int stall;              // > 0 (tests only): the MMA lane first waits that many
                          // polls on an mbarrier that nothing arrives at
};

// TMA descriptors of the two images (128-byte swizzled boxes of 32 K values)
// and of the forward partials sf (boxes of 128 rows x one m1's columns)
struct KMaps {
  CUtensorMap zf, wb, sf;
};

KGemm kgemm_plan (int version, PhaseTables t, const int2 *rowm, int R);
bool kgemm_fits (const KGemm &g);
size_t kgemm_sf_floats (const KGemm &g);      // partial structure factors
size_t kgemm_zf_floats (const KGemm &g);      // image sizes, both planes
size_t kgemm_wb_floats (const KGemm &g);
size_t kgemm_ypart_floats (const KGemm &g);   // partial y, [ksplit][ntile_b][np][c]
int kgemm_ypart_chunks (const KGemm &g);       // ksplit * ntile_b
int kgemm_maps (const KGemm &g, float *sf, KMaps *m);   // 0 on success

// forward GEMM -> per-k operators (image WB); then the backward GEMM into
// ypart.  The image ZF is written beforehand by mk_prep.
struct Ctx;
cudaError_t launch_kspace_forward (int version, const KGemm &g, const KMaps &maps, const MixK *kt,
                                   int nk, int *status, cudaStream_t st, Ctx *prof);
cudaError_t launch_kspace_backward (int version, const KGemm &g, const KMaps &maps, float *ypart,
                                    int *status, cudaStream_t st, Ctx *prof);

}  // namespace lsg
