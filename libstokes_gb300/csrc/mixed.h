// mixed.h -- data shared by the mixed-precision host code (mixed.cu) and its
// reciprocal-space tensor-core kernels (kspace_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace lsg {

// one half-space reciprocal vector (64 bytes); r: its (m2, m3) row of the
// tensor-core contraction
struct __align__ (16) MixK {
  int m1, m2, m3, r;
  float ex, ey, ez;
  float ya, yb, yc, yg, yh, ym;
  float f0, f1, f2;
};

// per-axis phase tables e^{2 pi i m u_j}: tab[off_d + m * np + j], m = 0..M_d
struct PhaseTables {
  const float2 *tab;
  size_t off1, off2;
  int M0, M1, M2;
  int np;
};

// plan of the separable tensor-core reciprocal sum (kspace_tc.cu).  The k
// vectors of the list are (m1, row) with row = one (m2, m3) combination that
// occurs in it; R rows, n1 = M0 + 1 values of m1.
struct KGemm {
  PhaseTables t;
  const int2 *rowm;       // (m2, m3) of each row, R entries
  int R;                  // rows
  int c;                  // components per particle (3, 6, 11)
  int n1;                 // M0 + 1
  int nrt;                // forward row tiles of 64 rows
  int gf, ntile_f, nf;    // m1 per forward column tile, tiles, MMA N
  int jper, nsplit;       // particles per forward K slice, number of slices
  int gb, ntile_b, nb;    // m1 per backward column tile, tiles, MMA N
  int mtiles;             // 128-particle row tiles of the backward GEMM
  int rper, ksplit;       // rows per backward K slice, number of slices
  float2 *T;              // T_r(j) = t1[m2](j) t2[m3](j), [R][ldT]
  int ldT;                // particles padded to a multiple of 16
};

KGemm kgemm_plan (int version, PhaseTables t, const int2 *rowm, int R);
bool kgemm_fits (const KGemm &g);
size_t kgemm_sf_floats (const KGemm &g);      // partial structure factors
size_t kgemm_w_elems (const KGemm &g);        // complex operators W (float2)
size_t kgemm_t_elems (const KGemm &g);        // row phase table T (float2)
size_t kgemm_ypart_floats (const KGemm &g);   // partial y, [ksplit][ntile_b][np][c]
int kgemm_ypart_chunks (const KGemm &g);       // ksplit * ntile_b

// forward GEMM -> per-k operators W -> backward GEMM into ypart
struct Ctx;
cudaError_t launch_kspace_gemm (int version, const KGemm &g, const MixK *kt, int nk,
                                const float *xf, float *sf, float2 *W, float *ypart,
                                int *status, cudaStream_t st, Ctx *prof);

}  // namespace lsg
