// engine.h -- internal interface between the host engine (gpu_engine.cu)
// and the kernel files.  Not installed; the public ABI is include/*.h.
#pragma once

#include <cuda_runtime.h>

#define NCOMP(v) ((v) == 0 ? 3 : ((v) == 1 ? 6 : 11))

namespace lsg {

// particle kinds: equal spheres, unequal radii, slip
enum Mode { MODE_MONO = 0, MODE_POLY = 1, MODE_SLIP = 2 };

// one real-space image: displacement (x, y, z) added to r_j - r_i; w unused
struct __align__ (32) Img4 { double x, y, z, w; };

// reciprocal-vector table, one row of KT_STRIDE doubles per k
enum {
  KT_KX = 0, KT_KY, KT_KZ,      // k vector (shear-shifted)
  KT_EX, KT_EY, KT_EZ,          // k / |k|
  KT_K, KT_KK, KT_KEXP,         // |k|, |k|^2, pi/V (1 + k4z (1 + 2 k4z)) / k^2 exp(-k4z)
  KT_YA, KT_YB, KT_YC, KT_YG, KT_YH, KT_YM,  // equal-sphere weights
  // unequal radii: factors of the G coefficient and of all the others on
  // the weights the kernels derive from KT_KEXP (1 and 1 but in the tuned
  // split's G correction)
  KT_GF, KT_AF,
  KT_STRIDE = 18
};

// structure-factor row per k: C | S | Cq | Sq, each up to 11 values
constexpr int SF_STRIDE = 44;

struct RealArgs {
  const double *pos;    // [np*3]
  const double *x;      // [np*c]
  const Img4 *img;   // images (dx, dy, dz, 0), shear shift included
  int nimg;
  int np;
  int nchunk;           // source chunks per target (parallel slack)
  double rmax2;
  double rmin;
  double xi, xisp;      // xi, xi/sqrt(pi)
  const double *rad;    // radii (or 1) [np], NULL for equal spheres
  const double *slipa;  // slip-effective radii [np] (slip mode)
  double *partial;      // [nchunk][np][c]
  int open = 0;         // non-periodic: free-space scalars (src/non-ewald.c)
  // rmin clamp at a split other than the struct's own: the clamped pairs
  // take the clamp's change at the struct's split xi_ref (clampfix = 1)
  int clampfix = 0;
  double xi_ref = 0.0, xisp_ref = 0.0;
};

struct RecipArgs {
  const double *x;
  const double2 *ph;    // [nk][np] (cos, sin)(k.r_j)
  const double *kt;     // [nk][KT_STRIDE]
  const double *rad;    // [np] radii (or 1)   (poly / slip)
  const double *qa;     // [np] squared Laplacian radius (poly / slip)
  int nk, np;
  double *sf;           // [nk][SF_STRIDE]
  double *yrec;         // [np*c]
};

struct MatArgs {
  const double *pos;
  const Img4 *img;
  int nimg, np, nk;
  double rmax2, rmin, xi, xisp;
  const double *rad, *slipa, *qa;
  const double *selfc;  // [np][3] self_a, self_c, self_m
  const double *kt;
  const double2 *ph;
  double *mat;
  int open = 0;         // non-periodic: free-space scalars (src/non-ewald.c)
  int f32 = 0;          // equal spheres: FP32 terms (k_matrix_f32), with
  const float4 *imgf = nullptr;   // the images as hi + lo floats,
  const float4 *imgl = nullptr;
  const float *ktf = nullptr;     // [nk][KTF_STRIDE]: e, ya, yb, yc, yg, yh, ym
  const float2 *phf = nullptr;    // [nk][np] phases
};

cudaError_t launch_real_fp64 (int version, int mode, const RealArgs &a, cudaStream_t st);
cudaError_t launch_phase_fp64 (const double *pos, const double *kt, int nk, int np,
                               double2 *ph, cudaStream_t st);
cudaError_t launch_recip_fp64 (int version, int mode, const RecipArgs &a, cudaStream_t st);
cudaError_t launch_combine_fp64 (int version, const double *x, const double *partial,
                                 int nchunk, const double *yrec, const double *selfc,
                                 int np, double *y, cudaStream_t st);
cudaError_t launch_matrix_fp64 (int version, int mode, const MatArgs &a, cudaStream_t st);
constexpr int KTF_STRIDE = 12;   // floats per reciprocal vector of the FP32 builder

// thread-per-pair split-precision dense builder (equal spheres, no shear, no
// clamp) at its own split: the lattice images of each pair are enumerated
// from the box, the reciprocal vectors form a half-space table with doubled
// weights
struct MatPairArgs {
  const double *pos;
  int np;
  double *mat;
  double lx, ly, lz, ilx, ily, ilz;    // box and its inverse
  float lxh, lyh, lzh, lxl, lyl, lzl;  // box as hi + lo floats
  float ilxf, ilyf, ilzf;
  float rc, rc2, xi, xisp;
  double xi64;                         // xi in FP64 (the diagonal blocks)
  double self[3];                      // self_a, self_c, self_m of the split
  const float *kco;                    // [nk][matrix_kco_stride]: moments per unit phase
  const float2 *phf;                   // [nk][np]
  int nk;
  const float *selfmo;                 // moments of the diagonal blocks
};
int matrix_kco_stride (int version);
cudaError_t launch_matrix_kco (int version, const double *kt, int nk, float *kco,
                               cudaStream_t st);
cudaError_t launch_matrix_self (int version, const MatPairArgs &a, const double *kt,
                                float *selfmo, cudaStream_t st);
cudaError_t launch_matrix_pairs (int version, const MatPairArgs &a, cudaStream_t st);
cudaError_t launch_phase_f32 (const double *pos, const double *kt, int nk, int np, float2 *phf,
                              cudaStream_t st);
cudaError_t launch_gemv_fp64 (int version, const double *mat, const double *x,
                              double *zbuf, int np, double *y, cudaStream_t st);

cudaError_t launch_gemv_rect_fp64 (const double *mat, int n1, int n2, const double *x,
                                   double *y, cudaStream_t st);

}  // namespace lsg
