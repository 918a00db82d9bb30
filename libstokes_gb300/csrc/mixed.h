// mixed.h -- data shared by the mixed-precision host code (mixed.cu) and its
// reciprocal-space tensor-core kernels (kspace_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace lsg {

// one half-space reciprocal vector (64 bytes)
struct __align__ (16) MixK {
  int m1, m2, m3, pad;
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

// structure factors and per-k operators: pq[q * nkh + k] holds P_k[q] for
// q < c and Q_k[q - c] for c <= q < 2c
cudaError_t launch_sfac_tc (int version, const MixK *kt, int nkh, PhaseTables t,
                            const float *xf, float *pq, int *status, cudaStream_t st);

// y_i partial sums over k slices: partial[split][i][q]
cudaError_t launch_backproj_tc (int version, const MixK *kt, int nkh, PhaseTables t,
                                const float *pq, int nsplit, float *partial, int *status,
                                cudaStream_t st);

// number of k slices the back-projection uses for np particles, nkh vectors
int backproj_splits (int np, int nkh);

}  // namespace lsg
