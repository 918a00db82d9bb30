// tc_selftest.cu -- known-answer check of the tcgen05 path used by the
// reciprocal-space kernels: one 128 x 16 x 32 product in 3xTF32 through
// TMEM, compared on the host with an FP64 product of the same operands.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gpu_engine.h"
#include "stokes_gpu.h"
#include "tc_umma.cuh"
#include "tma_host.h"

namespace lsg {

// A: 128 x 32 row-major, B: 16 x 32 row-major (rows of B^T); D = A B^T
__global__ void __launch_bounds__ (128)
k_umma_selftest (const float *A, const float *B, float *D, int *status)
{
  __shared__ __align__ (1024) unsigned char sA[2][128 * 32 * 4];
  __shared__ __align__ (1024) unsigned char sB[2][16 * 32 * 4];
  __shared__ __align__ (8) uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int k = 0; k < 32; k++)
    {
      uint32_t hi, lo;
      umma::split_tf32 (A[tid * 32 + k], hi, lo);
      const uint32_t o = umma::off (tid, k, 128);
      *reinterpret_cast<uint32_t *> (&sA[0][o]) = hi;
      *reinterpret_cast<uint32_t *> (&sA[1][o]) = lo;
    }
  if (tid < 16)
    for (int k = 0; k < 32; k++)
      {
        uint32_t hi, lo;
        umma::split_tf32 (B[tid * 32 + k], hi, lo);
        const uint32_t o = umma::off (tid, k, 16);
        *reinterpret_cast<uint32_t *> (&sB[0][o]) = hi;
        *reinterpret_cast<uint32_t *> (&sB[1][o]) = lo;
      }
  if (warp == 0) umma::tmem_alloc (&tslot, 32);
  if (tid == 0)
    {
      umma::mbar_init (&mbar, 1);
      umma::fence_mbar_init ();
    }
  umma::fence_async_smem ();
  umma::fence_before_sync ();
  __syncthreads ();
  umma::fence_after_sync ();
  const uint32_t tmem = tslot;
  if (tid == 0)
    {
      const uint32_t idesc = umma::idesc_tf32 (128, 16);
      for (int s = 0; s < 4; s++)
        {
          const uint64_t ahi = umma::smem_desc (umma::smem_u32 (sA[0]) + s * 4096, 128, 256);
          const uint64_t alo = umma::smem_desc (umma::smem_u32 (sA[1]) + s * 4096, 128, 256);
          const uint64_t bhi = umma::smem_desc (umma::smem_u32 (sB[0]) + s * 512, 128, 256);
          const uint64_t blo = umma::smem_desc (umma::smem_u32 (sB[1]) + s * 512, 128, 256);
          umma::mma_tf32 (tmem, ahi, bhi, idesc, s > 0 ? 1u : 0u);
          umma::mma_tf32 (tmem, ahi, blo, idesc, 1u);
          umma::mma_tf32 (tmem, alo, bhi, idesc, 1u);
        }
      umma::mma_commit (&mbar);
    }
  // every thread must agree before the warp-collective TMEM load
  const bool ok = __syncthreads_and (umma::mbar_wait (&mbar, 0, 1u << 24) ? 1 : 0) != 0;
  umma::fence_after_sync ();
  if (ok)
    {
      float v[16];
      umma::tmem_ld16 (tmem + ((uint32_t) (warp * 32) << 16), v);
      for (int q = 0; q < 16; q++) D[tid * 16 + q] = v[q];
    }
  else if (tid == 0)
    atomicExch (status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, 32);
}

// A: [2 planes (hi, lo)][128][64], B: [2][24][64] FP32 through TMA (box
// 32 columns x 128 or 32 rows, 128-byte swizzle; B rows 24..31 fill zeros),
// D = A B^T over K = 64 in 3xTF32 with the swizzled descriptors
__global__ void __launch_bounds__ (128)
k_tma_selftest (const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                float *D, int *status)
{
  extern __shared__ unsigned char dsm[];
  __shared__ __align__ (8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *base = dsm + ((1024u - (umma::smem_u32 (dsm) & 1023u)) & 1023u);
  // per K tile kt: A hi, A lo (16 KB each), B hi, B lo (4 KB each)
  auto sa = [&] (int kt, int h) { return base + kt * 40960 + h * 16384; };
  auto sb = [&] (int kt, int h) { return base + kt * 40960 + 32768 + h * 4096; };
  if (warp == 0) umma::tmem_alloc (&tslot, 32);
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
  if (tid == 0)
    {
      umma::mbar_expect_tx (&mbar[0], 2 * (16384 + 4096) * 2);
      for (int kt = 0; kt < 2; kt++)
        for (int h = 0; h < 2; h++)
          {
            umma::tma_load_3d (sa (kt, h), &tmA, 32 * kt, 0, h, &mbar[0]);
            umma::tma_load_3d (sb (kt, h), &tmB, 32 * kt, 0, h, &mbar[0]);
          }
      bool ok = umma::mbar_wait (&mbar[0], 0, 1u << 24);
      if (ok)
        {
          umma::fence_after_sync ();
          const uint32_t idesc = umma::idesc_tf32 (128, 32);
          for (int kt = 0; kt < 2; kt++)
            for (int s = 0; s < 4; s++)
              {
                const uint64_t ahi = umma::smem_desc_sw128 (umma::smem_u32 (sa (kt, 0)) + 32 * s);
                const uint64_t alo = umma::smem_desc_sw128 (umma::smem_u32 (sa (kt, 1)) + 32 * s);
                const uint64_t bhi = umma::smem_desc_sw128 (umma::smem_u32 (sb (kt, 0)) + 32 * s);
                const uint64_t blo = umma::smem_desc_sw128 (umma::smem_u32 (sb (kt, 1)) + 32 * s);
                umma::mma_tf32 (tmem, ahi, bhi, idesc, (kt | s) ? 1u : 0u);
                umma::mma_tf32 (tmem, ahi, blo, idesc, 1u);
                umma::mma_tf32 (tmem, alo, bhi, idesc, 1u);
              }
        }
      else
        atomicExch (status, 1);
      umma::mma_commit (&mbar[1]);
    }
  const bool ok = __syncthreads_and (umma::mbar_wait (&mbar[1], 0, 1u << 24) ? 1 : 0) != 0;
  umma::fence_after_sync ();
  if (ok)
    {
      float v[16];
      for (int c = 0; c < 32; c += 16)
        {
          umma::tmem_ld16 (tmem + ((uint32_t) (warp * 32) << 16) + c, v);
          for (int q = 0; q < 16; q++) D[tid * 32 + c + q] = v[q];
        }
    }
  else if (tid == 0)
    atomicExch (status, 1);
  umma::fence_before_sync ();
  __syncthreads ();
  if (warp == 0) umma::tmem_dealloc (tmem, 32);
}

}  // namespace lsg

using namespace lsg;

// round to TF32 (nearest, ties away from zero), as cvt.rna.tf32.f32
static float
host_tf32 (float x)
{
  uint32_t u;
  memcpy (&u, &x, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;
  float r;
  memcpy (&r, &u, 4);
  return r;
}

extern "C" int
stokes_gpu_selftest_tma (double *max_rel_err)
{
  clear_error ();
  if (!max_rel_err) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  const int KK = 64, NB = 24;
  std::vector<float> A (128 * KK), B (NB * KK), pa (2 * 128 * KK), pb (2 * NB * KK), D (128 * 32);
  uint32_t s = 777u;
  auto rnd = [&] () { s = s * 1664525u + 1013904223u; return ((s >> 8) / 16777216.0f) * 2.0f - 1.0f; };
  for (auto &v : A) v = rnd ();
  for (auto &v : B) v = rnd ();
  for (size_t e = 0; e < A.size (); e++)
    {
      pa[e] = host_tf32 (A[e]);
      pa[A.size () + e] = host_tf32 (A[e] - pa[e]);
    }
  for (size_t e = 0; e < B.size (); e++)
    {
      pb[e] = host_tf32 (B[e]);
      pb[B.size () + e] = host_tf32 (B[e] - pb[e]);
    }
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int *dS = nullptr;
  cudaError_t e = cudaMalloc (&dA, sizeof (float) * pa.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dB, sizeof (float) * pb.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dD, sizeof (float) * D.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dS, sizeof (int));
  if (e == cudaSuccess) e = cudaMemcpy (dA, pa.data (), sizeof (float) * pa.size (), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy (dB, pb.data (), sizeof (float) * pb.size (), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset (dS, 0, sizeof (int));
  if (e == cudaSuccess) e = cudaMemset (dD, 0xFF, sizeof (float) * D.size ());
  int status = 0, enc = 0;
  CUtensorMap ma, mb;
  if (e == cudaSuccess)
    {
      enc = encode_planes_sw128 (&ma, dA, 2, 128, KK, 128);
      if (!enc) enc = encode_planes_sw128 (&mb, dB, 2, NB, KK, 32);
    }
  if (e == cudaSuccess && !enc)
    {
      const int smem = 2 * 40960 + 1024;
      e = cudaFuncSetAttribute (k_tma_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e == cudaSuccess)
        {
          k_tma_selftest<<<1, 128, smem>>> (ma, mb, dD, dS);
          e = cudaGetLastError ();
        }
      if (e == cudaSuccess) e = cudaDeviceSynchronize ();
      if (e == cudaSuccess) e = cudaMemcpy (D.data (), dD, sizeof (float) * D.size (), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy (&status, dS, sizeof (int), cudaMemcpyDeviceToHost);
    }
  cudaFree (dA);
  cudaFree (dB);
  cudaFree (dD);
  cudaFree (dS);
  if (e != cudaSuccess) return cuda_fail (e, "TMA self-test");
  if (enc) return set_error (STOKES_GPU_ECUDA, "TMA self-test: tensor map encoding failed (%d)", enc);
  if (status) return set_error (STOKES_GPU_ETIMEOUT, "TMA self-test: a wait ran out");
  double worst = 0.0;
  for (int m = 0; m < 128; m++)
    for (int n = 0; n < 32; n++)
      {
        double ref = 0.0, mag = 0.0;
        if (n < NB)
          for (int k = 0; k < KK; k++)
            {
              ref += (double) A[m * KK + k] * (double) B[n * KK + k];
              mag += fabs ((double) A[m * KK + k] * (double) B[n * KK + k]);
            }
        const double err = fabs ((double) D[m * 32 + n] - ref) / (mag > 0 ? mag : 1.0);
        if (!(err <= worst)) worst = err;   // NaN-propagating max
      }
  *max_rel_err = worst;
  return STOKES_GPU_OK;
}

extern "C" int
stokes_gpu_selftest_tensor (double *max_rel_err)
{
  clear_error ();
  if (!max_rel_err) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  std::vector<float> A (128 * 32), B (16 * 32), D (128 * 16);
  uint32_t s = 12345u;
  auto rnd = [&] () { s = s * 1664525u + 1013904223u; return ((s >> 8) / 16777216.0f) * 2.0f - 1.0f; };
  for (auto &v : A) v = rnd ();
  for (auto &v : B) v = rnd ();
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int *dS = nullptr;
  cudaError_t e = cudaMalloc (&dA, sizeof (float) * A.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dB, sizeof (float) * B.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dD, sizeof (float) * D.size ());
  if (e == cudaSuccess) e = cudaMalloc (&dS, sizeof (int));
  if (e == cudaSuccess) e = cudaMemcpy (dA, A.data (), sizeof (float) * A.size (), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy (dB, B.data (), sizeof (float) * B.size (), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset (dS, 0, sizeof (int));
  if (e == cudaSuccess) e = cudaMemset (dD, 0, sizeof (float) * D.size ());
  int status = 0;
  if (e == cudaSuccess)
    {
      k_umma_selftest<<<1, 128>>> (dA, dB, dD, dS);
      e = cudaGetLastError ();
      if (e == cudaSuccess) e = cudaDeviceSynchronize ();
      if (e == cudaSuccess) e = cudaMemcpy (D.data (), dD, sizeof (float) * D.size (), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy (&status, dS, sizeof (int), cudaMemcpyDeviceToHost);
    }
  cudaFree (dA);
  cudaFree (dB);
  cudaFree (dD);
  cudaFree (dS);
  if (e != cudaSuccess) return cuda_fail (e, "tensor self-test");
  if (status) return set_error (STOKES_GPU_ETIMEOUT, "tensor self-test: MMA completion wait ran out");
  double worst = 0.0;
  for (int m = 0; m < 128; m++)
    for (int n = 0; n < 16; n++)
      {
        double ref = 0.0, mag = 0.0;
        for (int k = 0; k < 32; k++)
          {
            ref += (double) A[m * 32 + k] * (double) B[n * 32 + k];
            mag += fabs ((double) A[m * 32 + k] * (double) B[n * 32 + k]);
          }
        const double err = fabs ((double) D[m * 16 + n] - ref) / (mag > 0 ? mag : 1.0);
        if (!(err <= worst)) worst = err;   // NaN-propagating max
      }
  *max_rel_err = worst;
  return STOKES_GPU_OK;
}
