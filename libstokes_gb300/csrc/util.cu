// util.cu -- measurement helpers exported next to the operators:
//   stokes_gpu_count_real_terms: exact number of real-space (i, j, image)
//     terms inside the cutoff, the unit of the real-space roofline;
//   stokes_gpu_peak_fma: FP64 / FP32 FMA throughput of this GPU, measured
//     with an FMA-chain kernel (the denominator of the pipe rooflines).
#include <cuda_runtime.h>

#include "stokes_gpu.h"
#include "gpu_engine.h"

namespace lsg {

__global__ void
k_count_real (const double *pos, const Img4 *img, int nimg, int np, double rmax2,
              unsigned long long *count)
{
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (t < (long long) np * np)
    {
      const int i = (int) (t / np), j = (int) (t % np);
      const double dx0 = pos[3 * j] - pos[3 * i];
      const double dy0 = pos[3 * j + 1] - pos[3 * i + 1];
      const double dz0 = pos[3 * j + 2] - pos[3 * i + 2];
      for (int m = 0; m < nimg; m++)
        {
          const double dx = dx0 + img[m].x, dy = dy0 + img[m].y, dz = dz0 + img[m].z;
          const double rr = dx * dx + dy * dy + dz * dz;
          c += (rr != 0.0 && rr <= rmax2) ? 1ull : 0ull;
        }
    }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync (0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd (count, c);
}

template <typename R>
__global__ void __launch_bounds__ (256)
k_fma_chain (R seed, int iters, R *sink)
{
  R a[8];
#pragma unroll
  for (int q = 0; q < 8; q++) a[q] = seed + R (threadIdx.x + q);
  const R b = R (0.999999), c = R (1e-7);
  for (int it = 0; it < iters; it++)
    {
#pragma unroll
      for (int q = 0; q < 8; q++) a[q] = a[q] * b + c;
    }
  R s = R (0);
#pragma unroll
  for (int q = 0; q < 8; q++) s += a[q];
  if (s == R (-12345.0)) sink[0] = s;  // keeps the chain alive
}

int g_test_gemm_stall = 0;
long long g_test_bar_spins = 0;

}  // namespace lsg

using namespace lsg;

extern "C" {

static int
count_terms (struct stokes *sys, int tables, long long *count)
{
  if (!count) return set_error (STOKES_GPU_EINVAL, "NULL count");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, false, tables);
  if (rc) return rc;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * sys->np)) != cudaSuccess) return cuda_fail (e, "pos");
  DevBuf cnt;
  if ((e = cnt.ensure (sizeof (unsigned long long))) != cudaSuccess) return cuda_fail (e, "count");
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * sys->np, cudaMemcpyHostToDevice,
                   c->stream);
  cudaMemsetAsync (cnt.p, 0, sizeof (unsigned long long), c->stream);
  const long long nt = (long long) sys->np * sys->np;
  k_count_real<<<(int) ((nt + 255) / 256), 256, 0, c->stream>>> (
    (const double *) c->pos.p, (const Img4 *) c->img.p, c->nimg, sys->np, c->rmax2,
    (unsigned long long *) cnt.p);
  unsigned long long h = 0;
  e = cudaMemcpyAsync (&h, cnt.p, sizeof h, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  cnt.release ();
  if (e != cudaSuccess) return cuda_fail (e, "count");
  *count = (long long) h;
  return STOKES_GPU_OK;
}

// terms of the FP64 product's split (the tuned one where it applies)
int
stokes_gpu_count_real_terms (struct stokes *sys, long long *count)
{
  return count_terms (sys, 1, count);
}

// terms of the dense builder's split (the reference's)
int
stokes_gpu_count_real_terms_dense (struct stokes *sys, long long *count)
{
  return count_terms (sys, 2, count);
}

// failure injection for the tests of the bounded device waits
int
stokes_gpu_test_stall_waits (int gemm_polls, long long barrier_spins)
{
  if (gemm_polls < 0 || barrier_spins < 0)
    return set_error (STOKES_GPU_EINVAL, "negative wait limit");
  g_test_gemm_stall = gemm_polls;
  g_test_bar_spins = barrier_spins;
  return STOKES_GPU_OK;
}

// GFLOP/s (2 flops per FMA) of an FMA-chain kernel filling the GPU
int
stokes_gpu_peak_fma (int fp64, double *gflops)
{
  if (!gflops) return set_error (STOKES_GPU_EINVAL, "NULL gflops");
  int dev = 0, nsm = 0;
  cudaGetDevice (&dev);
  cudaDeviceGetAttribute (&nsm, cudaDevAttrMultiProcessorCount, dev);
  DevBuf sink;
  cudaError_t e = sink.ensure (64);
  if (e != cudaSuccess) return cuda_fail (e, "sink");
  cudaEvent_t a, b;
  cudaEventCreate (&a);
  cudaEventCreate (&b);
  const int blocks = nsm * 8, threads = 256;
  const int iters = fp64 ? 2048 : 65536;
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++)
    {
      cudaEventRecord (a);
      if (fp64) k_fma_chain<double><<<blocks, threads>>> (1.0, iters, (double *) sink.p);
      else k_fma_chain<float><<<blocks, threads>>> (1.0f, iters, (float *) sink.p);
      cudaEventRecord (b);
      cudaEventSynchronize (b);
      float ms = 0.f;
      cudaEventElapsedTime (&ms, a, b);
      if (rep > 0 && ms < best) best = ms;
    }
  e = cudaGetLastError ();
  cudaEventDestroy (a);
  cudaEventDestroy (b);
  sink.release ();
  if (e != cudaSuccess) return cuda_fail (e, "peak kernel");
  const double flops = 2.0 * 8.0 * (double) iters * blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return STOKES_GPU_OK;
}

}  // extern "C"
