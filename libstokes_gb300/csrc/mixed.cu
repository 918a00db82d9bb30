// mixed.cu -- mixed-precision mobility product (placeholder until built).
#include "gpu_engine.h"
#include "stokes_gpu.h"

namespace lsg {

int
atimes_mixed_dev (Ctx *, const double *, const double *, double *, cudaStream_t, bool)
{
  return set_error (STOKES_GPU_EINVAL, "mixed precision is not available in this build");
}

int
matrix_mixed_dev (Ctx *, const double *, double *, cudaStream_t)
{
  return set_error (STOKES_GPU_EINVAL, "mixed precision is not available in this build");
}

void release_mixed (Ctx *) {}

}  // namespace lsg
