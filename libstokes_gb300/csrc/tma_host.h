// tma_host.h -- host-side encoding of TMA tensor maps through the driver
// entry point (no link against libcuda).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace lsg {

typedef CUresult (*EncodeTiledFn) (CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                    const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                    const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// A [planes][rows][cols] FP32 array, row-major, cols a multiple of 4 (rows
// start on 16-byte boundaries), as a 3-d tensor map whose box is
// {32 columns (128 bytes), box_rows rows, 1 plane} in the 128-byte swizzled
// layout; reads outside [rows] x [cols] fill zeros.  Returns 0 on success.
inline EncodeTiledFn
encode_fn ()
{
  static EncodeTiledFn fn = nullptr;
  if (!fn)
    {
      void *p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion ("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q)
            == cudaSuccess
          && q == cudaDriverEntryPointSuccess && p)
        fn = (EncodeTiledFn) p;
    }
  return fn;
}

inline int
encode_planes_sw128 (CUtensorMap *map, const float *base, unsigned long long planes,
                     unsigned long long rows, unsigned long long cols, unsigned box_rows)
{
  EncodeTiledFn fn = encode_fn ();
  if (!fn) return -1;
  if (cols % 4 || ((unsigned long long) base & 15ull) || box_rows == 0 || box_rows > 256) return -2;
  const cuuint64_t dims[3] = {cols, rows, planes};
  const cuuint64_t strides[2] = {cols * 4ull, rows * cols * 4ull};
  const cuuint32_t box[3] = {32u, box_rows, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  const CUresult r = fn (map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *) base, dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int) r;
}

// A [rows][cols] FP32 array, row-major, cols a multiple of 4, as a 2-d
// tensor map without swizzle whose box is {box_cols, box_rows}; used for
// TMA stores of tiles kept row-major in shared memory.  0 on success.
inline int
encode_rows_plain (CUtensorMap *map, const float *base, unsigned long long rows,
                   unsigned long long cols, unsigned box_cols, unsigned box_rows)
{
  EncodeTiledFn fn = encode_fn ();
  if (!fn) return -1;
  if (cols % 4 || ((unsigned long long) base & 15ull) || box_rows == 0 || box_rows > 256
      || box_cols == 0 || box_cols > 256 || (box_cols * 4) % 16)
    return -2;
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * 4ull};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1u, 1u};
  const CUresult r = fn (map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *) base, dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int) r;
}

}  // namespace lsg
