// tc_umma.cuh -- minimal tcgen05 (5th-generation tensor core) helpers for
// sm_103a: TMEM allocation, shared-memory matrix descriptors, the TF32 MMA,
// commit to an mbarrier, bounded mbarrier waits and TMEM loads.
//
// Operand layout used throughout (K-major, no swizzle): a tile of R rows by
// 8 TF32 values (one MMA K step) is a grid of 8-row x 16-byte "core
// matrices"; the two core matrices of a row group sit side by side
// (LBO = 128 B apart along K) and consecutive 8-row groups are 256 B apart
// (SBO).  umma_off() gives the byte offset of element (row, k) in a tile of
// R rows and KT = 8 * nsteps columns.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lsg {
namespace umma {

// byte offset of (row, k) inside a K-major no-swizzle tile of `rows` rows
__host__ __device__ __forceinline__ uint32_t
off (uint32_t row, uint32_t k, uint32_t rows)
{
  const uint32_t step = k >> 3, kk = (k >> 2) & 1u, e = k & 3u;
  const uint32_t g = row >> 3, r = row & 7u;
  return step * (rows * 32u) + g * 256u + kk * 128u + r * 16u + e * 4u;
}

// shared-memory matrix descriptor (tcgen05 format, version 1):
// start >> 4 [0,14), LBO >> 4 [16,30), SBO >> 4 [32,46), version [46,48),
// base offset [49,52) = 0, layout type [61,64) = 0 (no swizzle)
__device__ __forceinline__ uint64_t
smem_desc (uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = 0;
  d |= (uint64_t) ((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t) 1u << 46;
  return d;
}

// descriptor of a K-major tile in the 128-byte swizzled layout that a TMA
// load with CU_TENSOR_MAP_SWIZZLE_128B writes: rows of 128 bytes (32 TF32
// values), 8-row groups 1024 bytes apart (SBO), the 16-byte chunks of row r
// permuted by r % 8; the tile must start on a 1024-byte boundary.  The k-th
// K step of 8 values starts 32 k bytes in (the swizzle is applied to the
// address, so the start moves within the atom).  LBO is unused in this mode.
__device__ __forceinline__ uint64_t
smem_desc_sw128 (uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t) ((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t) 1u << 16;                 // LBO (ignored): 16 bytes
  d |= (uint64_t) (1024u >> 4) << 32;       // SBO: 1024 bytes
  d |= (uint64_t) 1u << 46;                 // descriptor version
  d |= (uint64_t) 2u << 61;                 // layout: 128-byte swizzle
  return d;
}

// instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major
__host__ __device__ __forceinline__ uint32_t
idesc_tf32 (uint32_t M, uint32_t N)
{
  return (1u << 4)            // D format: f32
    | (2u << 7)               // A format: tf32
    | (2u << 10)              // B format: tf32
    | ((N >> 3) << 17)        // N / 8
    | ((M >> 4) << 24);       // M / 16
}

__device__ __forceinline__ uint32_t
smem_u32 (const void *p)
{
  return (uint32_t) __cvta_generic_to_shared (p);
}

__device__ __forceinline__ uint32_t
to_tf32 (float x)
{
  uint32_t r;
  asm volatile ("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// TF32 rounding of an FP32 bit pattern, to nearest with ties away from zero
// (the rounding of cvt.rna.tf32.f32): add half a TF32 unit to the magnitude
// bits and clear the 13 bits below TF32's mantissa; a carry moves into the
// exponent as it should.  Finite inputs.
__device__ __forceinline__ uint32_t
rna_tf32_bits (uint32_t u)
{
  return (u + 0x1000u) & 0xFFFFE000u;
}

// x = hi + lo with hi, lo representable in TF32 (the 3xTF32 split), in
// integer and FP32 arithmetic
__device__ __forceinline__ void
split_tf32 (float x, uint32_t &hi, uint32_t &lo)
{
  hi = rna_tf32_bits (__float_as_uint (x));
  lo = rna_tf32_bits (__float_as_uint (x - __uint_as_float (hi)));
}

// an L1 prefetch of the line holding p (no register result)
__device__ __forceinline__ void
prefetch_l1 (const void *p)
{
  asm volatile ("prefetch.global.L1 [%0];" :: "l"(p));
}

// TMEM allocation by one full warp; the column address lands in *slot
__device__ __forceinline__ void
tmem_alloc (uint32_t *slot, uint32_t ncols)
{
  asm volatile ("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                :: "r"(smem_u32 (slot)), "r"(ncols) : "memory");
  asm volatile ("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void
tmem_dealloc (uint32_t taddr, uint32_t ncols)
{
  asm volatile ("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                :: "r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void
mma_tf32 (uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate)
{
  asm volatile (
    "{\n\t.reg .pred p;\n\t"
    "setp.ne.b32 p, %4, 0;\n\t"
    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
    :: "r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

// arrive on an mbarrier once all previously issued MMAs of this thread are done
__device__ __forceinline__ void
mma_commit (uint64_t *mbar)
{
  asm volatile ("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                :: "r"(smem_u32 (mbar)) : "memory");
}

__device__ __forceinline__ void
mbar_init (uint64_t *mbar, uint32_t count)
{
  asm volatile ("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32 (mbar)), "r"(count)
                : "memory");
}

__device__ __forceinline__ void
fence_mbar_init ()
{
  asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// wait for phase `parity` of the mbarrier with at most `limit` polls;
// returns false when the limit ran out
__device__ __forceinline__ bool
mbar_wait (uint64_t *mbar, uint32_t parity, uint32_t limit)
{
  const uint32_t a = smem_u32 (mbar);
  for (uint32_t it = 0; it < limit; it++)
    {
      uint32_t done;
      asm volatile (
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(a), "r"(parity) : "memory");
      if (done) return true;
    }
  return false;
}

// one arrival on an mbarrier (release at CTA scope)
__device__ __forceinline__ void
mbar_arrive (uint64_t *mbar)
{
  asm volatile ("{\n\t.reg .b64 st;\n\t"
                "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}"
                :: "r"(smem_u32 (mbar)) : "memory");
}

// wait for phase `parity`, giving up early when *abort (a CTA-wide error flag
// in shared memory) becomes non-zero; returns false when the wait did not
// complete.  Each poll lets the thread sleep until the phase completes or
// about 20 us pass (the try_wait suspend-time hint), so waiting warps do not
// take issue slots from working ones; `limit` polls bound the wait to about
// limit x 20 us.
__device__ __forceinline__ bool
mbar_wait_or_abort (uint64_t *mbar, uint32_t parity, uint32_t limit, volatile int *abort)
{
  const uint32_t a = smem_u32 (mbar);
  for (uint32_t it = 0; it < limit; it++)
    {
      uint32_t done;
      asm volatile (
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(a), "r"(parity), "r"(20000u) : "memory");
      if (done) return true;
      if (*abort) return false;
    }
  *abort = 1;
  return false;
}

// arrive once on an mbarrier and add `bytes` to the transaction count its
// current phase waits for (the TMA loads that follow complete them)
__device__ __forceinline__ void
mbar_expect_tx (uint64_t *mbar, uint32_t bytes)
{
  asm volatile ("{\n\t.reg .b64 st;\n\t"
                "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
                :: "r"(smem_u32 (mbar)), "r"(bytes) : "memory");
}

// 3-d tiled TMA load of one box at coordinates (c0, c1, c2) into shared
// memory, completing `bytes of the box` on the mbarrier; tmap: the address of
// a __grid_constant__ CUtensorMap kernel parameter
__device__ __forceinline__ void
tma_load_3d (void *dst, const void *tmap, int c0, int c1, int c2, uint64_t *mbar)
{
  asm volatile (
    "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
    " [%0], [%1, {%2, %3, %4}], [%5];"
    :: "r"(smem_u32 (dst)), "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32 (mbar))
    : "memory");
}

// 2-d tiled TMA store of one box from shared memory (128-byte aligned, the
// box's rows back to back) to coordinates (c0, c1); parts of the box outside
// the tensor are not written.  Completes asynchronously: commit the group and
// wait before the shared memory is reused.
__device__ __forceinline__ void
tma_store_2d (const void *tmap, const void *src, int c0, int c1)
{
  asm volatile ("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
                :: "l"(tmap), "r"(smem_u32 (src)), "r"(c0), "r"(c1) : "memory");
}

__device__ __forceinline__ void
bulk_commit ()
{
  asm volatile ("cp.async.bulk.commit_group;" ::: "memory");
}

// wait until every committed bulk store has finished reading shared memory
__device__ __forceinline__ void
bulk_wait_read ()
{
  asm volatile ("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ void
tma_prefetch_desc (const void *tmap)
{
  asm volatile ("prefetch.tensormap [%0];" :: "l"(tmap) : "memory");
}

// generic-proxy smem writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void
fence_async_smem ()
{
  asm volatile ("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void
fence_before_sync ()
{
  asm volatile ("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void
fence_after_sync ()
{
  asm volatile ("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape):
// warp w of a warpgroup reads lanes 32 w .. 32 w + 31
__device__ __forceinline__ void
tmem_ld16 (uint32_t taddr, float v[16])
{
  uint32_t r[16];
  asm volatile (
    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
      "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
      "=r"(r[14]), "=r"(r[15])
    : "r"(taddr));
  asm volatile ("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float (r[q]);
}

}  // namespace umma
}  // namespace lsg
