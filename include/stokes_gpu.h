/* stokes_gpu.h -- additive GPU API of libstokes_gb300.
 *
 * These entry points have no counterpart in libstokes; they sit beside the
 * drop-in functions of stokes_abi.h.  Every one returns an int status
 * (STOKES_GPU_OK = 0) instead of exiting, takes plain pointers and sizes,
 * and runs on the calling thread's current CUDA device.
 *
 * Device pointers ("d_" prefix) must point to memory of that device.
 * A "stream" argument is a cudaStream_t passed as void*; NULL selects the
 * library's own stream for that system.
 */
#ifndef LIBSTOKES_GB300_STOKES_GPU_H
#define LIBSTOKES_GB300_STOKES_GPU_H

#include "stokes_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  STOKES_GPU_OK = 0,
  STOKES_GPU_EINVAL = 1,      /* bad argument (n, version, NULL pointer, ...) */
  STOKES_GPU_ENOTPERIODIC = 2,/* a lattice-sum entry point called on an open system */
  STOKES_GPU_ECUDA = 3,       /* a CUDA runtime call failed */
  STOKES_GPU_ENOMEM = 4,      /* device allocation failed */
  STOKES_GPU_ETIMEOUT = 5,    /* a bounded device wait ran out */
  STOKES_GPU_EACCURACY = 6,   /* Chebyshev error above the requested bound */
  STOKES_GPU_ETOOBIG = 7      /* size above a fixed capacity */
};

/* precision modes of the mobility product */
enum {
  STOKES_GPU_FP64 = 0,        /* IEEE FP64, the reference's image and k sets */
  STOKES_GPU_MIXED = 1        /* FP32 real space + split-BF16 tensor-core
                                 reciprocal space on a re-tuned Ewald split;
                                 relative L2 error <= 1e-6 vs FP64 */
};

/* status of the last failing call on this thread and its message */
int stokes_gpu_last_error (void);
const char *stokes_gpu_last_error_message (void);
/* 0 (default): a failing drop-in (void) function prints its reason and
 * exits with status 1, like libstokes on allocation failure.
 * 1: it records the error, fills its outputs with NaN and returns. */
void stokes_gpu_set_error_mode (int mode);

/* precision of the products of this system (default: STOKES_GPU_FP64, or
 * the value of the LIBSTOKES_GB300_PRECISION environment variable,
 * "fp64" or "mixed", at the first product of a system).  Mixed precision
 * (<= 1e-6 against FP64) serves open systems, and periodic equal or unequal
 * spheres without slip (unequal ones with rmin = 0); other periodic systems
 * report an error in it. */
int stokes_gpu_set_precision (struct stokes *sys, int mode);
int stokes_gpu_get_precision (const struct stokes *sys, int *mode);

/* free the device state kept for sys (stokes_free does this too) */
int stokes_gpu_release (struct stokes *sys);

/* called by stokes_set_xi: notes the split and tables it built, so that
 * the FP64 products may run at a cheaper split while the struct still holds
 * exactly those tables (tables set by hand are used as they are) */
void stokes_gpu_note_split (const struct stokes *sys);

/* y = M x with host buffers; the status-returning form of atimes_3all:
 * the Ewald sum of a periodic system, the free-space sum of an open one
 * (sys->periodic == 0, which needs neither a box nor a split) */
int stokes_gpu_atimes (struct stokes *sys, const double *x, double *y);

/* y = M x with device buffers.  d_pos: positions [np*3] on the device, or
 * NULL to upload sys->pos.  Asynchronous on `stream`; NULL is the legacy
 * default stream (the work is ordered after and before the caller's other
 * work on it). */
int stokes_gpu_atimes_dev (struct stokes *sys, const double *d_pos,
                           const double *d_x, double *d_y, void *stream);

/* y = M x in FP64 without allocating device memory.  No counterpart in
 * libstokes.  For callers that may not allocate on the device while they
 * run (a fixed memory budget owned by another framework, steps that must
 * never enter the driver's allocator): all scratch lives in one fixed
 * 5.06 MiB device array per GPU, reserved when this library's device module
 * is loaded on that GPU.  With lazy module loading (CUDA's default) that
 * happens during the first call on the device, so make one warm-up call per
 * device before the allocation-free region (or set
 * CUDA_MODULE_LOADING=EAGER).  Limits: np <= 512, at most 2048 real-space
 * images and 512 reciprocal vectors; larger systems get STOKES_GPU_ETOOBIG.
 * d_pos [np*3], d_x, d_y [np*{3,6,11}] are device buffers of the caller;
 * stream may be NULL (the default stream).  No call can be captured into a
 * CUDA graph: each waits for its small table uploads, and a call on a
 * capturing stream returns STOKES_GPU_EINVAL.  All calls share the array:
 * calls that overlap on one GPU race on it. */
int stokes_gpu_atimes_noalloc (struct stokes *sys, const double *d_pos,
                               const double *d_x, double *d_y, void *stream);

/* dense mobility matrix with host / device output (stream as for
 * stokes_gpu_atimes_dev) */
int stokes_gpu_matrix (struct stokes *sys, double *mat);
int stokes_gpu_matrix_dev (struct stokes *sys, const double *d_pos,
                           double *d_mat, void *stream);

/* y = mat . x (extracted form for FTS) on device buffers */
int stokes_gpu_matvec_dev (int version, int np, const double *d_mat,
                           const double *d_x, double *d_y, void *stream);

/* device milliseconds of the last host-buffer product: total, real space,
 * the rest (the real space runs beside the reciprocal part in mixed
 * precision; the rest is then total - real) */
int stokes_gpu_last_times (const struct stokes *sys, double *ms3);

/* Profiling window for the device entry points: between begin and end, each
 * product of sys (up to max_products) records CUDA events on its stream at
 * its phase boundaries.  end waits for them and returns the summed device
 * milliseconds (total, real space, reciprocal space) and the product count. */
int stokes_gpu_profile_begin (struct stokes *sys, int max_products);
int stokes_gpu_profile_end (struct stokes *sys, double *sum_ms3, int *count);

/* Vector-Jacobian product of the mobility product (FP64): for
 * L = g . M(r, box) f (g, f: host vectors in the product's layout), the
 * gradient dLdr[3 np] with respect to the positions and, when dLdbox is not
 * NULL, dLdbox[3] = dL/dl_x, dL/dl_y, dL/dl_z with the particles held fixed,
 * both at the system's image and k sets and its xi.  Lval (optional)
 * receives L.  F and FT versions, equal spheres without slip; the box
 * derivatives need shear_mode 0.  No counterpart in libstokes. */
int stokes_gpu_vjp (struct stokes *sys, const double *g, const double *f, double *dLdr,
                    double *dLdbox, double *Lval);

/* Batches: many independent periodic systems (each a struct stokes set up
 * as for atimes_ewald_3all) whose products run together, a few launches for
 * the whole batch replayed from a CUDA graph.  Vectors are packed: the
 * systems' vectors in libstokes' per-particle layout, one after the other
 * (offsets from stokes_gpu_batch_offsets).  STOKES_GPU_FP64 batches use each
 * system's own split (parity with atimes_ewald_3all); STOKES_GPU_MIXED
 * batches (F and FT equal spheres) re-split every system as the mixed
 * product does and tune their launch shapes on the first product.  The
 * positions are read at creation (and by stokes_gpu_batch_set_positions);
 * the box, split and version of every system are fixed for the batch's life.
 * No counterpart in libstokes (there: a loop over systems). */
typedef struct stokes_gpu_batch stokes_gpu_batch;
int stokes_gpu_batch_create (struct stokes **systems, int nsys, int precision,
                             stokes_gpu_batch **out);
int stokes_gpu_batch_destroy (stokes_gpu_batch *b);
/* particles and vector length over the whole batch */
int stokes_gpu_batch_size (const stokes_gpu_batch *b, int *np_total, int *n_total);
/* per system: first particle (p_off[s]) and first vector element (x_off[s]) */
int stokes_gpu_batch_offsets (const stokes_gpu_batch *b, int *p_off, int *x_off);
/* packed positions (3 per particle) of every system; also written back to
 * each system's pos */
int stokes_gpu_batch_set_positions (stokes_gpu_batch *b, const double *pos_packed);
/* y = M x for every system, packed host vectors */
int stokes_gpu_batch_atimes (stokes_gpu_batch *b, const double *x, double *y);
/* device ms of the last batch product, chosen real-space chunking and warps
 * per CTA, total k vectors (mixed) */
int stokes_gpu_batch_stats (const stokes_gpu_batch *b, double *out4);
/* mixed batches: the split of system s, eta = xi V^(1/3) and xi (the split
 * is autotuned with the chunking on the first product) */
int stokes_gpu_batch_split (const stokes_gpu_batch *b, int s, double *eta, double *xi);
/* nsteps Brownian-dynamics mid-point steps of every system of the batch
 * (no repulsion, no imposed flow): f = sqrt(2 / (peclet dt)) z with
 * z = M^{-1/2} y by an n_cheb-term Chebyshev series on per-system bounds
 * eig[2 s], eig[2 s + 1] (NULL: FP64 Lanczos on the batch products,
 * n_lanczos steps, widened by 0.8 and 1.05); y read from y_host (n_total
 * values per step) or, when y_host is NULL, drawn on the device (Philox,
 * seed).  pos_out (optional) receives the packed positions. */
int stokes_gpu_batch_bd (stokes_gpu_batch *b, double peclet, double dt, int n_cheb,
                         int n_lanczos, const double *eig, const double *y_host,
                         unsigned long long seed, int nsteps, double *pos_out);

/* Kernel profiling window: between begin and end, every product of sys
 * records a CUDA event on its own stream after each kernel it launches (at
 * most max_marks events in all).  end waits for them and returns, per kernel
 * name (32-byte slots in names, at most max_kernels), the summed device
 * milliseconds between the kernel's event and the previous one and the
 * number of launches; *nkernels is the number of names filled. */
int stokes_gpu_kprof_begin (struct stokes *sys, int max_marks);
int stokes_gpu_kprof_end (struct stokes *sys, int max_kernels, char *names, double *sum_ms,
                          int *count, int *nkernels);

/* number of kernel launches issued by the last product of sys */
int stokes_gpu_last_launches (const struct stokes *sys, int *count);

/* number of real-space (i, j, image) terms with 0 < r^2 <= rmax2 -- the
 * unit count of the real-space roofline -- at the split of the FP64
 * product (the tuned split where it applies) and at that of the dense
 * builder (the reference's split) */
int stokes_gpu_count_real_terms (struct stokes *sys, long long *count);
int stokes_gpu_count_real_terms_dense (struct stokes *sys, long long *count);

/* number of real-space (i, j, image) terms the mixed product evaluates
 * (0 < r^2 < rc^2 at the mixed split, after its first mixed product): the
 * unit count of the mixed real-space roofline.  No counterpart in libstokes. */
int stokes_gpu_count_mixed_real_terms (struct stokes *sys, long long *count);

/* split chosen by the mixed path for sys (after its first mixed product):
 * xi, rc, kc, eta = xi V^(1/3), eps, half-space k count, max |m| per axis */
int stokes_gpu_mixed_split (struct stokes *sys, double *info9);

/* known-answer test of the tensor-core (tcgen05, 3xTF32) path on the
 * current GPU: largest error of a 128x16x32 product relative to the sum of
 * absolute products (expect ~1e-7) */
int stokes_gpu_selftest_tensor (double *max_rel_err);

/* known-answer test of the TMA path of the reciprocal-space GEMMs: operand
 * images (TF32 hi/lo planes) loaded by 3-d TMA boxes with 128-byte swizzle
 * (including zero-filled rows past the end), a 128 x 32 x 64 product in
 * 3xTF32 on the swizzled descriptors; largest error relative to the sum of
 * absolute products (expect ~1e-7) */
int stokes_gpu_selftest_tma (double *max_rel_err);

/* measured FMA throughput of the current GPU in GFLOP/s (2 flops per FMA),
 * fp64 = 1 for FP64, 0 for FP32 */
int stokes_gpu_peak_fma (int fp64, double *gflops);

/* Failure injection for tests of the bounded device waits (no counterpart
 * in libstokes; process-wide, 0 and 0 restore normal operation).
 * gemm_polls > 0: the MMA lane of every tensor-core k-space GEMM first waits
 * that many polls (about 20 us each) on an mbarrier that nothing arrives at;
 * the wait runs out, the CTA's roles stop, the kernel raises its status word
 * and the mixed product reports STOKES_GPU_ETIMEOUT.  barrier_spins > 0: the
 * GMRES grid barrier gives up after that many polls, and the solve reports
 * STOKES_GPU_ETIMEOUT. */
int stokes_gpu_test_stall_waits (int gemm_polls, long long barrier_spins);

#ifdef __cplusplus
}
#endif

#endif /* LIBSTOKES_GB300_STOKES_GPU_H */
