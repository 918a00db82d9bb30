// gpu_engine.h -- per-system device context shared by the host engine files.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <array>
#include <vector>

#include "stokes_abi.h"
#include "engine.h"

namespace lsg {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure (size_t bytes);
  void release ();
};

struct MixedState;   // mixed-precision state (mixed.cu)

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {};
  cudaEvent_t join[2] = {};   // orders the context's stream inside the legacy default stream
  int precision = 0;

  // geometry of the last prepared system
  const struct stokes *sys = nullptr;
  int version = 0, np = 0, mode = 0;
  double xi = 0, xisp = 0, rmax2 = 0, rmin = 0;
  double xi_ref = 0;      // the struct's own split (differs from xi at the tuned split)
  int nimg = 0, nk = 0;
  uint64_t fp_img = 0, fp_kt = 0, fp_pp = 0;
  std::vector<Img4> h_img;
  std::vector<double> h_kt, h_pp;

  DevBuf pos, x, y, img, kt, pp, ph, sf, yrec, partial, mat, zbuf;

  double times[3] = {0, 0, 0};
  int launches = 0;
  bool timed = false;

  // profiling window: 4 events per product (start, reciprocal done,
  // real space done, end), read back by stokes_gpu_profile_end
  bool prof_on = false;
  int prof_n = 0;
  std::vector<cudaEvent_t> prof_ev;

  // kernel profiling window: one event after each launch, tagged with the
  // kernel's name (nullptr marks the start of a product)
  bool kprof_on = false;
  // non-periodic (free-space) operator: set for systems with periodic = 0 and
  // by the *_nonewald_* entry points (force_open), src/non-ewald.c
  bool open = false, force_open = false;
  // FP64 products of an equal-sphere periodic system run at a cheaper
  // Ewald split than the reference's (prepare): a private copy of the
  // system set up at that split, its key, and whether prepare may use it
  struct stokes *tuned = nullptr;
  double tuned_key[7] = {0, 0, 0, 0, 0, 0, 0};
  bool tune = true;
  size_t kprof_n = 0;
  std::vector<cudaEvent_t> kprof_ev;
  std::vector<const char *> kprof_name;

  MixedState *mixed = nullptr;

  DevBuf openf;   // scratch of the mixed-precision free-space product
  DevBuf imgf;    // the images in FP32 (split-precision dense builder)
  // the thread-per-pair dense builder's split: a private copy of the system
  // at it, its key, the half-space tables (FP64 rows for the phases, floats
  // for the terms) and their count
  bool cube = false;   // the last prepare's image set is the _notbl cube
  struct stokes *dense = nullptr;
  double dense_key[7] = {0, 0, 0, 0, 0, 0, 0};
  int dense_nk = 0;
  std::vector<double> h_dkt;
  DevBuf dkt, dktf, dself;   // FP64 rows, moment coefficients, diagonal moments
  uint64_t fp_dkt = 0;

  // pinned, mapped mirror of sys->pos for the host entry points of the
  // mixed paths, whose kernels read the positions once
  double *hpos = nullptr;
  const double *hpos_dev = nullptr;   // its device address
  size_t hpos_bytes = 0;

  std::array<DevBuf *, 17> all_buffers ()
  {
    return {&pos, &x, &y, &img, &kt, &pp, &ph, &sf, &yrec, &partial, &mat, &zbuf, &openf, &imgf,
            &dkt, &dktf, &dself};
  }
};

int set_error (int code, const char *fmt, ...);
void clear_error ();
int cuda_fail (cudaError_t e, const char *where);
void dropin_failed (const char *fn, double *out, size_t nout);

Ctx *get_ctx (const struct stokes *sys, bool create);
// host tables of one system (gpu_engine.cu)
int check_sys (const struct stokes *sys, bool open = false);
// STOKES_GPU_EINVAL when a coordinate of the host positions pos[3 np] is NaN
// or infinite (the kernels would turn it into a wrong result, not an error)
int check_positions (const double *pos, int np);
void build_images (const struct stokes *sys, bool cube, std::vector<Img4> &img);
void build_ktable (const struct stokes *sys, std::vector<double> &kt);
void build_particles (const struct stokes *sys, int mode, std::vector<double> &pp,
                      bool open = false, const struct stokes *split = nullptr);
int release_ctx (const struct stokes *sys);
// u = (I + M L)^-1 M f on device buffers (krylov.cu), F and FT, the
// context's product at positions d_pos, GMRES settings from sys->it
int lub_mobility_dev (Ctx *c, struct stokes *sys, const double *d_pos, const double *d_f,
                      double *d_u, cudaStream_t st, int *iters);
// f = L u on device buffers (lub.cu): version 0 (F) or 1 (FT)
int lub_dev (const struct stokes *sys, int version, const double *d_pos, const double *d_u,
             double *d_f, cudaStream_t st);
// check sys and bring the context's device tables up to date.  tables: 1
// builds the FP64 image and reciprocal tables of the FP64 product (the
// tuned split where it applies), 2 those of the dense builder (the
// reference's split), 0 skips them (the mixed product never reads them),
// -1 chooses by the context's precision.
int prepare (Ctx *c, const struct stokes *sys, bool cube, int tables = -1);

// drops the adjoint's private copy of sys, if any (adjoint.cu)
void release_adjoint (const struct stokes *sys);
int atimes_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                cudaStream_t st, bool timed);
int atimes_fp64_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                     cudaStream_t st, bool timed);
void collect_times (Ctx *c);
cudaEvent_t *phase_events (Ctx *c, bool timed);
// record a kernel-profiling mark on st when the window is open
void kmark (Ctx *c, cudaStream_t st, const char *name);

// mixed-precision path (mixed.cu)
int atimes_mixed_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                      cudaStream_t st, bool timed);
// free-space product of an open system in mixed precision (open_f32.cu)
int atimes_open_f32_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                         cudaStream_t st, bool timed);
void release_mixed (Ctx *c);
// mixed-precision VJP (adjoint_f32.cu): 1 when it served the call, 0 when
// the system needs the FP64 adjoint, -status on error
int vjp_mixed (Ctx *c, const struct stokes *sys, const double *g, const double *f, double *dLdr,
               double *dLdbox);
void release_vjp_mixed (const Ctx *c);
// after the stream of a mixed product was synchronised: STOKES_GPU_ETIMEOUT
// (and the status word cleared) when a bounded wait of its tensor-core
// kernels ran out, else STOKES_GPU_OK
int mixed_check_status (Ctx *c);

// failure-injection settings of stokes_gpu_test_stall_waits (util.cu): polls
// of an extra wait of the k-space GEMMs' MMA lane on an mbarrier that nothing
// arrives at (0: no such wait), and the spin limit of the GMRES grid barrier
// (0: the default)
extern int g_test_gemm_stall;
extern long long g_test_bar_spins;

}  // namespace lsg
