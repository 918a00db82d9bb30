// noalloc.cu -- an allocation-free variant of the FP64 mobility product.
//
// Who needs it: callers that must not allocate device memory while they run
// -- code that executes under a fixed, pre-reserved memory budget (another
// framework owns the device heap), code that is not allowed to enter the
// driver's allocator in its steady state (hard real-time steps, callbacks
// invoked from inside another library's allocator-free region), and
// programs that treat any cudaMalloc after start-up as an error.  The
// regular entry points keep growable per-system device buffers; this one
// uses only the fixed array below, reserved once when the library's module
// is loaded on a device.
//
// Limits (checked, STOKES_GPU_ETOOBIG beyond them): at most 512 particles,
// 2048 real-space images and 512 reciprocal vectors -- systems of up to a
// few hundred spheres, such as the members of an ensemble.  The array takes
// 5,304,320 bytes (5.06 MiB) on every GPU that loads the library and stays
// there until the process exits.
//
// The first call on each device looks up the array's device address
// (cudaGetSymbolAddress) with that device current.  With lazy module loading
// (CUDA's default) that lookup is also what loads this library's device
// module on the device, and loading a module reserves its static arrays
// through the driver: make one warm-up call on each device before the
// region in which nothing may allocate, or run with
// CUDA_MODULE_LOADING=EAGER, which loads the module (and reserves the array)
// when the CUDA context is created.
//
// No call of this entry point can be recorded into a CUDA graph: every call
// copies its small tables from host memory and waits for those copies
// (cudaStreamSynchronize) before it returns, and a synchronize is illegal on
// a capturing stream.  A call on a stream that is being captured is refused
// with STOKES_GPU_EINVAL before it touches the stream.  The kernels
// themselves run asynchronously on the caller's stream.
//
// Every call uses the same array and leaves its last contents in it.  Calls
// that overlap on the same GPU -- on different streams, or from different
// host threads without ordering between them -- race on the array and can
// corrupt each other's results.  Each device has its own copy, so calls on
// different GPUs do not interact.  Nothing in the array has to start at
// zero: each kernel of this product writes every scratch element before it
// reads it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "engine.h"
#include "gpu_engine.h"
#include "stokes_gpu.h"

namespace lsg {
namespace {

constexpr int NA_MAX_NP = 512;
constexpr int NA_MAX_IMG = 2048;
constexpr int NA_MAX_K = 512;
constexpr int NA_NCHUNK = 16;   // source chunks of the real-space kernel

// byte offsets inside the scratch array (each region 256-byte aligned)
constexpr size_t na_align (size_t b) { return (b + 255) & ~(size_t) 255; }
constexpr size_t NA_IMG = 0;
constexpr size_t NA_KT = NA_IMG + na_align (sizeof (Img4) * NA_MAX_IMG);
constexpr size_t NA_PP = NA_KT + na_align (sizeof (double) * KT_STRIDE * NA_MAX_K);
constexpr size_t NA_PART = NA_PP + na_align (sizeof (double) * 6 * NA_MAX_NP);
constexpr size_t NA_YREC = NA_PART + na_align (sizeof (double) * NA_NCHUNK * NA_MAX_NP * 11);
constexpr size_t NA_SF = NA_YREC + na_align (sizeof (double) * NA_MAX_NP * 11);
constexpr size_t NA_PH = NA_SF + na_align (sizeof (double) * SF_STRIDE * NA_MAX_K);
constexpr size_t NA_BYTES = NA_PH + na_align (sizeof (double2) * NA_MAX_K * NA_MAX_NP);

}  // namespace

// the scratch of stokes_gpu_atimes_noalloc, one copy per device
static __device__ __align__ (256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {

// host copies of the derived tables, in static storage (no heap), guarded
// by a mutex for the time a call builds and uploads them
struct NaHost {
  Img4 img[NA_MAX_IMG];
  double kt[KT_STRIDE * NA_MAX_K];
  double pp[6 * NA_MAX_NP];
};
NaHost t_host;
std::mutex g_host_mu;

std::mutex g_na_mu;
void *g_na_ptr[64];   // device address of the scratch per device ordinal

// Device address of the scratch on the current device.  In host code the
// array's name is only a stand-in, so the address is taken once per device
// with cudaGetSymbolAddress while that device is current.
int
na_scratch (void **out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice (&dev);
  if (e != cudaSuccess) return cuda_fail (e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return set_error (STOKES_GPU_EINVAL, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lk (g_na_mu);
  if (!g_na_ptr[dev])
    {
      void *p = nullptr;
      e = cudaGetSymbolAddress (&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_fail (e, "cudaGetSymbolAddress(scratch)");
      g_na_ptr[dev] = p;
    }
  *out = g_na_ptr[dev];
  return STOKES_GPU_OK;
}

// image list (table form with the shear shift folded in), as the regular
// product builds it from the struct (src/ewald.c:678-686)
int
na_images (const struct stokes *sys, int *nimg)
{
  if (sys->nr > NA_MAX_IMG)
    return set_error (STOKES_GPU_ETOOBIG, "%d real-space images; this entry point takes at most %d",
                      sys->nr, NA_MAX_IMG);
  for (int m = 0; m < sys->nr; m++)
    {
      double sx = 0.0;
      if (sys->shear_mode == 1) sx = (double) sys->rmy[m] * sys->shear_shift;
      else if (sys->shear_mode == 2) sx = (double) sys->rmz[m] * sys->shear_shift;
      t_host.img[m] = Img4{sys->rlx[m] + sx, sys->rly[m], sys->rlz[m], 0.0};
    }
  *nimg = sys->nr;
  return STOKES_GPU_OK;
}

// reciprocal vectors and weights (src/ewald.c:923-958)
int
na_ktable (const struct stokes *sys, int *nk_out)
{
  const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly, k0z = 2.0 * M_PI / sys->lz;
  const double sl = sys->shear_shift / sys->lx;
  int nk = 0;
  for (int m1 = -sys->kmaxx; m1 <= sys->kmaxx; m1++)
    for (int m2 = -sys->kmaxy; m2 <= sys->kmaxy; m2++)
      for (int m3 = -sys->kmaxz; m3 <= sys->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          const double k1 = k0x * m1;
          double k2 = k0y * m2, k3 = k0z * m3;
          if (sys->shear_mode == 1) k2 = k0y * ((double) m2 - sl * (double) m1);
          else if (sys->shear_mode == 2) k3 = k0z * ((double) m3 - sl * (double) m1);
          const double kk = k1 * k1 + k2 * k2 + k3 * k3;
          const double k = sqrt (kk);
          if (sys->kmax != 0.0 && k > sys->kmax) continue;
          if (nk == NA_MAX_K)
            return set_error (STOKES_GPU_ETOOBIG,
                              "more than %d reciprocal vectors; this entry point takes at most %d",
                              NA_MAX_K, NA_MAX_K);
          const double k4z = kk / 4.0 / sys->xi2;
          const double kexp = sys->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          double *r = t_host.kt + (size_t) KT_STRIDE * nk;
          for (int q = 0; q < KT_STRIDE; q++) r[q] = 0.0;
          r[KT_KX] = k1; r[KT_KY] = k2; r[KT_KZ] = k3;
          r[KT_EX] = k1 / k; r[KT_EY] = k2 / k; r[KT_EZ] = k3 / k;
          r[KT_K] = k; r[KT_KK] = kk; r[KT_KEXP] = kexp;
          r[KT_GF] = r[KT_AF] = 1.0;
          r[KT_YA] = 6.0 * (1.0 - kk / 3.0) * kexp;
          r[KT_YB] = 3.0 * k * kexp;
          r[KT_YC] = 1.5 * kk * kexp;
          r[KT_YG] = 3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp;
          r[KT_YH] = 1.5 * kk * kexp;
          r[KT_YM] = 3.0 * (1.0 - kk / 5.0) * kk * kexp;
          nk++;
        }
  *nk_out = nk;
  return STOKES_GPU_OK;
}

// radii, slip radii, Laplacian radii squared, self scalars (src/ewald.c:540-643)
void
na_particles (const struct stokes *sys, int mode)
{
  const int np = sys->np;
  double *rad = t_host.pp, *slipa = rad + np, *qa = slipa + np, *selfc = qa + np;
  for (int i = 0; i < np; i++)
    {
      const double a = sys->a ? sys->a[i] : 1.0;
      rad[i] = a;
      slipa[i] = sys->slip ? sys->slip_a[i] : a;
      qa[i] = (mode == MODE_SLIP) ? slipa[i] * slipa[i] : a * a;
      double sa = sys->self_a, sc = sys->self_c, sm = sys->self_m;
      if (mode != MODE_MONO)
        {
          const double a2 = a * a, a3 = a2 * a;
          double fa = 1.0, fc = 1.0, fm = 1.0;
          if (sys->slip) { fa = sys->slip_G32[i]; fc = sys->slip_G30[i]; fm = sys->slip_G52[i]; }
          sa = fa - a * sys->xiaspi * (6.0 - 40.0 / 3.0 * sys->xia2 * a2);
          sc = 0.75 * fc - a3 * sys->xiaspi * sys->xia2 * 10.0;
          sm = 0.9 * fm - a3 * sys->xiaspi * sys->xia2 * (12.0 - 30.24 * sys->xia2 * a2);
        }
      selfc[3 * i] = sa;
      selfc[3 * i + 1] = sc;
      selfc[3 * i + 2] = sm;
    }
}

}  // namespace
}  // namespace lsg

using namespace lsg;

extern "C" int
stokes_gpu_atimes_noalloc (struct stokes *sys, const double *d_pos, const double *d_x,
                           double *d_y, void *stream)
{
  clear_error ();
  if (sys == nullptr) return set_error (STOKES_GPU_EINVAL, "struct stokes is NULL");
  if (!d_pos || !d_x || !d_y) return set_error (STOKES_GPU_EINVAL, "NULL device pointer");
  if (sys->periodic == 0)
    return set_error (STOKES_GPU_ENOTPERIODIC, "this entry point serves periodic systems");
  if (sys->version < 0 || sys->version > 2)
    return set_error (STOKES_GPU_EINVAL, "invalid version %d", sys->version);
  if (sys->np <= 0) return set_error (STOKES_GPU_EINVAL, "no particles");
  if (!(sys->lx > 0.0 && sys->ly > 0.0 && sys->lz > 0.0))
    return set_error (STOKES_GPU_EINVAL, "box size not set");
  if (!(sys->xi > 0.0)) return set_error (STOKES_GPU_EINVAL, "Ewald xi not set");
  if (sys->np > NA_MAX_NP)
    return set_error (STOKES_GPU_ETOOBIG, "%d particles; this entry point takes at most %d",
                      sys->np, NA_MAX_NP);
  if (sys->nr > 0 && (!sys->rlx || !sys->rly || !sys->rlz))
    return set_error (STOKES_GPU_EINVAL, "image table missing (stokes_set_xi not called?)");
  cudaStream_t st = (cudaStream_t) stream;
  {
    // the table uploads end in a synchronize, which a capture cannot record
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing (st, &cs);
    if (ce != cudaSuccess) return cuda_fail (ce, "cudaStreamIsCapturing");
    if (cs != cudaStreamCaptureStatusNone)
      return set_error (STOKES_GPU_EINVAL,
                        "stokes_gpu_atimes_noalloc cannot be captured into a CUDA graph "
                        "(it waits for its table uploads)");
  }
  const int np = sys->np;
  const int mode = sys->slip ? MODE_SLIP : (sys->a ? MODE_POLY : MODE_MONO);
  void *base = nullptr;
  int rc = na_scratch (&base);
  if (rc) return rc;
  std::lock_guard<std::mutex> host_lock (g_host_mu);
  int nimg = 0, nk = 0;
  rc = na_images (sys, &nimg);
  if (!rc) rc = na_ktable (sys, &nk);
  if (rc) return rc;
  na_particles (sys, mode);

  unsigned char *b = (unsigned char *) base;
  Img4 *img = (Img4 *) (b + NA_IMG);
  double *kt = (double *) (b + NA_KT);
  double *pp = (double *) (b + NA_PP);
  double *part = (double *) (b + NA_PART);
  double *yrec = (double *) (b + NA_YREC);
  double *sf = (double *) (b + NA_SF);
  double2 *ph = (double2 *) (b + NA_PH);

  // derived tables into the scratch; the copies complete before the host
  // staging is released
  cudaError_t e = cudaSuccess;
  if (nimg) e = cudaMemcpyAsync (img, t_host.img, sizeof (Img4) * nimg, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nk)
    e = cudaMemcpyAsync (kt, t_host.kt, sizeof (double) * KT_STRIDE * nk, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync (pp, t_host.pp, sizeof (double) * 6 * np, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "scratch upload");

  if (nk > 0 && (e = launch_phase_fp64 (d_pos, kt, nk, np, ph, st)) != cudaSuccess)
    return cuda_fail (e, "phase kernel");
  RecipArgs ra;
  ra.x = d_x; ra.ph = ph; ra.kt = kt; ra.rad = pp; ra.qa = pp + 2 * np;
  ra.nk = nk; ra.np = np; ra.sf = sf; ra.yrec = yrec;
  if ((e = launch_recip_fp64 (sys->version, mode, ra, st)) != cudaSuccess)
    return cuda_fail (e, "reciprocal kernels");
  RealArgs a;
  a.pos = d_pos; a.x = d_x; a.img = img; a.nimg = nimg; a.np = np;
  a.nchunk = np < NA_NCHUNK ? np : NA_NCHUNK;
  a.rmax2 = sys->rmax2; a.rmin = sys->rmin; a.xi = sys->xi; a.xisp = sys->xi / sqrt (M_PI);
  a.rad = pp; a.slipa = pp + np; a.partial = part;
  if ((e = launch_real_fp64 (sys->version, mode, a, st)) != cudaSuccess)
    return cuda_fail (e, "real-space kernel");
  if ((e = launch_combine_fp64 (sys->version, d_x, part, a.nchunk, yrec, pp + 3 * np, np, d_y,
                                st)) != cudaSuccess)
    return cuda_fail (e, "combine kernel");
  return STOKES_GPU_OK;
}
