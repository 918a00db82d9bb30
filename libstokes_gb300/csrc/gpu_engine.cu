// gpu_engine.cu -- host engine and C ABI of libstokes_gb300.
//
// Keeps one device context per struct stokes (keyed by its address):
// a stream, timing events, grow-only device buffers and the device copies
// of the lattice tables.  Every product re-derives the image list, the
// reciprocal table and the per-particle constants from the struct on the
// host (cheap, O(images + k + np)) and re-uploads only what changed, so a
// caller may poke struct members directly between calls, as libstokes'
// own tests do (test/check-ewald.c:73-125).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "stokes_gpu.h"
#include "engine.h"
#include "gpu_engine.h"

namespace lsg {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local int t_err = STOKES_GPU_OK;
static thread_local char t_msg[512] = "";
static int g_error_mode = 0;

int
set_error (int code, const char *fmt, ...)
{
  t_err = code;
  va_list ap;
  va_start (ap, fmt);
  vsnprintf (t_msg, sizeof t_msg, fmt, ap);
  va_end (ap);
  return code;
}

int
cuda_fail (cudaError_t e, const char *where)
{
  if (e == cudaErrorMemoryAllocation)
    return set_error (STOKES_GPU_ENOMEM, "%s: %s", where, cudaGetErrorString (e));
  return set_error (STOKES_GPU_ECUDA, "%s: %s", where, cudaGetErrorString (e));
}

// called by the void drop-in functions on failure
void
dropin_failed (const char *fn, double *out, size_t nout)
{
  fprintf (stderr, "libstokes_gb300 %s: %s\n", fn, t_msg);
  if (g_error_mode == 0) exit (1);
  if (out)
    for (size_t q = 0; q < nout; q++) out[q] = NAN;
}

// ---------------------------------------------------------------------------
// buffers and contexts
// ---------------------------------------------------------------------------
cudaError_t
DevBuf::ensure (size_t bytes)
{
  if (bytes <= cap) return cudaSuccess;
  if (p) cudaFree (p);
  p = nullptr;
  cap = 0;
  size_t want = bytes + bytes / 4 + 256;
  cudaError_t e = cudaMalloc (&p, want);
  if (e != cudaSuccess) { p = nullptr; return e; }
  cap = want;
  return cudaSuccess;
}

void
DevBuf::release ()
{
  if (p) cudaFree (p);
  p = nullptr;
  cap = 0;
}

static std::mutex g_mu;
static std::unordered_map<const void *, Ctx *> g_ctx;

static uint64_t
fnv (const void *data, size_t n, uint64_t h = 1469598103934665603ull)
{
  // FNV-1a over 8-byte words (the tail byte-wise): a change detector for
  // host tables, so word granularity is enough and 8x cheaper
  const unsigned char *b = (const unsigned char *) data;
  size_t q = 0;
  for (; q + 8 <= n; q += 8)
    {
      uint64_t w;
      memcpy (&w, b + q, 8);
      h ^= w;
      h *= 1099511628211ull;
    }
  for (; q < n; q++) { h ^= b[q]; h *= 1099511628211ull; }
  return h;
}

Ctx *
get_ctx (const struct stokes *sys, bool create)
{
  std::lock_guard<std::mutex> lk (g_mu);
  auto it = g_ctx.find (sys);
  if (it != g_ctx.end ()) return it->second;
  if (!create) return nullptr;
  Ctx *c = new Ctx ();
  cudaGetDevice (&c->device);
  if (cudaStreamCreateWithFlags (&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    { delete c; return nullptr; }
  for (int q = 0; q < 4; q++) cudaEventCreate (&c->ev[q]);
  for (int q = 0; q < 2; q++) cudaEventCreateWithFlags (&c->join[q], cudaEventDisableTiming);
  const char *env = getenv ("LIBSTOKES_GB300_PRECISION");
  c->precision = (env && strcmp (env, "mixed") == 0) ? STOKES_GPU_MIXED : STOKES_GPU_FP64;
  g_ctx[sys] = c;
  return c;
}

static void
free_ctx (Ctx *c)
{
  for (cudaEvent_t e : c->prof_ev) cudaEventDestroy (e);
  for (cudaEvent_t e : c->kprof_ev) cudaEventDestroy (e);
  for (DevBuf *b : c->all_buffers ()) b->release ();
  for (int q = 0; q < 4; q++) cudaEventDestroy (c->ev[q]);
  for (int q = 0; q < 2; q++) cudaEventDestroy (c->join[q]);
  if (c->hpos) cudaFreeHost (c->hpos);
  cudaStreamDestroy (c->stream);
  release_mixed (c);
  release_vjp_mixed (c);
  if (c->tuned) stokes_free (c->tuned);
  if (c->dense) stokes_free (c->dense);
  delete c;
}

int
release_ctx (const struct stokes *sys)
{
  Ctx *c = nullptr;
  {
    std::lock_guard<std::mutex> lk (g_mu);
    auto it = g_ctx.find (sys);
    if (it == g_ctx.end ()) return STOKES_GPU_OK;
    c = it->second;
    g_ctx.erase (it);
  }
  cudaStreamSynchronize (c->stream);
  free_ctx (c);
  return STOKES_GPU_OK;
}

// ---------------------------------------------------------------------------
// host-side tables
// ---------------------------------------------------------------------------
int
check_sys (const struct stokes *sys, bool open)
{
  if (sys == nullptr) return set_error (STOKES_GPU_EINVAL, "struct stokes is NULL");
  if (sys->version < 0 || sys->version > 2)
    return set_error (STOKES_GPU_EINVAL, "invalid version %d", sys->version);
  if (sys->np <= 0 || sys->pos == nullptr)
    return set_error (STOKES_GPU_EINVAL, "no particles (np = %d)", sys->np);
  // the free-space operator needs neither a box nor a split
  if (open) return STOKES_GPU_OK;
  if (!(sys->lx > 0.0 && sys->ly > 0.0 && sys->lz > 0.0))
    return set_error (STOKES_GPU_EINVAL, "box size not set");
  if (sys->xi <= 0.0) return set_error (STOKES_GPU_EINVAL, "Ewald xi not set");
  return STOKES_GPU_OK;
}

int
check_positions (const double *pos, int np)
{
  for (int k = 0; k < 3 * np; k++)
    if (!std::isfinite (pos[k]))
      return set_error (STOKES_GPU_EINVAL, "non-finite position of particle %d (%c = %g)", k / 3,
                        "xyz"[k % 3], pos[k]);
  return STOKES_GPU_OK;
}

// real-space image list.  Table form: images of sys->rl* with the shear
// shift of src/ewald.c:678-686 folded in.  Cube form ("_notbl"): the cube
// |m| <= rmax{x,y,z} with the running shear shift of src/ewald.c:1843-1861
// (rlx is reset per m1 only, so the shift accumulates over m2, m3).
void
build_images (const struct stokes *sys, bool cube, std::vector<Img4> &img)
{
  img.clear ();
  if (!cube)
    {
      img.reserve (sys->nr);
      for (int m = 0; m < sys->nr; m++)
        {
          double sx = 0.0;
          if (sys->shear_mode == 1) sx = (double) sys->rmy[m] * sys->shear_shift;
          else if (sys->shear_mode == 2) sx = (double) sys->rmz[m] * sys->shear_shift;
          img.push_back (Img4{sys->rlx[m] + sx, sys->rly[m], sys->rlz[m], 0.0});
        }
      return;
    }
  for (int m1 = -sys->rmaxx; m1 <= sys->rmaxx; m1++)
    {
      double rlx = sys->lx * (double) m1;
      for (int m2 = -sys->rmaxy; m2 <= sys->rmaxy; m2++)
        {
          const double rly = sys->ly * (double) m2;
          for (int m3 = -sys->rmaxz; m3 <= sys->rmaxz; m3++)
            {
              const double rlz = sys->lz * (double) m3;
              if (sys->shear_mode == 1) rlx += (double) m2 * sys->shear_shift;
              else if (sys->shear_mode == 2) rlx += (double) m3 * sys->shear_shift;
              img.push_back (Img4{rlx, rly, rlz, 0.0});
            }
        }
    }
}

// reciprocal table: the k cube |m_i| <= kmax{x,y,z} without 0, the sphere
// |k| <= kmax unless kmax == 0, Lees-Edwards shifted (src/ewald.c:923-958)
void
build_ktable (const struct stokes *sys, std::vector<double> &kt)
{
  kt.clear ();
  const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly, k0z = 2.0 * M_PI / sys->lz;
  const double sl = sys->shear_shift / sys->lx;
  for (int m1 = -sys->kmaxx; m1 <= sys->kmaxx; m1++)
    for (int m2 = -sys->kmaxy; m2 <= sys->kmaxy; m2++)
      for (int m3 = -sys->kmaxz; m3 <= sys->kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          const double k1 = k0x * (double) m1;
          double k2 = k0y * (double) m2;
          double k3 = k0z * (double) m3;
          if (sys->shear_mode == 1) k2 = k0y * ((double) m2 - sl * (double) m1);
          else if (sys->shear_mode == 2) k3 = k0z * ((double) m3 - sl * (double) m1);
          const double kk = k1 * k1 + k2 * k2 + k3 * k3;
          const double k = sqrt (kk);
          if (sys->kmax != 0.0 && k > sys->kmax) continue;
          const double k4z = kk / 4.0 / sys->xi2;
          const double kexp = sys->pivol * (1.0 + k4z * (1.0 + 2.0 * k4z)) / kk * exp (-k4z);
          double row[KT_STRIDE] = {0};
          row[KT_KX] = k1; row[KT_KY] = k2; row[KT_KZ] = k3;
          row[KT_EX] = k1 / k; row[KT_EY] = k2 / k; row[KT_EZ] = k3 / k;
          row[KT_K] = k; row[KT_KK] = kk; row[KT_KEXP] = kexp;
          row[KT_GF] = row[KT_AF] = 1.0;
          row[KT_YA] = 6.0 * (1.0 - kk / 3.0) * kexp;
          row[KT_YB] = 3.0 * k * kexp;
          row[KT_YC] = 1.5 * kk * kexp;
          row[KT_YG] = 3.0 * (1.0 - 4.0 / 15.0 * kk) * k * kexp;
          row[KT_YH] = 1.5 * kk * kexp;
          row[KT_YM] = 3.0 * (1.0 - kk / 5.0) * kk * kexp;
          kt.insert (kt.end (), row, row + KT_STRIDE);
        }
}

// per-particle arrays: radii (1 when a == NULL), slip radii, squared
// Laplacian radii, and self scalars (src/ewald.c:540-643)
void
build_particles (const struct stokes *sys, int mode, std::vector<double> &pp, bool open,
                 const struct stokes *split)
{
  // the self terms follow the split of `split` (the tuned one), the radii
  // and slip factors are the system's own
  const struct stokes *sp = split ? split : sys;
  const int np = sys->np;
  pp.assign ((size_t) 6 * np, 0.0);
  double *rad = pp.data (), *slipa = rad + np, *qa = slipa + np, *selfc = qa + np;
  for (int i = 0; i < np; i++)
    {
      const double a = sys->a ? sys->a[i] : 1.0;
      rad[i] = a;
      slipa[i] = sys->slip ? sys->slip_a[i] : a;
      qa[i] = (mode == MODE_SLIP) ? slipa[i] * slipa[i] : a * a;
      double sa, sc, sm;
      if (open)
        {
          // free-space self terms (src/non-ewald.c:344-358), slip factors
          sa = 1.0; sc = 0.75; sm = 0.9;
          if (sys->slip) { sa *= sys->slip_G32[i]; sc *= sys->slip_G30[i]; sm *= sys->slip_G52[i]; }
        }
      else if (mode == MODE_MONO)
        { sa = sp->self_a; sc = sp->self_c; sm = sp->self_m; }
      else
        {
          const double a2 = a * a, a3 = a2 * a;
          double fa = 1.0, fc = 1.0, fm = 1.0;
          if (sys->slip) { fa = sys->slip_G32[i]; fc = sys->slip_G30[i]; fm = sys->slip_G52[i]; }
          sa = 1.0 * fa - a * sp->xiaspi * (6.0 - 40.0 / 3.0 * sp->xia2 * a2);
          sc = 0.75 * fc - a3 * sp->xiaspi * sp->xia2 * 10.0;
          sm = 0.9 * fm - a3 * sp->xiaspi * sp->xia2 * (12.0 - 30.24 * sp->xia2 * a2);
        }
      selfc[3 * i] = sa;
      selfc[3 * i + 1] = sc;
      selfc[3 * i + 2] = sm;
    }
}

static int
upload_if_changed (DevBuf &buf, uint64_t &fp, const void *host, size_t bytes,
                   cudaStream_t st, const char *what)
{
  const uint64_t h = fnv (host, bytes, fnv (&bytes, sizeof bytes));
  if (h == fp && buf.p) return STOKES_GPU_OK;
  cudaError_t e = buf.ensure (bytes > 0 ? bytes : 64);
  if (e != cudaSuccess) return cuda_fail (e, what);
  if (bytes)
    {
      e = cudaMemcpyAsync (buf.p, host, bytes, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return cuda_fail (e, what);
      // pageable source: make the copy complete before the host vector changes
      e = cudaStreamSynchronize (st);
      if (e != cudaSuccess) return cuda_fail (e, what);
    }
  fp = h;
  return STOKES_GPU_OK;
}

// ---- the tuned FP64 split ---------------------------------------------------
// The reference's split xi = sqrt(pi) / L puts nearly all of the work in
// real space (hundreds of lattice images at N = 1000).  The FP64 products
// of equal and unequal spheres (not slip: libstokes' slip sum depends on xi
// beyond the G term, 1e-2 between splits) run at xi = eta / V^(1/3) instead (eta 6 up to 1024
// particles, 8 up to 4096, 10 above; LIBSTOKES_GB300_FP64_ETA sets it, 0
// keeps the reference's split), set up by the reference's own rules on a
// private copy of the system.  The sum is split-invariant to rounding
// (measured 5e-15 to 8e-15 against the reference's split) -- except under
// the rmin clamp, which changes only the real-space part of the clamped
// (overlapping) pairs: the real-space kernel adds that change at the
// reference's split to each clamped pair (clamp_term, ewald_fp64.cu), which
// needs the clamp radius below half the box (only the minimum image of a pair
// can be clamped).  libstokes' FTS result depends on its
// xi through the sign of its reciprocal G term (src/ewald.c:1060-1066):
// y(xi) = y_inv + 2 G(xi), G the reciprocal G part as libstokes evaluates
// it.  The tuned table therefore carries the invariant sign (-G on the tuned
// k set) and adds 2 G(xi_ref) on the reference's k set, which reproduces
// y(xi_ref).  For unequal radii the kernels derive the weights from KT_KEXP;
// G is linear in it, so the table's factors KT_GF (G) and KT_AF (the rest)
// express the same correction.
static double
tuned_eta (int np)
{
  static const double env = [] {
    const char *s = getenv ("LIBSTOKES_GB300_FP64_ETA");
    return s ? atof (s) : -1.0;
  }();
  if (env >= 0.0) return env;
  return np <= 1024 ? 6.0 : (np <= 4096 ? 8.0 : 10.0);
}

// the split and tables stokes_set_xi built for each system
struct SplitNote {
  double v[8];
  const void *rl[3];
};
static std::unordered_map<const void *, SplitNote> g_split;   // guarded by g_mu

static SplitNote
split_note (const struct stokes *sys)
{
  SplitNote n;
  const double v[8] = {sys->xi, sys->ewald_eps, sys->rmax2, sys->kmax, (double) sys->nr,
                       (double) sys->kmaxx, (double) sys->kmaxy, (double) sys->kmaxz};
  memcpy (n.v, v, sizeof v);
  n.rl[0] = sys->rlx;
  n.rl[1] = sys->rly;
  n.rl[2] = sys->rlz;
  return n;
}

static bool
split_is_as_set (const struct stokes *sys)
{
  const SplitNote now = split_note (sys);
  std::lock_guard<std::mutex> lk (g_mu);
  auto it = g_split.find (sys);
  return it != g_split.end () && memcmp (&it->second, &now, sizeof now) == 0;
}

static bool
tuned_applies (const Ctx *c, const struct stokes *sys, bool cube)
{
  const double eta = tuned_eta (sys->np);
  // the clamp (rmin > 0) of equal spheres, when only the minimum image of a
  // pair can be clamped
  bool clamp_ok = sys->rmin == 0.0;
  if (!clamp_ok && sys->rmin > 0.0 && sys->a == nullptr)
    {
      const double lmin = std::min (sys->lx, std::min (sys->ly, sys->lz));
      clamp_ok = 2.0 * sys->rmin < 0.5 * lmin;
    }
  return c->tune && eta > 0.0 && !cube && !c->open && sys->periodic && split_is_as_set (sys)
         && sys->slip == nullptr && sys->shear_mode == 0
         && clamp_ok && sys->np > 0 && eta > sys->xi * cbrt (sys->lx * sys->ly * sys->lz);
}

// the private copy at the tuned split (rebuilt when the box, size, version
// or accuracy change)
static const struct stokes *
tuned_system (Ctx *c, const struct stokes *sys)
{
  const double eps = sys->ewald_eps > 0.0 ? sys->ewald_eps : 1e-12;
  const double eta = tuned_eta (sys->np);
  const double key[7] = {sys->lx, sys->ly, sys->lz, (double) sys->np, (double) sys->version,
                         eta, eps};
  if (c->tuned && memcmp (c->tuned_key, key, sizeof key) == 0) return c->tuned;
  if (c->tuned) stokes_free (c->tuned);
  struct stokes *sv = stokes_init ();
  if (!sv) return nullptr;
  sv->version = sys->version;
  sv->periodic = 1;
  stokes_set_np (sv, sys->np, sys->nm);
  stokes_set_l (sv, sys->lx, sys->ly, sys->lz);
  stokes_set_xi (sv, eta / cbrt (sys->lx * sys->ly * sys->lz), eps);
  c->tuned = sv;
  memcpy (c->tuned_key, key, sizeof key);
  return sv;
}

// FTS: -G on the tuned k set, +2 G(xi_ref) on the reference's k set (merged
// into a tuned entry with the same k, appended otherwise)
static void
g_correction (const struct stokes *sys, std::vector<double> &kt)
{
  const double k0x = 2.0 * M_PI / sys->lx, k0y = 2.0 * M_PI / sys->ly, k0z = 2.0 * M_PI / sys->lz;
  auto key = [] (long long a, long long b, long long c) {
    return (a + 4096) * 8192 * 8192 + (b + 4096) * 8192 + (c + 4096);
  };
  std::unordered_map<long long, size_t> at;
  const size_t nk = kt.size () / KT_STRIDE;
  for (size_t q = 0; q < nk; q++)
    {
      double *row = &kt[q * KT_STRIDE];
      row[KT_YG] = -row[KT_YG];
      row[KT_GF] = -1.0;        // the same for the weights derived from KT_KEXP
      at.emplace (key (llrint (row[KT_KX] / k0x), llrint (row[KT_KY] / k0y),
                       llrint (row[KT_KZ] / k0z)), q);
    }
  std::vector<double> ref;
  build_ktable (sys, ref);
  const size_t nr = ref.size () / KT_STRIDE;
  for (size_t q = 0; q < nr; q++)
    {
      const double *row = &ref[q * KT_STRIDE];
      const double g2 = 2.0 * row[KT_YG];
      const auto hit = at.find (key (llrint (row[KT_KX] / k0x), llrint (row[KT_KY] / k0y),
                                     llrint (row[KT_KZ] / k0z)));
      if (hit != at.end ())
        {
          // G is linear in kexp: -G(kexp_t) + 2 G(kexp_ref) = G(kexp_t) (-1 +
          // 2 kexp_ref / kexp_t) for the derived weights
          double *t = &kt[hit->second * KT_STRIDE];
          t[KT_YG] += g2;
          t[KT_GF] = -1.0 + 2.0 * row[KT_KEXP] / t[KT_KEXP];
          continue;
        }
      double add[KT_STRIDE];
      memcpy (add, row, sizeof add);
      add[KT_YA] = add[KT_YB] = add[KT_YC] = add[KT_YH] = add[KT_YM] = 0.0;
      add[KT_YG] = g2;
      add[KT_GF] = 2.0;
      add[KT_AF] = 0.0;
      kt.insert (kt.end (), add, add + KT_STRIDE);
    }
}

int
prepare (Ctx *c, const struct stokes *sys, bool cube, int tables)
{
  int rc = check_sys (sys, sys && (sys->periodic == 0 || c->force_open));
  if (rc) return rc;
  c->open = sys->periodic == 0 || c->force_open;
  if (!c->open && !cube && (sys->nr > 0) && (!sys->rlx || !sys->rly || !sys->rlz))
    return set_error (STOKES_GPU_EINVAL, "image table missing (stokes_set_xi not called?)");
  c->sys = sys;
  c->cube = cube;
  c->version = sys->version;
  c->np = sys->np;
  c->mode = sys->slip ? MODE_SLIP : (sys->a ? MODE_POLY : MODE_MONO);
  c->xi = sys->xi;
  c->xi_ref = sys->xi;
  c->xisp = sys->xi / sqrt (M_PI);
  c->rmax2 = sys->rmax2;
  c->rmin = sys->rmin;
  if (c->open)
    {
      // every pair, once, in free space: one zero image, no cutoff, no k
      c->xi = c->xisp = 0.0;
      c->rmax2 = DBL_MAX;
    }

  // the free-space products (FP64 and mixed) read the particle table and the
  // FP64 set-up of the open system
  if (tables < 0) tables = c->precision == STOKES_GPU_MIXED && !c->open ? 0 : 1;
  // the dense builder pays for every k vector once per pair: it keeps the
  // reference's split, which is light in reciprocal space
  const bool dense = tables == 2;
  if (dense) tables = 1;
  if (!tables)
    {
      // the particle table only (radii for the BD interactions); equal
      // spheres without slip need none
      if (c->mode == MODE_MONO) return STOKES_GPU_OK;
      build_particles (sys, c->mode, c->h_pp, c->open);
      return upload_if_changed (c->pp, c->fp_pp, c->h_pp.data (), sizeof (double) * c->h_pp.size (),
                                c->stream, "particle table");
    }
  // the system whose split the FP64 tables follow
  const struct stokes *ts = sys;
  if (!dense && tuned_applies (c, sys, cube))
    {
      ts = tuned_system (c, sys);
      if (!ts) return set_error (STOKES_GPU_ENOMEM, "tuned split");
      c->xi = ts->xi;
      c->xisp = ts->xi / sqrt (M_PI);
      c->rmax2 = ts->rmax2;
    }
  if (c->open)
    c->h_img.assign (1, Img4 {0.0, 0.0, 0.0, 0.0});
  else
    build_images (ts, cube, c->h_img);
  c->nimg = (int) c->h_img.size ();
  rc = upload_if_changed (c->img, c->fp_img, c->h_img.data (), sizeof (Img4) * c->h_img.size (),
                          c->stream, "image table");
  if (rc) return rc;
  if (c->open)
    c->h_kt.clear ();
  else
    {
      build_ktable (ts, c->h_kt);
      if (ts != sys && sys->version == 2) g_correction (sys, c->h_kt);
    }
  c->nk = (int) (c->h_kt.size () / KT_STRIDE);
  rc = upload_if_changed (c->kt, c->fp_kt, c->h_kt.data (), sizeof (double) * c->h_kt.size (),
                          c->stream, "reciprocal table");
  if (rc) return rc;
  // self terms at the split of the tables (radii: the system's own)
  build_particles (sys, c->mode, c->h_pp, c->open, ts);
  rc = upload_if_changed (c->pp, c->fp_pp, c->h_pp.data (), sizeof (double) * c->h_pp.size (),
                          c->stream, "particle table");
  if (rc) return rc;
  return STOKES_GPU_OK;
}

// ---------------------------------------------------------------------------
// FP64 product on device buffers
// ---------------------------------------------------------------------------
static int
choose_nchunk (int np)
{
  // about 8 warps of work per SM slot; a chunk holds at least one source
  const int target = 152 * 32;
  int nc = (target + np - 1) / np;
  if (nc < 1) nc = 1;
  if (nc > np) nc = np;
  if (nc > 64) nc = 64;
  return nc;
}

int
atimes_fp64_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y,
                 cudaStream_t st, bool timed)
{
  const int np = c->np, C = NCOMP (c->version);
  const int nchunk = choose_nchunk (np);
  cudaError_t e;
  if ((e = c->partial.ensure (sizeof (double) * (size_t) nchunk * np * C)) != cudaSuccess)
    return cuda_fail (e, "real-space scratch");
  if ((e = c->yrec.ensure (sizeof (double) * (size_t) np * C)) != cudaSuccess)
    return cuda_fail (e, "reciprocal scratch");
  if ((e = c->ph.ensure (sizeof (double2) * (size_t) (c->nk > 0 ? c->nk : 1) * np)) != cudaSuccess)
    return cuda_fail (e, "phase table");
  if ((e = c->sf.ensure (sizeof (double) * (size_t) SF_STRIDE * (c->nk > 0 ? c->nk : 1))) != cudaSuccess)
    return cuda_fail (e, "structure factors");

  const double *pp = (const double *) c->pp.p;
  const double *rad = pp, *slipa = pp + np, *qa = pp + 2 * np, *selfc = pp + 3 * np;
  int launches = 0;
  cudaEvent_t *E = phase_events (c, timed);
  if (E) cudaEventRecord (E[0], st);
  kmark (c, st, nullptr);

  // reciprocal space
  if (c->nk > 0)
    {
      if ((e = launch_phase_fp64 (d_pos, (const double *) c->kt.p, c->nk, np,
                                  (double2 *) c->ph.p, st)) != cudaSuccess)
        return cuda_fail (e, "phase kernel");
      launches++;
      kmark (c, st, "k_phase");
    }
  RecipArgs ra;
  ra.x = d_x;
  ra.ph = (const double2 *) c->ph.p;
  ra.kt = (const double *) c->kt.p;
  ra.rad = rad;
  ra.qa = qa;
  ra.nk = c->nk;
  ra.np = np;
  ra.sf = (double *) c->sf.p;
  ra.yrec = (double *) c->yrec.p;
  if ((e = launch_recip_fp64 (c->version, c->mode, ra, st)) != cudaSuccess)
    return cuda_fail (e, "reciprocal kernels");
  launches += c->nk > 0 ? 2 : 0;
  if (c->nk > 0) kmark (c, st, "k_sfac+k_backproj");
  if (E) cudaEventRecord (E[1], st);

  // real space
  RealArgs a;
  a.pos = d_pos;
  a.x = d_x;
  a.img = (const Img4 *) c->img.p;
  a.nimg = c->nimg;
  a.np = np;
  a.nchunk = nchunk;
  a.rmax2 = c->rmax2;
  a.rmin = c->rmin;
  a.xi = c->xi;
  a.xisp = c->xisp;
  a.rad = rad;
  a.slipa = slipa;
  a.partial = (double *) c->partial.p;
  a.open = c->open ? 1 : 0;
  a.clampfix = (!c->open && c->rmin > 0.0 && c->xi != c->xi_ref) ? 1 : 0;
  a.xi_ref = c->xi_ref;
  a.xisp_ref = c->xi_ref / sqrt (M_PI);
  if ((e = launch_real_fp64 (c->version, c->mode, a, st)) != cudaSuccess)
    return cuda_fail (e, "real-space kernel");
  launches++;
  kmark (c, st, "k_real");
  if (E) cudaEventRecord (E[2], st);

  if ((e = launch_combine_fp64 (c->version, d_x, (const double *) c->partial.p, nchunk,
                                (const double *) c->yrec.p, selfc, np, d_y, st)) != cudaSuccess)
    return cuda_fail (e, "combine kernel");
  launches++;
  kmark (c, st, "k_combine");
  if (E) cudaEventRecord (E[3], st);
  c->launches = launches;
  c->timed = timed;
  return STOKES_GPU_OK;
}

// Event set for one product: the context's own set for host-buffer calls
// (read back right after), or the next slot of the profiling ring while a
// profile window is open (read back at stokes_gpu_profile_end).
cudaEvent_t *
phase_events (Ctx *c, bool timed)
{
  if (timed) return c->ev;
  if (c->prof_on && c->prof_n < (int) (c->prof_ev.size () / 4))
    return &c->prof_ev[4 * (size_t) c->prof_n++];
  return nullptr;
}

void
kmark (Ctx *c, cudaStream_t st, const char *name)
{
  if (!c || !c->kprof_on || c->kprof_n >= c->kprof_ev.size ()) return;
  cudaEventRecord (c->kprof_ev[c->kprof_n], st);
  c->kprof_name[c->kprof_n] = name;
  c->kprof_n++;
}

void
collect_times (Ctx *c)
{
  if (!c->timed) return;
  // events: start, end of the reciprocal part before the real space, end of
  // the real space, end; the reciprocal time is the rest of the product
  float t_real = 0.f, t_all = 0.f;
  if (cudaEventElapsedTime (&t_all, c->ev[0], c->ev[3]) != cudaSuccess)
    {
      cudaGetLastError ();   // leave no error for the next launch check
      return;
    }
  if (cudaEventElapsedTime (&t_real, c->ev[1], c->ev[2]) != cudaSuccess)
    {
      cudaGetLastError ();
      t_real = (float) c->times[1];
    }
  c->times[0] = t_all;
  c->times[1] = t_real;
  c->times[2] = t_all - t_real;
}

int
atimes_dev (Ctx *c, const double *d_pos, const double *d_x, double *d_y, cudaStream_t st,
            bool timed)
{
  if (c->precision == STOKES_GPU_MIXED)
    return c->open ? atimes_open_f32_dev (c, d_pos, d_x, d_y, st, timed)
                   : atimes_mixed_dev (c, d_pos, d_x, d_y, st, timed);
  return atimes_fp64_dev (c, d_pos, d_x, d_y, st, timed);
}

// host buffers in and out; positions from sys->pos
void clear_error () { t_err = STOKES_GPU_OK; t_msg[0] = 0; }

// the device address of a pinned (page-locked, mapped) host buffer, or
// nullptr for any other memory
static void *
mapped_host (const void *p)
{
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes (&at, p) != cudaSuccess)
    {
      cudaGetLastError ();
      return nullptr;
    }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// the positions as the mixed kernels read them from a host call: sys->pos in
// place when it is pinned, else a copy in the context's pinned mirror. The
// mixed kernels read each coordinate once (mk_prep, k_open_prep convert
// them), so a read over the CPU-GPU link replaces the staging copy of
// pageable memory. Called only between synchronised host calls, so no
// kernel is reading the mirror while it is rewritten.
static const double *
mapped_positions (Ctx *c, const struct stokes *sys)
{
  const size_t bytes = sizeof (double) * 3 * sys->np;
  if (const double *p = (const double *) mapped_host (sys->pos)) return p;
  if (c->hpos_bytes < bytes)
    {
      if (c->hpos) cudaFreeHost (c->hpos);
      c->hpos = nullptr;
      c->hpos_bytes = 0;
      if (cudaHostAlloc ((void **) &c->hpos, bytes, cudaHostAllocMapped) != cudaSuccess)
        {
          cudaGetLastError ();
          c->hpos = nullptr;
          return nullptr;
        }
      c->hpos_dev = (const double *) mapped_host (c->hpos);
      if (!c->hpos_dev) return nullptr;
      c->hpos_bytes = bytes;
    }
  memcpy (c->hpos, sys->pos, bytes);
  return c->hpos_dev;
}

int
atimes_host (struct stokes *sys, const double *x, double *y, bool cube)
{
  clear_error ();
  if (x == nullptr || y == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL x or y");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, cube);
  if (rc) return rc;
  if ((rc = check_positions (sys->pos, sys->np))) return rc;
  const int np = sys->np, n = NCOMP (sys->version) * np;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess) return cuda_fail (e, "pos");
  // pinned host buffers (cudaHostAlloc, cudaHostRegister) are used in place
  // through their device mapping -- over the CPU-GPU link -- without a
  // staging copy and its latency: y always (each element is written once),
  // x on the mixed paths, which read it twice (the FP64 kernels read x once
  // per reciprocal vector or pair and take a device copy); other host
  // memory goes through device copies
  const double *d_x = c->precision == STOKES_GPU_MIXED ? (const double *) mapped_host (x) : nullptr;
  double *d_y = (double *) mapped_host (y);
  if (!d_x)
    {
      if ((e = c->x.ensure (sizeof (double) * n)) != cudaSuccess) return cuda_fail (e, "x");
      cudaMemcpyAsync (c->x.p, x, sizeof (double) * n, cudaMemcpyHostToDevice, c->stream);
      d_x = (const double *) c->x.p;
    }
  if (!d_y)
    {
      if ((e = c->y.ensure (sizeof (double) * n)) != cudaSuccess) return cuda_fail (e, "y");
    }
  const double *d_pos = c->precision == STOKES_GPU_MIXED ? mapped_positions (c, sys) : nullptr;
  if (!d_pos)
    {
      cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice,
                       c->stream);
      d_pos = (const double *) c->pos.p;
    }
  rc = atimes_dev (c, d_pos, d_x, d_y ? d_y : (double *) c->y.p, c->stream, true);
  if (rc) return rc;
  e = d_y ? cudaSuccess
          : cudaMemcpyAsync (y, c->y.p, sizeof (double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  if (e != cudaSuccess) return cuda_fail (e, "atimes");
  // a bounded wait of this product's tensor-core kernels that ran out
  if (c->precision == STOKES_GPU_MIXED && !c->open && (rc = mixed_check_status (c)) != 0)
    return rc;
  collect_times (c);
  sys->cpu1 = c->times[0];
  sys->cpu2 = c->times[1];
  sys->cpu3 = c->times[2];
  return STOKES_GPU_OK;
}

// ---- the thread-per-pair dense builder ---------------------------------------
// The split-precision builder of equal spheres pays for every real-space
// image and every reciprocal vector once per pair.  At xi = eta / V^(1/3)
// with eta about 2 and libstokes' cutoff rule at eps = 1e-6, a pair holds
// about 35 images and 125 half-space vectors (the reference's split at its
// 1e-12 holds about 110 images).  LIBSTOKES_GB300_DENSE_ETA sets
// eta (0: the warp-per-pair builder at the reference's split).  FTS takes
// the G correction of the tuned FP64 split (g_correction), so that the
// matrix is that of the reference's split.
static double
dense_eta ()
{
  static const double env = [] {
    const char *s = getenv ("LIBSTOKES_GB300_DENSE_ETA");
    return s ? atof (s) : -1.0;
  }();
  return env >= 0.0 ? env : 2.2;
}

static bool
dense_pairs_apply (const Ctx *c, const struct stokes *sys)
{
  return dense_eta () > 0.0 && c->precision == STOKES_GPU_MIXED && !c->open && !c->cube
         && c->mode == MODE_MONO && sys->periodic && sys->shear_mode == 0 && sys->rmin == 0.0
         && sys->np > 0 && split_is_as_set (sys);
}

// the private copy at the dense split and its half-space tables
static int
dense_tables (Ctx *c, const struct stokes *sys, cudaStream_t st)
{
  // truncation: 1e-6 in libstokes' cutoff rule leaves about 7e-8 of the
  // largest entry (measured against eps 1e-14 on the FP64 oracle)
  const double eps = 1e-6;
  const double eta = dense_eta ();
  const double key[7] = {sys->lx, sys->ly, sys->lz, (double) sys->np, (double) sys->version,
                         eta, sys->xi};
  if (!c->dense || memcmp (c->dense_key, key, sizeof key) != 0)
    {
      if (c->dense) stokes_free (c->dense);
      c->dense = nullptr;
      struct stokes *sv = stokes_init ();
      if (!sv) return set_error (STOKES_GPU_ENOMEM, "dense split");
      sv->version = sys->version;
      sv->periodic = 1;
      stokes_set_np (sv, sys->np, sys->nm);
      stokes_set_l (sv, sys->lx, sys->ly, sys->lz);
      stokes_set_xi (sv, eta / cbrt (sys->lx * sys->ly * sys->lz), eps);
      c->dense = sv;
      memcpy (c->dense_key, key, sizeof key);
      std::vector<double> full;
      build_ktable (sv, full);
      if (sys->version == 2) g_correction (sys, full);
      // half space: the terms of k and -k are equal (cos even, sin odd with
      // the odd moments), so keep one of each pair with doubled weights
      const double k0[3] = {2.0 * M_PI / sys->lx, 2.0 * M_PI / sys->ly, 2.0 * M_PI / sys->lz};
      c->h_dkt.clear ();
      const size_t nk = full.size () / KT_STRIDE;
      for (size_t q = 0; q < nk; q++)
        {
          const double *row = &full[q * KT_STRIDE];
          const long long m1 = llrint (row[KT_KX] / k0[0]), m2 = llrint (row[KT_KY] / k0[1]),
                          m3 = llrint (row[KT_KZ] / k0[2]);
          if (!(m1 > 0 || (m1 == 0 && (m2 > 0 || (m2 == 0 && m3 > 0))))) continue;
          double h[KT_STRIDE];
          memcpy (h, row, sizeof h);
          for (int w : {KT_YA, KT_YB, KT_YC, KT_YG, KT_YH, KT_YM}) h[w] *= 2.0;
          c->h_dkt.insert (c->h_dkt.end (), h, h + KT_STRIDE);
        }
      c->dense_nk = (int) (c->h_dkt.size () / KT_STRIDE);
    }
  return upload_if_changed (c->dkt, c->fp_dkt, c->h_dkt.data (),
                            sizeof (double) * c->h_dkt.size (), st, "dense reciprocal table");
}

static int
matrix_pairs_dev (Ctx *c, const struct stokes *sys, const double *d_pos, double *d_mat,
                  cudaStream_t st)
{
  int rc = dense_tables (c, sys, st);
  if (rc) return rc;
  const int np = c->np, nk = c->dense_nk;
  const struct stokes *sv = c->dense;
  cudaError_t e;
  kmark (c, st, nullptr);
  int launches = 0;
  if (nk > 0)
    {
      if ((e = c->ph.ensure (sizeof (float2) * (size_t) nk * np)) != cudaSuccess)
        return cuda_fail (e, "phase table");
      if ((e = launch_phase_f32 (d_pos, (const double *) c->dkt.p, nk, np, (float2 *) c->ph.p,
                                 st)) != cudaSuccess)
        return cuda_fail (e, "phase kernel");
      launches++;
      kmark (c, st, "k_phase");
    }
  MatPairArgs a;
  a.pos = d_pos;
  a.np = np;
  a.mat = d_mat;
  a.lx = sys->lx; a.ly = sys->ly; a.lz = sys->lz;
  a.ilx = 1.0 / sys->lx; a.ily = 1.0 / sys->ly; a.ilz = 1.0 / sys->lz;
  a.lxh = (float) sys->lx; a.lyh = (float) sys->ly; a.lzh = (float) sys->lz;
  a.lxl = (float) (sys->lx - (double) a.lxh);
  a.lyl = (float) (sys->ly - (double) a.lyh);
  a.lzl = (float) (sys->lz - (double) a.lzh);
  a.ilxf = (float) a.ilx; a.ilyf = (float) a.ily; a.ilzf = (float) a.ilz;
  a.rc2 = (float) sv->rmax2;
  a.rc = sqrtf (a.rc2);
  a.xi = (float) sv->xi;
  a.xisp = (float) (sv->xi / sqrt (M_PI));
  a.xi64 = sv->xi;
  a.self[0] = sv->self_a;
  a.self[1] = sv->self_c;
  a.self[2] = sv->self_m;
  if ((e = c->dktf.ensure (sizeof (float) * matrix_kco_stride (c->version)
                           * (size_t) std::max (nk, 1))) != cudaSuccess)
    return cuda_fail (e, "reciprocal coefficients");
  if ((e = launch_matrix_kco (c->version, (const double *) c->dkt.p, nk, (float *) c->dktf.p,
                              st)) != cudaSuccess)
    return cuda_fail (e, "matrix kernel");
  if (nk > 0) launches++;
  a.kco = (const float *) c->dktf.p;
  a.phf = (const float2 *) c->ph.p;
  a.nk = nk;
  if ((e = c->dself.ensure (sizeof (float) * 80)) != cudaSuccess)
    return cuda_fail (e, "diagonal moments");
  a.selfmo = (const float *) c->dself.p;
  if ((e = launch_matrix_self (c->version, a, (const double *) c->dkt.p, (float *) c->dself.p,
                               st)) != cudaSuccess)
    return cuda_fail (e, "matrix kernel");
  launches++;
  if ((e = launch_matrix_pairs (c->version, a, st)) != cudaSuccess)
    return cuda_fail (e, "matrix kernel");
  kmark (c, st, "k_matrix_pairs");
  c->launches = launches + 1;
  return STOKES_GPU_OK;
}

// dense matrix on device
int
matrix_dev (Ctx *c, const double *d_pos, double *d_mat, cudaStream_t st)
{
  if (c->sys && dense_pairs_apply (c, c->sys)) return matrix_pairs_dev (c, c->sys, d_pos, d_mat, st);
  const int np = c->np;
  cudaError_t e;
  if ((e = c->ph.ensure (sizeof (double2) * (size_t) (c->nk > 0 ? c->nk : 1) * np)) != cudaSuccess)
    return cuda_fail (e, "phase table");
  int launches = 0;
  // mixed precision: FP32 terms for equal spheres (unequal radii and slip,
  // and open systems, keep the FP64 builder)
  const bool f32 = c->precision == STOKES_GPU_MIXED && !c->open && c->mode == MODE_MONO;
  kmark (c, st, nullptr);
  if (c->nk > 0)
    {
      e = f32 ? launch_phase_f32 (d_pos, (const double *) c->kt.p, c->nk, np, (float2 *) c->ph.p, st)
              : launch_phase_fp64 (d_pos, (const double *) c->kt.p, c->nk, np, (double2 *) c->ph.p,
                                   st);
      if (e != cudaSuccess) return cuda_fail (e, "phase kernel");
      launches++;
      kmark (c, st, "k_phase");
    }
  const double *pp = (const double *) c->pp.p;
  MatArgs a;
  a.pos = d_pos;
  a.img = (const Img4 *) c->img.p;
  a.nimg = c->nimg;
  a.np = np;
  a.nk = c->nk;
  a.rmax2 = c->rmax2;
  a.rmin = c->rmin;
  a.xi = c->xi;
  a.xisp = c->xisp;
  a.rad = pp;
  a.slipa = pp + np;
  a.qa = pp + 2 * np;
  a.selfc = pp + 3 * np;
  a.kt = (const double *) c->kt.p;
  a.ph = (const double2 *) c->ph.p;
  a.mat = d_mat;
  a.open = c->open ? 1 : 0;
  a.f32 = f32 ? 1 : 0;
  if (f32)
    {
      // float copies: images as hi + lo pairs, then the k table (e, ya..ym)
      const size_t ni = (size_t) c->nimg, nk = (size_t) c->nk;
      std::vector<float> f (8 * ni + KTF_STRIDE * nk + 4, 0.0f);
      for (size_t q = 0; q < ni; q++)
        {
          const double v[3] = {c->h_img[q].x, c->h_img[q].y, c->h_img[q].z};
          for (int d = 0; d < 3; d++)
            {
              const float hi = (float) v[d];
              f[4 * q + d] = hi;
              f[4 * (ni + q) + d] = (float) (v[d] - (double) hi);
            }
        }
      float *kf = f.data () + 8 * ni;
      for (size_t k = 0; k < nk; k++)
        {
          const double *K = c->h_kt.data () + KT_STRIDE * k;
          const int src[9] = {KT_EX, KT_EY, KT_EZ, KT_YA, KT_YB, KT_YC, KT_YG, KT_YH, KT_YM};
          for (int q = 0; q < 9; q++) kf[KTF_STRIDE * k + q] = (float) K[src[q]];
        }
      if ((e = c->imgf.ensure (sizeof (float) * f.size ())) != cudaSuccess)
        return cuda_fail (e, "FP32 tables");
      // pageable source: the copy is staged before the call returns, so the
      // vector may go out of scope
      if ((e = cudaMemcpyAsync (c->imgf.p, f.data (), sizeof (float) * f.size (),
                                cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail (e, "FP32 tables");
      a.imgf = (const float4 *) c->imgf.p;
      a.imgl = a.imgf + ni;
      a.ktf = (const float *) c->imgf.p + 8 * ni;
      a.phf = (const float2 *) c->ph.p;
    }
  if ((e = launch_matrix_fp64 (c->version, c->mode, a, st)) != cudaSuccess)
    return cuda_fail (e, "matrix kernel");
  kmark (c, st, a.f32 ? "k_matrix_f32" : "k_matrix");
  c->launches = launches + 1;
  return STOKES_GPU_OK;
}

int
matrix_host (struct stokes *sys, double *mat, bool cube)
{
  clear_error ();
  if (mat == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL mat");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, cube, 2);
  if (rc) return rc;
  if ((rc = check_positions (sys->pos, sys->np))) return rc;
  const int np = sys->np;
  const size_t n = (size_t) NCOMP (sys->version) * np;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess) return cuda_fail (e, "pos");
  if ((e = c->mat.ensure (sizeof (double) * n * n)) != cudaSuccess) return cuda_fail (e, "matrix");
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice, c->stream);
  cudaEventRecord (c->ev[0], c->stream);
  rc = matrix_dev (c, (const double *) c->pos.p, (double *) c->mat.p, c->stream);
  if (rc) return rc;
  cudaEventRecord (c->ev[3], c->stream);
  e = cudaMemcpyAsync (mat, c->mat.p, sizeof (double) * n * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  if (e != cudaSuccess) return cuda_fail (e, "matrix");
  float t = 0.f;
  cudaEventElapsedTime (&t, c->ev[0], c->ev[3]);
  sys->cpu1 = t;
  sys->cpu2 = t;
  sys->cpu3 = 0.0;
  return STOKES_GPU_OK;
}

// build the matrix on the device and apply it there (src/ewald.c:484-505)
int
atimes_matrix_host (struct stokes *sys, const double *x, double *y, bool cube)
{
  clear_error ();
  if (x == nullptr || y == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL x or y");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, cube, 2);
  if (rc) return rc;
  const int np = sys->np;
  const size_t n = (size_t) NCOMP (sys->version) * np;
  cudaError_t e;
  if ((e = c->pos.ensure (sizeof (double) * 3 * np)) != cudaSuccess) return cuda_fail (e, "pos");
  if ((e = c->mat.ensure (sizeof (double) * n * n)) != cudaSuccess) return cuda_fail (e, "matrix");
  if ((e = c->x.ensure (sizeof (double) * n)) != cudaSuccess) return cuda_fail (e, "x");
  if ((e = c->y.ensure (sizeof (double) * n)) != cudaSuccess) return cuda_fail (e, "y");
  if ((e = c->zbuf.ensure (sizeof (double) * n)) != cudaSuccess) return cuda_fail (e, "z");
  cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * np, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync (c->x.p, x, sizeof (double) * n, cudaMemcpyHostToDevice, c->stream);
  rc = matrix_dev (c, (const double *) c->pos.p, (double *) c->mat.p, c->stream);
  if (rc) return rc;
  if ((e = launch_gemv_fp64 (sys->version, (const double *) c->mat.p, (const double *) c->x.p,
                             (double *) c->zbuf.p, np, (double *) c->y.p, c->stream)) != cudaSuccess)
    return cuda_fail (e, "gemv");
  e = cudaMemcpyAsync (y, c->y.p, sizeof (double) * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize (c->stream);
  if (e != cudaSuccess) return cuda_fail (e, "atimes_3all_matrix");
  return STOKES_GPU_OK;
}

}  // namespace lsg

using namespace lsg;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int stokes_gpu_last_error (void) { return t_err; }
const char *stokes_gpu_last_error_message (void) { return t_msg; }
void stokes_gpu_set_error_mode (int mode) { g_error_mode = mode; }

int
stokes_gpu_set_precision (struct stokes *sys, int mode)
{
  if (sys == nullptr) return set_error (STOKES_GPU_EINVAL, "struct stokes is NULL");
  if (mode != STOKES_GPU_FP64 && mode != STOKES_GPU_MIXED)
    return set_error (STOKES_GPU_EINVAL, "invalid precision mode %d", mode);
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  c->precision = mode;
  return STOKES_GPU_OK;
}

int
stokes_gpu_get_precision (const struct stokes *sys, int *mode)
{
  if (sys == nullptr || mode == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  *mode = c->precision;
  return STOKES_GPU_OK;
}

int
stokes_gpu_release (struct stokes *sys)
{
  release_adjoint (sys);
  {
    std::lock_guard<std::mutex> lk (g_mu);
    g_split.erase (sys);
  }
  return release_ctx (sys);
}

void
stokes_gpu_note_split (const struct stokes *sys)
{
  if (!sys) return;
  const SplitNote n = split_note (sys);
  std::lock_guard<std::mutex> lk (g_mu);
  g_split[sys] = n;
}

int
stokes_gpu_atimes (struct stokes *sys, const double *x, double *y)
{
  return atimes_host (sys, x, y, false);
}

// Work for a caller's stream.  NULL names the legacy default stream (as
// everywhere in CUDA); the work then runs on the context's own non-blocking
// stream, ordered after the caller's earlier work and before its later work
// by two events, which keeps graph capture and the side stream usable.
static int
on_caller_stream (Ctx *c, void *stream, const std::function<int (cudaStream_t)> &f)
{
  if (stream) return f ((cudaStream_t) stream);
  cudaStream_t legacy = (cudaStream_t) 0;
  cudaError_t e = cudaEventRecord (c->join[0], legacy);
  if (e == cudaSuccess) e = cudaStreamWaitEvent (c->stream, c->join[0], 0);
  if (e != cudaSuccess) return cuda_fail (e, "ordering after the default stream");
  const int rc = f (c->stream);
  e = cudaEventRecord (c->join[1], c->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent (legacy, c->join[1], 0);
  if (e != cudaSuccess && rc == STOKES_GPU_OK) return cuda_fail (e, "ordering before the default stream");
  return rc;
}

int
stokes_gpu_atimes_dev (struct stokes *sys, const double *d_pos, const double *d_x,
                       double *d_y, void *stream)
{
  clear_error ();
  if (d_x == nullptr || d_y == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL x or y");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, false);
  if (rc) return rc;
  return on_caller_stream (c, stream, [&] (cudaStream_t st) {
    if (d_pos == nullptr)
      {
        cudaError_t e = c->pos.ensure (sizeof (double) * 3 * sys->np);
        if (e != cudaSuccess) return cuda_fail (e, "pos");
        cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * sys->np,
                         cudaMemcpyHostToDevice, st);
        d_pos = (const double *) c->pos.p;
      }
    return atimes_dev (c, d_pos, d_x, d_y, st, false);
  });
}

int
stokes_gpu_matrix (struct stokes *sys, double *mat)
{
  return matrix_host (sys, mat, false);
}

int
stokes_gpu_matrix_dev (struct stokes *sys, const double *d_pos, double *d_mat, void *stream)
{
  clear_error ();
  if (d_mat == nullptr) return set_error (STOKES_GPU_EINVAL, "NULL mat");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  int rc = prepare (c, sys, false, 2);
  if (rc) return rc;
  return on_caller_stream (c, stream, [&] (cudaStream_t st) {
    if (d_pos == nullptr)
      {
        cudaError_t e = c->pos.ensure (sizeof (double) * 3 * sys->np);
        if (e != cudaSuccess) return cuda_fail (e, "pos");
        cudaMemcpyAsync (c->pos.p, sys->pos, sizeof (double) * 3 * sys->np,
                         cudaMemcpyHostToDevice, st);
        d_pos = (const double *) c->pos.p;
      }
    return matrix_dev (c, d_pos, d_mat, st);
  });
}

int
stokes_gpu_matvec_dev (int version, int np, const double *d_mat, const double *d_x,
                       double *d_y, void *stream)
{
  if (version < 0 || version > 2 || np <= 0 || !d_mat || !d_x || !d_y)
    return set_error (STOKES_GPU_EINVAL, "bad matvec arguments");
  static thread_local DevBuf zb;
  cudaError_t e = zb.ensure (sizeof (double) * NCOMP (version) * (size_t) np);
  if (e != cudaSuccess) return cuda_fail (e, "z buffer");
  e = launch_gemv_fp64 (version, d_mat, d_x, (double *) zb.p, np, d_y, (cudaStream_t) stream);
  if (e != cudaSuccess) return cuda_fail (e, "gemv");
  return STOKES_GPU_OK;
}

int
stokes_gpu_last_times (const struct stokes *sys, double *ms3)
{
  if (!sys || !ms3) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c) return set_error (STOKES_GPU_EINVAL, "no product run for this system yet");
  ms3[0] = c->times[0];
  ms3[1] = c->times[1];
  ms3[2] = c->times[2];
  return STOKES_GPU_OK;
}

int
stokes_gpu_profile_begin (struct stokes *sys, int max_products)
{
  if (!sys || max_products <= 0) return set_error (STOKES_GPU_EINVAL, "bad profile window");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  const size_t want = 4 * (size_t) max_products;
  while (c->prof_ev.size () < want)
    {
      cudaEvent_t e;
      if (cudaEventCreate (&e) != cudaSuccess)
        return set_error (STOKES_GPU_ECUDA, "cannot create events");
      c->prof_ev.push_back (e);
    }
  c->prof_on = true;
  c->prof_n = 0;
  return STOKES_GPU_OK;
}

int
stokes_gpu_profile_end (struct stokes *sys, double *sum_ms3, int *count)
{
  if (!sys || !sum_ms3 || !count) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c) return set_error (STOKES_GPU_EINVAL, "no profile window open");
  c->prof_on = false;
  sum_ms3[0] = sum_ms3[1] = sum_ms3[2] = 0.0;
  for (int q = 0; q < c->prof_n; q++)
    {
      cudaEvent_t *E = &c->prof_ev[4 * (size_t) q];
      cudaError_t e = cudaEventSynchronize (E[3]);
      if (e != cudaSuccess) return cuda_fail (e, "profile events");
      float t_all = 0.f, t_real = 0.f;
      cudaEventElapsedTime (&t_real, E[1], E[2]);
      cudaEventElapsedTime (&t_all, E[0], E[3]);
      const float t_rec = t_all - t_real;
      sum_ms3[0] += t_all;
      sum_ms3[1] += t_real;
      sum_ms3[2] += t_rec;
    }
  *count = c->prof_n;
  return STOKES_GPU_OK;
}

int
stokes_gpu_kprof_begin (struct stokes *sys, int max_marks)
{
  if (!sys || max_marks <= 0) return set_error (STOKES_GPU_EINVAL, "bad profile window");
  Ctx *c = get_ctx (sys, true);
  if (!c) return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  while (c->kprof_ev.size () < (size_t) max_marks)
    {
      cudaEvent_t e;
      if (cudaEventCreate (&e) != cudaSuccess)
        return set_error (STOKES_GPU_ECUDA, "cannot create events");
      c->kprof_ev.push_back (e);
    }
  c->kprof_name.assign (c->kprof_ev.size (), nullptr);
  c->kprof_n = 0;
  c->kprof_on = true;
  return STOKES_GPU_OK;
}

int
stokes_gpu_kprof_end (struct stokes *sys, int max_kernels, char *names, double *sum_ms,
                      int *count, int *nkernels)
{
  if (!sys || !names || !sum_ms || !count || !nkernels || max_kernels <= 0)
    return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c || !c->kprof_on) return set_error (STOKES_GPU_EINVAL, "no kernel profile window open");
  c->kprof_on = false;
  int nk = 0;
  for (int k = 0; k < max_kernels; k++) { sum_ms[k] = 0.0; count[k] = 0; }
  if (c->kprof_n > 0)
    {
      cudaError_t e = cudaEventSynchronize (c->kprof_ev[c->kprof_n - 1]);
      if (e != cudaSuccess) return cuda_fail (e, "kernel profile events");
    }
  for (size_t m = 1; m < c->kprof_n; m++)
    {
      const char *nm = c->kprof_name[m];
      if (!nm) continue;
      int k = 0;
      while (k < nk && strncmp (names + 32 * k, nm, 31) != 0) k++;
      if (k == nk)
        {
          if (nk == max_kernels) continue;
          strncpy (names + 32 * k, nm, 31);
          names[32 * k + 31] = 0;
          nk++;
        }
      float ms = 0.f;
      cudaEventElapsedTime (&ms, c->kprof_ev[m - 1], c->kprof_ev[m]);
      sum_ms[k] += ms;
      count[k] += 1;
    }
  *nkernels = nk;
  return STOKES_GPU_OK;
}

int
stokes_gpu_last_launches (const struct stokes *sys, int *count)
{
  if (!sys || !count) return set_error (STOKES_GPU_EINVAL, "NULL argument");
  Ctx *c = get_ctx (sys, false);
  if (!c) return set_error (STOKES_GPU_EINVAL, "no product run for this system yet");
  *count = c->launches;
  return STOKES_GPU_OK;
}

// ---- drop-in replacements of src/ewald.c ----------------------------------

// the Ewald-named entry points evaluate lattice sums: periodic systems only
static int
need_periodic (const struct stokes *sys, const char *fn)
{
  if (sys && sys->periodic == 0)
    return set_error (STOKES_GPU_ENOTPERIODIC,
                      "%s: the system is not periodic (the free-space operator is "
                      "atimes_nonewald_3all)", fn);
  return STOKES_GPU_OK;
}

static int
check_n (const struct stokes *sys, int n)
{
  clear_error ();
  if (sys == nullptr) return set_error (STOKES_GPU_EINVAL, "user_data is NULL");
  if (sys->version < 0 || sys->version > 2)
    return set_error (STOKES_GPU_EINVAL, "invalid version %d", sys->version);
  if (n != NCOMP (sys->version) * sys->np)
    return set_error (STOKES_GPU_EINVAL, "n = %d but np * %d = %d", n, NCOMP (sys->version),
                      NCOMP (sys->version) * sys->np);
  return STOKES_GPU_OK;
}

void
atimes_ewald_3all (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || need_periodic (sys, "atimes_ewald_3all") || atimes_host (sys, x, y, false))
    dropin_failed ("atimes_ewald_3all", y, n > 0 ? (size_t) n : 0);
}

void
atimes_ewald_3all_notbl (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || need_periodic (sys, "atimes_ewald_3all_notbl")
      || atimes_host (sys, x, y, true))
    dropin_failed ("atimes_ewald_3all_notbl", y, n > 0 ? (size_t) n : 0);
}

void
atimes_3all (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || atimes_host (sys, x, y, false))
    dropin_failed ("atimes_3all", y, n > 0 ? (size_t) n : 0);
}

void
make_matrix_mob_ewald_3all (struct stokes *sys, double *mat)
{
  if (need_periodic (sys, "make_matrix_mob_ewald_3all") || matrix_host (sys, mat, false))
    {
      size_t n = sys && sys->version >= 0 && sys->version <= 2
        ? (size_t) NCOMP (sys->version) * (sys->np > 0 ? sys->np : 0) : 0;
      dropin_failed ("make_matrix_mob_ewald_3all", mat, n * n);
    }
}

void
make_matrix_mob_ewald_3all_notbl (struct stokes *sys, double *mat)
{
  if (need_periodic (sys, "make_matrix_mob_ewald_3all_notbl") || matrix_host (sys, mat, true))
    {
      size_t n = sys && sys->version >= 0 && sys->version <= 2
        ? (size_t) NCOMP (sys->version) * (sys->np > 0 ? sys->np : 0) : 0;
      dropin_failed ("make_matrix_mob_ewald_3all_notbl", mat, n * n);
    }
}

void
make_matrix_mob_3all (struct stokes *sys, double *mat)
{
  if (matrix_host (sys, mat, false))
    {
      size_t n = sys && sys->version >= 0 && sys->version <= 2
        ? (size_t) NCOMP (sys->version) * (sys->np > 0 ? sys->np : 0) : 0;
      dropin_failed ("make_matrix_mob_3all", mat, n * n);
    }
}

void
atimes_3all_matrix (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || atimes_matrix_host (sys, x, y, false))
    dropin_failed ("atimes_3all_matrix", y, n > 0 ? (size_t) n : 0);
}

void
atimes_ewald_3all_matrix_notbl (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || need_periodic (sys, "atimes_ewald_3all_matrix_notbl")
      || atimes_matrix_host (sys, x, y, true))
    dropin_failed ("atimes_ewald_3all_matrix_notbl", y, n > 0 ? (size_t) n : 0);
}

// the free-space (non-periodic) operator, whatever sys->periodic says
// (src/non-ewald.c:330-706): the forced-open context around the common path
static int
open_call (struct stokes *sys, const std::function<int ()> &f)
{
  Ctx *c = sys ? get_ctx (sys, true) : nullptr;
  if (!c) return set_error (sys ? STOKES_GPU_ECUDA : STOKES_GPU_EINVAL, "no context");
  c->force_open = true;
  const int rc = f ();
  c->force_open = false;
  return rc;
}

void
atimes_nonewald_3all (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || open_call (sys, [&] { return atimes_host (sys, x, y, false); }))
    dropin_failed ("atimes_nonewald_3all", y, n > 0 ? (size_t) n : 0);
}

void
make_matrix_mob_nonewald_3all (struct stokes *sys, double *mat)
{
  if (open_call (sys, [&] { return matrix_host (sys, mat, false); }))
    {
      size_t n = sys && sys->version >= 0 && sys->version <= 2
        ? (size_t) NCOMP (sys->version) * (sys->np > 0 ? sys->np : 0) : 0;
      dropin_failed ("make_matrix_mob_nonewald_3all", mat, n * n);
    }
}

void
atimes_nonewald_3all_matrix (int n, const double *x, double *y, void *user_data)
{
  struct stokes *sys = (struct stokes *) user_data;
  if (check_n (sys, n) || open_call (sys, [&] { return atimes_matrix_host (sys, x, y, false); }))
    dropin_failed ("atimes_nonewald_3all_matrix", y, n > 0 ? (size_t) n : 0);
}

}  // extern "C"

// ---- dense helpers (replace src/matrix.c:365-399 and :447-478) ------------
// The matrix, x and y are host arrays; the product runs on the device.
namespace lsg {
static int
dense_host (int version, int n1, int n2, int np, const double *mat, const double *x, double *y)
{
  static thread_local DevBuf dm, dx, dy, dz;
  static thread_local cudaStream_t st = nullptr;
  if (!st && cudaStreamCreateWithFlags (&st, cudaStreamNonBlocking) != cudaSuccess)
    return set_error (STOKES_GPU_ECUDA, "cannot create a CUDA stream");
  cudaError_t e;
  if ((e = dm.ensure (sizeof (double) * (size_t) n1 * n2)) != cudaSuccess) return cuda_fail (e, "mat");
  if ((e = dx.ensure (sizeof (double) * (size_t) n2)) != cudaSuccess) return cuda_fail (e, "x");
  if ((e = dy.ensure (sizeof (double) * (size_t) n1)) != cudaSuccess) return cuda_fail (e, "y");
  if ((e = dz.ensure (sizeof (double) * (size_t) n2)) != cudaSuccess) return cuda_fail (e, "z");
  cudaMemcpyAsync (dm.p, mat, sizeof (double) * (size_t) n1 * n2, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync (dx.p, x, sizeof (double) * (size_t) n2, cudaMemcpyHostToDevice, st);
  if (version == 2)
    e = launch_gemv_fp64 (2, (const double *) dm.p, (const double *) dx.p, (double *) dz.p, np,
                          (double *) dy.p, st);
  else
    e = launch_gemv_rect_fp64 ((const double *) dm.p, n1, n2, (const double *) dx.p,
                               (double *) dy.p, st);
  if (e != cudaSuccess) return cuda_fail (e, "gemv");
  e = cudaMemcpyAsync (y, dy.p, sizeof (double) * (size_t) n1, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize (st);
  if (e != cudaSuccess) return cuda_fail (e, "gemv");
  return STOKES_GPU_OK;
}
}  // namespace lsg

extern "C" {

void
dot_prod_matrix (const double *mat, int n1, int n2, const double *x, double *y)
{
  if (n1 <= 0 || n2 <= 0) return;
  if (!mat || !x || !y)
    {
      set_error (STOKES_GPU_EINVAL, "NULL argument");
      dropin_failed ("dot_prod_matrix", y, y ? (size_t) n1 : 0);
      return;
    }
  if (dense_host (0, n1, n2, 0, mat, x, y)) dropin_failed ("dot_prod_matrix", y, (size_t) n1);
}

void
multiply_extmat_with_extvec_3fts (int np, const double *m, const double *x, double *y)
{
  if (np <= 0) return;
  const int n = 11 * np;
  if (!m || !x || !y)
    {
      set_error (STOKES_GPU_EINVAL, "NULL argument");
      dropin_failed ("multiply_extmat_with_extvec_3fts", y, y ? (size_t) n : 0);
      return;
    }
  if (dense_host (2, n, n, np, m, x, y))
    dropin_failed ("multiply_extmat_with_extvec_3fts", y, (size_t) n);
}

}  // extern "C"
