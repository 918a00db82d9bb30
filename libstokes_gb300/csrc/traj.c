/* traj.c -- trajectory and checkpoint files (include/stokes_traj.h).
 *
 * Host C.  The content follows libstokes' NetCDF output (src/stokes-nc.c):
 * the box and shear parameters, the radii, and per frame the time, the
 * shear shift, the particle arrays and the generator state.  Frames have a
 * fixed size, so frame k sits at header + radii + k * frame bytes.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "stokes_traj.h"

#define TRAJ_MAGIC "LSGTRJ01"
#define TRAJ_BOM 0x01020304u
#define TRAJ_HEADER 128

struct stokes_traj {
  FILE *fp;
  int np, nf, version, fields, flags;
  double box[3];
  int shear_mode;
  double shear_rate;
  long long data0;   /* offset of the first frame */
  long long fbytes;  /* bytes per frame */
  int nframes;
  double *a, *af;    /* radii, or NULL */
};

/* doubles per particle of each field, in bit order (X U O E F T S Q XF) */
static const int k_width[9] = {3, 3, 3, 5, 3, 3, 5, 4, 3};
#define RNG_BYTES (624 * 4 + 4 + 4 + 8)

static long long
frame_bytes (int np, int nf, int fields)
{
  long long b = 16;
  for (int q = 0; q < 9; q++)
    if (fields & (1 << q)) b += 8LL * k_width[q] * (q == 8 ? nf : np);
  if (fields & STOKES_TRAJ_RNG) b += RNG_BYTES;
  return b;
}

static int
write_all (FILE *fp, const void *p, size_t n)
{
  return fwrite (p, 1, n, fp) == n ? 0 : -1;
}

static int
read_all (FILE *fp, void *p, size_t n)
{
  return fread (p, 1, n, fp) == n ? 0 : -1;
}

struct stokes_traj *
stokes_traj_create (const char *path, int np, int nf, int fields, const struct stokes *sys)
{
  if (!path || np < 0 || nf < 0) return NULL;
  FILE *fp = fopen (path, "w+b");
  if (!fp) return NULL;
  struct stokes_traj *t = (struct stokes_traj *) calloc (1, sizeof *t);
  if (!t)
    {
      fclose (fp);
      return NULL;
    }
  t->fp = fp;
  t->np = np;
  t->nf = nf;
  t->fields = fields & 1023;
  t->version = sys ? sys->version : -1;
  /* radii when sys has them for every particle of the file */
  t->flags = (sys && sys->a && np + nf <= sys->np) ? 1 : 0;
  if (sys)
    {
      t->box[0] = sys->lx;
      t->box[1] = sys->ly;
      t->box[2] = sys->lz;
      t->shear_mode = sys->shear_mode;
      t->shear_rate = sys->shear_rate;
    }
  unsigned char h[TRAJ_HEADER];
  memset (h, 0, sizeof h);
  uint32_t bom = TRAJ_BOM;
  int32_t iv[5] = {np, nf, t->version, t->fields, t->flags};
  int32_t sm = t->shear_mode;
  memcpy (h, TRAJ_MAGIC, 8);
  memcpy (h + 8, &bom, 4);
  memcpy (h + 12, iv, sizeof iv);
  memcpy (h + 32, t->box, sizeof t->box);
  memcpy (h + 56, &sm, 4);
  memcpy (h + 64, &t->shear_rate, 8);
  int rc = write_all (fp, h, sizeof h);
  if (!rc && t->flags)
    {
      /* the radii of the mobile particles, then of the fixed ones
       * (sys->a holds np + nf entries in libstokes' convention) */
      rc = write_all (fp, sys->a, sizeof (double) * (size_t) np);
      if (!rc && nf > 0) rc = write_all (fp, sys->a + np, sizeof (double) * (size_t) nf);
    }
  if (rc || fflush (fp))
    {
      fclose (fp);
      free (t);
      return NULL;
    }
  t->data0 = TRAJ_HEADER + (t->flags ? 8LL * (np + nf) : 0);
  t->fbytes = frame_bytes (np, nf, t->fields);
  return t;
}

struct stokes_traj *
stokes_traj_open (const char *path)
{
  if (!path) return NULL;
  FILE *fp = fopen (path, "r+b");
  if (!fp) return NULL;
  unsigned char h[TRAJ_HEADER];
  uint32_t bom = 0;
  if (read_all (fp, h, sizeof h) || memcmp (h, TRAJ_MAGIC, 8) != 0
      || (memcpy (&bom, h + 8, 4), bom != TRAJ_BOM))
    {
      fclose (fp);
      return NULL;
    }
  struct stokes_traj *t = (struct stokes_traj *) calloc (1, sizeof *t);
  if (!t)
    {
      fclose (fp);
      return NULL;
    }
  int32_t iv[5], sm;
  memcpy (iv, h + 12, sizeof iv);
  memcpy (t->box, h + 32, sizeof t->box);
  memcpy (&sm, h + 56, 4);
  memcpy (&t->shear_rate, h + 64, 8);
  t->fp = fp;
  t->np = iv[0];
  t->nf = iv[1];
  t->version = iv[2];
  t->fields = iv[3] & 1023;
  t->flags = iv[4];
  t->shear_mode = sm;
  if (t->np < 0 || t->nf < 0)
    {
      stokes_traj_close (t);
      return NULL;
    }
  if (t->flags & 1)
    {
      t->a = (double *) malloc (sizeof (double) * (size_t) (t->np > 0 ? t->np : 1));
      t->af = (double *) malloc (sizeof (double) * (size_t) (t->nf > 0 ? t->nf : 1));
      if (!t->a || !t->af || read_all (fp, t->a, sizeof (double) * (size_t) t->np)
          || read_all (fp, t->af, sizeof (double) * (size_t) t->nf))
        {
          stokes_traj_close (t);
          return NULL;
        }
    }
  t->data0 = TRAJ_HEADER + ((t->flags & 1) ? 8LL * (t->np + t->nf) : 0);
  t->fbytes = frame_bytes (t->np, t->nf, t->fields);
  /* complete frames only: a frame cut short by a crash is overwritten by
   * the next append */
  if (fseek (fp, 0, SEEK_END) == 0)
    {
      const long long end = ftell (fp);
      t->nframes = end > t->data0 ? (int) ((end - t->data0) / t->fbytes) : 0;
    }
  return t;
}

void
stokes_traj_close (struct stokes_traj *t)
{
  if (!t) return;
  if (t->fp) fclose (t->fp);
  free (t->a);
  free (t->af);
  free (t);
}

int
stokes_traj_nframes (const struct stokes_traj *t)
{
  return t ? t->nframes : -1;
}

int
stokes_traj_info (const struct stokes_traj *t, int *np, int *nf, int *version, int *fields,
                  double *box, double *a, double *af)
{
  if (!t) return -1;
  if (np) *np = t->np;
  if (nf) *nf = t->nf;
  if (version) *version = t->version;
  if (fields) *fields = t->fields;
  if (box) memcpy (box, t->box, sizeof t->box);
  for (int i = 0; a && i < t->np; i++) a[i] = t->a ? t->a[i] : 1.0;
  for (int i = 0; af && i < t->nf; i++) af[i] = t->af ? t->af[i] : 1.0;
  return 0;
}

static double *
field_ptr (const struct stokes_traj_frame *fr, int q)
{
  switch (q)
    {
    case 0: return fr->x;
    case 1: return fr->u;
    case 2: return fr->o;
    case 3: return fr->e;
    case 4: return fr->f;
    case 5: return fr->t;
    case 6: return fr->s;
    case 7: return fr->q;
    default: return fr->xf;
    }
}

int
stokes_traj_append (struct stokes_traj *t, const struct stokes_traj_frame *fr)
{
  if (!t || !fr) return -1;
  if (fseek (t->fp, (long) (t->data0 + (long long) t->nframes * t->fbytes), SEEK_SET)) return -1;
  double head[2] = {fr->time, fr->shear_shift};
  if (write_all (t->fp, head, sizeof head)) return -1;
  for (int q = 0; q < 9; q++)
    {
      if (!(t->fields & (1 << q))) continue;
      const double *p = field_ptr (fr, q);
      const size_t n = (size_t) k_width[q] * (q == 8 ? t->nf : t->np);
      if (!p) return -1;
      if (write_all (t->fp, p, sizeof (double) * n)) return -1;
    }
  if (t->fields & STOKES_TRAJ_RNG)
    {
      if (!fr->rng) return -1;
      uint32_t mt[624];
      for (int i = 0; i < 624; i++) mt[i] = (uint32_t) (fr->rng->mt[i] & 0xffffffffUL);
      int32_t iv[2] = {fr->rng->mti, fr->rng->Gaussian_has_saved};
      if (write_all (t->fp, mt, sizeof mt) || write_all (t->fp, iv, sizeof iv)
          || write_all (t->fp, &fr->rng->Gaussian_saved, sizeof (double)))
        return -1;
    }
  if (fflush (t->fp)) return -1;
  t->nframes++;
  return 0;
}

int
stokes_traj_read (struct stokes_traj *t, int k, struct stokes_traj_frame *fr)
{
  if (!t || !fr || k < 0 || k >= t->nframes) return -1;
  if (fseek (t->fp, (long) (t->data0 + (long long) k * t->fbytes), SEEK_SET)) return -1;
  double head[2];
  if (read_all (t->fp, head, sizeof head)) return -1;
  fr->time = head[0];
  fr->shear_shift = head[1];
  for (int q = 0; q < 9; q++)
    {
      if (!(t->fields & (1 << q))) continue;
      double *p = field_ptr (fr, q);
      const size_t n = (size_t) k_width[q] * (q == 8 ? t->nf : t->np);
      if (p)
        {
          if (read_all (t->fp, p, sizeof (double) * n)) return -1;
        }
      else if (fseek (t->fp, (long) (sizeof (double) * n), SEEK_CUR))
        return -1;
    }
  if ((t->fields & STOKES_TRAJ_RNG) && fr->rng)
    {
      uint32_t mt[624];
      int32_t iv[2];
      if (read_all (t->fp, mt, sizeof mt) || read_all (t->fp, iv, sizeof iv)
          || read_all (t->fp, &fr->rng->Gaussian_saved, sizeof (double)))
        return -1;
      for (int i = 0; i < 624; i++) fr->rng->mt[i] = mt[i];
      fr->rng->mti = iv[0];
      fr->rng->Gaussian_has_saved = iv[1];
    }
  return 0;
}
