/* stokes_traj.h -- trajectories and checkpoints of libstokes_gb300 runs.
 *
 * libstokes writes its trajectories and the state of its random-number
 * generator to NetCDF files (src/stokes-nc.c: stokes_nc_init :1445,
 * stokes_nc_set_time :2118, stokes_nc_set_x :2235, stokes_nc_set_q :2263,
 * stokes_nc_set_rng :2646; src/stokes-nc-read.c: stokes_nc_open :742,
 * stokes_nc_get_rng :1420).  NetCDF is not part of this library; this is a
 * plain binary file with the same content, fixed-size frames for random
 * access, and the complete MT19937 state, so that a Brownian-dynamics run
 * can be stopped and resumed bit for bit.  (The NetCDF checkpoint copies
 * sizeof (int) x 624 bytes of the unsigned long state array,
 * src/stokes-nc.c:2668 and src/stokes-nc-read.c:1452, which on LP64
 * systems is the first half of the state only.)
 *
 * File layout (native byte order, marked by a byte-order word):
 *   header  128 bytes: "LSGTRJ01", 0x01020304, np, nf, version, fields,
 *           flags (1: radii follow), lx, ly, lz, shear_mode, shear_rate,
 *           zero padding
 *   radii   a[np], af[nf] when flags & 1
 *   frames  time, shear_shift, then for each field bit set, in bit order:
 *           X 3np, U 3np, O 3np, E 5np, F 3np, T 3np, S 5np, Q 4np,
 *           XF 3nf (doubles); RNG: 624 uint32 words, mti, has_saved (int32),
 *           saved (double)
 */
#ifndef STOKES_TRAJ_H
#define STOKES_TRAJ_H

#include "stokes_abi.h"
#include "stokes_bd.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  STOKES_TRAJ_X = 1, STOKES_TRAJ_U = 2, STOKES_TRAJ_O = 4, STOKES_TRAJ_E = 8,
  STOKES_TRAJ_F = 16, STOKES_TRAJ_T = 32, STOKES_TRAJ_S = 64, STOKES_TRAJ_Q = 128,
  STOKES_TRAJ_XF = 256, STOKES_TRAJ_RNG = 512
};

/* one frame: the arrays of the fields the file holds (others ignored).
 * stokes_traj_append reads them; stokes_traj_read fills them. */
struct stokes_traj_frame {
  double time;
  double shear_shift;
  double *x, *u, *o, *e, *f, *t, *s, *q, *xf;
  struct KIrand *rng;
};

struct stokes_traj;

/* a new file (an existing one is replaced): np mobile and nf fixed
 * particles, the fields to store per frame, the box, shear and radii of
 * sys (sys may be NULL: no box, equal spheres).  NULL on failure. */
struct stokes_traj *stokes_traj_create (const char *path, int np, int nf, int fields,
                                        const struct stokes *sys);
/* an existing file, for reading and for appending frames after the last
 * complete one.  NULL when the file is missing or not a trajectory. */
struct stokes_traj *stokes_traj_open (const char *path);
void stokes_traj_close (struct stokes_traj *t);

/* 0 on success */
int stokes_traj_append (struct stokes_traj *t, const struct stokes_traj_frame *fr);
int stokes_traj_read (struct stokes_traj *t, int k, struct stokes_traj_frame *fr);
int stokes_traj_nframes (const struct stokes_traj *t);
/* np, nf, version, fields, box[3], radii a[np] / af[nf] (NULL to skip;
 * filled with 1 for equal spheres) */
int stokes_traj_info (const struct stokes_traj *t, int *np, int *nf, int *version, int *fields,
                      double *box, double *a, double *af);

#ifdef __cplusplus
}
#endif

#endif /* STOKES_TRAJ_H */
