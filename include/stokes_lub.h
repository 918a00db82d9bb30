/* stokes_lub.h -- the lubrication correction of libstokes (src/lub.h),
 * computed on the GPU for equal spheres without slip.
 *
 * f = L u: the sum over close pairs (0 < r < sys->lubmax, or every pair of
 * the image cube when lubmax is 0; r clamped from below at
 * sqrt(sys->lubmin2)) of the two-sphere resistance minus its far-field
 * part, with the lattice images of a periodic system in the cube
 * |n_x,y,z| <= lubmax / L + 1 (src/lub.c:129-157).  Errors (unequal radii,
 * slip) are reported as the other drop-in entry points report them
 * (stokes_gpu_last_error; exit unless the error mode is 1). */
#ifndef STOKES_LUB_H
#define STOKES_LUB_H

#include "stokes_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/lub.h: calc_lub_3f (u, f [np*3]), calc_lub_3ft (uo, ft [np*6]),
 * calc_lub_3fts (uoe, fts [np*11], the extracted 5-component stresslet and
 * strain as in libstokes) */
void calc_lub_3f (struct stokes *sys, const double *u, double *f);
void calc_lub_3ft (struct stokes *sys, const double *uo, double *ft);
void calc_lub_3fts (struct stokes *sys, const double *uoe, double *fts);

/* status-returning forms: version 0 (F), 1 (FT) or 2 (FTS); host vectors,
 * or device vectors on the caller's stream (d_pos [np*3]) */
int stokes_gpu_lub (struct stokes *sys, int version, const double *u, double *f);
int stokes_gpu_lub_dev (struct stokes *sys, int version, const double *d_pos,
                        const double *d_u, double *d_f, void *stream);
/* src/lub-matrix.c:76-507: the dense L, mat [n*n] row-major with
 * n = np*{3, 6, 11}, fully overwritten; f = mat u equals calc_lub_3f / 3ft
 * (u, f), and for FTS mat acts in libstokes' extracted form (as
 * multiply_extmat_with_extvec_3fts, src/matrix.c:447-478, applies it).
 * make_matrix_lub_3f / 3ft / 3fts are the drop-ins; the status-returning
 * forms take the version, host memory or a device buffer on the caller's
 * stream (d_pos [np*3], d_mat [n*n]). */
void make_matrix_lub_3f (struct stokes *sys, double *mat);
void make_matrix_lub_3ft (struct stokes *sys, double *mat);
void make_matrix_lub_3fts (struct stokes *sys, double *mat);
int stokes_gpu_lub_matrix (struct stokes *sys, int version, double *mat);
int stokes_gpu_lub_matrix_dev (struct stokes *sys, int version, const double *d_pos,
                               double *d_mat, void *stream);
/* the power-series coefficients of the 22 lubrication-form functions
 * (x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c x11g x12g y11g y12g
 * y11h y12h x11m x12m y11m y12m z11m z12m; 26 each, out[572]), generated on
 * the host from the Jeffrey-Onishi recurrences */
int stokes_gpu_lub_coefficients (double *out);

#ifdef __cplusplus
}
#endif

#endif /* STOKES_LUB_H */
