/* stokes_abi.h -- the reference-facing C ABI of libstokes_gb300.
 *
 * libstokes_gb300 is a drop-in replacement for the Ewald-summed mobility path
 * of libstokes 0.4.1 (kichiki/libstokes).  Every function declared here keeps
 * the name, signature and meaning of the libstokes function it replaces, so a
 * program (or the rest of libstokes: solve_mob_3f, BD_evolve_mid, ...) that is
 * linked against libstokes_gb300.so ahead of libstokes runs its periodic
 * mobility products on the GPU without edits.
 *
 * struct stokes below is byte-identical to libstokes' struct stokes
 * (src/stokes.h:27-154): same members, same order, same types.  The layout is
 * an interface, not an implementation choice; tests/test_abi_layout.py checks
 * every member offset against the reference header.
 */
#ifndef LIBSTOKES_GB300_STOKES_ABI_H
#define LIBSTOKES_GB300_STOKES_ABI_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* opaque to this library: only the lubrication code of libstokes reads them */
struct twobody_f_list;
struct twobody_slip_f_list;
struct iter;

/* System description shared by every mobility routine.
 * Mirrors src/stokes.h:27-154 member for member. */
struct stokes {
  int version;          /* 0 = F, 1 = FT, 2 = FTS */

  int np;               /* all particles */
  int nm;               /* mobile particles (the first nm of np) */
  double *pos;          /* pos[np*3] */

  double *a;            /* radii[np]; NULL = monodisperse, a = 1 */
  double rmin;          /* r is clamped to rmin*(ai+aj) before the pair terms */
  int twobody_nmax;     /* lubrication table order (not used on the GPU) */
  int twobody_lub;      /* lubrication form flag (not used on the GPU) */
  int *poly_table;      /* lubrication table index (not used on the GPU) */
  struct twobody_f_list *twobody_f_list;

  double *slip;         /* slip length[np]; NULL = no-slip */
  double *slip_a;       /* effective radius of the Laplacian terms */
  double *slip_G32;     /* Lambda(3,2), a-self factor */
  double *slip_G30;     /* Lambda(3,0), c-self factor */
  double *slip_G52;     /* Lambda(5,2), m-self factor */
  int *slip_table;
  struct twobody_slip_f_list *twobody_slip_f_list;

  double Ui[3];         /* imposed flow */
  double Oi[3];
  double Ei[5];

  int shear_mode;       /* 0: none, 1: flow x / gradient y, 2: flow x / gradient z */
  double shear_rate;
  double shear_shift;   /* Lees-Edwards cell shift */

  int periodic;         /* 0 = open system, 1 = periodic box */

  double ewald_eps;
  double rmax2;         /* real-space cutoff squared */
  int rmaxx, rmaxy, rmaxz;
  double kmax;          /* reciprocal cutoff; 0 = take the whole k cube */
  int kmaxx, kmaxy, kmaxz;

  double xi, xi2, xiaspi, xia2;
  double pivol;         /* pi / volume */

  double lx, ly, lz;
  int ilx[27], ily[27], ilz[27];

  double self_a;        /* Ewald self terms of the monodisperse system */
  double self_c;
  double self_m;

  int flag_table;       /* 1 when the lattice tables below are valid */
  int nr;               /* real-space image table */
  double *rlx;
  double *rly;
  double *rlz;
  int *rmx;
  int *rmy;
  int *rmz;
  int nk;               /* reciprocal table (filled, not read by the product) */
  double *ex;
  double *ey;
  double *ez;
  double *k;
  double *k1;
  double *k2;
  double *k3;
  double *ya;
  double *yb;
  double *yc;
  double *yg;
  double *yh;
  double *ym;

  double lubmin2;
  double lubmax;

  double cpu1, cpu2, cpu3;  /* ms spent: total, real space, reciprocal space */

  struct iter *it;
};

/* ---- system set-up (replaces src/stokes.c) ----------------------------- */

/* src/stokes.c:317-418 -- allocate and zero a struct stokes */
struct stokes *stokes_init (void);
/* src/stokes.c:422-445 */
void stokes_free (struct stokes *sys);
/* src/stokes.c:451-466 -- set np, nm and allocate pos[np*3] */
void stokes_set_np (struct stokes *sys, int np, int nm);
/* src/stokes.c:469-495 */
void stokes_set_Ui (struct stokes *sys, double uix, double uiy, double uiz);
void stokes_set_Oi (struct stokes *sys, double oix, double oiy, double oiz);
void stokes_set_Ei (struct stokes *sys, double eixx, double eixy, double eixz,
                    double eiyz, double eiyy);
/* src/stokes.c:506-543 */
void stokes_set_shear (struct stokes *sys, int shear_mode, double shear_rate);
/* src/stokes.c:554-589 */
double stokes_get_shear_shift (struct stokes *sys, double t, double t0,
                               double s0);
/* src/stokes.c:599-604 */
void stokes_set_shear_shift (struct stokes *sys, double t, double t0,
                             double s0);
/* src/stokes.c:607-651 -- box size, pi/V and the 27-cell integer table */
void stokes_set_l (struct stokes *sys, double lx, double ly, double lz);
/* src/stokes.c:703-762 -- Ewald split, self terms, cutoffs, lattice tables */
void stokes_set_xi (struct stokes *sys, double xi, double ewald_eps);
/* src/stokes.c:766-776 */
double xi_by_tratio (struct stokes *sys, double tratio);
/* src/stokes.c:822-830 */
void stokes_set_pos (struct stokes *sys, const double *pos);
/* src/stokes.c:840-848 */
void stokes_set_pos_mobile (struct stokes *sys, const double *pos);
/* src/stokes.c:858-868 */
void stokes_set_pos_fixed (struct stokes *sys, const double *pos);
/* src/stokes.c:902-960 -- radii.  The lubrication tables (poly_table,
 * twobody_f_list) are not built: the GPU path reads only a[]. */
void stokes_set_radius (struct stokes *sys, const double *a);
/* src/stokes.c:972-985 */
void stokes_unset_radius (struct stokes *sys);
/* src/stokes.c:1109-1180 -- slip arrays.  The slip lubrication table is not
 * built: the GPU path reads only slip, slip_a and slip_G**. */
void stokes_set_slip (struct stokes *sys, const double *gamma);
/* src/stokes.c:1193-1217 */
void stokes_unset_slip (struct stokes *sys);

/* ---- mobility operators (replace src/ewald.c) --------------------------- */

/* src/ewald.c:519-1081 (declared src/ewald.h:155-156).
 * y = M x for the Ewald-summed F/FT/FTS mobility, n = np*{3,6,11}.
 * x holds F | FT | FTS (stresslet as xx,xy,xz,yz,yy) per particle, y the
 * matching U | UO | UOE.  y is fully overwritten.  sys->cpu1/2/3 are set to
 * the GPU time (ms) of the whole product / real part / the rest
 * (cpu1 = cpu2 + cpu3, as in the reference).  In mixed precision the real
 * part runs on a second stream beside the reciprocal part: cpu2 is its span
 * there (as measured on the configuration's last launch outside its CUDA
 * graph) and cpu3 the rest of the product's span.
 * On a device or input error the library prints the reason, records it for
 * stokes_gpu_last_error() and exits the process with status 1 -- the
 * reference's own behaviour on allocation failure (src/memory-check.h:22-25). */
void atimes_ewald_3all (int n, const double *x, double *y, void *user_data);

/* src/ewald.c:1092-1677 (src/ewald.h:167-168).
 * mat[n*n], row-major, fully overwritten; FTS in the extracted form. */
void make_matrix_mob_ewald_3all (struct stokes *sys, double *mat);

/* src/ewald.c:432-447: the Ewald operator for periodic systems, the
 * free-space one (atimes_nonewald_3all) otherwise. */
void atimes_3all (int n, const double *x, double *y, void *user_data);
/* src/ewald.c:459-472 */
void make_matrix_mob_3all (struct stokes *sys, double *mat);
/* src/ewald.c:484-505 -- build the dense matrix, then y = mat . x
 * (FTS through the extracted-form product). */
void atimes_3all_matrix (int n, const double *x, double *y, void *user_data);

/* src/ewald.c:1691, 2149, 2628 -- the "_notbl" variants enumerate the image
 * cube rmaxx/rmaxy/rmaxz instead of the table.  They give the same sums as
 * the table versions and are served by the same kernels. */
void atimes_ewald_3all_notbl (int n, const double *x, double *y,
                              void *user_data);

/* Free-space (non-periodic) Rotne-Prager-Yamakawa operator, FP64 on the
 * device: the self term plus every pair j != i with the scalars of
 * src/non-ewald.c:49-210 (mono, poly, slip; rmin clamp).  atimes_3all,
 * make_matrix_mob_3all and atimes_3all_matrix dispatch here when
 * sys->periodic is 0; the Ewald-named entry points reject such systems.
 * src/non-ewald.c:330-475 */
void atimes_nonewald_3all (int n, const double *x, double *y, void *user_data);
/* src/non-ewald.c:494-666 -- dense, row-major, FTS in the extracted form */
void make_matrix_mob_nonewald_3all (struct stokes *sys, double *mat);
/* src/non-ewald.c:677-706 -- dense matrix, then y = mat . x */
void atimes_nonewald_3all_matrix (int n, const double *x, double *y, void *user_data);
void make_matrix_mob_ewald_3all_notbl (struct stokes *sys, double *mat);
void atimes_ewald_3all_matrix_notbl (int n, const double *x, double *y,
                                     void *user_data);

/* ---- dense helpers (replace src/matrix.c:365-478) ----------------------- */

/* src/matrix.c:365-399: y[n1] = mat[n1,n2] . x[n2] */
void dot_prod_matrix (const double *mat, int n1, int n2, const double *x,
                      double *y);
/* src/matrix.c:447-478: FTS extracted-form product y = m . x */
void multiply_extmat_with_extvec_3fts (int np, const double *m,
                                       const double *x, double *y);

/* ---- Chebyshev routines (replace src/chebyshev.c) ------------------------ */

/* src/chebyshev.c:33-61 */
void chebyshev_coef (int ncheb, double (*func) (double), double x0, double x1,
                     double *a);
/* src/chebyshev.c:74-105 (Clenshaw) */
double chebyshev_eval (int ncheb, const double *a, double x0, double x1,
                       double x);
/* src/chebyshev.c:117-148 (explicit recurrence) */
double chebyshev_eval_ (int ncheb, const double *a, double x0, double x1,
                        double x);
/* src/chebyshev.c:163-228.  z = sum_k a_k T_k(M) y by Clenshaw.  When atimes
 * is this library's Ewald operator (atimes_ewald_3all or atimes_3all) on a
 * periodic system, every product stays on the GPU and only z comes back. */
void chebyshev_eval_atimes (int ncheb, const double *a, int n, const double *y,
                            double *z, double eign0, double eign1,
                            void (*atimes) (int, const double *, double *,
                                            void *),
                            void *user_data);
/* src/chebyshev.c:241-269: |z.Mz - y.y| / z.Mz */
double chebyshev_error_minvsqrt (int n, const double *y, const double *z,
                                 void (*atimes) (int, const double *, double *,
                                                 void *),
                                 void *user_data);
/* src/chebyshev.c:282-310: |y.Ry - z.z| / y.Ry */
double chebyshev_error_Rsqrt (int n, const double *y, const double *z,
                              void (*atimes) (int, const double *, double *,
                                              void *),
                              void *user_data);

#ifdef __cplusplus
}
#endif

#endif /* LIBSTOKES_GB300_STOKES_ABI_H */
