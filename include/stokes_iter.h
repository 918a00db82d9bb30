/* stokes_iter.h -- the iterative solves of libstokes' mobility and
 * resistance problems, on the device.
 *
 * libstokes hands its linear systems to an external iterative-solver
 * library ("libiter", not part of the libstokes sources) through three
 * calls: iter_init (from stokes_set_iter, src/stokes.c:790-812), solve_iter
 * (src/ewald-3f.c:94, :308; src/ewald-3ft.c:113, :368; src/ewald-3fts.c:71,
 * :286-297, :567-578) and iter_free (src/stokes.c:440).  This library
 * exports the same three calls.  solve_iter runs restarted GMRES with its
 * Krylov vectors in device memory; when the operator is one of this
 * library's (atimes_3all, atimes_ewald_3all, atimes_nonewald_3all) every
 * product stays on the device too, otherwise the caller's atimes is called
 * on host copies of the vectors.
 *
 * struct iter is this library's own: libiter's layout is not part of
 * libstokes, and a program that links this library gets iter_init,
 * solve_iter and iter_free together, so only they touch the fields.
 */
#ifndef STOKES_ITER_H
#define STOKES_ITER_H

#include <stdio.h>

#include "stokes_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

struct iter {
  char *solver;    /* the name given to iter_init; every name runs GMRES(restart) */
  int max;         /* maximum number of operator applications */
  int restart;     /* Krylov dimension of one GMRES cycle */
  double eps;      /* stop when |b - A x| <= eps |b| */
  int n;           /* length of guess */
  double *guess;   /* start vector when flag_guess != 0 (zero at first) */
  int flag_guess;  /* 1: start from guess and keep each solution there */
  int debug;       /* 1: print the residual of every iteration to out */
  FILE *out;
  int niter;       /* operator applications of the last solve */
  double res;      /* relative residual |b - A x| / |b| of the last solve */
};

/* replaces libiter's iter_init as called by stokes_set_iter
 * (src/stokes.c:809-812); guess may be NULL */
struct iter *iter_init (const char *solver, int max, int restart, double eps, int n,
                        const double *guess, int flag_guess, int debug, FILE *out);
void iter_free (struct iter *it);

/* sys->it for the problem solvers (src/stokes.c:790-812): n from the
 * version and np, no initial guess, the solution kept as the next guess */
void stokes_set_iter (struct stokes *sys, const char *solver, int max, int restart, double eps,
                      int debug, FILE *out);

/* x = A^{-1} b; A given by atimes(n, in, out, user_data).  it == NULL takes
 * GMRES(20), at most 2000 applications, eps 1e-6, a zero start vector.
 * Failure (a CUDA error, a bad argument) ends the program with a message,
 * or, with stokes_gpu_set_error_mode (1), fills x with NaN and records the
 * reason for stokes_gpu_last_error (). */
void solve_iter (int n, const double *b, double *x,
                 void (*atimes) (int, const double *, double *, void *), void *user_data,
                 struct iter *it);

/* the natural FTS mobility problem in the fluid-rest frame
 * (src/ewald-3fts.c:263-314): given f, t [np*3] and e [np*5], the velocity
 * u, o [np*3] and stresslet s [np*5] from
 *   (u, o, 0) - M (0, 0, s) = M (f, t, 0) - (0, 0, e)
 * (src/ewald-3fts.c:146-247), with both the operator and the right-hand
 * side on the device.  iter == NULL takes sys->it. */
void solve_mob_3fts_0 (struct stokes *sys, struct iter *iter, const double *f,
                       const double *t, const double *e, double *u, double *o, double *s);

/* Status-returning form, no counterpart in libstokes.  op selects A:
 *   STOKES_GPU_SOLVE_RES     A = M (the resistance problems of
 *                            src/ewald-3f*.c: M x = b)
 *   STOKES_GPU_SOLVE_MOB_FTS A (u,o,s) = (u,o,0) - M (0,0,s) (FTS only)
 *   STOKES_GPU_SOLVE_MOB_LUB A = I + M L, L the lubrication correction of
 *                            calc_lub_3f / calc_lub_3ft (F and FT, equal
 *                            spheres; the operator of src/ewald-3f.c:411
 *                            and src/ewald-3ft.c, b = M f)
 * b, x [n] host buffers, n = np * {3, 6, 11}; x holds the start vector on
 * entry.  restart <= 0 and max <= 0 take 20 and 2000.  iters and res (may
 * be NULL) receive the operator applications and |b - A x| / |b|. */
enum { STOKES_GPU_SOLVE_RES = 0, STOKES_GPU_SOLVE_MOB_FTS = 1, STOKES_GPU_SOLVE_MOB_LUB = 2 };
int stokes_gpu_solve (struct stokes *sys, int op, const double *b, double *x, int restart,
                      int max, double eps, int *iters, double *res);

#ifdef __cplusplus
}
#endif

#endif /* STOKES_ITER_H */
