/* stokes_bd.h -- Brownian dynamics with Chebyshev noise: the libstokes
 * interface it keeps (struct KIrand, struct EV_LJ, struct BD_params and
 * the noise / mid-point routines) and the additive device-resident engine.
 *
 * The three structs are byte-identical to libstokes' (src/KIrand.h:51-58,
 * src/ev-LJ.h:26-51, src/brownian.h:28-96); tests/test_abi.py checks their
 * member offsets against the reference headers.
 */
#ifndef LIBSTOKES_GB300_STOKES_BD_H
#define LIBSTOKES_GB300_STOKES_BD_H

#include "stokes_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- random numbers (replaces src/KIrand.c) ----------------------------- */

#define KIRAND_MT_N 624
struct KIrand {
  unsigned long mt[KIRAND_MT_N]; /* MT19937 state */
  int mti;                       /* KIRAND_MT_N + 1: not seeded yet */
  int Gaussian_has_saved;        /* a second deviate is kept */
  double Gaussian_saved;
};

/* src/KIrand.c:57-67 */
struct KIrand *KIrand_init (void);
/* src/KIrand.c:70-74 */
void KIrand_free (struct KIrand *r);
/* src/KIrand.c:78-88 */
void KIrand_load_mt (struct KIrand *r, unsigned long *mt, int mti);
/* src/KIrand.c:92-103 */
void KIrand_load_Gaussian (struct KIrand *r, unsigned long *mt, int mti,
                           int flag_saved, double x_saved);
/* src/KIrand.c:137-156 */
void KIrand_init_genrand (struct KIrand *r, unsigned long s);
/* src/KIrand.c:200-244 */
unsigned long KIrand_genrand_int32 (struct KIrand *r);
/* src/KIrand.c:246-276 */
long KIrand_genrand_int31 (struct KIrand *r);
double KIrand_genrand_real1 (struct KIrand *r);
double KIrand_genrand_real2 (struct KIrand *r);
double KIrand_genrand_real3 (struct KIrand *r);
/* src/KIrand.c:277-284 */
double KIrand_genrand_res53 (struct KIrand *r);
/* src/KIrand.c:107-133: polar Box-Muller, second deviate saved */
double KIrand_Gaussian (struct KIrand *r);

/* ---- soft repulsion (src/ev-LJ.h:26-51) ---------------------------------- */

struct EV_LJ {
  int n;          /* particles */
  int *flag;      /* how e was made dimensionless (0: e/kT, 1: e/(kT Pe r0)) */
  double *e;      /* strength per particle */
  double *r0;     /* potential-minimum distance per particle */
};

/* src/ev-LJ.c:35-81: zero-initialised per-particle coefficients; the scale
 * turns e into e / (peclet r0) for entries with flag 0 and sets their flag */
struct EV_LJ *EV_LJ_init (int np);
void EV_LJ_free (struct EV_LJ *ev_LJ);
void EV_LJ_scale (struct EV_LJ *ev_LJ, double peclet);

/* ---- Brownian dynamics parameters (src/brownian.h:28-96) ------------------ */

struct BeadRod;
struct BONDS;
struct BONDS_GROUPS;
struct EV;
struct angles;
struct EV_DH;
struct confinement;

struct BD_params {
  struct stokes *sys;
  struct KIrand *rng;
  double *F;
  double *T;
  double *E;
  double *uf;
  double *of;
  double *ef;

  int flag_noHI;
  int flag_mat;
  int flag_lub;
  int flag_lub_B;

  double t0;        /* reference time of the shear shift s0 */
  double s0;

  double st;

  struct BeadRod *br;
  struct BONDS *bonds;
  struct BONDS_GROUPS *groups;
  double gamma;
  struct EV *ev;
  struct angles *ang;
  struct EV_DH *ev_dh;
  struct EV_LJ *ev_LJ;
  struct confinement *cf;

  int flag_Q;

  double peclet;
  double eps;       /* bound on the Chebyshev error before re-estimating */

  int n_minv;       /* Chebyshev coefficients of M^{-1/2} */
  double eig_minv[2];
  double *a_minv;
  int n_lub;
  double eig_lub[2];
  double *a_lub;

  int scheme;       /* 0: mid-point */
  double BB_n;

  double rmin;      /* overlap factor for dt adjustment (0: none) */
  double dt_lim;
};

/* ---- drop-in routines (replace src/brownian.c) ---------------------------- */

/* src/brownian.c:105-260: the RNG is seeded with `seed`, a_minv / a_lub are
 * zeroed and eig_minv = eig_lub = {0, 0} (bounds not set yet) */
struct BD_params *
BD_params_init (struct stokes *sys, unsigned long seed, double *F, double *T, double *E,
                double *uf, double *of, double *ef, int flag_noHI, int flag_lub, int flag_mat,
                double st, struct BeadRod *br, struct BONDS *bonds, double gamma, struct EV *ev,
                struct angles *ang, struct EV_DH *ev_dh, struct EV_LJ *ev_LJ,
                struct confinement *cf, int flag_Q, double peclet, double eps, int n_minv,
                int n_lub, int scheme, double BB_n, double rmin, double dt_lim);
/* src/brownian.c:262-277 (F, T, E, uf, of, ef stay the caller's); also
 * releases the device state the BD routines keep for this BD */
void BD_params_free (struct BD_params *BD);

/* src/brownian.c:2177-2187: sqrt(2 / (Pe dt)), 0 without Brownian force */
double BD_params_get_fact (struct BD_params *BD, double dt);
/* src/brownian.c:2033-2058: nm*3 (F) or nm*6 (FT, FTS) */
int BD_get_n (struct stokes *sys);
/* src/brownian.c:1545-1874, Chebyshev branch (n_minv > 0, HI on, no fixed
 * particles, equal or unequal spheres): z = M^{-1/2} y with y ~ N(0,1) from
 * BD->rng.  When eig_minv[0] == eig_minv[1] the bounds are estimated first
 * (20-step FP64 Lanczos on the device, in place of ARPACK) and a_minv is
 * fitted.  With BD->flag_lub_B (equal spheres without slip, n_lub > 0) the
 * lubrication noise L^{1/2} y_lub is added, y_lub drawn after y: Chebyshev
 * of sqrt on [eig_lub[0], eig_lub[1]] with the device lubrication operator,
 * bounds by Lanczos when eig_lub[0] == eig_lub[1] (lower bound at least 0),
 * re-estimated when |y.Ly - z.z| / y.Ly > BD->eps (src/brownian.c:1734-1849).
 * Unsupported branches (the matrix forms n_minv <= 0, n_lub <= 0) exit with
 * a message. */
void BD_calc_FB (struct BD_params *BD, double *z);
/* src/brownian.c:2352-2560 (scheme 0, F and FT, quaternions q when given,
 * constant force F/T, EV_LJ repulsion, imposed flow and shear, dt halving on
 * overlap when sys->rmin == 0 and BD->rmin > 0; with BD->flag_lub the
 * velocities solve (I + M L) u = M f on the device, GMRES settings from
 * sys->it; BD->flag_lub_B adds the lubrication noise as in BD_calc_FB): one
 * mid-point step with noise from BD_calc_FB; returns the dt
 * done.  The products run on the GPU
 * in the precision set for sys (stokes_gpu_set_precision). */
double BD_evolve_mid (double t, struct BD_params *BD, double *x, double *q, double dt);

/* ---- device-resident engine (no counterpart in libstokes) ----------------- */

struct stokes_gpu_bd_params {
  double peclet;            /* fact = sqrt(2 / (peclet dt)) */
  double dt;
  int n_cheb;               /* Chebyshev coefficients of M^{-1/2} */
  int n_lanczos;            /* Lanczos steps for the eigenvalue bounds */
  double cheb_eps;          /* re-estimate the bounds above this error */
  int check_every;          /* Chebyshev error check every n steps (0: never) */
  double lj_e;              /* EV_LJ strength (0: no repulsion) */
  double lj_r0;             /* EV_LJ distance */
  unsigned long long seed;  /* device noise (Philox) */
  int precision;            /* STOKES_GPU_FP64 or STOKES_GPU_MIXED */
};

typedef struct stokes_gpu_bd stokes_gpu_bd;

/* positions of sys (its pos[]) are the initial configuration */
int stokes_gpu_bd_create (struct stokes *sys, const struct stokes_gpu_bd_params *p,
                          stokes_gpu_bd **out);
int stokes_gpu_bd_destroy (stokes_gpu_bd *bd);
int stokes_gpu_bd_set_positions (stokes_gpu_bd *bd, const double *x);
int stokes_gpu_bd_get_positions (stokes_gpu_bd *bd, double *x);
/* constant external force / torque per particle (host, nm*3 each; NULL = 0) */
int stokes_gpu_bd_set_force (stokes_gpu_bd *bd, const double *F, const double *T);
/* eigenvalue bounds of M at the current positions by Lanczos (FP64), widened
 * by the safety factors; also refits the Chebyshev coefficients */
int stokes_gpu_bd_estimate_bounds (stokes_gpu_bd *bd, double *eig2);
int stokes_gpu_bd_set_bounds (stokes_gpu_bd *bd, const double *eig2);
/* z = M^{-1/2} y at the current positions (host vectors of BD_get_n) and the
 * Chebyshev error |z.Mz - y.y| / z.Mz */
int stokes_gpu_bd_noise (stokes_gpu_bd *bd, const double *y, double *z, double *err);
/* one mid-point step at time t with the given noise y (host, particle
 * order), as BD_evolve_mid does with rmin = 0 */
int stokes_gpu_bd_step_noise (stokes_gpu_bd *bd, double t, const double *y);
/* nsteps mid-point steps from time t, noise from the device generator */
int stokes_gpu_bd_run (stokes_gpu_bd *bd, double t, int nsteps);
/* products issued, bound estimates, last Chebyshev error, steps done */
int stokes_gpu_bd_stats (stokes_gpu_bd *bd, double *out4);

#ifdef __cplusplus
}
#endif

#endif /* LIBSTOKES_GB300_STOKES_BD_H */
