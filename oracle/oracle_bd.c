/* oracle_bd.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of libstokes' Brownian-dynamics mid-point step with
 * Chebyshev noise, for checking the device engine on identical inputs:
 *  - Clenshaw evaluation of z = sum_k a_k T_k(M~) y      (src/chebyshev.c:163-228)
 *  - EV_LJ soft repulsion over the 27 neighbour cells     (src/ev-LJ.c:105-265)
 *  - forces f = F + fact z + F_LJ                         (src/brownian.c:2273-2311)
 *  - mid-point scheme with rmin = 0 (no dt adjustment)    (src/brownian.c:2352-2560)
 * The mobility products are those of oracle_ewald.c (oracle_atimes).  F and
 * FT versions, no fixed particles, no imposed flow.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

void oracle_atimes (void *h, const double *x, double *y);
void oracle_set_pos (void *h, const double *pos);

static int ncomp_of (int version) { return version == 0 ? 3 : (version == 1 ? 6 : 11); }

/* z = M^{-1/2} y by Clenshaw; y, z in the product's layout (n = c np) */
void
oracle_cheb_eval (void *h, int n, int ncheb, const double *a, double e0, double e1,
                  const double *y, double *z)
{
  double *x = calloc ((size_t) n, sizeof (double));
  double *b = calloc ((size_t) 3 * n, sizeof (double));
  const double da = 2.0 / (e1 - e0), db = -(e1 + e0) / (e1 - e0);
  for (int i = 0; i < ncheb - 1; i++)
    {
      double *b2 = b + (size_t) ((i + 2) % 3) * n, *b1 = b + (size_t) ((i + 1) % 3) * n,
             *b0 = b + (size_t) (i % 3) * n;
      oracle_atimes (h, b1, x);
      const double aj = a[ncheb - 1 - i];
      for (int k = 0; k < n; k++) b2[k] = 2.0 * da * x[k] + 2.0 * db * b1[k] - b0[k] + aj * y[k];
    }
  const int i = ncheb - 1;
  double *b1 = b + (size_t) ((i + 1) % 3) * n, *b0 = b + (size_t) (i % 3) * n;
  oracle_atimes (h, b1, x);
  for (int k = 0; k < n; k++) z[k] = da * x[k] + db * b1[k] - b0[k] + a[0] * y[k];
  free (x);
  free (b);
}

/* EV_LJ force on each particle, added to f (stride c).  image = 0: the
 * reference's force (src/ev-LJ.c:185-262), along the primary-cell vector over
 * the image distance; image = 1: the nearest image and the force along the
 * image vector (the convention of this library's own BD engine); image = 2:
 * an open system, the pair vector itself (src/ev-LJ.c:222-233) */
static void
lj_add (int np, int c, const double *pos, double lx, double ly, double lz, double e, double r0,
        int image, double *f)
{
  for (int i = 0; i < np; i++)
    for (int j = i + 1; j < np; j++)
      {
        const double x = pos[3 * i] - pos[3 * j], y = pos[3 * i + 1] - pos[3 * j + 1],
                     z = pos[3 * i + 2] - pos[3 * j + 2];
        if (image)
          {
            const int wrap = image == 1;
            const double xx = wrap ? x - lx * rint (x / lx) : x;
            const double yy = wrap ? y - ly * rint (y / ly) : y;
            const double zz = wrap ? z - lz * rint (z / lz) : z;
            const double r = sqrt (xx * xx + yy * yy + zz * zz);
            const double ov = 2.0 - r;
            if (!(ov > 0.0)) continue;
            double rl = r0 - ov;
            if (rl < 0.0) rl = 1.0e-12;
            const double ri = r0 / rl, ri6 = pow (ri, 6.0);
            const double fr = 12.0 * e * ri6 * ri * (ri6 - 1.0);
            f[c * i] += fr * xx / r;
            f[c * i + 1] += fr * yy / r;
            f[c * i + 2] += fr * zz / r;
            f[c * j] -= fr * xx / r;
            f[c * j + 1] -= fr * yy / r;
            f[c * j + 2] -= fr * zz / r;
            continue;
          }
        for (int kx = -1; kx <= 1; kx++)
          for (int ky = -1; ky <= 1; ky++)
            for (int kz = -1; kz <= 1; kz++)
              {
                const double xx = x + kx * lx, yy = y + ky * ly, zz = z + kz * lz;
                const double r = sqrt (xx * xx + yy * yy + zz * zz);
                const double ov = 2.0 - r;
                if (!(ov > 0.0)) continue;
                double rl = r0 - ov;
                if (rl < 0.0) rl = 1.0e-12;
                const double ri = r0 / rl, ri6 = pow (ri, 6.0);
                const double fr = 12.0 * e * ri6 * ri * (ri6 - 1.0);
                f[c * i] += fr * x / r;
                f[c * i + 1] += fr * y / r;
                f[c * i + 2] += fr * z / r;
                f[c * j] -= fr * x / r;
                f[c * j + 1] -= fr * y / r;
                f[c * j + 2] -= fr * z / r;
              }
      }
}

/* one mid-point step.  y: noise in the product layout (c per particle,
 * torque slots used for FT; stresslet slots absent); x: positions (in/out);
 * z_out (optional): the Chebyshev noise */
void
oracle_bd_step_ex (void *h, int version, int np, double lx, double ly, double lz, double dt,
                   double peclet, int ncheb, const double *a, double e0, double e1,
                   const double *y, const double *F, double lj_e, double lj_r0, int lj_image,
                   double *x, double *z_out)
{
  const int c = ncomp_of (version), n = c * np;
  double *z = calloc ((size_t) n, sizeof (double));
  double *f = calloc ((size_t) n, sizeof (double));
  double *u = calloc ((size_t) n, sizeof (double));
  double *xm = malloc (sizeof (double) * 3 * np);
  const double fact = peclet > 0.0 ? sqrt (2.0 / (peclet * dt)) : 0.0;

  oracle_set_pos (h, x);
  oracle_cheb_eval (h, n, ncheb, a, e0, e1, y, z);
  if (z_out) memcpy (z_out, z, sizeof (double) * n);

  for (int pass = 0; pass < 2; pass++)
    {
      const double *pcur = pass == 0 ? x : xm;
      for (int k = 0; k < n; k++) f[k] = fact * z[k] + (F ? F[k] : 0.0);
      if (lj_e != 0.0) lj_add (np, c, pcur, lx, ly, lz, lj_e, lj_r0, lj_image, f);
      oracle_set_pos (h, pcur);
      oracle_atimes (h, f, u);
      const double hstep = pass == 0 ? 0.5 * dt : dt;
      double *dst = pass == 0 ? xm : x;
      for (int i = 0; i < np; i++)
        for (int d = 0; d < 3; d++) dst[3 * i + d] = x[3 * i + d] + hstep * u[c * i + d];
    }
  free (z);
  free (f);
  free (u);
  free (xm);
}

/* the step with the reference's EV_LJ force */
void
oracle_bd_step (void *h, int version, int np, double lx, double ly, double lz, double dt,
                double peclet, int ncheb, const double *a, double e0, double e1,
                const double *y, const double *F, double lj_e, double lj_r0, double *x,
                double *z_out)
{
  oracle_bd_step_ex (h, version, np, lx, ly, lz, dt, peclet, ncheb, a, e0, e1, y, F, lj_e, lj_r0,
                     0, x, z_out);
}
