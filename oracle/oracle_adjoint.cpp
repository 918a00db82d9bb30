// oracle_adjoint.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU FP64 gradient of L = g . M(r, box) f for the F and FT Ewald mobility
// (equal spheres, no slip, no shear), written as direct pair sums so that it
// shares no structure with the device adjoint:
//   real space  (src/ewald.c:649-789): sum over (i, j, image) of
//               g_i . R(d) f_j,  d = r_j - r_i + t_m;
//   reciprocal  (src/ewald.c:923-1075): sum over (i, j, k) of
//               g_i . [cos(k.d) Bc(k) - sin(k.d) Bs(k)] f_j,  d = r_j - r_i;
//   self        (src/ewald.c:540-643): g_i . self f_i.
// Derivatives by forward-mode dual numbers: in d for dL/dr, in the box
// lengths (through the images t_m = n_m l and k = 2 pi n / l, pi/V) for
// dL/dl.  Scalars restate src/ewald.c:49-120 (the F and FT rows of
// scalars_ewald_real) and the y-functions of src/ewald.c:955-983.
#include <cmath>
#include <cstring>

namespace {

struct D {
  double v, d[3];
  D (double x = 0.0) : v (x), d{0.0, 0.0, 0.0} {}
};
D operator+ (const D &a, const D &b) { D r (a.v + b.v); for (int k = 0; k < 3; k++) r.d[k] = a.d[k] + b.d[k]; return r; }
D operator- (const D &a, const D &b) { D r (a.v - b.v); for (int k = 0; k < 3; k++) r.d[k] = a.d[k] - b.d[k]; return r; }
D operator- (const D &a) { D r (-a.v); for (int k = 0; k < 3; k++) r.d[k] = -a.d[k]; return r; }
D operator* (const D &a, const D &b) { D r (a.v * b.v); for (int k = 0; k < 3; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
D operator/ (const D &a, const D &b)
{ D r (a.v / b.v); for (int k = 0; k < 3; k++) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v); return r; }
D fn (const D &a, double f, double df) { D r (f); for (int k = 0; k < 3; k++) r.d[k] = df * a.d[k]; return r; }
D Derfc (const D &x) { return fn (x, std::erfc (x.v), -2.0 / std::sqrt (M_PI) * std::exp (-x.v * x.v)); }
D Dexp (const D &x) { double e = std::exp (x.v); return fn (x, e, e); }
D Dsqrt (const D &x) { double s = std::sqrt (x.v); return fn (x, s, 0.5 / s); }
D Dcos (const D &x) { return fn (x, std::cos (x.v), -std::sin (x.v)); }
D Dsin (const D &x) { return fn (x, std::sin (x.v), std::cos (x.v)); }

// xa, ya (F); yb, xc, yc (FT) at distance r, unit radius
void
scalars (int version, double xi, const D &r, D s[5])
{
  const D u2 = D (xi) * r * D (xi) * r;
  const D r2 = r * r;
  const D ec = Derfc (D (xi) * r);
  const D ex = D (xi / std::sqrt (M_PI)) * Dexp (-u2);
  const D a1 = (D (0.75) + D (0.5) / r2) / r * ec
    + ((D (1.0) + u2 * (D (14.0) + D (4.0) * u2 * (u2 - D (5.0)))) / r2 - D (4.5) + D (3.0) * u2) * ex;
  const D a2 = (D (0.75) - D (1.5) / r2) / r * ec
    + ((D (-3.0) + u2 * (D (-2.0) + D (4.0) * u2 * (D (4.0) - u2))) / r2 + D (1.5) - D (3.0) * u2) * ex;
  s[0] = a1 + a2;   // xa
  s[1] = a1;        // ya
  s[2] = s[3] = s[4] = D (0.0);
  if (version == 0) return;
  s[2] = D (-0.75) / r2 * ec - D (1.5) * (D (1.0) + u2 * (D (-6.0) + D (2.0) * u2)) / r * ex;
  const D c1 = D (-0.375) / (r2 * r) * ec
    - D (0.75) * (D (1.0) + u2 * (D (14.0) + u2 * (D (-20.0) + D (4.0) * u2))) / r2 * ex;
  const D c2 = D (1.125) / (r2 * r) * ec
    - D (0.75) * (D (-3.0) + u2 * (D (-2.0) + u2 * (D (16.0) - D (4.0) * u2))) / r2 * ex;
  s[3] = c1 + c2;   // xc
  s[4] = c1;        // yc
}

D dot (const D *a, const D *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
void cross (const D *a, const D *b, D *c)
{
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// g_i . R f_j for the real-space pair block with unit vector e from i to j
D
real_pair (int version, const D *e, const D *s, const double *gi, const double *fj)
{
  D F[3], G[3];
  for (int a = 0; a < 3; a++) { F[a] = D (fj[a]); G[a] = D (gi[a]); }
  const D eF = dot (e, F), eG = dot (e, G);
  D out = s[1] * dot (G, F) + (s[0] - s[1]) * eF * eG;
  if (version == 0) return out;
  D T[3], Gt[3], Txe[3], Fxe[3];
  for (int a = 0; a < 3; a++) { T[a] = D (fj[3 + a]); Gt[a] = D (gi[3 + a]); }
  cross (T, e, Txe);
  cross (F, e, Fxe);
  const D eT = dot (e, T), eGt = dot (e, Gt);
  out = out + s[2] * dot (G, Txe) + s[2] * dot (Gt, Fxe) + s[4] * dot (Gt, T)
    + (s[3] - s[4]) * eT * eGt;
  return out;
}

// g_i . [c Bc - s Bs] f_j for one k (unit vector e, weights ya, yb, yc)
D
recip_pair (int version, const D *e, const D &ya, const D &yb, const D &yc, const D &cs,
            const D &sn, const double *gi, const double *fj)
{
  D F[3], G[3];
  for (int a = 0; a < 3; a++) { F[a] = D (fj[a]); G[a] = D (gi[a]); }
  const D eF = dot (e, F), eG = dot (e, G);
  D out = cs * ya * (dot (G, F) - eF * eG);
  if (version == 0) return out;
  D T[3], Gt[3], Txe[3], Fxe[3];
  for (int a = 0; a < 3; a++) { T[a] = D (fj[3 + a]); Gt[a] = D (gi[3 + a]); }
  cross (T, e, Txe);
  cross (F, e, Fxe);
  const D eT = dot (e, T), eGt = dot (e, Gt);
  out = out + cs * yc * (dot (Gt, T) - eT * eGt)
    - sn * yb * (dot (G, Txe) + dot (Gt, Fxe));
  return out;
}

}  // namespace

extern "C" {

/* dLdr[3 np], dLdbox[3], *Lout for L = g . M f.  rl, rm: the image table
 * (3 per image); the k set is the cube |m| <= kmax{x,y,z} without 0, cut at
 * |k| <= kmax unless kmax == 0. */
void
oracle_vjp (int version, int np, const double *pos, double lx, double ly, double lz, double xi,
            double rmax2, double rmin, int nr, const double *rl, const int *rm, int kmaxx,
            int kmaxy, int kmaxz, double kmax, double self_a, double self_c, const double *g,
            const double *f, double *dLdr, double *dLdbox, double *Lout)
{
  const int c = version == 0 ? 3 : 6;
  const double L3[3] = {lx, ly, lz};
  std::memset (dLdr, 0, sizeof (double) * 3 * np);
  double box[3] = {0.0, 0.0, 0.0}, Lval = 0.0;
  // self
  for (int i = 0; i < np; i++)
    for (int q = 0; q < c; q++) Lval += g[c * i + q] * (q < 3 ? self_a : self_c) * f[c * i + q];
  // real space: seeds in d for the positions, in l for the box
  for (int i = 0; i < np; i++)
    for (int j = 0; j < np; j++)
      for (int m = 0; m < nr; m++)
        {
          double dv[3];
          for (int a = 0; a < 3; a++) dv[a] = pos[3 * j + a] - pos[3 * i + a] + rl[3 * m + a];
          const double rr = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
          if (rr == 0.0 || rr > rmax2) continue;
          for (int pass = 0; pass < 2; pass++)
            {
              D d[3];
              for (int a = 0; a < 3; a++)
                {
                  d[a] = D (dv[a]);
                  if (pass == 0) d[a].d[a] = 1.0;                     // d/dd
                  else d[a].d[a] = (double) rm[3 * m + a];            // d/dl_a
                }
              D r = Dsqrt (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
              if (r.v < 2.0 * rmin) r = D (2.0 * rmin);
              const D e[3] = {d[0] / r, d[1] / r, d[2] / r};
              D s[5];
              scalars (version, xi, r, s);
              const D phi = real_pair (version, e, s, g + c * i, f + c * j);
              if (pass == 0)
                {
                  Lval += phi.v;
                  // d = r_j - r_i + t: dL/dr_i -= grad, dL/dr_j += grad
                  for (int a = 0; a < 3; a++)
                    {
                      dLdr[3 * i + a] -= phi.d[a];
                      dLdr[3 * j + a] += phi.d[a];
                    }
                }
              else
                for (int a = 0; a < 3; a++) box[a] += phi.d[a];
            }
        }
  // reciprocal space
  const double pi_ = M_PI, xi2 = xi * xi;
  for (int m1 = -kmaxx; m1 <= kmaxx; m1++)
    for (int m2 = -kmaxy; m2 <= kmaxy; m2++)
      for (int m3 = -kmaxz; m3 <= kmaxz; m3++)
        {
          if (m1 == 0 && m2 == 0 && m3 == 0) continue;
          const double kv[3] = {2.0 * pi_ * m1 / lx, 2.0 * pi_ * m2 / ly, 2.0 * pi_ * m3 / lz};
          const double kn = std::sqrt (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
          if (kmax != 0.0 && kn > kmax) continue;
          // k, weights and unit vector as functions of the box lengths
          D Ll[3];
          for (int a = 0; a < 3; a++) { Ll[a] = D (L3[a]); Ll[a].d[a] = 1.0; }
          const int mm[3] = {m1, m2, m3};
          D k[3];
          for (int a = 0; a < 3; a++) k[a] = D (2.0 * pi_ * mm[a]) / Ll[a];
          const D kk = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
          const D kr = Dsqrt (kk);
          const D k4z = kk / D (4.0 * xi2);
          const D pivol = D (pi_) / (Ll[0] * Ll[1] * Ll[2]);
          const D kexp = pivol * (D (1.0) + k4z * (D (1.0) + D (2.0) * k4z)) / kk * Dexp (-k4z);
          const D ya = D (6.0) * (D (1.0) - kk / D (3.0)) * kexp;
          const D yb = D (3.0) * kr * kexp;
          const D yc = D (1.5) * kk * kexp;
          const D eL[3] = {k[0] / kr, k[1] / kr, k[2] / kr};
          // constants for the position pass
          D ec[3];
          for (int a = 0; a < 3; a++) ec[a] = D (eL[a].v);
          for (int i = 0; i < np; i++)
            for (int j = 0; j < np; j++)
              {
                double dv[3];
                for (int a = 0; a < 3; a++) dv[a] = pos[3 * j + a] - pos[3 * i + a];
                // positions: seed d (pair terms with i != j depend on r)
                {
                  D d[3];
                  for (int a = 0; a < 3; a++) { d[a] = D (dv[a]); d[a].d[a] = 1.0; }
                  const D kd = D (kv[0]) * d[0] + D (kv[1]) * d[1] + D (kv[2]) * d[2];
                  const D phi = recip_pair (version, ec, D (ya.v), D (yb.v), D (yc.v), Dcos (kd),
                                            Dsin (kd), g + c * i, f + c * j);
                  Lval += phi.v;
                  if (i != j)
                    for (int a = 0; a < 3; a++)
                      {
                        dLdr[3 * i + a] -= phi.d[a];
                        dLdr[3 * j + a] += phi.d[a];
                      }
                }
                // box: k and the weights depend on l, d does not
                {
                  const D kd = k[0] * D (dv[0]) + k[1] * D (dv[1]) + k[2] * D (dv[2]);
                  const D phi = recip_pair (version, eL, ya, yb, yc, Dcos (kd), Dsin (kd),
                                            g + c * i, f + c * j);
                  for (int a = 0; a < 3; a++) box[a] += phi.d[a];
                }
              }
        }
  for (int a = 0; a < 3; a++) dLdbox[a] = box[a];
  *Lout = Lval;
}

}  // extern "C"
