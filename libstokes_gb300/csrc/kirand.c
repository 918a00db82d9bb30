/* kirand.c -- host random numbers with libstokes' KIrand interface
 * (replaces src/KIrand.c): the Mersenne Twister MT19937 of Matsumoto and
 * Nishimura (ACM TOMACS 8, 1998) and the polar Box-Muller method with the
 * second deviate kept for the next call.  The generator's constants and
 * steps are those of the published algorithm; they have to be alike for the
 * same seed to give the same stream, which the Brownian-dynamics parity
 * tests rely on.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "stokes_bd.h"

#define MT_N KIRAND_MT_N
#define MT_M 397
#define MT_MATRIX_A 0x9908b0dfUL
#define MT_UPPER 0x80000000UL
#define MT_LOWER 0x7fffffffUL

struct KIrand *
KIrand_init (void)
{
  struct KIrand *r = (struct KIrand *) calloc (1, sizeof (struct KIrand));
  if (r == NULL)
    {
      fprintf (stderr, "libstokes_gb300 KIrand_init: out of memory\n");
      exit (1);
    }
  r->mti = MT_N + 1;   /* not seeded */
  return r;
}

void
KIrand_free (struct KIrand *r)
{
  free (r);
}

void
KIrand_load_mt (struct KIrand *r, unsigned long *mt, int mti)
{
  for (int i = 0; i < MT_N; i++) r->mt[i] = mt[i];
  r->mti = mti;
}

void
KIrand_load_Gaussian (struct KIrand *r, unsigned long *mt, int mti, int flag_saved,
                      double x_saved)
{
  KIrand_load_mt (r, mt, mti);
  r->Gaussian_has_saved = flag_saved;
  r->Gaussian_saved = x_saved;
}

/* seeding by the linear recurrence of the published generator */
void
KIrand_init_genrand (struct KIrand *r, unsigned long s)
{
  r->mt[0] = s & 0xffffffffUL;
  for (int i = 1; i < MT_N; i++)
    {
      unsigned long prev = r->mt[i - 1];
      r->mt[i] = (1812433253UL * (prev ^ (prev >> 30)) + (unsigned long) i) & 0xffffffffUL;
    }
  r->mti = MT_N;
}

/* regenerate the whole state vector (twist) */
static void
mt_twist (struct KIrand *r)
{
  for (int k = 0; k < MT_N; k++)
    {
      const unsigned long y = (r->mt[k] & MT_UPPER) | (r->mt[(k + 1) % MT_N] & MT_LOWER);
      r->mt[k] = r->mt[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1UL) ? MT_MATRIX_A : 0UL);
    }
  r->mti = 0;
}

unsigned long
KIrand_genrand_int32 (struct KIrand *r)
{
  if (r->mti >= MT_N)
    {
      if (r->mti == MT_N + 1) KIrand_init_genrand (r, 5489UL);
      mt_twist (r);
    }
  unsigned long y = r->mt[r->mti++];
  /* tempering */
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680UL;
  y ^= (y << 15) & 0xefc60000UL;
  y ^= (y >> 18);
  return y & 0xffffffffUL;
}

long
KIrand_genrand_int31 (struct KIrand *r)
{
  return (long) (KIrand_genrand_int32 (r) >> 1);
}

/* [0,1] */
double
KIrand_genrand_real1 (struct KIrand *r)
{
  return (double) KIrand_genrand_int32 (r) * (1.0 / 4294967295.0);
}

/* [0,1) */
double
KIrand_genrand_real2 (struct KIrand *r)
{
  return (double) KIrand_genrand_int32 (r) * (1.0 / 4294967296.0);
}

/* (0,1) */
double
KIrand_genrand_real3 (struct KIrand *r)
{
  return ((double) KIrand_genrand_int32 (r) + 0.5) * (1.0 / 4294967296.0);
}

/* [0,1) with 53-bit resolution */
double
KIrand_genrand_res53 (struct KIrand *r)
{
  const unsigned long a = KIrand_genrand_int32 (r) >> 5, b = KIrand_genrand_int32 (r) >> 6;
  return ((double) a * 67108864.0 + (double) b) * (1.0 / 9007199254740992.0);
}

/* N(0,1) by the polar method; every second call returns the saved deviate */
double
KIrand_Gaussian (struct KIrand *r)
{
  if (r->Gaussian_has_saved)
    {
      r->Gaussian_has_saved = 0;
      return r->Gaussian_saved;
    }
  double x, y, s;
  do
    {
      x = 2.0 * KIrand_genrand_real2 (r) - 1.0;
      y = 2.0 * KIrand_genrand_real2 (r) - 1.0;
      s = x * x + y * y;
    }
  while (s > 1.0 || s == 0.0);
  s = sqrt (-2.0 * log (s) / s);
  r->Gaussian_saved = y * s;
  r->Gaussian_has_saved = 1;
  return x * s;
}
