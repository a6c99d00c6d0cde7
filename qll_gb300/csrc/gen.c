/*
 * gen.c -- seeded synthetic inputs: SU(3) gauge links and Gaussian
 * sources, computed on the host so that the GPU library and the CPU
 * oracle see bit-identical inputs, independent of thread count.
 *
 * Random numbers: SplitMix64 (Steele, Lea and Flood, "Fast splittable
 * pseudorandom number generators", OOPSLA 2014; the finaliser constants of
 * Vigna's public-domain splitmix64.c) applied to a counter built from
 * (seed, lexicographic site, direction, entry): every number depends only
 * on its key.  Gaussians by the Box-Muller transform.
 *
 * Links: U = exp(i eps H) with H = (A + A^dagger)/2 minus its trace/3 and A
 * a 3x3 matrix of unit-variance complex Gaussians; the exponential by
 * scaling and squaring with a degree-18 Taylor series, then projected to
 * SU(3) (row 1 normalised, row 2 orthogonalised and normalised,
 * row 3 = conj(row1 x row2), so det U = 1 exactly up to rounding).
 */
#include "qll_gb300.h"
#include "qllg_internal.h"
#include "gen_core.h"

int
qllg_gen_gauge(const int dims[4], unsigned long long seed, double eps, int ks, double *u[4])
{
  qllg_geom g;
  if(qllg_geom_from_dims(&g, dims)) return -1;
  gen_gauge_fill(g.L, seed, eps, ks, u);
  return 0;
}

int
qllg_gen_source(const int dims[4], unsigned long long seed, int nelem, const char *sub, double *v)
{
  qllg_geom g;
  if(qllg_geom_from_dims(&g, dims)) return -1;
  gen_source_fill(g.L, seed, nelem, sub, v);
  return 0;
}

void
qllg_asqtad_coeffs(Fat7Coeffs *c)
{
  c->one_link = 5.0/8.0;
  c->three_staple = -1.0/16.0;
  c->five_staple = 1.0/64.0;
  c->seven_staple = -1.0/384.0;
  c->lepage = -1.0/16.0;
  c->naik = -1.0/24.0;
}
