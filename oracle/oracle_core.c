/*
 * oracle_core.c -- precision-independent part of the CPU oracle
 * (TEST INFRASTRUCTURE ONLY; see qll_oracle.h).
 *
 * Geometry, neighbour tables and gamma matrices, restated from the
 * reference for one rank and VLEN=1, plus the known-answer tests of the
 * reference's stress.c and fieldtest.c run on the oracle's own transporter.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "qll_oracle.h"

int
or_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* the thread count of the oracle's parallel loops (a host process that
 * also runs other OpenMP code may have changed it) */
void
or_set_num_threads(int n)
{
#ifdef _OPENMP
  if(n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int
or_nsites(const int dims[4])
{
  return dims[0]*dims[1]*dims[2]*dims[3];
}

/* layoutIndex for one rank and innerGeom = 1 (lib/layout.c:120-142):
 * lexicographic index oi (x0 fastest, lex_i :95-103), then oi/2 for even
 * parity and (oi+nSitesOuter)/2 for odd parity. */
int
or_site_index(const int dims[4], const int x[4])
{
  int oi = 0;
  for(int i=3; i>=0; --i) oi = oi*dims[i] + (x[i] % dims[i]);
  int p = x[0] + x[1] + x[2] + x[3];
  int V = or_nsites(dims);
  int oi2 = oi/2;
  if(p & 1) oi2 = (oi + V)/2;
  return oi2;
}

/* layoutCoord for one rank and innerGeom = 1 (lib/layout.c:144-205):
 * undo the parity split, expand 2*ii lexicographically, and if the parity
 * is odd step the coordinate by one in lexicographic order. */
void
or_site_coord(const int dims[4], int idx, int x[4])
{
  int V = or_nsites(dims);
  int nEven = V - V/2;
  int ii = idx, p = 0;
  if(ii >= nEven) { ii -= nEven; p++; }
  ii *= 2;
  for(int i=0; i<4; i++) {
    int k = ii % dims[i];
    x[i] = k;
    p += k;
    ii /= dims[i];
  }
  if(p & 1) {
    for(int i=0; i<4; i++) {
      x[i]++;
      if(x[i] >= dims[i]) x[i] = 0;
      else break;
    }
  }
}

/* map() of lib/shifts.c:312-358 restricted to one rank: destination i takes
 * its value from coord(i) - disp, or nothing (-1) when the parity filter of
 * the subset excludes it (SUB2PAR :370).  With VLEN=1 the pidx of
 * makeShiftMultiSub (:657-670) is that source index. */
void
or_shift_table(const int dims[4], const int disp[4], int parity, int *pidx)
{
  int V = or_nsites(dims);
#pragma omp parallel for
  for(int i=0; i<V; i++) {
    int x[4], y[4];
    or_site_coord(dims, i, x);
    int p = x[0] + x[1] + x[2] + x[3];
    if(parity >= 0 && (p & 1) != parity) { pidx[i] = -1; continue; }
    for(int k=0; k<4; k++) y[k] = (x[k] - disp[k] + dims[k]) % dims[k];
    pidx[i] = or_site_index(dims, y);
  }
}

/* slot s of a staggered link set: with Naik (SHIFT13 pairing,
 * lib/stagDslash.c:853-856) slot 2i is the one-hop and 2i+1 the three-hop
 * shift of direction i/2; i even gathers from forward (disp -len), i odd
 * from backward (:829-832).  Without Naik slot i is the one-hop shift i. */
void
or_stag_slot_table(const int dims[4], int slot, int naik, int parity, int *pidx)
{
  int i = naik ? slot/2 : slot;
  int len = (naik && (slot & 1)) ? 3 : 1;
  int disp[4] = {0,0,0,0};
  disp[i/2] = len*(2*(i & 1) - 1);
  or_shift_table(dims, disp, parity, pidx);
}

/* gammaMatrix of lib/Gamma.lua:5-26: gammaDir[d] = gammaMatrix[2^d] for
 * d<4, gammaDir[4] = gammaMatrix[15] = g1 g2 g4 g8 (product order of the
 * generator loop). */
static void
gmul(double *r, const double *a, const double *b)
{
  double t[32];
  for(int i=0; i<4; i++) for(int j=0; j<4; j++) {
    double sr = 0, si = 0;
    for(int k=0; k<4; k++) {
      double ar = a[(i*4+k)*2], ai = a[(i*4+k)*2+1];
      double br = b[(k*4+j)*2], bi = b[(k*4+j)*2+1];
      sr += ar*br - ai*bi;
      si += ar*bi + ai*br;
    }
    t[(i*4+j)*2] = sr; t[(i*4+j)*2+1] = si;
  }
  memcpy(r, t, sizeof(t));
}

void
or_gamma(int d, double g[32])
{
  /* entries as (re,im); I = (0,1) */
  static const double G[4][32] = {
    /* gammaMatrix[1] */
    {0,0, 0,0, 0,0, 0,1,   0,0, 0,0, 0,1, 0,0,   0,0, 0,-1, 0,0, 0,0,   0,-1, 0,0, 0,0, 0,0},
    /* gammaMatrix[2] */
    {0,0, 0,0, 0,0, -1,0,  0,0, 0,0, 1,0, 0,0,   0,0, 1,0, 0,0, 0,0,    -1,0, 0,0, 0,0, 0,0},
    /* gammaMatrix[4] */
    {0,0, 0,0, 0,1, 0,0,   0,0, 0,0, 0,0, 0,-1,  0,-1, 0,0, 0,0, 0,0,   0,0, 0,1, 0,0, 0,0},
    /* gammaMatrix[8] */
    {0,0, 0,0, 1,0, 0,0,   0,0, 0,0, 0,0, 1,0,   1,0, 0,0, 0,0, 0,0,    0,0, 1,0, 0,0, 0,0},
  };
  if(d < 4) { memcpy(g, G[d], sizeof(G[d])); return; }
  double m[32];
  memcpy(m, G[0], sizeof(m));
  gmul(m, m, G[1]);
  gmul(m, m, G[2]);
  gmul(m, m, G[3]);
  memcpy(g, m, sizeof(m));
}

/* ---- known-answer tests held by the reference's own test programs ---- */

void or_makeUD(double *m, int nsites);
void or_transportD(const int dims[4], double *dest, const double *u,
                   const double *src, int nelem, int dir, int fwd);
void or_doublestoreD(const int dims[4], double *ua, const double *u, int dir, int len);

static double
norm2d(const double *x, long n)
{
  double s = 0;
  for(long i=0; i<n; i++) s += x[i]*x[i];
  return s;
}

/* stress.c:132-234: constant unitary links (makeU of element values 1..18),
 * constant vector 1..6; v2 accumulates nrep rounds of the 8 one-hop
 * transports; |v2|^2 must equal V*64*nrep^2*|U v1|^2 and repeat bitwise. */
double
or_stress_kat(const int dims[4], int nrep, int npass, int *bitwise_ok)
{
  int V = or_nsites(dims);
  double *v1 = malloc(sizeof(double)*6*V);
  double *v2 = malloc(sizeof(double)*6*V);
  double *u = malloc(sizeof(double)*18*V);
  for(int i=0; i<V; i++) {
    for(int j=0; j<6; j++) v1[6*i+j] = j + 1;
    for(int j=0; j<18; j++) u[18*i+j] = j + 1;
  }
  or_makeUD(u, V);
  /* check = |u(0) v1(0)|^2 as X_peq_M_times_xXp on one site (stress.c:171-174) */
  double t[6] = {0,0,0,0,0,0};
  for(int i=0; i<3; i++) {
    double vr = v1[2*i], vi = v1[2*i+1];
    for(int j=0; j<3; j++) {
      t[2*j]   += u[(3*i+j)*2]*vr - u[(3*i+j)*2+1]*vi;
      t[2*j+1] += u[(3*i+j)*2]*vi + u[(3*i+j)*2+1]*vr;
    }
  }
  double check = t[0]*t[0]+t[1]*t[1]+t[2]*t[2]+t[3]*t[3]+t[4]*t[4]+t[5]*t[5];
  double ratio0 = 0, prev = 0;
  *bitwise_ok = 1;
  for(int its=0; its<npass; its++) {
    memset(v2, 0, sizeof(double)*6*V);
    for(int r=0; r<nrep; r++)
      for(int d=0; d<8; d++)
        or_transportD(dims, v2, u, v1, 6, d/2, (d & 1) == 0);
    double nv = norm2d(v2, 6L*V);
    if(its == 0) {
      ratio0 = nv/check/V/nrep/nrep/64.0;
      prev = nv;
    } else if(nv != prev) {
      *bitwise_ok = 0;
    }
  }
  free(v1); free(v2); free(u);
  return ratio0;
}

/* fieldtest.c:92-191: v1 = real index, u = makeU of the site-dependent
 * pattern, ua = double-stored adjoint of u in direction 3; forward
 * transport with u then backward transport with ua returns v1. */
double
or_fieldtest_kat(const int dims[4])
{
  int V = or_nsites(dims);
  double *v1 = malloc(sizeof(double)*6*V);
  double *v2 = calloc(6L*V, sizeof(double));
  double *v3 = calloc(6L*V, sizeof(double));
  double *u = malloc(sizeof(double)*18*V);
  double *ua = malloc(sizeof(double)*18*V);
  for(int i=0; i<V; i++) {
    int k = i*6;
    for(int j=0; j<6; j++) v1[k+j] = k + j;
    int km = i*18;
    for(int j1=0; j1<3; j1++) for(int j2=0; j2<3; j2++) {
      int j0 = km + (j1 + j2*3)*2;
      u[j0]   = 1 + j0/(double)(1 + j1 + j2);
      u[j0+1] = 1 + j0/(double)(1 + j1*j2);
    }
  }
  or_makeUD(u, V);
  int dir = 3;
  or_doublestoreD(dims, ua, u, dir, -1);
  or_transportD(dims, v2, u, v1, 6, dir, 1);
  or_transportD(dims, v3, ua, v2, 6, dir, 0);
  double s = 0;
  for(long i=0; i<6L*V; i++) { double d = v3[i] - v1[i]; s += d*d; }
  free(v1); free(v2); free(v3); free(u); free(ua);
  return s;
}
