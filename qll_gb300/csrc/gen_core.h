/*
 * gen_core.h -- the seeded input generator itself (gauge links and
 * sources), as static functions, so that the library (gen.c) and the CPU
 * oracle compile the same code and produce bit-identical inputs on one
 * machine.  The algorithms are described in gen.c.  Extents must have
 * been checked by the caller (even, >= 4).
 */
#ifndef QLLG_GEN_CORE_H
#define QLLG_GEN_CORE_H
#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint64_t
splitmix64(uint64_t z)
{
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

/* uniform in (0,1] */
static inline double
unif(uint64_t seedh, uint64_t ctr)
{
  uint64_t h = splitmix64(seedh ^ splitmix64(ctr));
  return ((double)(h >> 11) + 1.0)*(1.0/9007199254740992.0);
}

/* Gaussian pair of counter ctr */
static inline void
gauss2(uint64_t seedh, uint64_t ctr, double *g1, double *g2)
{
  double u1 = unif(seedh, 2*ctr), u2 = unif(seedh, 2*ctr + 1);
  double r = sqrt(-2.0*log(u1));
  double t = 6.283185307179586476925*u2;
  *g1 = r*cos(t);
  *g2 = r*sin(t);
}

typedef struct { double r, i; } cplx;

static inline cplx cmul(cplx a, cplx b) { cplx c = {a.r*b.r - a.i*b.i, a.r*b.i + a.i*b.r}; return c; }
static inline cplx cconj(cplx a) { cplx c = {a.r, -a.i}; return c; }

/* row-major 3x3 */
static void
mmul(cplx *c, const cplx *a, const cplx *b)
{
  cplx t[9];
  for(int i=0; i<3; i++) for(int j=0; j<3; j++) {
    cplx s = {0, 0};
    for(int k=0; k<3; k++) { cplx p = cmul(a[3*i+k], b[3*k+j]); s.r += p.r; s.i += p.i; }
    t[3*i+j] = s;
  }
  memcpy(c, t, sizeof(t));
}

/* exp(X) by scaling and squaring with a Taylor polynomial */
static void
mexp(cplx *E, const cplx *X)
{
  double nrm = 0;
  for(int i=0; i<3; i++) {
    double rs = 0;
    for(int j=0; j<3; j++) rs += hypot(X[3*i+j].r, X[3*i+j].i);
    if(rs > nrm) nrm = rs;
  }
  int s = 0;
  while(nrm > 0.25) { nrm *= 0.5; s++; }
  double sc = ldexp(1.0, -s);
  cplx Y[9], T[9];
  for(int k=0; k<9; k++) { Y[k].r = X[k].r*sc; Y[k].i = X[k].i*sc; }
  /* Horner: E = I + Y(I + Y/2(I + Y/3(...))) */
  for(int k=0; k<9; k++) { E[k].r = (k % 4 == 0) ? 1 : 0; E[k].i = 0; }
  for(int n=18; n>=1; n--) {
    mmul(T, Y, E);
    for(int k=0; k<9; k++) {
      E[k].r = T[k].r/n + ((k % 4 == 0) ? 1 : 0);
      E[k].i = T[k].i/n;
    }
  }
  for(int q=0; q<s; q++) mmul(E, E, E);
}

static void
su3_project(cplx *U)
{
  cplx *r1 = U, *r2 = U + 3, *r3 = U + 6;
  double n = 0;
  for(int j=0; j<3; j++) n += r1[j].r*r1[j].r + r1[j].i*r1[j].i;
  n = 1/sqrt(n);
  for(int j=0; j<3; j++) { r1[j].r *= n; r1[j].i *= n; }
  cplx d = {0, 0};
  for(int j=0; j<3; j++) { cplx p = cmul(cconj(r1[j]), r2[j]); d.r += p.r; d.i += p.i; }
  for(int j=0; j<3; j++) { cplx p = cmul(d, r1[j]); r2[j].r -= p.r; r2[j].i -= p.i; }
  n = 0;
  for(int j=0; j<3; j++) n += r2[j].r*r2[j].r + r2[j].i*r2[j].i;
  n = 1/sqrt(n);
  for(int j=0; j<3; j++) { r2[j].r *= n; r2[j].i *= n; }
  /* r3 = conj(r1 x r2) */
  for(int j=0; j<3; j++) {
    int a = (j + 1) % 3, b = (j + 2) % 3;
    cplx p = cmul(r1[a], r2[b]), q = cmul(r1[b], r2[a]);
    cplx c = {p.r - q.r, p.i - q.i};
    r3[j] = cconj(c);
  }
}

static void
coords_of(const int L[4], int V, int idx, int x[4])
{
  int p = idx >= V/2;
  int i = idx - p*(V/2);
  int X0h = L[0]/2;
  int x0h = i % X0h, r = i / X0h;
  x[1] = r % L[1]; r /= L[1];
  x[2] = r % L[2]; x[3] = r / L[2];
  x[0] = 2*x0h + ((p + x[1] + x[2] + x[3]) & 1);
}

static void
gen_gauge_fill(const int L[4], unsigned long long seed, double eps, int ks, double *u[4])
{
  const int V = L[0]*L[1]*L[2]*L[3];
  const uint64_t sh = splitmix64((uint64_t)seed ^ 0x51ed2701f3a5c7e9ULL);
#pragma omp parallel for schedule(static)
  for(int s=0; s<V; s++) {
    int x[4];
    coords_of(L, V, s, x);
    uint64_t lex = (uint64_t)x[0] + (uint64_t)L[0]*(x[1] + (uint64_t)L[1]*(x[2] + (uint64_t)L[2]*x[3]));
    for(int mu=0; mu<4; mu++) {
      cplx A[9], H[9], X[9], U[9];
      for(int k=0; k<9; k++) {
        double a, b;
        gauss2(sh, (lex*4 + mu)*16 + k, &a, &b);
        A[k].r = a*0.70710678118654752440; A[k].i = b*0.70710678118654752440;
      }
      for(int i=0; i<3; i++) for(int j=0; j<3; j++) {
        H[3*i+j].r = 0.5*(A[3*i+j].r + A[3*j+i].r);
        H[3*i+j].i = 0.5*(A[3*i+j].i - A[3*j+i].i);
      }
      double tr = (H[0].r + H[4].r + H[8].r)/3.0;
      H[0].r -= tr; H[4].r -= tr; H[8].r -= tr;
      for(int k=0; k<9; k++) { X[k].r = -eps*H[k].i; X[k].i = eps*H[k].r; }
      mexp(U, X);
      su3_project(U);
      double eta = 1;
      if(ks) { int sum = 0; for(int nu=0; nu<mu; nu++) sum += x[nu]; if(sum & 1) eta = -1; }
      double *m = u[mu] + 18L*s;
      for(int row=0; row<3; row++) for(int col=0; col<3; col++) {
        m[(3*col + row)*2] = eta*U[3*row+col].r;
        m[(3*col + row)*2 + 1] = eta*U[3*row+col].i;
      }
    }
  }
}


static void
gen_source_fill(const int L[4], unsigned long long seed, int nelem, const char *sub, double *v)
{
  const int V = L[0]*L[1]*L[2]*L[3];
  int i0 = 0, i1 = V;
  if(sub && sub[0] == 'e') i1 = V/2;
  else if(sub && sub[0] == 'o') i0 = V/2;
  const uint64_t sh = splitmix64((uint64_t)seed ^ 0x3c6ef372fe94f82bULL);
#pragma omp parallel for schedule(static)
  for(int s=0; s<V; s++) {
    double *vs = v + (long)nelem*s;
    if(s < i0 || s >= i1) { for(int e=0; e<nelem; e++) vs[e] = 0; continue; }
    int x[4];
    coords_of(L, V, s, x);
    uint64_t lex = (uint64_t)x[0] + (uint64_t)L[0]*(x[1] + (uint64_t)L[1]*(x[2] + (uint64_t)L[2]*x[3]));
    for(int e=0; e<nelem; e+=2) {
      double a, b;
      gauss2(sh, lex*64 + e/2, &a, &b);
      vs[e] = a;
      if(e + 1 < nelem) vs[e+1] = b;
    }
  }
}

#endif
