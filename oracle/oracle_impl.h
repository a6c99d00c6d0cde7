/*
 * oracle_impl.h -- precision-templated CPU oracle (TEST INFRASTRUCTURE ONLY;
 * see qll_oracle.h).  Included by oracle_d.c (real=double, S=D) and
 * oracle_f.c (real=float, S=F), mirroring the reference's XD.c/XF.c
 * wrappers (lib/stagDslashD.c, lib/stagDslashF.c).
 *
 * Each routine restates the reference routine named in its comment, with
 * the same operation order inside a site, so that the float variant rounds
 * where the reference's F variant rounds (scalars handed to a `real`
 * argument are converted to real first, reductions accumulate in double).
 */
#ifndef real
#error "define real and S before including oracle_impl.h"
#endif

#define OCAT_(a,b) a##b
#define OCAT(a,b) OCAT_(a,b)
#define OFN(n) OCAT(n, S)

/* ---------------------------------------------------------------- tables */

/* neighbour tables are built once per (dims, displacement) and kept, like
 * the static shift tables of lib/stagDslash.c:715-719 */
typedef struct { int dims[4]; int disp[4]; int *t; } OFN(tcache_t);
#define OR_NCACHE 512
static OFN(tcache_t) OFN(tcache)[OR_NCACHE];
static int OFN(ntcache) = 0, OFN(next_evict) = 0;

static const int *
OFN(table)(const int dims[4], const int disp[4])
{
  for(int i=0; i<OFN(ntcache); i++) {
    OFN(tcache_t) *c = &OFN(tcache)[i];
    if(!memcmp(c->dims, dims, sizeof(int)*4) && !memcmp(c->disp, disp, sizeof(int)*4))
      return c->t;
  }
  /* full: replace the oldest entry only, so tables handed out earlier in
   * the same call (at most 16) stay valid */
  OFN(tcache_t) *c;
  if(OFN(ntcache) < OR_NCACHE) c = &OFN(tcache)[OFN(ntcache)++];
  else {
    c = &OFN(tcache)[OFN(next_evict)];
    OFN(next_evict) = (OFN(next_evict) + 1) % OR_NCACHE;
    free(c->t);
  }
  memcpy(c->dims, dims, sizeof(int)*4);
  memcpy(c->disp, disp, sizeof(int)*4);
  c->t = malloc(sizeof(int)*or_nsites(dims));
  or_shift_table(dims, disp, -1, c->t);
  return c->t;
}

/* table of getShift(dir, len) (lib/stagDslash.c:735-749): len>0 gathers
 * from x + len*dir, len<0 from x - |len|*dir */
static const int *
OFN(shift_table)(const int dims[4], int dir, int len)
{
  int disp[4] = {0,0,0,0};
  disp[dir] = -len;
  return OFN(table)(dims, disp);
}

static void
OFN(sub_range)(const int dims[4], const char *sub, int *i0, int *i1)
{
  int V = or_nsites(dims);
  int nEven = V - V/2;
  *i0 = 0; *i1 = V;                           /* layoutSubset, lib/layout.c:5-19 */
  if(sub && sub[0] == 'e') *i1 = nEven;
  else if(sub && sub[0] == 'o') *i0 = V/2;
}

/* --------------------------------------------------------- site kernels */

/* PeqM3AtimesV3o (lib/vla0.c.lua:193-213): r += M v, M column-major;
 * real parts of v_i first, then imaginary parts, per input colour i */
static inline void
OFN(peq_m_v)(real *r, const real *m, const real *v)
{
  real r0r=r[0], r0i=r[1], r1r=r[2], r1i=r[3], r2r=r[4], r2i=r[5];
  for(int i=0; i<3; i++) {
    real vr = v[2*i], vi = v[2*i+1];
    const real *c = m + 6*i;
    r0r += vr*c[0]; r0i += vr*c[1];
    r1r += vr*c[2]; r1i += vr*c[3];
    r2r += vr*c[4]; r2i += vr*c[5];
    r0r -= vi*c[1]; r0i += vi*c[0];
    r1r -= vi*c[3]; r1i += vi*c[2];
    r2r -= vi*c[5]; r2i += vi*c[4];
  }
  r[0]=r0r; r[1]=r0i; r[2]=r1r; r[3]=r1i; r[4]=r2r; r[5]=r2i;
}

/* ------------------------------------------------------ staggered Dslash */

/* dslash2 / dslash2T (lib/stagDslash.c:259-420, 531-544) with the link
 * slots of createStaggeredLinks (:422-462): slot s uses u[s/2] (even s) or
 * u3[s/2] (odd s) and the SHIFT13 table of that slot. */
void
OFN(or_dslash)(const int dims[4], real *x, real *const u[8], real *const u3[8],
               real mass, const real *y, const char *sub)
{
  int i0, i1;
  OFN(sub_range)(dims, sub, &i0, &i1);
  if(sub && (sub[0] == 'e' || sub[0] == 'o')) mass *= 0;   /* massFac = 0 */
  int nl = u3 ? 16 : 8;
  const int *tab[16];
  const real *lk[16];
  for(int s=0; s<nl; s++) {
    int i = u3 ? s/2 : s;
    int len = (u3 && (s & 1)) ? 3 : 1;
    int disp[4] = {0,0,0,0};
    disp[i/2] = len*(2*(i & 1) - 1);
    tab[s] = OFN(table)(dims, disp);
    lk[s] = u3 ? ((s & 1) ? u3[s/2] : u[s/2]) : u[s];
  }
#pragma omp parallel for schedule(static)
  for(int i=i0; i<i1; i++) {
    real *xi = x + 6L*i;
    /* VeqRtimesV (:8-9): zero when the scale is zero, else scale */
    if(mass == 0) { for(int c=0; c<6; c++) xi[c] = 0; }
    else { for(int c=0; c<6; c++) xi[c] = mass*y[6L*i+c]; }
    for(int s=0; s<nl; s++) {
      int k = tab[s][i];
      if(k >= 0) OFN(peq_m_v)(xi, lk[s] + 18L*i, y + 6L*k);
    }
  }
}

/* ----------------------------------------------------------- vector ops */

double
OFN(or_norm2)(const int dims[4], const real *x, int nelem, const char *sub)
{
  int i0, i1;
  OFN(sub_range)(dims, sub, &i0, &i1);
  double s = 0;
  long a = (long)nelem*i0, b = (long)nelem*i1;
#pragma omp parallel for reduction(+:s) schedule(static)
  for(long i=a; i<b; i++) { double t = x[i]; s += t*t; }
  return s;
}

static double
OFN(vnorm2)(const real *x, long n)
{
  double s = 0;
#pragma omp parallel for reduction(+:s) schedule(static)
  for(long i=0; i<n; i++) { double t = x[i]; s += t*t; }
  return s;
}

static double
OFN(vdot)(const real *x, const real *y, long n)
{
  double s = 0;
#pragma omp parallel for reduction(+:s) schedule(static)
  for(long i=0; i<n; i++) { double a = x[i], b = y[i]; s += a*b; }
  return s;
}

/* X_veq_X_plus_r_times_X (lib/vla.c:767-786): r = v + a w */
static void
OFN(vxpay)(real *r, const real *v, real a, const real *w, long n)
{
#pragma omp parallel for schedule(static)
  for(long i=0; i<n; i++) r[i] = v[i] + a*w[i];
}

/* X_veq_r_times_X (lib/vla.c:732-747), with VeqRtimesV's zero case */
static void
OFN(vscale)(real *r, real a, const real *v, long n)
{
  if(a == 0) {
#pragma omp parallel for schedule(static)
    for(long i=0; i<n; i++) r[i] = 0;
  } else {
#pragma omp parallel for schedule(static)
    for(long i=0; i<n; i++) r[i] = a*v[i];
  }
}

/* X_eq_scale_plus_X (lib/vla.c:788-804): r = a r + v */
static void
OFN(vscale_plus)(real *r, real a, const real *v, long n)
{
#pragma omp parallel for schedule(static)
  for(long i=0; i<n; i++) r[i] = a*r[i] + v[i];
}

/* X_eq_scale_plus_r_times_X (lib/vla.c:806-825): r = a r + b v */
static void
OFN(vscale_plus_b)(real *r, real a, real b, const real *v, long n)
{
#pragma omp parallel for schedule(static)
  for(long i=0; i<n; i++) { real t = b*v[i]; r[i] = a*r[i] + t; }
}

/* ----------------------------------------------- staggered normal operator */

/* dslashp2 (lib/stagDslash.c:546-575): v_o = D_oe x, Ax = m^2 x - D_eo v,
 * <x,Ax> = m^2 |x|^2 + |v_o|^2 */
double
OFN(or_dslashp2)(const int dims[4], real *Ax, const real *x, real *const u[8],
                 real *const u3[8], double mass, real *v)
{
  int V = or_nsites(dims);
  int nEven = V - V/2;
  OFN(or_dslash)(dims, v, u, u3, 0, x, "odd");
  OFN(or_dslash)(dims, Ax, u, u3, 0, v, "even");
  long n = 6L*nEven;
  OFN(vscale)(Ax, -1, Ax, n);
  double m2 = mass*mass;
  OFN(vxpay)(Ax, Ax, (real)m2, x, n);
  double n0 = OFN(vnorm2)(x, n);
  double n1 = OFN(vnorm2)(v + 6L*(V/2), 6L*(V - V/2));
  return m2*n0 + n1;
}

/* cgSolveT (lib/cg.c:43-122) with Aop = dslashp2 and no preconditioner,
 * then solve2's scaling by the mass (lib/stagDslash.c:600-623) */
int
OFN(or_solve2)(const int dims[4], real *x, real *const u[8], real *const u3[8],
               real mass, const real *b, double rsqin, int itnlim, int noscale,
               double *final_rsq)
{
  int V = or_nsites(dims);
  long n = 6L*(V - V/2);
  if(rsqin < 0) rsqin = -rsqin;
  real *r = malloc(sizeof(real)*n);
  real *p = malloc(sizeof(real)*n);
  real *Ap = malloc(sizeof(real)*n);
  real *v = malloc(sizeof(real)*6L*V);
  for(long i=0; i<n; i++) { x[i] = 0; p[i] = 0; r[i] = b[i]; }
  double rsq = OFN(vnorm2)(r, n);
  double bsq = rsq;
  double rsqstop = rsqin*bsq;
  int itn = 0;
  do {
    itn++;
    double beta = 1/rsq;
    OFN(vxpay)(p, p, (real)beta, r, n);
    double pAp = OFN(or_dslashp2)(dims, Ap, p, u, u3, mass, v);
    double alpha = 1/pAp;
    OFN(vxpay)(x, x, (real)alpha, p, n);
    OFN(vxpay)(r, r, -(real)alpha, Ap, n);
    rsq = OFN(vnorm2)(r, n);
  } while(rsq >= rsqstop && itn < itnlim);
  if(final_rsq) *final_rsq = rsq/bsq;
  if(!noscale) OFN(vscale)(x, mass, x, n);
  free(r); free(p); free(Ap); free(v);
  return itn;
}

/* cgmsSolveT (lib/cgms.c:6-179) with Aop = dslashp2, then solveMulti2's
 * shifts m_i^2 - m_0^2 and scaling (lib/stagDslash.c:625-657) */
int
OFN(or_solveMulti2)(const int dims[4], real *const out[], real *const u[8],
                    real *const u3[8], const double masses[], int nshifts,
                    const real *in, double rsqin, int itnlim, int noscale)
{
  int V = or_nsites(dims);
  long n = 6L*(V - V/2);
  if(rsqin < 0) rsqin = -rsqin;
  double mass0 = masses[0];
  double shifts[64], a[64], b[64], s[64], bo[64], z[64], zo[64], zn[64];
  for(int i=0; i<nshifts; i++) shifts[i] = masses[i]*masses[i] - masses[0]*masses[0];
  double insq = OFN(vnorm2)(in, n);
  int iteration = 0;
  if(insq == 0) {
    for(int i=0; i<nshifts; i++) for(long k=0; k<n; k++) out[i][k] = 0;
  } else {
    real *r = malloc(sizeof(real)*n);
    real *Ap = malloc(sizeof(real)*n);
    real *v = malloc(sizeof(real)*6L*V);
    real *ps[64];
    for(int i=0; i<nshifts; i++) ps[i] = malloc(sizeof(real)*n);
    for(long k=0; k<n; k++) r[k] = in[k];
    for(int i=0; i<nshifts; i++) {
      for(long k=0; k<n; k++) { out[i][k] = 0; ps[i][k] = r[k]; }
      zo[i] = z[i] = 1;
      bo[i] = -1;
      a[i] = 0;
      s[i] = 1;
    }
    double rsqstop = rsqin*insq;
    double rsq = insq, oldrsq, pkp;
    while(1) {
      oldrsq = rsq;
      pkp = OFN(or_dslashp2)(dims, Ap, ps[0], u, u3, mass0, v);
      iteration++;
      pkp *= s[0]*s[0];
      if(pkp <= 0) break;
      b[0] = rsq/pkp;
      zn[0] = 1;
      for(int i=1; i<nshifts; i++) {
        double c1;
        zn[i] = z[i]*zo[i]*bo[0];
        c1 = b[0]*a[0]*(zo[i] - z[i]);
        c1 += zo[i]*bo[0]*(1 + shifts[i]*b[0]);
        if(c1 != 0.0) zn[i] /= c1;
        else zn[i] = 0;
        if(z[i] != 0.0) b[i] = b[0]*zn[i]/z[i];
        else zn[i] = b[i] = 0;
      }
      for(int i=0; i<nshifts; i++) {
        double t = b[i]*s[i];
        OFN(vxpay)(out[i], out[i], (real)t, ps[i], n);
      }
      {
        double t = b[0]*s[0];
        OFN(vxpay)(r, r, -(real)t, Ap, n);
      }
      rsq = OFN(vnorm2)(r, n);
      if((iteration >= itnlim) || (rsqstop <= 0 || rsq < rsqstop)) break;
      a[0] = rsq/oldrsq;
      for(int i=1; i<nshifts; i++) {
        double c2 = z[i]*b[0];
        if(c2 != 0.0) a[i] = a[0]*zn[i]*b[i]/c2;
        else a[i] = 0;
      }
      OFN(vscale_plus)(ps[0], (real)a[0], r, n);
      for(int i=1; i<nshifts; i++) {
        if(s[i] != 0) OFN(vscale_plus_b)(ps[i], (real)a[i], (real)zn[i], r, n);
      }
      for(int i=0; i<nshifts; i++) {
        bo[i] = b[i];
        zo[i] = z[i];
        z[i] = zn[i];
      }
    }
    for(int i=0; i<nshifts; i++) free(ps[i]);
    free(r); free(Ap); free(v);
  }
  if(!noscale) {
    for(int i=0; i<nshifts; i++) OFN(vscale)(out[i], (real)masses[i], out[i], n);
  }
  return iteration;
}

/* --------------------------------------------------- 3x3 matrix fields */

/* PeqMtimesX with ldv columns (lib/vla.c:929-964): r(j,i) += M(j,l) V(l,i) */
static inline void
OFN(mpeq_m_x)(real *r, const real *m, const real *v, int ldv)
{
  for(int i=0; i<ldv; i++) {
    for(int l=0; l<3; l++) {
      real vr = v[(3*i+l)*2], vi = v[(3*i+l)*2+1];
      for(int j=0; j<3; j++) {
        const real *mj = m + (j + 3*l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] += mj[0]*vr;
        rj[1] += mj[0]*vi;
      }
      for(int j=0; j<3; j++) {
        const real *mj = m + (j + 3*l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] -= mj[1]*vi;
        rj[1] += mj[1]*vr;
      }
    }
  }
}

/* PeqMtimesXa (lib/vla.c:1002-1038): r(j,i) += M(j,l) conj(V(i,l)) */
static inline void
OFN(mpeq_m_xa)(real *r, const real *m, const real *v)
{
  for(int i=0; i<3; i++) {
    for(int l=0; l<3; l++) {
      real vr = v[(3*l+i)*2], vi = v[(3*l+i)*2+1];
      for(int j=0; j<3; j++) {
        const real *mj = m + (j + 3*l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] += mj[0]*vr;
        rj[1] -= mj[0]*vi;
      }
      for(int j=0; j<3; j++) {
        const real *mj = m + (j + 3*l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] += mj[1]*vi;
        rj[1] += mj[1]*vr;
      }
    }
  }
}

/* PeqMatimesX (lib/vla.c:1040-1078): r(j,i) += conj(M(l,j)) V(l,i) */
static inline void
OFN(mpeq_ma_x)(real *r, const real *m, const real *v)
{
  for(int i=0; i<3; i++) {
    for(int l=0; l<3; l++) {
      real vr = v[(3*i+l)*2], vi = v[(3*i+l)*2+1];
      for(int j=0; j<3; j++) {
        const real *mj = m + (j*3 + l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] += mj[0]*vr;
        rj[1] += mj[0]*vi;
      }
      for(int j=0; j<3; j++) {
        const real *mj = m + (j*3 + l)*2;
        real *rj = r + (3*i+j)*2;
        rj[0] += mj[1]*vi;
        rj[1] -= mj[1]*vr;
      }
    }
  }
}

/* transporter with td>0 (lib/transporter.c:75-92, X_peq_M_times_xXp
 * lib/vla.c:1279-1307): dest(x) += u(x) src(nbr(x)) */
void
OFN(or_transport)(const int dims[4], real *dest, const real *u, const real *src,
                  int nelem, int dir, int fwd)
{
  int V = or_nsites(dims);
  const int *t = OFN(shift_table)(dims, dir, fwd ? 1 : -1);
  int ldv = nelem/6;
#pragma omp parallel for schedule(static)
  for(int i=0; i<V; i++) {
    int k = t[i];
    if(k >= 0) OFN(mpeq_m_x)(dest + (long)nelem*i, u + 18L*i, src + (long)nelem*k, ldv);
  }
}

/* X_eq_xXp (lib/vla.c:294-319): dest(x) = src(nbr(x)) */
static void
OFN(mshift)(const int dims[4], real *dest, const real *src, int nelem, int dir, int len)
{
  int V = or_nsites(dims);
  const int *t = OFN(shift_table)(dims, dir, len);
#pragma omp parallel for schedule(static)
  for(int i=0; i<V; i++) {
    int k = t[i];
    if(k >= 0) for(int e=0; e<nelem; e++) dest[(long)nelem*i+e] = src[(long)nelem*k+e];
  }
}

void
OFN(or_shift)(const int dims[4], real *x, const real *y, int nelem, int dir, int len)
{
  int d = (dir > 0 ? dir : -dir) - 1;
  OFN(mshift)(dims, x, y, nelem, d, dir > 0 ? len : -len);
}

/* M_eq_M_times_M / M_eq_M_times_Ma / M_eq_Ma_times_M (lib/gauge.c:13-18) */
static void
OFN(m_eq)(const int dims[4], real *r, const real *m, const real *v, int kind)
{
  int V = or_nsites(dims);
#pragma omp parallel for schedule(static)
  for(int i=0; i<V; i++) {
    real *ri = r + 18L*i;
    for(int e=0; e<18; e++) ri[e] = 0;
    if(kind == 0) OFN(mpeq_m_x)(ri, m + 18L*i, v + 18L*i, 3);
    else if(kind == 1) OFN(mpeq_m_xa)(ri, m + 18L*i, v + 18L*i);
    else OFN(mpeq_ma_x)(ri, m + 18L*i, v + 18L*i);
  }
}

/* X_vpeq_r_times_X (lib/vla.c:749-765): r += a v */
static void
OFN(mpeq_r)(real *r, real a, const real *v, long n)
{
#pragma omp parallel for schedule(static)
  for(long i=0; i<n; i++) r[i] = r[i] + a*v[i];
}

/* Xadj (lib/vla.c:827-854): in-place adjoint */
static void
OFN(madj)(real *r, long nsites)
{
#pragma omp parallel for schedule(static)
  for(long s=0; s<nsites; s++) {
    real *m = r + 18*s;
    for(int a=0; a<3; a++) {
      for(int b=0; b<a; b++) {
        int k1 = (a*3+b)*2, k2 = (b*3+a)*2;
        real xr = m[k1], xi = m[k1+1], yr = m[k2], yi = m[k2+1];
        m[k2] = xr; m[k2+1] = -xi;
        m[k1] = yr; m[k1+1] = -yi;
      }
      int k = a*4*2;
      m[k+1] = -m[k+1];
    }
  }
}

void
OFN(or_doublestore)(const int dims[4], real *ua, const real *u, int dir, int len)
{
  OFN(mshift)(dims, ua, u, 18, dir, len);
  OFN(madj)(ua, or_nsites(dims));
}

void
OFN(or_negadj_back)(const int dims[4], real *ub, const real *u, int dir, int len)
{
  int V = or_nsites(dims);
  OFN(mshift)(dims, ub, u, 18, dir, -len);
#pragma omp parallel for schedule(static)
  for(long s=0; s<V; s++) {                 /* adjM of testdslash.c:59-85 */
    real *m = ub + 18*s;
    for(int ic=0; ic<3; ic++) {
      for(int jc=ic; jc<3; jc++) {
        real a0 = m[(ic*3+jc)*2], a1 = m[(ic*3+jc)*2+1];
        real b0 = m[(jc*3+ic)*2], b1 = m[(jc*3+ic)*2+1];
        m[(ic*3+jc)*2] = -b0; m[(ic*3+jc)*2+1] = b1;
        m[(jc*3+ic)*2] = -a0; m[(jc*3+ic)*2+1] = a1;
      }
    }
  }
}

/* makeU / makeUsite (lib/vla.c:1635-1665): Gram-Schmidt of the columns */
void
OFN(or_makeU)(real *mm, int nsites)
{
#pragma omp parallel for schedule(static)
  for(int s=0; s<nsites; s++) {
    real *m = mm + 18L*s;
    for(int i=0; i<3; i++) {
      real *mi = m + 6*i;
      real n = 0;
      for(int k=0; k<6; k++) n += mi[k]*mi[k];
      real ni = 1/sqrt(n);
      for(int k=0; k<6; k++) mi[k] *= ni;
      for(int j=0; j<i; j++) {
        real *mj = m + 6*j;
        real dr = mj[0]*mi[0], di = mj[0]*mi[1];
        dr += mj[1]*mi[1]; di -= mj[1]*mi[0];
        for(int k=2; k<6; k+=2) {
          dr += mj[k]*mi[k]; di += mj[k]*mi[k+1];
          dr += mj[k+1]*mi[k+1]; di -= mj[k+1]*mi[k];
        }
        for(int k=0; k<6; k+=2) {
          real x0 = mi[k], x1 = mi[k+1];
          x0 -= dr*mj[k]; x1 -= dr*mj[k+1];
          x0 += di*mj[k+1]; x1 -= di*mj[k];
          mi[k] = x0; mi[k+1] = x1;
        }
        n = 0;
        for(int k=0; k<6; k++) n += mi[k]*mi[k];
        ni = 1/sqrt(n);
        for(int k=0; k<6; k++) mi[k] *= ni;
      }
    }
  }
}

/* gaugePlaq (lib/gauge.c:114-183) */
void
OFN(or_plaq)(const int dims[4], double plaqs[6], real *const u[4])
{
  int V = or_nsites(dims);
  real *A = malloc(sizeof(real)*18L*V);
  real *B = malloc(sizeof(real)*18L*V);
  int l = 0;
  for(int i=0; i<4; i++) {
    for(int j=0; j<i; j++) {
      /* f[j][i] = u_i(x) u_j(x+i), f[i-1][j] = u_j(x) u_i(x+j) */
      memset(A, 0, sizeof(real)*18L*V);
      memset(B, 0, sizeof(real)*18L*V);
      OFN(or_transport)(dims, A, u[i], u[j], 18, i, 1);
      OFN(or_transport)(dims, B, u[j], u[i], 18, j, 1);
      plaqs[l++] = OFN(vdot)(A, B, 18L*V)/(3.0*V);
    }
  }
  free(A); free(B);
}

/* genStaple (lib/gauge.c:188-262) */
static void
OFN(gen_staple)(const int dims[4], real *staple, int mu, int nu, const real *link,
                double coef, real *const gauge[4], real *const fl[4],
                const real *ts1, real *tmat1, real *tmat2)
{
  int V = or_nsites(dims);
  long n = 18L*V;
  memset(tmat1, 0, sizeof(real)*n);
  OFN(or_transport)(dims, tmat1, gauge[nu], link, 18, nu, 1);
  if(staple) {
    OFN(m_eq)(dims, staple, tmat1, ts1, 1);
  } else {
    OFN(m_eq)(dims, tmat2, tmat1, ts1, 1);
    OFN(mpeq_r)(fl[mu], (real)coef, tmat2, n);
  }
  OFN(m_eq)(dims, tmat1, gauge[nu], link, 2);
  OFN(m_eq)(dims, tmat2, tmat1, ts1, 0);
  OFN(mshift)(dims, tmat1, tmat2, 18, nu, -1);
  if(staple) {
    OFN(mpeq_r)(staple, 1, tmat1, n);
    OFN(mpeq_r)(fl[mu], (real)coef, staple, n);
  } else {
    OFN(mpeq_r)(fl[mu], (real)coef, tmat1, n);
  }
}

/* smearFat7 (lib/gauge.c:264-416) */
void
OFN(or_smearFat7)(const int dims[4], real *const fl[4], real *const ll[4],
                  const or_fat7_coeffs *coef, real *const u[4], real *const uLong[4])
{
  int V = or_nsites(dims);
  long n = 18L*V;
  double coef1 = coef->one_link;
  double coef3 = coef->three_staple;
  double coef5 = coef->five_staple;
  double coef7 = coef->seven_staple;
  double coefL = coef->lepage;
  coef1 -= 6*coefL;
  int have5 = coef5 || coef7 || coefL;
  int have3 = coef3 || have5;
  real *staple = NULL, *tempmat1 = NULL, *t1 = NULL, *t2 = NULL, *tsg[4][4];
  if(have3 || ll) {
    staple = malloc(sizeof(real)*n);
    tempmat1 = malloc(sizeof(real)*n);
  }
  if(have3) {
    t1 = malloc(sizeof(real)*n);
    t2 = malloc(sizeof(real)*n);
    for(int dir=0; dir<4; dir++) for(int nu=0; nu<4; nu++) {
      tsg[dir][nu] = NULL;
      if(dir != nu) {
        tsg[dir][nu] = malloc(sizeof(real)*n);
        OFN(mshift)(dims, tsg[dir][nu], u[dir], 18, nu, 1);
      }
    }
  }
  for(int dir=0; dir<4; dir++) {
    OFN(vscale)(fl[dir], (real)coef1, u[dir], n);
    if(have3) {
      for(int nu=0; nu<4; nu++) {
        if(nu == dir) continue;
        OFN(gen_staple)(dims, staple, dir, nu, u[dir], coef3, u, fl,
                        tsg[nu][dir], t1, t2);
        if(coefL) {
          OFN(gen_staple)(dims, NULL, dir, nu, staple, coefL, u, fl,
                          tsg[nu][dir], t1, t2);
        }
        if(coef5 || coef7) {
          for(int rho=0; rho<4; rho++) {
            if(rho == dir || rho == nu) continue;
            OFN(gen_staple)(dims, tempmat1, dir, rho, staple, coef5, u, fl,
                            tsg[rho][dir], t1, t2);
            if(coef7) {
              for(int sig=0; sig<4; sig++) {
                if(sig != dir && sig != nu && sig != rho) {
                  OFN(gen_staple)(dims, NULL, dir, sig, tempmat1, coef7, u, fl,
                                  tsg[sig][dir], t1, t2);
                }
              }
            }
          }
        }
      }
    }
  }
  if(ll) {
    double naik = coef->naik;
    for(int dir=0; dir<4; dir++) {
      memset(tempmat1, 0, sizeof(real)*n);
      OFN(or_transport)(dims, tempmat1, uLong[dir], uLong[dir], 18, dir, 1);
      memset(ll[dir], 0, sizeof(real)*n);
      OFN(or_transport)(dims, ll[dir], uLong[dir], tempmat1, 18, dir, 1);
      OFN(vscale)(ll[dir], (real)naik, ll[dir], n);
    }
  }
  free(staple); free(tempmat1); free(t1); free(t2);
  if(have3) for(int dir=0; dir<4; dir++) for(int nu=0; nu<4; nu++) free(tsg[dir][nu]);
}

/* --------------------------------------------------------- Wilson Dslash */

/* sprojMat / sreconMat of lib/Gamma.lua:49-73 for d=0..4, s=0 (+) and
 * s=1 (-), as complex 2x4 and 4x2 row-major matrices */
static double OFN(wP)[5][2][16], OFN(wR)[5][2][16];
static int OFN(winit) = 0;

static void
OFN(wilson_init)(void)
{
  if(OFN(winit)) return;
  for(int d=0; d<5; d++) {
    double g[32];
    or_gamma(d, g);
    for(int s=0; s<2; s++) {
      double sg = 1 - 2*s, t[32];
      for(int k=0; k<16; k++) {
        int a = k/4, b = k%4;
        t[2*k] = (a == b ? 1 : 0) + sg*g[2*k];
        t[2*k+1] = sg*g[2*k+1];
        if(d == 4) { t[2*k] *= 0.5; t[2*k+1] *= 0.5; }
      }
      int r0 = (d == 4 && s == 1) ? 2 : 0;
      for(int i=0; i<2; i++) for(int a=0; a<4; a++) {
        OFN(wP)[d][s][(i*4+a)*2] = t[((r0+i)*4+a)*2];
        OFN(wP)[d][s][(i*4+a)*2+1] = t[((r0+i)*4+a)*2+1];
      }
      /* R = f * t * P^dagger, f = 1 for d=4 else 1/2 */
      double f = (d == 4) ? 1 : 0.5;
      for(int a=0; a<4; a++) for(int k=0; k<2; k++) {
        double sr = 0, si = 0;
        for(int c=0; c<4; c++) {
          double tr = t[(a*4+c)*2], ti = t[(a*4+c)*2+1];
          double pr = OFN(wP)[d][s][(k*4+c)*2], pi = -OFN(wP)[d][s][(k*4+c)*2+1];
          sr += tr*pr - ti*pi;
          si += tr*pi + ti*pr;
        }
        OFN(wR)[d][s][(a*2+k)*2] = f*sr;
        OFN(wR)[d][s][(a*2+k)*2+1] = f*si;
      }
    }
  }
  OFN(winit) = 1;
}

/* MeqSproj<d><s>M3timesD3 (lib/vlaw0.c.lua:580-601): per projected spin k,
 * h_k = P_k f (one or two phase terms), t_k = U h_k, r -= R(:,k) t_k */
static inline void
OFN(wmeq_sproj)(real *r, const real *m, const real *f, int d, int s)
{
  const double *P = OFN(wP)[d][s], *R = OFN(wR)[d][s];
  for(int k=0; k<2; k++) {
    real t[6] = {0,0,0,0,0,0};
    for(int j=0; j<3; j++) {
      /* h_kj: first nonzero term, plus the second one if present */
      real hr = 0, hi = 0;
      int first = 1;
      for(int a=0; a<4; a++) {
        double pr = P[(k*4+a)*2], pi = P[(k*4+a)*2+1];
        if(pr == 0 && pi == 0) continue;
        real fr = f[(3*a+j)*2], fi = f[(3*a+j)*2+1];
        real yr = (real)(pr*fr - pi*fi), yi = (real)(pr*fi + pi*fr);
        if(first) { hr = yr; hi = yi; first = 0; }
        else { hr = hr + yr; hi = hi + yi; }
      }
      const real *c = m + 6*j;
      t[0] += hr*c[0]; t[1] += hr*c[1];
      t[2] += hr*c[2]; t[3] += hr*c[3];
      t[4] += hr*c[4]; t[5] += hr*c[5];
      t[0] -= hi*c[1]; t[1] += hi*c[0];
      t[2] -= hi*c[3]; t[3] += hi*c[2];
      t[4] -= hi*c[5]; t[5] += hi*c[4];
    }
    for(int a=0; a<4; a++) {
      double qr = -R[(a*2+k)*2], qi = -R[(a*2+k)*2+1];
      if(qr == 0 && qi == 0) continue;
      for(int j=0; j<3; j++) {
        real tr = t[2*j], ti = t[2*j+1];
        real *ra = r + (3*a+j)*2;
        ra[0] = ra[0] + (real)(qr*tr - qi*ti);
        ra[1] = ra[1] + (real)(qr*ti + qi*tr);
      }
    }
  }
}

void
OFN(or_wilson_dslash)(const int dims[4], real *x, real *const u[8], real mass,
                      int sign, const real *y, const char *sub)
{
  (void)sign;   /* ignored, as in lib/wilsonDslash.c:272-285 */
  OFN(wilson_init)();
  int i0, i1;
  OFN(sub_range)(dims, sub, &i0, &i1);
  real massFac = (sub && (sub[0] == 'e' || sub[0] == 'o')) ? 0 : 1;
  mass = massFac*(4 + mass);
  const int *tab[8];
  for(int s=0; s<8; s++) {
    int disp[4] = {0,0,0,0};
    disp[s/2] = 2*(s & 1) - 1;
    tab[s] = OFN(table)(dims, disp);
  }
#pragma omp parallel for schedule(static)
  for(int i=i0; i<i1; i++) {
    real *xi = x + 24L*i;
    if(mass == 0) { for(int c=0; c<24; c++) xi[c] = 0; }
    else { for(int c=0; c<24; c++) xi[c] = mass*y[24L*i+c]; }
    for(int sl=0; sl<8; sl++) {
      int k = tab[sl][i];
      /* slot 2mu: (1-gamma_mu) from x+mu; slot 2mu+1: (1+gamma_mu) from x-mu */
      if(k >= 0) OFN(wmeq_sproj)(xi, u[sl] + 18L*i, y + 24L*k, sl/2, (sl & 1) ? 0 : 1);
    }
  }
}

/* wilsonSolve = cgSolveT with the Wilson dslashp2 (lib/wilsonDslash.c:287-364)
 * and norms over the full 24 reals per site */
int
OFN(or_wilson_solve)(const int dims[4], real *x, real *const u[8], real mass,
                     const real *b, double rsqin, int itnlim, int noscale)
{
  int V = or_nsites(dims);
  long n = 24L*(V - V/2);
  if(rsqin < 0) rsqin = -rsqin;
  real *r = malloc(sizeof(real)*n);
  real *p = malloc(sizeof(real)*n);
  real *Ap = malloc(sizeof(real)*n);
  real *v = malloc(sizeof(real)*24L*V);
  for(long i=0; i<n; i++) { x[i] = 0; p[i] = 0; r[i] = b[i]; }
  double rsq = OFN(vnorm2)(r, n);
  double rsqstop = rsqin*rsq;
  double m2 = (double)mass*mass;
  int itn = 0;
  do {
    itn++;
    double beta = 1/rsq;
    OFN(vxpay)(p, p, (real)beta, r, n);
    OFN(or_wilson_dslash)(dims, v, u, 0, 1, p, "odd");
    OFN(or_wilson_dslash)(dims, Ap, u, 0, 1, v, "even");
    OFN(vscale)(Ap, -1, Ap, n);
    OFN(vxpay)(Ap, Ap, (real)m2, p, n);
    double pAp = m2*OFN(vnorm2)(p, n) + OFN(vnorm2)(v + 24L*(V/2), 24L*(V - V/2));
    double alpha = 1/pAp;
    OFN(vxpay)(x, x, (real)alpha, p, n);
    OFN(vxpay)(r, r, -(real)alpha, Ap, n);
    rsq = OFN(vnorm2)(r, n);
  } while(rsq >= rsqstop && itn < itnlim);
  if(!noscale) OFN(vscale)(x, mass, x, n);
  free(r); free(p); free(Ap); free(v);
  return itn;
}

/* gamma5 on a spinor field of n sites */
static void
OFN(g5)(real *y, const real *x, long nsites)
{
  double g[32];
  or_gamma(4, g);
#pragma omp parallel for schedule(static)
  for(long s=0; s<nsites; s++) {
    real t[24];
    for(int a=0; a<4; a++) for(int c=0; c<3; c++) {
      double sr = 0, si = 0;
      for(int b=0; b<4; b++) {
        double gr = g[(a*4+b)*2], gi = g[(a*4+b)*2+1];
        double xr = x[24*s+(3*b+c)*2], xi = x[24*s+(3*b+c)*2+1];
        sr += gr*xr - gi*xi;
        si += gr*xi + gi*xr;
      }
      t[(3*a+c)*2] = (real)sr; t[(3*a+c)*2+1] = (real)si;
    }
    for(int k=0; k<24; k++) y[24*s+k] = t[k];
  }
}

void
OFN(or_wilson_schur)(const int dims[4], real *Sy, real *const u[8], double mass,
                     const real *y, int dag, real *tmp)
{
  int V = or_nsites(dims);
  long ne = V - V/2;
  long n = 24L*ne;
  double a = 4 + mass;
  real *src = (real *)y;
  real *g = NULL;
  if(dag) { g = malloc(sizeof(real)*n); OFN(g5)(g, y, ne); src = g; }
  OFN(or_wilson_dslash)(dims, tmp, u, 0, 1, src, "odd");
  OFN(or_wilson_dslash)(dims, Sy, u, 0, 1, tmp, "even");
#pragma omp parallel for schedule(static)
  for(long i=0; i<n; i++) Sy[i] = (real)(a*src[i] - Sy[i]/a);
  if(dag) { OFN(g5)(Sy, Sy, ne); free(g); }
}

/* CGNR on the Schur complement */
int
OFN(or_wilson_cgnr)(const int dims[4], real *x, real *const u[8], double mass,
                    const real *b, double rsqin, int maxits, double *final_rsq)
{
  int V = or_nsites(dims);
  long n = 24L*(V - V/2);
  real *r = malloc(sizeof(real)*n), *p = malloc(sizeof(real)*n);
  real *Sp = malloc(sizeof(real)*n), *Ap = malloc(sizeof(real)*n);
  real *tmp = malloc(sizeof(real)*24L*V);
  OFN(or_wilson_schur)(dims, r, u, mass, b, 1, tmp);
  for(long i=0; i<n; i++) { x[i] = 0; p[i] = r[i]; }
  double rsq = OFN(vnorm2)(r, n);
  double stop = rsqin*rsq, r0 = rsq;
  int itn = 0;
  while(rsq >= stop && itn < maxits) {
    itn++;
    OFN(or_wilson_schur)(dims, Sp, u, mass, p, 0, tmp);
    double pAp = OFN(vnorm2)(Sp, n);
    OFN(or_wilson_schur)(dims, Ap, u, mass, Sp, 1, tmp);
    double alpha = rsq/pAp;
    OFN(vxpay)(x, x, (real)alpha, p, n);
    OFN(vxpay)(r, r, -(real)alpha, Ap, n);
    double rsqn = OFN(vnorm2)(r, n);
    double beta = rsqn/rsq;
    rsq = rsqn;
    OFN(vscale_plus)(p, (real)beta, r, n);
  }
  if(final_rsq) *final_rsq = rsq/r0;
  free(r); free(p); free(Sp); free(Ap); free(tmp);
  return itn;
}

#undef OFN
#undef OCAT
#undef OCAT_
