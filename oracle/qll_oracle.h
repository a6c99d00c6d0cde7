/*
 * qll_oracle.h -- CPU ORACLE for the QLL solver hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * library's algorithms (jcosborn/qll, files cited per function below), used
 * as the checker for the GPU library.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product library
 * (qll_gb300/libqll_gb300.so) never links or calls it.
 *
 * Parity status: the reference cannot be compiled here (it needs sources
 * generated by Lua scripts -- lib/vla0.c, lib/vlaw0.c, include/vec_ops_c.h --
 * and the external QMP message-passing library), and it ships no golden
 * output vectors.  This restatement is pinned to the known-answer tests the
 * reference's own test programs hold (stress.c:196-234 analytic transport
 * norm and bitwise repeatability; fieldtest.c:183-191 transport followed by
 * back-transport with double-stored adjoint links is the identity) and to
 * analytic properties (anti-Hermiticity, gauge covariance, unit-link
 * plaquette, free-field spectrum).  No reference output vector pins it.
 *
 * Layout: the reference's VLEN=1 (-DC1) site layout.  A field with nelem
 * reals per site is an array [nSites][nelem]; sites are numbered by
 * layoutIndex (lib/layout.c:120-142): even-parity sites first, in
 * lexicographic order with x0 fastest, then odd-parity sites.  3x3 complex
 * matrices are column-major: element (row j, column i) sits at reals
 * (3*i+j)*2 + {0: re, 1: im} (lib/vla.c:9-11).
 *
 * Every function exists as ..D (double fields) and ..F (float fields), like
 * the reference's P() macro (include/vla.h:4-8).  Global sums and the CG /
 * multishift recurrences are double in both, as in the reference.
 */
#ifndef QLL_ORACLE_H
#define QLL_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double one_link, three_staple, five_staple, seven_staple, lepage, naik;
} or_fat7_coeffs;   /* same member order as Fat7Coeffs, include/qll.h:7-14 */

/* geometry: dims[4], all even */
int  or_nsites(const int dims[4]);
int  or_site_index(const int dims[4], const int x[4]);        /* lib/layout.c:120-142 */
void or_site_coord(const int dims[4], int idx, int x[4]);     /* lib/layout.c:144-205 */
/* pidx of makeShiftSub for one rank, VLEN=1: dest i gathers from
 * coord(i) - disp; -1 where i is outside the parity (0 even, 1 odd, -1 all).
 * lib/shifts.c:312-358 (map) and :516-736 (makeShiftMultiSub). */
void or_shift_table(const int dims[4], const int disp[4], int parity, int *pidx);
/* the neighbour table of staggered slot s (0..15) of createStaggeredLinks
 * (lib/stagDslash.c:422-462 with getStaggeredSI :721-733, disp :829-832) */
void or_stag_slot_table(const int dims[4], int slot, int naik, int parity, int *pidx);

/* gamma matrices of lib/Gamma.lua:5-26 (DeGrand-Rossi): g[d] for d=0..4
 * (4 = gamma5), 4x4 row-major complex as re/im pairs */
void or_gamma(int d, double g[32]);

#define OR_DECLARE(S, real)                                                   \
  /* x = mass*massFac*y + sum_s u_s(x) y(x+d_s)  (lib/stagDslash.c:259-420,  \
   * 531-544); sub 'e','o' or all; u3 may be NULL (no Naik) */               \
  void or_dslash##S(const int dims[4], real *x, real *const u[8],            \
                    real *const u3[8], real mass, const real *y,             \
                    const char *sub);                                        \
  /* Ax = m^2 x - D_eo D_oe x on even sites, returns <x,Ax>                  \
   * (dslashp2, lib/stagDslash.c:546-575); v: odd scratch, 6*nSites */       \
  double or_dslashp2##S(const int dims[4], real *Ax, const real *x,          \
                        real *const u[8], real *const u3[8], double mass,     \
                        real *v);                                            \
  /* solve2 / cgSolve (lib/stagDslash.c:600-623, lib/cg.c:43-136) */         \
  int or_solve2##S(const int dims[4], real *x, real *const u[8],             \
                   real *const u3[8], real mass, const real *y, double rsq,  \
                   int maxits, int noscale, double *final_rsq);              \
  /* solveMulti2 / cgmsSolve (lib/stagDslash.c:625-657, lib/cgms.c:6-195) */ \
  int or_solveMulti2##S(const int dims[4], real *const x[], real *const u[8],\
                        real *const u3[8], const double masses[],            \
                        int nmasses, const real *y, double rsq, int maxits,  \
                        int noscale);                                        \
  /* smearFat7 (lib/gauge.c:188-416); fl/ll are outputs (ll may be NULL) */  \
  void or_smearFat7##S(const int dims[4], real *const fl[4],                 \
                       real *const ll[4], const or_fat7_coeffs *coef,        \
                       real *const u[4], real *const ulong_[4]);             \
  /* gaugeDoublestore: ua = (shift_{dir,len} u)^dagger (lib/gauge.c:34-63) */\
  void or_doublestore##S(const int dims[4], real *ua, const real *u,         \
                         int dir, int len);                                  \
  /* backward staggered link -(shift_{dir,-len} u)^dagger, the caller-built  \
   * negative adjoint of testdslash.c:59-85,277-278 */                       \
  void or_negadj_back##S(const int dims[4], real *ub, const real *u,         \
                         int dir, int len);                                  \
  /* gaugePlaq (lib/gauge.c:114-183): 6 plaquettes, normalised by nc*V */    \
  void or_plaq##S(const int dims[4], double plaqs[6], real *const u[4]);     \
  /* makeU: Gram-Schmidt of the columns (lib/vla.c:1635-1665) */             \
  void or_makeU##S(real *m, int nsites);                                     \
  /* shift (lib/stagDslash.c:91-101): x = y shifted by dir (+-1..4), len */  \
  void or_shift##S(const int dims[4], real *x, const real *y, int nelem,     \
                   int dir, int len);                                        \
  /* transporterDo with td>0 and links: dest(x) += u(x) src(x+-dir)          \
   * (lib/transporter.c:32-193, lib/vla.c:929-1230); nelem 6 or 18;          \
   * fwd=1 gathers from x+dir, fwd=0 from x-dir */                           \
  void or_transport##S(const int dims[4], real *dest, const real *u,         \
                       const real *src, int nelem, int dir, int fwd);        \
  /* Wilson: x = massFac*(4+m) y - sum_mu [R P U y(x+-mu)]                   \
   * (lib/wilsonDslash.c:21-179,272-285; lib/vlaw0.c.lua:545-652) */         \
  void or_wilson_dslash##S(const int dims[4], real *x, real *const u[8],     \
                           real mass, int sign, const real *y,               \
                           const char *sub);                                 \
  /* wilsonSolve (lib/wilsonDslash.c:287-364) with the norms over all 24     \
   * reals of a site (the reference sums a 6-real window, :308,310, which    \
   * reads memory that was never written) */                                 \
  int or_wilson_solve##S(const int dims[4], real *x, real *const u[8],       \
                         real mass, const real *y, double rsq, int maxits,   \
                         int noscale);                                       \
  /* Schur complement of the even-odd Wilson matrix on even sites,           \
   * S y = a y - W_e(W_o y)/a with a = 4+m and W the massless e/o Dslash;    \
   * dag=1 applies S^dagger = g5 S g5 */                                     \
  void or_wilson_schur##S(const int dims[4], real *Sy, real *const u[8],     \
                          double mass, const real *y, int dag, real *tmp);   \
  /* CG on S^dagger S x = S^dagger b (CGNR), FP64 recurrences; stops when    \
   * |S^dag(b - S x)|^2 < rsq |S^dag b|^2; returns iterations */             \
  int or_wilson_cgnr##S(const int dims[4], real *x, real *const u[8],        \
                        double mass, const real *b, double rsq, int maxits,  \
                        double *final_rsq);                                  \
  /* vector helpers over the site range of sub */                            \
  double or_norm2##S(const int dims[4], const real *x, int nelem,            \
                     const char *sub);

OR_DECLARE(D, double)
OR_DECLARE(F, float)

/* stress.c:196-234 known-answer test on the oracle's transporter: returns
 * the ratio that stress.c requires to be 1 within 1e-10 (first pass) */
double or_stress_kat(const int dims[4], int nrep, int npass, int *bitwise_ok);
/* fieldtest.c:133-191 known-answer test: |v3 - v1|^2 after forward
 * transport and back-transport with the double-stored adjoint */
double or_fieldtest_kat(const int dims[4]);

/* number of OpenMP threads the oracle uses */
int or_num_threads(void);
void or_set_num_threads(int n);
int or_gen_gauge(const int dims[4], unsigned long long seed, double eps, int ks, double *u[4]);
int or_gen_source(const int dims[4], unsigned long long seed, int nelem, const char *sub, double *v);

#ifdef __cplusplus
}
#endif
#endif
