/*
 * gauge.c -- link preparation on the GPU: fat7/asqtad smearing
 * (lib/gauge.c:188-416), the plaquette (:114-183), double-stored links
 * (:34-63), the Field API (lib/field.c) and the generic transporter and
 * shift (lib/transporter.c, lib/stagDslash.c:25-101), plus the native entry
 * that builds a resident asqtad operator from thin links without a host
 * round trip of the fat and long links.
 *
 * smearFat7 runs the reference's sequence of field operations (genStaple
 * and the Naik products) as device kernels over full-lattice matrix fields
 * in the precision of the call (FP64 for D, FP32 for F).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"
#include "vla.h"

void qllg_stag_set_single_store(qllg_stag *S);

int qllg_geom_from_layout(qllg_geom *g, const Layout *l);
int qllg_stag_attach_links(qllg_stag *S, int prec, void *links);
qllg_stag *qllg_stag_alloc(const int dims[4], int nslots, int prec);

/* ------------------------------------------------------------ fat7 */

typedef struct {
  int prec;
  qllg_geom g;
  size_t n;      /* reals of one field */
  size_t bytes;
} fctx;

static void *
fnew(const fctx *c)
{
  return qllg_dmalloc(c->bytes);
}

/* genStaple (lib/gauge.c:188-262):
 *   upper  U_nu(x) link(x+nu) U_nu(x+mu)^dagger
 *   lower  shift_{-nu}[ U_nu^dagger(x) link(x) U_nu(x+mu) ]
 * staple (if given) = upper + lower and fl_mu += coef*staple; without a
 * staple both pieces go straight into fl_mu. */
static int
gen_staple(const fctx *c, void *staple, int mu, int nu, const void *link, double coef,
           void *const gauge[4], void *const fl[4], const void *ts1, void *t1, void *t2)
{
  int p = c->prec;
  /* tmat1 = U_nu(x) link(x+nu), the tf[nu] transport with td=2 */
  if(qllg_k_mat_mul(p, t1, gauge[nu], link, &c->g, 0, nu, 1, 0)) return -1;
  if(staple) {
    if(qllg_k_mat_mul(p, staple, t1, ts1, &c->g, 1, 0, 0, 0)) return -1;
  } else {
    if(qllg_k_mat_mul(p, t2, t1, ts1, &c->g, 1, 0, 0, 0)) return -1;
    if(qllg_k_mat_peq(p, fl[mu], t2, coef, c->n)) return -1;
  }
  if(qllg_k_mat_mul(p, t1, gauge[nu], link, &c->g, 2, 0, 0, 0)) return -1;
  if(qllg_k_mat_mul(p, t2, t1, ts1, &c->g, 0, 0, 0, 0)) return -1;
  if(qllg_k_mat_shift(p, t1, t2, &c->g, nu, -1, 0, 1.0)) return -1;
  if(staple) {
    if(qllg_k_mat_peq(p, staple, t1, 1.0, c->n)) return -1;
    if(qllg_k_mat_peq(p, fl[mu], staple, coef, c->n)) return -1;
  } else {
    if(qllg_k_mat_peq(p, fl[mu], t1, coef, c->n)) return -1;
  }
  return 0;
}

/* smearFat7 (lib/gauge.c:264-416) on device fields */
int
qllg_fat7_device(int prec, const qllg_geom *g, void *const fl[4], void *const ll[4],
                 const Fat7Coeffs *coef, void *const u[4], void *const uLong[4])
{
  fctx c;
  c.prec = prec;
  c.g = *g;
  c.n = 18*(size_t)g->V;
  c.bytes = c.n*(prec == QLLG_F64 ? 8 : 4);
  double coef1 = coef->one_link, coef3 = coef->three_staple, coef5 = coef->five_staple;
  double coef7 = coef->seven_staple, coefL = coef->lepage;
  coef1 -= 6*coefL;
  int have5 = coef5 || coef7 || coefL;
  int have3 = coef3 || have5;
  void *staple = NULL, *tempmat1 = NULL, *t1 = NULL, *t2 = NULL, *tsg[4][4];
  memset(tsg, 0, sizeof(tsg));
  int rc = -1;
  if(have3 || ll) {
    if(!(staple = fnew(&c)) || !(tempmat1 = fnew(&c))) goto out;
  }
  if(have3) {
    if(!(t1 = fnew(&c)) || !(t2 = fnew(&c))) goto out;
    for(int dir=0; dir<4; dir++) for(int nu=0; nu<4; nu++) {
      if(dir == nu) continue;
      if(!(tsg[dir][nu] = fnew(&c))) goto out;
      if(qllg_k_mat_shift(prec, tsg[dir][nu], u[dir], g, nu, 1, 0, 1.0)) goto out;
    }
  }
  for(int dir=0; dir<4; dir++) {
    if(qllg_k_mat_axpy(prec, fl[dir], u[dir], 0.0, coef1, c.n)) goto out;
    if(!have3) continue;
    for(int nu=0; nu<4; nu++) {
      if(nu == dir) continue;
      if(gen_staple(&c, staple, dir, nu, u[dir], coef3, u, fl, tsg[nu][dir], t1, t2)) goto out;
      if(coefL &&
         gen_staple(&c, NULL, dir, nu, staple, coefL, u, fl, tsg[nu][dir], t1, t2)) goto out;
      if(coef5 || coef7) {
        for(int rho=0; rho<4; rho++) {
          if(rho == dir || rho == nu) continue;
          if(gen_staple(&c, tempmat1, dir, rho, staple, coef5, u, fl, tsg[rho][dir], t1, t2))
            goto out;
          if(coef7) {
            for(int sig=0; sig<4; sig++) {
              if(sig != dir && sig != nu && sig != rho &&
                 gen_staple(&c, NULL, dir, sig, tempmat1, coef7, u, fl, tsg[sig][dir], t1, t2))
                goto out;
            }
          }
        }
      }
    }
  }
  if(ll) {
    for(int dir=0; dir<4; dir++) {
      /* L = naik * U(x) U(x+dir) U(x+2dir) as two transports (:368-392) */
      if(qllg_k_mat_mul(prec, tempmat1, uLong[dir], uLong[dir], g, 0, dir, 1, 0)) goto out;
      if(qllg_k_mat_mul(prec, ll[dir], uLong[dir], tempmat1, g, 0, dir, 1, 0)) goto out;
      if(qllg_k_mat_axpy(prec, ll[dir], ll[dir], 0.0, coef->naik, c.n)) goto out;
    }
  }
  rc = qllg_sync();
out:
  qllg_sync();
  qllg_dfree(staple); qllg_dfree(tempmat1); qllg_dfree(t1); qllg_dfree(t2);
  for(int dir=0; dir<4; dir++) for(int nu=0; nu<4; nu++) qllg_dfree(tsg[dir][nu]);
  return rc;
}

/* host [V][18] <-> device matrix field [9][V] */
static int
mfield_up(int prec, void *dev, const void *host, int V)
{
  int dbl = prec == QLLG_F64;
  size_t hb = (dbl ? 8 : 4)*18*(size_t)V;
  void *st = qllg_stage(hb);
  if(!st || qllg_h2d(st, host, hb)) return -1;
  return qllg_k_link_from_aos(prec, dev, NULL, st, dbl, V);
}

static int
mfield_down(int prec, void *host, const void *dev, int V)
{
  int dbl = prec == QLLG_F64;
  size_t hb = (dbl ? 8 : 4)*18*(size_t)V;
  void *st = qllg_stage(hb);
  if(!st) return -1;
  if(qllg_k_link_to_aos(prec, dev, st, dbl, V)) return -1;
  return qllg_d2h(host, st, hb);
}

static int
smear_host(int prec, const int dims[4], void *const flh[4], void *const llh[4],
           const Fat7Coeffs *coef, void *const uh[4], void *const ulh[4])
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return -1;
  size_t bytes = 18*(size_t)g.V*(prec == QLLG_F64 ? 8 : 4);
  void *u[4] = {0}, *ul[4] = {0}, *fl[4] = {0}, *ll[4] = {0};
  int rc = -1;
  for(int d=0; d<4; d++) {
    if(!(u[d] = qllg_dmalloc(bytes)) || !(fl[d] = qllg_dmalloc(bytes))) goto out;
    if(mfield_up(prec, u[d], uh[d], g.V)) goto out;
    if(llh) {
      if(!(ll[d] = qllg_dmalloc(bytes))) goto out;
      if(ulh[d] == uh[d]) ul[d] = u[d];
      else {
        if(!(ul[d] = qllg_dmalloc(bytes)) || mfield_up(prec, ul[d], ulh[d], g.V)) goto out;
      }
    }
  }
  if(qllg_fat7_device(prec, &g, fl, llh ? ll : NULL, coef, u, ul)) goto out;
  for(int d=0; d<4; d++) {
    if(mfield_down(prec, flh[d], fl[d], g.V)) goto out;
    if(llh && mfield_down(prec, llh[d], ll[d], g.V)) goto out;
  }
  rc = 0;
out:
  qllg_sync();
  for(int d=0; d<4; d++) {
    if(ul[d] && ul[d] != u[d]) qllg_dfree(ul[d]);
    qllg_dfree(u[d]); qllg_dfree(fl[d]); qllg_dfree(ll[d]);
  }
  return rc;
}

/* ------------------------------------------------------------ native */

int
qllg_smear_fat7(const int dims[4], double *const fl[4], double *const ll[4],
                const Fat7Coeffs *coef, double *const u[4], double *const ulong_[4])
{
  return smear_host(QLLG_F64, dims, (void *const *)fl, (void *const *)ll, coef,
                    (void *const *)u, (void *const *)(ulong_ ? ulong_ : u));
}

/* thin links -> fat7 -> the links of a resident operator, all on the GPU:
 * 16 slots (forward and negative-adjoint backward), or with single_store
 * the 8 forward slots [fat mu, long mu] whose backward links the kernels
 * make on the fly */
static qllg_stag *
create_asqtad(const int dims[4], double *const thin[4], const Fat7Coeffs *coef, int single_store)
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return NULL;
  size_t fb = 144*(size_t)g.V;
  const int stored = single_store ? 8 : 16, per_mu = stored/4;
  void *u[4] = {0}, *fl[4] = {0}, *ll[4] = {0};
  qllg_stag *S = NULL;
  char *links = qllg_dmalloc(fb*stored);
  if(!links) return NULL;
  for(int d=0; d<4; d++) {
    if(!(u[d] = qllg_dmalloc(fb))) goto out;
    if(mfield_up(QLLG_F64, u[d], thin[d], g.V)) goto out;
    fl[d] = links + fb*(per_mu*d + 0);
    ll[d] = links + fb*(per_mu*d + 1);
  }
  if(qllg_fat7_device(QLLG_F64, &g, fl, ll, coef, u, u)) goto out;
  for(int d=0; d<4 && !single_store; d++) {
    /* slot 4mu+2: -F_mu(x-mu)^dagger; slot 4mu+3: -L_mu(x-3mu)^dagger */
    if(qllg_k_mat_shift(QLLG_F64, links + fb*(4*d + 2), fl[d], &g, d, -1, 1, -1.0)) goto out;
    if(qllg_k_mat_shift(QLLG_F64, links + fb*(4*d + 3), ll[d], &g, d, -3, 1, -1.0)) goto out;
  }
  if(qllg_sync()) goto out;
  S = qllg_stag_alloc(dims, 16, QLLG_F64);
  if(S && single_store) qllg_stag_set_single_store(S);
  if(S && qllg_stag_attach_links(S, QLLG_F64, links)) { qllg_stag_destroy(S); S = NULL; }
  if(S) links = NULL;
out:
  qllg_sync();
  for(int d=0; d<4; d++) qllg_dfree(u[d]);
  qllg_dfree(links);
  return S;
}

qllg_stag *
qllg_stag_create_asqtad(const int dims[4], double *const thin[4], const Fat7Coeffs *coef)
{
  return create_asqtad(dims, thin, coef, 0);
}

qllg_stag *
qllg_stag_create_asqtad_fb(const int dims[4], double *const thin[4], const Fat7Coeffs *coef)
{
  return create_asqtad(dims, thin, coef, 1);
}

int
qllg_plaq(const int dims[4], double *const u[4], double plaqs[6])
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return -1;
  size_t fb = 144*(size_t)g.V;
  void *ud[4] = {0};
  double *res = NULL;
  qllg_redbuf rb = {0};
  int rc = -1;
  if(qllg_redbuf_init(&rb) || !(res = qllg_dmalloc(sizeof(double)*6))) goto out;
  for(int d=0; d<4; d++) {
    if(!(ud[d] = qllg_dmalloc(fb)) || mfield_up(QLLG_F64, ud[d], u[d], g.V)) goto out;
  }
  {
    int l = 0;
    for(int i=0; i<4; i++) for(int j=0; j<i; j++, l++)
      if(qllg_k_plaq(QLLG_F64, ud[i], ud[j], &g, i, j, res + l, &rb)) goto out;
  }
  if(qllg_d2h(plaqs, res, sizeof(double)*6)) goto out;
  for(int l=0; l<6; l++) plaqs[l] /= 3.0*g.V;
  rc = 0;
out:
  qllg_sync();
  for(int d=0; d<4; d++) qllg_dfree(ud[d]);
  qllg_dfree(res);
  qllg_redbuf_free(&rb);
  return rc;
}

/* ------------------------------------------------- drop-in: gauge */

#define DEFINE_GAUGE_DROPIN(S_, real, PREC)                                       \
void                                                                              \
smearFat7##S_(Field##S_ *fl[], Field##S_ *ll[], Fat7Coeffs *coef, Field##S_ *u[], \
              Field##S_ *uLong[])                                                 \
{                                                                                 \
  qllg_geom g;                                                                    \
  if(qllg_geom_from_layout(&g, u[0]->l)) return;                                  \
  void *flh[4], *llh[4], *uh[4], *ulh[4];                                         \
  for(int d=0; d<4; d++) {                                                        \
    flh[d] = fl[d]->f;                                                            \
    llh[d] = ll ? ll[d]->f : NULL;                                                \
    uh[d] = u[d]->f;                                                              \
    ulh[d] = uLong ? uLong[d]->f : u[d]->f;                                       \
  }                                                                               \
  smear_host(PREC, g.L, flh, ll ? llh : NULL, coef, uh, ulh);                     \
}                                                                                 \
                                                                                  \
void                                                                              \
gaugePlaq##S_(double plaqs[], Field##S_ *u[])                                     \
{                                                                                 \
  qllg_geom g;                                                                    \
  if(qllg_geom_from_layout(&g, u[0]->l)) return;                                  \
  size_t fb = 18*(size_t)g.V*sizeof(real);                                        \
  void *ud[4] = {0};                                                              \
  double *res = NULL;                                                             \
  qllg_redbuf rb = {0};                                                           \
  if(qllg_redbuf_init(&rb) || !(res = qllg_dmalloc(sizeof(double)*6))) goto out;  \
  for(int d=0; d<4; d++)                                                          \
    if(!(ud[d] = qllg_dmalloc(fb)) || mfield_up(PREC, ud[d], u[d]->f, g.V)) goto out; \
  {                                                                               \
    int l = 0;                                                                    \
    for(int i=0; i<4; i++) for(int j=0; j<i; j++, l++)                            \
      if(qllg_k_plaq(PREC, ud[i], ud[j], &g, i, j, res + l, &rb)) goto out;       \
  }                                                                               \
  if(qllg_d2h(plaqs, res, sizeof(double)*6)) goto out;                            \
  for(int l=0; l<6; l++) plaqs[l] /= 3.0*g.V;                                     \
out:                                                                              \
  qllg_sync();                                                                    \
  for(int d=0; d<4; d++) qllg_dfree(ud[d]);                                       \
  qllg_dfree(res);                                                                \
  qllg_redbuf_free(&rb);                                                          \
}                                                                                 \
                                                                                  \
void                                                                              \
gaugeDoublestore##S_(Field##S_ *ua[], Field##S_ *u[], int dirs[], int lens[], int n) \
{                                                                                 \
  for(int i=0; i<n; i++) {                                                        \
    qllg_geom g;                                                                  \
    if(qllg_geom_from_layout(&g, u[i]->l)) return;                                \
    if(u[i]->nelem != 18) { qllg_set_error("gaugeDoublestore: nelem %d", u[i]->nelem); return; } \
    size_t fb = 18*(size_t)g.V*sizeof(real);                                      \
    void *a = qllg_dmalloc(fb), *b = qllg_dmalloc(fb);                            \
    if(a && b && !mfield_up(PREC, a, u[i]->f, g.V) &&                             \
       !qllg_k_mat_shift(PREC, b, a, &g, dirs[i], lens[i], 1, 1.0))               \
      mfield_down(PREC, ua[i]->f, b, g.V);                                        \
    qllg_sync();                                                                  \
    qllg_dfree(a); qllg_dfree(b);                                                 \
  }                                                                               \
}

DEFINE_GAUGE_DROPIN(D, double, QLLG_F64)
DEFINE_GAUGE_DROPIN(F, float, QLLG_F32)

/* ------------------------------------------------- makeU (drop-in) */
/* makeU (include/vla.h:85, lib/vla.c:1635-1665): re-unitarise sites [i0, i1)
 * of host matrices, 2 nc^2 reals a site in QLL's one-lane order, by
 * Gram-Schmidt of the nc vectors (make_u_k on the GPU).  void, as the
 * reference's: a failure leaves the matrices untouched and records the
 * message (qllg_last_error). */
static void
make_u_host(int prec, void *mm, int nc, int i0, int i1)
{
  if(i1 <= i0) return;
  if(nc < 1 || nc > 3) { qllg_set_error("makeU: nc %d (1 to 3)", nc); return; }
  if(qllg_runtime_init()) return;
  const size_t per = (prec == QLLG_F64 ? 8 : 4)*2*(size_t)nc*nc;
  const size_t bytes = per*(size_t)(i1 - i0);
  char *h = (char *)mm + per*(size_t)i0;
  void *d = qllg_stage(bytes);
  if(!d || qllg_h2d(d, h, bytes) || qllg_k_make_u(prec, d, nc, 0, (size_t)(i1 - i0))) {
    qllg_sync();
    return;
  }
  /* into a host copy first, so that a failed copy leaves mm as it was */
  char *tmp = malloc(bytes);
  if(!tmp) { qllg_set_error("makeU: host buffer of %zu bytes", bytes); qllg_sync(); return; }
  if(qllg_d2h(tmp, d, bytes) == 0) memcpy(h, tmp, bytes);
  free(tmp);
}

void makeUD(double *mm, int nc, int i0, int i1) { make_u_host(QLLG_F64, mm, nc, i0, i1); }
void makeUF(float *mm, int nc, int i0, int i1) { make_u_host(QLLG_F32, mm, nc, i0, i1); }
