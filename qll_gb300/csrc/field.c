/*
 * field.c -- the Field API (lib/field.c:3-63), the generic transporter
 * (lib/transporter.c:12-193), shift (lib/stagDslash.c:91-101) and the
 * Dslash timers (lib/stagDslash.c:659-713, lib/wilsonDslash.c:403-456).
 *
 * Fields live in host memory, as in the reference.  Reductions, shifts and
 * transports run on the GPU on a device copy of the operands: the call
 * uploads the operands, runs the kernel and copies back the sites of the
 * subset.  The transporter's start/local/wait split exists for the
 * reference's halo overlap; with one GPU and no halo the whole transport
 * runs in transporterWaitT, and StartT/LocalT only record the operands.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

int qllg_geom_from_layout(qllg_geom *g, const Layout *l);
Layout *qllg_current_layout(void);

/* shared scratch for the field calls: two device buffers and a workspace */
static void *g_fa = NULL, *g_fb = NULL, *g_fu = NULL;
static size_t g_fa_n = 0, g_fb_n = 0, g_fu_n = 0;
static qllg_redbuf g_frb;
static double *g_fres = NULL;

static void *
fbuf(void **p, size_t *n, size_t bytes)
{
  if(bytes <= *n) return *p;
  if(*p) { qllg_sync(); qllg_dfree(*p); }
  *p = qllg_dmalloc(bytes);
  *n = *p ? bytes : 0;
  return *p;
}

static int
fred_init(void)
{
  if(g_fres) return 0;
  if(qllg_redbuf_init(&g_frb)) return -1;
  g_fres = qllg_dmalloc(sizeof(double)*4);
  return g_fres ? 0 : -1;
}

/* sum (sq = 0) or sum of squares (sq = 1) of a host field over sub */
static double
field_reduce(const void *f, int dbl, int nelem, const Subset *sub, int sq)
{
  size_t es = dbl ? 8 : 4;
  size_t n = (size_t)nelem*(sub->end - sub->begin);
  double r = 0;
  if(qllg_runtime_init() || fred_init()) return 0;
  void *d = fbuf(&g_fa, &g_fa_n, n*es + 16);
  if(!d) return 0;
  if(qllg_h2d(d, (const char *)f + es*nelem*(size_t)sub->begin, n*es)) return 0;
  if(qllg_k_aos_sum(dbl ? QLLG_F64 : QLLG_F32, d, nelem, 0, sub->end - sub->begin, sq, g_fres,
                    &g_frb)) return 0;
  qllg_d2h(&r, g_fres, sizeof(double));
  return r;
}

/* x = y gathered from x + len*mu (host [V][nelem]) */
static int
field_shift(void *x, const void *y, int dbl, int nelem, int mu, int len)
{
  Layout *l = qllg_current_layout();
  qllg_geom g;
  if(!l) { qllg_set_error("shift: call stagDslashSetup first"); return -1; }
  if(qllg_geom_from_layout(&g, l)) return -1;
  size_t bytes = (dbl ? 8 : 4)*(size_t)nelem*g.V;
  void *a = fbuf(&g_fa, &g_fa_n, bytes), *b = fbuf(&g_fb, &g_fb_n, bytes);
  if(!a || !b || qllg_h2d(a, y, bytes)) return -1;
  if(qllg_k_aos_shift(dbl ? QLLG_F64 : QLLG_F32, b, a, nelem, &g, mu, len)) return -1;
  return qllg_d2h(x, b, bytes);
}

/* dest(x) (+)= u(x) src(x + len*mu) on the sites [s0, s1) */
static int
field_transport(void *dest, const void *u, const void *src, int dbl, int nelem, int mu, int len,
                int s0, int s1, int with_u)
{
  Layout *l = qllg_current_layout();
  qllg_geom g;
  if(!l) { qllg_set_error("transporter: call stagDslashSetup first"); return -1; }
  if(qllg_geom_from_layout(&g, l)) return -1;
  if(with_u && nelem % 6) { qllg_set_error("transporter: nelem %d is not a multiple of 6", nelem); return -1; }
  size_t es = dbl ? 8 : 4;
  size_t bytes = es*(size_t)nelem*g.V;
  int prec = dbl ? QLLG_F64 : QLLG_F32;
  void *a = fbuf(&g_fa, &g_fa_n, bytes), *b = fbuf(&g_fb, &g_fb_n, bytes);
  if(!a || !b || qllg_h2d(a, src, bytes)) return -1;
  if(with_u) {
    void *du = fbuf(&g_fu, &g_fu_n, es*18*(size_t)g.V);
    if(!du || qllg_h2d(du, u, es*18*(size_t)g.V) || qllg_h2d(b, dest, bytes)) return -1;
    if(qllg_k_aos_transport(prec, b, du, a, nelem, &g, mu, len)) return -1;
  } else {
    if(qllg_k_aos_shift(prec, b, a, nelem, &g, mu, len)) return -1;
  }
  size_t off = es*(size_t)nelem*s0;
  return qllg_d2h((char *)dest + off, (char *)b + off, es*(size_t)nelem*(s1 - s0));
}

/* direction and length of a ShiftIndices (gathers from x - disp) */
static int
si_dir(const ShiftIndices *si, int *mu, int *len)
{
  if(!si->disp) { qllg_set_error("transporter: shift without displacement"); return -1; }
  for(int i=0; i<4; i++) if(si->disp[i]) { *mu = i; *len = -si->disp[i]; return 0; }
  *mu = 0; *len = 0;
  return 0;
}

static void
print_timer(const char *fam, double scale)
{
  int n; double ms;
  qllg_timing_read(fam, &n, &ms);
  printf("%13s: %12.2f\t(%d launches, GPU events)\n", fam, scale*ms*1e3, n);
  fflush(stdout);
}

#define DEFINE_FIELD_DROPIN(S_, real, DBL)                                        \
void fieldNew##S_(Field##S_ *f, Layout *l, int nelem)                             \
{                                                                                 \
  f->l = l;                                                                       \
  f->f = myalloc(sizeof(real)*(size_t)nelem*l->nSites);                           \
  f->nelem = nelem;                                                               \
}                                                                                 \
void fieldFree##S_(Field##S_ *f) { free(f->f); f->f = NULL; }                     \
void fieldSet##S_(Field##S_ *f, real *r, Layout *l, int nelem)                    \
{                                                                                 \
  f->l = l; f->f = r; f->nelem = nelem;                                           \
}                                                                                 \
void fieldZero##S_(Field##S_ *f, Subset *sub)                                     \
{                                                                                 \
  memset(f->f + (size_t)f->nelem*sub->begin, 0,                                   \
         sizeof(real)*(size_t)f->nelem*(sub->end - sub->begin));                  \
}                                                                                 \
double fieldSumElem##S_(Field##S_ *f, Subset *sub)                                \
{                                                                                 \
  return field_reduce(f->f, DBL, f->nelem, sub, 0);                               \
}                                                                                 \
double fieldNorm2##S_(Field##S_ *f, Subset *sub)                                  \
{                                                                                 \
  return field_reduce(f->f, DBL, f->nelem, sub, 1);                               \
}                                                                                 \
void shift##S_(real *x, real *y, int nelem, int dir, int len)                     \
{                                                                                 \
  int mu = (dir > 0 ? dir : -dir) - 1;                                            \
  field_shift(x, y, DBL, nelem, mu, dir > 0 ? len : -len);                        \
}                                                                                 \
void transporterNew##S_(Transporter##S_ *t, real *u, ShiftIndices *si,            \
                        Subset *sub, int nelem, int nc)                           \
{                                                                                 \
  memset(t, 0, sizeof(*t));                                                       \
  t->u = u;                                                                       \
  if(si) t->si = *si;                                                             \
  t->nelem = nelem;                                                               \
  t->nc = nc;                                                                     \
  t->sub = *sub;                                                                  \
}                                                                                 \
void transporterFree##S_(Transporter##S_ *t) { (void)t; }                         \
void transporterStartT##S_(Transporter##S_ *t, real *dest, real *src, int td,     \
                           ThreadCtx *TC)                                         \
{                                                                                 \
  (void)TC;                                                                       \
  t->dest = dest; t->src = src; t->td = td;                                       \
}                                                                                 \
void transporterLocalT##S_(Transporter##S_ *t, ThreadCtx *TC) { (void)t; (void)TC; } \
void transporterWaitT##S_(Transporter##S_ *t, ThreadCtx *TC)                      \
{                                                                                 \
  (void)TC;                                                                       \
  int mu, len;                                                                    \
  if(si_dir(&t->si, &mu, &len)) return;                                           \
  field_transport(t->dest, t->u, t->src, DBL, t->nelem, mu, len, t->sub.begin,    \
                  t->sub.end, t->td > 0 && t->u);                                 \
}                                                                                 \
void transporterDoT##S_(Transporter##S_ *t, real *dest, real *src, int td,        \
                        ThreadCtx *TC)                                            \
{                                                                                 \
  transporterStartT##S_(t, dest, src, td, TC);                                    \
  transporterLocalT##S_(t, TC);                                                   \
  transporterWaitT##S_(t, TC);                                                    \
}                                                                                 \
void transporterDo##S_(Transporter##S_ *t, real *dest, real *src, int td)         \
{                                                                                 \
  transporterDoT##S_(t, dest, src, td, NULL);                                     \
}                                                                                 \
void dslashResetTimer##S_(void) { qllg_timing_enable(1); qllg_timing_reset(); }   \
void dslashPrintTimer##S_(double scale) { print_timer(DBL ? "stag_dslash_f64_n1" : "stag_dslash_f32_n1", scale); }    \
void wilsonDslashResetTimer##S_(void) { qllg_timing_enable(1); qllg_timing_reset(); } \
void wilsonDslashPrintTimer##S_(double scale) { print_timer("wilson_dslash", scale); }

DEFINE_FIELD_DROPIN(D, double, 1)
DEFINE_FIELD_DROPIN(F, float, 0)
