/*
 * stag.c -- the asqtad staggered operator on the GPU: resident links,
 * dslash2, the even-odd normal operator of dslashp2, CG (cgSolveT) and the
 * drop-in entry points createStaggeredLinks / dslash2 /
 * createStaggeredSolver / solve2 / freeStaggeredSolver
 * (lib/stagDslash.c:422-657, lib/cg.c:8-136).
 *
 * A CG iteration is four launches: p += r/|r|^2; v = D_oe p with |v|^2;
 * Ap = m^2 p - D_eo v with |p|^2; x += a p, r -= a Ap with |r|^2 (a =
 * 1/(m^2|p|^2 + |v|^2), the fused <p,Ap> of dslashp2).  All scalars stay on
 * the GPU; convergence is tested by the last kernel, which retires right-hand
 * sides individually, and the host looks at the "done" flag once per batch
 * of iterations, so the iteration count equals the reference's exactly.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

void qllg_tm_begin(const char *name);
void qllg_tm_end(void);
int qllg_geom_from_layout(qllg_geom *g, const Layout *l);
Layout *qllg_current_layout(void);

enum { WS_X, WS_R, WS_P, WS_AP, WS_V, WS_B, WS_IO, WS_X64, WS_R64, WS_T64, WS_V64,
       WS_PS, WS_OUT, WS_XDF, WS_CGP, WS_N };

/* what one solver iteration launches */
typedef struct {
  int mixed;                 /* 0 plain CG, 1 mixed CG with reliable updates */
  int ps, pl, nrhs, reortho;
  void *x, *r, *p, *v;       /* sloppy (or only) vectors */
  void *x64, *r64, *t64, *w64;
  void *xdf;                 /* double-float copy of x64 for the intermediate
                                reliable updates, NULL: all in FP64 */
  const void *b;
} iter_ctx;

struct qllg_stag {
  qllg_geom g;
  int nslots;
  int master;              /* precision of the links handed in */
  void *links[QLLG_NLINKP];  /* per precision, lazily derived from the master */
  float *lscale;           /* 16-bit link scales [nslots] */
  qllg_redbuf rb;
  qllg_cg_scalars *sc;     /* device scalars */
  qllg_cg_scalars *hsc;    /* pinned host copy */
  qllg_cgms_scalars *cs;   /* multishift scalars, device */
  qllg_cgms_scalars *hcs;  /* pinned host copy */
  qllg_mcgms_scalars *mcs; /* multi-rhs multishift scalars, device (on first use) */
  void *ws[WS_N];
  size_t ws_bytes[WS_N];
  unsigned ws_gen;         /* bumped when a workspace buffer moves */
  cudaEvent_t ev0, ev1;
  struct {                 /* graph-captured solver loops */
    long key[11];
    cudaGraphExec_t exec;
    int body;              /* kernels in one trip of the loop body */
    int ifbody;            /* ... of it in the conditional reliable-update block */
  } graphs[6];
  int ngraph_next;
  int graph_body;          /* body of the graph the current solve launched, 0: none */
  int graph_ifbody;
  int cap_ifbody;          /* while capturing: kernels of the reliable-update block */
  int used_persistent;     /* the last solve ran the persistent CG */
  unsigned char shared[QLLG_NLINKP]; /* links[p] belong to another operator */
  int recon_bad;           /* the Naik links are not reconstructible (reconstruct-12 refused) */
  int fb;                  /* single-stored: the nslots/2 forward slots only */
  /* continuous batching (qllg_batch_*): a fixed-width mixed CG whose
   * columns are admitted and retired independently */
  int batch_on;
  iter_ctx bctx;
  void *bstage;            /* one column, [Vh][6] FP64, on the device */
  cudaEvent_t bev;         /* end of the last chunk and its scalar copy */
};

/* ------------------------------------------------------------ helpers */

static void *
ws_get(qllg_stag *S, int id, size_t bytes)
{
  if(bytes <= S->ws_bytes[id]) return S->ws[id];
  if(S->ws[id]) { qllg_sync(); qllg_dfree(S->ws[id]); }
  S->ws[id] = qllg_dmalloc(bytes);
  S->ws_bytes[id] = S->ws[id] ? bytes : 0;
  S->ws_gen++;
  return S->ws[id];
}

static size_t
vec_bytes(const qllg_stag *S, int prec, int nrhs)
{
  return qllg_spinor_bytes(prec, 3)*(size_t)S->g.Vh*nrhs;
}

/* link slots held in memory: all of them, or the forward half */
static int
stored_slots(const qllg_stag *S)
{
  return S->fb ? S->nslots/2 : S->nslots;
}

void
qllg_stag_set_single_store(qllg_stag *S)
{
  S->fb = 1;
}

/* bytes of the links of precision prec (the reconstruct-12 format keeps
 * fat slots at 72, Naik slots at 48 bytes a site, plus one sign byte) */
static size_t
links_bytes(const qllg_stag *S, int prec)
{
  const size_t V = (size_t)S->g.V;
  const int n = stored_slots(S);
  if(prec != QLLG_F32R) return qllg_link_bytes(prec)*V*n;
  return S->nslots == 16 ? (size_t)(n/2)*120*V + V : (size_t)n*72*V;
}

/* FP32 links in the reconstruct-12 format, from the FP64 master */
static int
make_f32r_links(qllg_stag *S)
{
  const size_t V = (size_t)S->g.V;
  const int n = stored_slots(S), n16 = S->nslots == 16;
  char *out = qllg_dmalloc(links_bytes(S, QLLG_F32R));
  int *bad = qllg_dmalloc(sizeof(int)), hbad = 0;
  if(!out || !bad) { qllg_dfree(out); qllg_dfree(bad); return -1; }
  unsigned char *signs = (unsigned char *)out + (n16 ? (size_t)(n/2)*120*V : (size_t)n*72*V);
  int rc = qllg_check_cuda(cudaMemsetAsync(bad, 0, sizeof(int), qllg_stream()), "clear");
  for(int s=0; s<n && !rc; s++) {
    const size_t base = n16 ? ((size_t)(s >> 1)*120 + (s & 1)*72)*V : (size_t)s*72*V;
    rc = qllg_k_link_to_f32r(out + base, (const double *)S->links[QLLG_F64] + (size_t)s*18*V,
                             S->g.V, n16 && (s & 1), signs, s >> 1, bad);
  }
  if(!rc) rc = qllg_d2h(&hbad, bad, sizeof(int));
  qllg_dfree(bad);
  if(rc || hbad) {
    qllg_sync();
    qllg_dfree(out);
    if(hbad) {
      S->recon_bad = 1;
      qllg_set_error("reconstruct-12: Naik links are not real multiples of SU(3) matrices");
    }
    return -1;
  }
  S->links[QLLG_F32R] = out;
  return 0;
}

static int ensure_links(qllg_stag *S, int prec);

/* links for the FP32 Dslash of the mixed solvers: the reconstruct-12
 * format when the parameter allows it and the Naik links are SU(3) up to a
 * real factor, else plain FP32 */
static int
f32_links(qllg_stag *S)
{
  if(qllg_get_param("links_recon12") != 0 && S->master == QLLG_F64 && S->nslots == 16 &&
     !S->recon_bad) {
    if(ensure_links(S, QLLG_F32R) == 0) return QLLG_F32R;
    qllg_clear_error();
  }
  return QLLG_F32;
}

static int ensure_links_make(qllg_stag *S, int prec);

/* Links of precision prec (FP64, FP32 or 16-bit) now exist for S, so
 * qllg_stag_dslash_norm2_noalloc can take S at that precision.  That call
 * must not allocate device memory, but with CUDA's lazy module loading
 * (the default) the first launch of a kernel loads its code into device
 * memory, and the first look-up of the fixed scratch loads the scratch.
 * This, an allocating call anyway, does both ahead of it: it resolves the
 * scratch's address on the current device and loads every Dslash kernel
 * the no-allocation call can reach at this precision and slot count. */
static int
noalloc_preload(qllg_stag *S, int prec)
{
  if(prec < QLLG_F64 || prec > QLLG_I16 || !S->links[prec]) return 0;
  qllg_redbuf rb;
  if(qllg_noalloc_redbuf(&rb)) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = S->g;
  A.nrhs = 1;
  A.nslots = S->nslots;
  A.fb = S->fb;
  A.links = S->links[prec];
  A.rb = &rb;
  A.preload = 1;
  return qllg_k_stag_dslash(prec, prec, &A);
}

static int
ensure_links(qllg_stag *S, int prec)
{
  if(S->links[prec]) return 0;
  int rc = ensure_links_make(S, prec);
  if(!rc) rc = noalloc_preload(S, prec);
  return rc;
}

static int
ensure_links_make(qllg_stag *S, int prec)
{
  if(prec == QLLG_F32R) {
    if(S->recon_bad) {
      qllg_set_error("reconstruct-12: Naik links are not real multiples of SU(3) matrices");
      return -1;
    }
    if(ensure_links(S, QLLG_F64)) return -1;
    return make_f32r_links(S);
  }
  if(S->master != QLLG_F64) {
    qllg_set_error("operator created from float links has no %s copy",
                   prec == QLLG_F64 ? "FP64" : "16-bit");
    return -1;
  }
  size_t per = qllg_link_bytes(prec)*(size_t)S->g.V;
  S->links[prec] = qllg_dmalloc(per*stored_slots(S));
  if(!S->links[prec]) return -1;
  const double *src = S->links[QLLG_F64];
  for(int s=0; s<stored_slots(S); s++) {
    if(qllg_k_link_convert(prec, (char *)S->links[prec] + per*s, S->lscale + s,
                           src + (size_t)s*18*S->g.V, S->g.V)) return -1;
  }
  return 0;
}

static qllg_stag *
stag_create(const int dims[4], void *const fat[8], void *const lng[8], int dbl)
{
  if(qllg_runtime_init()) return NULL;
  qllg_stag *S = calloc(1, sizeof(qllg_stag));
  if(qllg_geom_from_dims(&S->g, dims)) { free(S); return NULL; }
  S->nslots = lng ? 16 : 8;
  S->master = dbl ? QLLG_F64 : QLLG_F32;
  if(qllg_redbuf_init(&S->rb)) goto fail;
  S->sc = qllg_dmalloc(sizeof(qllg_cg_scalars));
  S->lscale = qllg_dmalloc(sizeof(float)*16);
  if(!S->sc || !S->lscale) goto fail;
  if(qllg_check_cuda(cudaMallocHost((void **)&S->hsc, sizeof(qllg_cg_scalars)), "cudaMallocHost"))
    goto fail;
  S->cs = qllg_dmalloc(sizeof(qllg_cgms_scalars));
  if(!S->cs) goto fail;
  if(qllg_check_cuda(cudaMallocHost((void **)&S->hcs, sizeof(qllg_cgms_scalars)), "cudaMallocHost"))
    goto fail;
  memset(S->hsc, 0, sizeof(qllg_cg_scalars));
  cudaEventCreate(&S->ev0);
  cudaEventCreate(&S->ev1);
  {
    int prec = S->master;
    size_t per = qllg_link_bytes(prec)*(size_t)S->g.V;
    size_t hbytes = (dbl ? 8 : 4)*18*(size_t)S->g.V;
    S->links[prec] = qllg_dmalloc(per*S->nslots);
    void *stage = qllg_stage(hbytes);
    if(!S->links[prec] || !stage) goto fail;
    for(int s=0; s<S->nslots; s++) {
      const void *h = (S->nslots == 16) ? ((s & 1) ? lng[s/2] : fat[s/2]) : fat[s];
      if(!h) { qllg_set_error("link slot %d is NULL", s); goto fail; }
      if(qllg_h2d(stage, h, hbytes)) goto fail;
      if(qllg_k_link_from_aos(prec, (char *)S->links[prec] + per*s, S->lscale + s, stage, dbl,
                              S->g.V)) goto fail;
    }
    if(qllg_sync()) goto fail;
  }
  if(noalloc_preload(S, S->master)) goto fail;
  return S;
fail:
  qllg_stag_destroy(S);
  return NULL;
}

/* an operator whose links are attached later (device-built links) */
qllg_stag *
qllg_stag_alloc(const int dims[4], int nslots, int prec)
{
  if(qllg_runtime_init()) return NULL;
  qllg_stag *S = calloc(1, sizeof(qllg_stag));
  if(qllg_geom_from_dims(&S->g, dims)) { free(S); return NULL; }
  S->nslots = nslots;
  S->master = prec;
  if(qllg_redbuf_init(&S->rb)) goto fail;
  S->sc = qllg_dmalloc(sizeof(qllg_cg_scalars));
  S->lscale = qllg_dmalloc(sizeof(float)*16);
  S->cs = qllg_dmalloc(sizeof(qllg_cgms_scalars));
  if(!S->sc || !S->lscale || !S->cs) goto fail;
  if(qllg_check_cuda(cudaMallocHost((void **)&S->hsc, sizeof(qllg_cg_scalars)), "cudaMallocHost") ||
     qllg_check_cuda(cudaMallocHost((void **)&S->hcs, sizeof(qllg_cgms_scalars)), "cudaMallocHost"))
    goto fail;
  cudaEventCreate(&S->ev0);
  cudaEventCreate(&S->ev1);
  return S;
fail:
  qllg_stag_destroy(S);
  return NULL;
}

/* hand a device link array [nslots][9][V] of prec to the operator, which
 * owns it from now on */
int
qllg_stag_attach_links(qllg_stag *S, int prec, void *links)
{
  if(S->links[prec]) qllg_dfree(S->links[prec]);
  S->links[prec] = links;
  return noalloc_preload(S, prec);
}

qllg_stag *
qllg_stag_create(const int dims[4], double *const fat[8], double *const lng[8])
{
  return stag_create(dims, (void *const *)fat, (void *const *)lng, 1);
}

qllg_stag *
qllg_stag_create_f(const int dims[4], float *const fat[8], float *const lng[8])
{
  return stag_create(dims, (void *const *)fat, (void *const *)lng, 0);
}

/* a second operator on the same resident links: its own workspaces,
 * scalars, reduction buffer and graphs, the links (FP64 and FP32, derived
 * here if missing) shared with S.  S must outlive it. */
qllg_stag *
qllg_stag_share(qllg_stag *S)
{
  if(ensure_links(S, QLLG_F64) || ensure_links(S, QLLG_F32)) return NULL;
  f32_links(S);               /* the reconstruct-12 copy too, when it applies */
  /* and the double-float copy of the reliable updates, so that the
   * operators sharing S do not each make their own */
  if(qllg_get_param("ru_df") != 0 && qllg_get_param("ru_compact") != 0 && S->master == QLLG_F64 &&
     ensure_links(S, QLLG_DF)) return NULL;
  int dims[4] = {S->g.L[0], S->g.L[1], S->g.L[2], S->g.L[3]};
  qllg_stag *T = qllg_stag_alloc(dims, S->nslots, S->master);
  if(!T) return NULL;
  T->fb = S->fb;
  T->recon_bad = S->recon_bad;
  for(int p=0; p<QLLG_NLINKP; p++) {
    T->links[p] = S->links[p];
    T->shared[p] = S->links[p] != NULL;
  }
  if(qllg_check_cuda(cudaMemcpyAsync(T->lscale, S->lscale, sizeof(float)*16,
                                     cudaMemcpyDeviceToDevice, qllg_stream()), "share scales")) {
    qllg_stag_destroy(T);
    return NULL;
  }
  return T;
}

void
qllg_stag_destroy(qllg_stag *S)
{
  if(!S) return;
  qllg_sync();
  for(int p=0; p<QLLG_NLINKP; p++) if(!S->shared[p]) qllg_dfree(S->links[p]);
  qllg_dfree(S->bstage);
  if(S->bev) cudaEventDestroy(S->bev);
  qllg_dfree(S->lscale);
  qllg_dfree(S->sc);
  if(S->hsc) cudaFreeHost(S->hsc);
  qllg_dfree(S->cs);
  qllg_dfree(S->mcs);
  if(S->hcs) cudaFreeHost(S->hcs);
  qllg_redbuf_free(&S->rb);
  for(int i=0; i<WS_N; i++) qllg_dfree(S->ws[i]);
  for(int i=0; i<6; i++) if(S->graphs[i].exec) cudaGraphExecDestroy(S->graphs[i].exec);
  if(S->ev0) cudaEventDestroy(S->ev0);
  if(S->ev1) cudaEventDestroy(S->ev1);
  free(S);
}

int qllg_k_mat_shift(int prec, void *out, const void *in, const qllg_geom *g, int mu, int len,
                     int adj, double sgn);

/* copy the operator's FP64 link slots to host arrays [V][18] (backward
 * slots of a single-stored operator are made from its forward ones) */
int
qllg_stag_get_links(qllg_stag *S, double *const out[16])
{
  if(ensure_links(S, QLLG_F64)) return -1;
  size_t per = qllg_link_bytes(QLLG_F64)*(size_t)S->g.V, hb = 8*18*(size_t)S->g.V;
  void *st = qllg_stage(hb);
  if(!st) return -1;
  for(int s=0; s<S->nslots; s++) {
    const char *src = (const char *)S->links[QLLG_F64] + per*s;
    void *tmp = NULL;
    if(S->fb) {
      /* single-stored: forward slots as held, backward ones made here */
      const int n16 = S->nslots == 16;
      const int mu = n16 ? s/4 : s/2, back = n16 ? (s/2) & 1 : s & 1, nk = n16 ? s & 1 : 0;
      src = (const char *)S->links[QLLG_F64] + per*(n16 ? 2*mu + nk : mu);
      if(back) {
        if(!(tmp = qllg_dmalloc(per)) ||
           qllg_k_mat_shift(QLLG_F64, tmp, src, &S->g, mu, nk ? -3 : -1, 1, -1.0)) {
          qllg_dfree(tmp);
          return -1;
        }
        src = tmp;
      }
    }
    int rc = qllg_k_link_to_aos(QLLG_F64, src, st, 1, S->g.V) || qllg_d2h(out[s], st, hb);
    if(tmp) { qllg_sync(); qllg_dfree(tmp); }
    if(rc) return -1;
  }
  return 0;
}

/* 1 when the operator's mixed FP32 solves use reconstruct-12 links
 * (deriving them now if the parameter allows it) */
int
qllg_stag_recon12(qllg_stag *S)
{
  return f32_links(S) == QLLG_F32R;
}

int
qllg_stag_nslots(const qllg_stag *S)
{
  return S->nslots;
}

size_t
qllg_stag_device_bytes(const qllg_stag *S)
{
  size_t b = 0;
  for(int p=0; p<QLLG_NLINKP; p++)
    if(S->links[p] && !S->shared[p]) b += links_bytes(S, p);
  for(int i=0; i<WS_N; i++) b += S->ws_bytes[i];
  if(S->bstage) b += 48*(size_t)S->g.Vh;
  return b;
}

/* one half-Dslash launch; compact: threads only over the rhs flagged in
 * active (modes 0 and 2, no norms) */
static int
dslash_half_x(qllg_stag *S, int ps, int pl, int out_parity, int nrhs, const void *in,
              const void *self, void *out, int mode, const double *a, double a0, double b,
              double *norm_out, double *norm_self, const int *active, const int *done,
              int compact, int active_eq)
{
  if(ensure_links(S, pl)) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = S->g;
  A.out_parity = out_parity;
  A.nrhs = nrhs;
  A.nslots = S->nslots;
  A.fb = S->fb;
  A.links = S->links[pl];
  A.lscale = S->lscale;
  A.in = in;
  A.self = self;
  A.out = out;
  A.mode = mode;
  A.a = a;
  A.a0 = a0;
  A.b = b;
  A.norm_out = norm_out;
  A.norm_self = norm_self;
  A.active = active;
  A.done = done;
  A.rb = &S->rb;
  A.compact = compact;
  A.active_eq = active_eq;
  static const char *pn[5] = {"f64", "f32", "i16", "f32r", "df"};
  char fam[32];
  snprintf(fam, sizeof(fam), "stag_dslash_%s_n%d", pn[ps], nrhs);
  qllg_tm_begin(fam);
  int rc = qllg_k_stag_dslash(ps, pl, &A);
  qllg_tm_end();
  return rc;
}

static int
dslash_half(qllg_stag *S, int ps, int pl, int out_parity, int nrhs, const void *in,
            const void *self, void *out, int mode, const double *a, double a0, double b,
            double *norm_out, double *norm_self, const int *active, const int *done)
{
  return dslash_half_x(S, ps, pl, out_parity, nrhs, in, self, out, mode, a, a0, b, norm_out,
                       norm_self, active, done, 0, 0);
}

/* host [V][6] parity block(s) <-> device single-rhs block */
static int
upload_block(qllg_stag *S, int prec, void *dev, const void *host, int dbl, int site0, int nsites)
{
  size_t bytes = (dbl ? 8 : 4)*6*(size_t)nsites;
  void *stage = qllg_stage(bytes);
  if(!stage) return -1;
  if(qllg_h2d(stage, (const char *)host + (dbl ? 8 : 4)*6*(size_t)site0, bytes)) return -1;
  return qllg_k_spinor_from_aos(prec, dev, stage, dbl, nsites, 3, 1, 0);
}

static int
download_block(qllg_stag *S, int prec, const void *dev, void *host, int dbl, int site0, int nsites)
{
  size_t bytes = (dbl ? 8 : 4)*6*(size_t)nsites;
  void *stage = qllg_stage(bytes);
  if(!stage) return -1;
  if(qllg_k_spinor_to_aos(prec, dev, stage, dbl, nsites, 3, 1, 0)) return -1;
  return qllg_d2h((char *)host + (dbl ? 8 : 4)*6*(size_t)site0, stage, bytes);
}

/* ------------------------------------------------------------ dslash2 */

int
qllg_stag_dslash(qllg_stag *S, void *x, double mass, const void *y, const char *sub)
{
  int prec = S->master, dbl = (prec == QLLG_F64);
  int Vh = S->g.Vh;
  size_t vb = vec_bytes(S, prec, 1);
  void *ye = ws_get(S, WS_IO, 4*vb);
  if(!ye) return -1;
  void *yo = (char *)ye + vb, *xe = (char *)ye + 2*vb, *xo = (char *)ye + 3*vb;
  int doe = !(sub && sub[0] == 'o'), doo = !(sub && sub[0] == 'e');
  int all = doe && doo;
  /* inputs: the opposite parity of each output, plus self for the mass term */
  if((doe && upload_block(S, prec, yo, y, dbl, Vh, Vh)) ||
     (doo && upload_block(S, prec, ye, y, dbl, 0, Vh))) return -1;
  if(all && mass != 0) {
    /* x = mass*y + D y, accumulated onto mass*y like VeqRtimesV then the slots */
    if(dslash_half(S, prec, prec, 0, 1, yo, ye, xe, 1, NULL, mass, 1, NULL, NULL, NULL, NULL) ||
       dslash_half(S, prec, prec, 1, 1, ye, yo, xo, 1, NULL, mass, 1, NULL, NULL, NULL, NULL))
      return -1;
  } else {
    if(doe && dslash_half(S, prec, prec, 0, 1, yo, NULL, xe, 0, NULL, 0, 1, NULL, NULL, NULL, NULL))
      return -1;
    if(doo && dslash_half(S, prec, prec, 1, 1, ye, NULL, xo, 0, NULL, 0, 1, NULL, NULL, NULL, NULL))
      return -1;
  }
  if(doe && download_block(S, prec, xe, x, dbl, 0, Vh)) return -1;
  if(doo && download_block(S, prec, xo, x, dbl, Vh, Vh)) return -1;
  return 0;
}

/* ------------------------------------------------------------ CG */

/* Ap = m^2 p - D_eo D_oe p (all rhs, masses from S->sc->mass2) */
static int
apply_normal(qllg_stag *S, int ps, int pl, int nrhs, const void *p, void *v, void *Ap,
             double *vnorm, double *pnorm, const int *active, const int *done)
{
  if(dslash_half(S, ps, pl, 1, nrhs, p, NULL, v, 0, NULL, 0, 1, vnorm, NULL, active, done))
    return -1;
  return dslash_half(S, ps, pl, 0, nrhs, v, p, Ap, 2, S->sc->mass2, 0, -1, NULL, pnorm,
                     active, done);
}

/* t = m^2 x - D_eo D_oe x for the rhs flagged in active only (the FP64
 * reliable update: threads over the flagged rhs, so its cost follows how
 * many are flagged); every launch returns at once when *done is set */
static int
apply_normal_flagged(qllg_stag *S, int prec, int nrhs, const void *x, void *w, void *t,
                     const int *active, int eq, const int *done)
{
  if(dslash_half_x(S, prec, prec, 1, nrhs, x, NULL, w, 0, NULL, 0, 1, NULL, NULL, active, done,
                   1, eq)) return -1;
  return dslash_half_x(S, prec, prec, 0, nrhs, w, x, t, 2, S->sc->mass2, 0, -1, NULL, NULL,
                       active, done, 1, eq);
}

/* one CG iteration in three launches (cgSolveT, lib/cg.c:77-115):
 *   p += r/|r|^2 with |p|^2;  v = D_oe p with |v|^2;
 *   Ap = m^2 p - D_eo v in registers, x += a p, r -= a Ap, |r|^2, bookkeeping
 * ps: precision of p, v, r; pl: of the links; x is FP64 for FP64 spinors,
 * else FP32; mixed selects the reliable-update bookkeeping */
static int
cg_iteration(qllg_stag *S, int ps, int pl, int nrhs, void *x, void *r, void *p, void *v, int mixed)
{
  qllg_cg_scalars *sc = S->sc;
  if(qllg_k_cg_update_p_norm(ps, p, r, S->g.Vh, nrhs, sc, &S->rb)) return -1;
  if(dslash_half(S, ps, pl, 1, nrhs, p, NULL, v, 0, NULL, 0, 1, sc->vnorm, NULL, sc->active,
                 &sc->done)) return -1;
  if(ensure_links(S, pl)) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = S->g;
  A.out_parity = 0;
  A.nrhs = nrhs;
  A.nslots = S->nslots;
  A.fb = S->fb;
  A.links = S->links[pl];
  A.lscale = S->lscale;
  A.in = v;
  A.self = p;
  A.mode = 3;
  A.a = sc->mass2;
  A.b = -1;
  A.active = sc->active;
  A.done = &sc->done;
  A.rb = &S->rb;
  A.x = x;
  A.r = r;
  A.sc = sc;
  A.mixed = mixed;
  static const char *pn[3] = {"f64", "f32", "i16"};
  char fam[40];
  snprintf(fam, sizeof(fam), "stag_cg_fused_%s_n%d", pn[ps], nrhs);
  qllg_tm_begin(fam);
  int rc = qllg_k_stag_dslash(ps, pl, &A);
  qllg_tm_end();
  return rc;
}

static int
push_scalars(qllg_stag *S)
{
  return qllg_check_cuda(cudaMemcpyAsync(S->sc, S->hsc, sizeof(qllg_cg_scalars),
                                         cudaMemcpyHostToDevice, qllg_stream()), "push scalars");
}

static int
pull_scalars(qllg_stag *S)
{
  if(qllg_check_cuda(cudaMemcpyAsync(S->hsc, S->sc, sizeof(qllg_cg_scalars),
                                     cudaMemcpyDeviceToHost, qllg_stream()), "pull scalars"))
    return -1;
  return qllg_sync();
}

static int
pull_done(qllg_stag *S)
{
  if(qllg_check_cuda(cudaMemcpyAsync(&S->hsc->done, &S->sc->done, sizeof(int),
                                     cudaMemcpyDeviceToHost, qllg_stream()), "pull done"))
    return -1;
  if(qllg_sync()) return -1;
  return S->hsc->done;
}

/* ------------------------------------------------ solver loop driver */

static int
issue_iteration(qllg_stag *S, const iter_ctx *c)
{
  qllg_cg_scalars *sc = S->sc;
  int Vh = S->g.Vh;
  if(cg_iteration(S, c->ps, c->pl, c->nrhs, c->x, c->r, c->p, c->v, c->mixed)) return -1;
  if(!c->mixed) return 0;
  /* reliable update of the flagged rhs; every launch returns at once when
   * no rhs is flagged.  In a captured loop the block is the body of a
   * conditional IF node, taken only in the iterations that flag an update */
  const int cond = qllg_capturing() && qllg_get_param("graph_ru_if") != 0;
  unsigned long long n1 = 0;
  if(cond) {
    unsigned long long h;
    if(qllg_capture_cond(&h) || qllg_k_ru_cond(h, &sc->no_ru, &sc->ru_trips) ||
       qllg_capture_if_begin(h)) return -1;
    n1 = qllg_launch_count();
  }
  if(qllg_k_mcg_accum(QLLG_F32, c->x64, c->x, Vh, 3, c->nrhs, sc)) return -1;
  if(qllg_get_param("ru_compact") != 0) {
    if(c->xdf) {
      /* intermediate updates (ru 1) in double-float: x64 to (hi, lo)
       * pairs, A x in the FP32 pipes, t back to FP64 in place; the final
       * candidates (ru 2) below in FP64 */
      if(qllg_k_spinor_df(1, c->xdf, c->x64, Vh, 3, c->nrhs, sc->ru, 1, &sc->no_ru) ||
         apply_normal_flagged(S, QLLG_DF, c->nrhs, c->xdf, c->w64, c->t64, sc->ru, 1, &sc->no_ru) ||
         qllg_k_spinor_df(0, c->t64, c->t64, Vh, 3, c->nrhs, sc->ru, 1, &sc->no_ru)) return -1;
    }
    if(apply_normal_flagged(S, QLLG_F64, c->nrhs, c->x64, c->w64, c->t64, sc->ru, c->xdf ? 2 : 0,
                            &sc->no_ru)) return -1;
  } else if(apply_normal(S, QLLG_F64, QLLG_F64, c->nrhs, c->x64, c->w64, c->t64, NULL, NULL,
                         sc->ru, &sc->no_ru)) return -1;
  if(qllg_k_mcg_residual(QLLG_F32, c->r64, c->r, c->b, c->t64, Vh, 3, c->nrhs, 0, sc, &S->rb))
    return -1;
  if(c->reortho && qllg_k_mcg_reortho(c->ps, c->p, c->r, Vh, c->nrhs, sc, &S->rb)) return -1;
  if(cond) {
    S->cap_ifbody = (int)(qllg_launch_count() - n1);
    if(qllg_capture_if_end()) return -1;
  }
  return 0;
}

/* a CUDA graph whose conditional WHILE node repeats one captured iteration
 * until the done flag is set (or the trip cap is reached) */
static cudaGraphExec_t
loop_graph(qllg_stag *S, const iter_ctx *c)
{
  long key[11] = {c->mixed, c->ps, c->pl, c->nrhs, c->reortho, (long)c->x, (long)c->b,
                  (long)c->x64, (long)S->ws_gen, (long)c->xdf,
                  2 + (qllg_get_param("graph_ru_if") != 0)};
  for(int i=0; i<6; i++)
    if(S->graphs[i].exec && !memcmp(S->graphs[i].key, key, sizeof(key))) {
      S->graph_body = S->graphs[i].body;
      S->graph_ifbody = S->graphs[i].ifbody;
      return S->graphs[i].exec;
    }
  S->cap_ifbody = 0;
  unsigned long long n0 = qllg_launch_count();
  cudaGraph_t g = NULL;
  cudaGraphExec_t exec = NULL;
  cudaGraphConditionalHandle h;
  cudaGraphNode_t node;
  struct cudaGraphNodeParams np;
  if(qllg_check_cuda(cudaGraphCreate(&g, 0), "graph create")) return NULL;
  if(qllg_check_cuda(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault),
                     "conditional handle")) goto fail;
  memset(&np, 0, sizeof(np));
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  if(qllg_check_cuda(cudaGraphAddNode(&node, g, NULL, NULL, 0, &np), "conditional node")) goto fail;
  if(qllg_capture_begin(np.conditional.phGraph_out[0])) goto fail;
  {
    int rc = issue_iteration(S, c);
    rc |= qllg_k_loop_cond((unsigned long long)h, &S->sc->done, &S->sc->loops,
                           &S->sc->loop_limit);
    rc |= qllg_capture_end(np.conditional.phGraph_out[0]);
    if(rc) goto fail;
  }
  if(qllg_check_cuda(cudaGraphInstantiate(&exec, g, 0), "graph instantiate")) goto fail;
  cudaGraphDestroy(g);
  {
    /* the capture counted the body's launches without running them; those
     * of the conditional block run only in the trips that take it */
    int all = (int)(qllg_launch_count() - n0);
    qllg_launch_adjust(-(long long)all);
    int i = S->ngraph_next;
    S->ngraph_next = (i + 1) % 6;
    if(S->graphs[i].exec) cudaGraphExecDestroy(S->graphs[i].exec);
    memcpy(S->graphs[i].key, key, sizeof(key));
    S->graphs[i].exec = exec;
    S->graphs[i].body = all - S->cap_ifbody;
    S->graphs[i].ifbody = S->cap_ifbody;
    S->graph_body = all - S->cap_ifbody;
    S->graph_ifbody = S->cap_ifbody;
  }
  return exec;
fail:
  if(qllg_capturing()) qllg_capture_end(np.conditional.phGraph_out[0]);
  if(g) cudaGraphDestroy(g);
  return NULL;
}

/* run iterations until every rhs is done: one graph launch, or (timing
 * enabled, or graphs switched off) batches of launches with a host check of
 * the done flag after each batch */
int qllg_timing_on(void);

/* after a graph-launched solve: the kernels its trips ran (sc->loops) */
static void
count_graph_trips(qllg_stag *S)
{
  if(S->graph_body)
    qllg_launch_adjust((long long)S->graph_body*S->hsc->loops +
                       (long long)S->graph_ifbody*S->hsc->ru_trips);
  S->graph_body = 0;
  S->graph_ifbody = 0;
}

/* the persistent CG (one cooperative launch for the whole loop) takes the
 * solve when the lattice is small enough for launch latency to dominate
 * (sites x rhs up to persistent_max) and the precisions are ones it has:
 * FP64 iterations, or FP32 iterations and links with FP64 reliable
 * updates (intermediate ones in FP64 too, not double-float) */
static int
persistent_ok(const qllg_stag *S, const iter_ctx *c)
{
  if(qllg_get_param("persistent") == 0) return 0;
  if((double)S->g.Vh*c->nrhs > qllg_get_param("persistent_max")) return 0;
  if(c->mixed) return c->ps == QLLG_F32 && c->pl == QLLG_F32 && S->links[QLLG_F64];
  return c->ps == QLLG_F64 && c->pl == QLLG_F64;
}

static int
run_persistent(qllg_stag *S, const iter_ctx *c, int maxits)
{
  /* control words: barrier arrivals and generation, the error flag */
  unsigned *ctl = ws_get(S, WS_CGP, 4*sizeof(unsigned));
  /* the second p buffer of the persistent loop (the Ap workspace, unused
   * by this path) */
  void *p2 = ws_get(S, WS_AP, vec_bytes(S, c->ps, c->nrhs));
  if(!ctl || !p2) return -1;
  if(qllg_check_cuda(cudaMemsetAsync(ctl, 0, 4*sizeof(unsigned), qllg_stream()),
                     "persistent CG: control words")) return -1;
  qllg_cgp_args a;
  memset(&a, 0, sizeof(a));
  a.g = S->g;
  a.nslots = S->nslots;
  a.fb = S->fb;
  a.mixed = c->mixed;
  a.reortho = c->reortho;
  a.nrhs = c->nrhs;
  a.links = S->links[c->pl];
  a.links64 = S->links[QLLG_F64];
  a.lscale = S->lscale;
  a.x = c->x; a.r = c->r; a.p = c->p; a.v = c->v;
  a.x64 = c->x64; a.r64 = c->r64; a.w64 = c->w64;
  a.p2 = p2;
  a.b = c->b;
  a.sc = S->sc;
  a.partial = S->rb.partial;
  a.bar = ctl;
  a.err = (int *)(ctl + 2);
  a.poll_limit = (long long)qllg_get_param("wait_polls");
  a.extra = (int)qllg_get_param("cg_barrier_extra");
  a.trips = maxits + 2;
  /* the launch takes at most 128 blocks, whose partials fit the
   * operator's reduction buffer (checked here, before the launch) */
  if(qllg_cgp_partial_bytes(128) > sizeof(double)*2*QLLG_MAXRHS*(size_t)S->rb.maxblocks) {
    qllg_set_error("persistent CG: the reduction buffer is too small");
    return -1;
  }
  int grid = 0;
  if(qllg_k_cg_persistent(&a, &grid)) return -1;
  int err = 0;
  if(qllg_check_cuda(cudaMemcpyAsync(&err, ctl + 2, sizeof(int), cudaMemcpyDeviceToHost,
                                     qllg_stream()), "persistent CG: error flag") ||
     qllg_sync()) return -1;
  if(err) {
    qllg_set_error("persistent CG: a grid barrier wait ran out (%lld polls)", a.poll_limit);
    return -1;
  }
  S->used_persistent = 1;
  return 0;
}

static int
run_loop(qllg_stag *S, const iter_ctx *c, int maxits)
{
  S->graph_body = 0;
  S->used_persistent = 0;
  if(persistent_ok(S, c)) return run_persistent(S, c, maxits);
  if(qllg_get_param("graph") != 0 && !qllg_timing_on()) {
    /* one iteration launched directly first: every kernel of the body is
     * then loaded before the capture starts */
    if(issue_iteration(S, c)) return -1;
    cudaGraphExec_t exec = loop_graph(S, c);
    if(!exec) return -1;
    return qllg_check_cuda(cudaGraphLaunch(exec, qllg_stream()), "graph launch");
  }
  int issued = 0, batch = (int)qllg_get_param("poll");
  if(batch < 1) batch = 1;
  while(issued < maxits + 2) {
    for(int it=0; it<batch; it++) if(issue_iteration(S, c)) return -1;
    issued += batch;
    int d = pull_done(S);
    if(d < 0) return -1;
    if(d) break;
    if(batch < 64) batch *= 2;
  }
  return 0;
}

/* plain CG of cgSolveT in one precision on device vectors x, b (even sites,
 * nrhs rhs).  Returns the largest iteration count, fills hsc. */
static int
cg_plain(qllg_stag *S, int prec, int nrhs, void *x, const void *b, const double mass[],
         double rsq, int maxits)
{
  if(ensure_links(S, prec)) return -1;
  size_t vb = vec_bytes(S, prec, nrhs);
  void *r = ws_get(S, WS_R, vb), *p = ws_get(S, WS_P, vb);
  void *v = ws_get(S, WS_V, vb);
  if(!r || !p || !v) return -1;
  memset(S->hsc, 0, sizeof(qllg_cg_scalars));
  for(int i=0; i<nrhs; i++) {
    S->hsc->mass2[i] = mass[i]*mass[i];
    S->hsc->rsq_stop[i] = rsq;
  }
  S->hsc->maxits = maxits;
  S->hsc->loop_limit = maxits + 2;
  if(push_scalars(S)) return -1;
  int Vh = S->g.Vh;
  qllg_cg_scalars *sc = S->sc;
  if(qllg_k_cg_init(prec, x, r, p, b, Vh, 3, nrhs, sc, &S->rb)) return -1;
  iter_ctx c;
  memset(&c, 0, sizeof(c));
  c.ps = c.pl = prec;
  c.nrhs = nrhs;
  c.x = x; c.r = r; c.p = p; c.v = v;
  c.b = b;
  if(run_loop(S, &c, maxits)) return -1;
  if(pull_scalars(S)) return -1;
  count_graph_trips(S);
  int its = 0;
  for(int i=0; i<nrhs; i++) if(S->hsc->iters[i] > its) its = S->hsc->iters[i];
  return its;
}

/* |b - A x|^2 / |b|^2 per rhs in FP64 (x, b FP64 device vectors) */
static int
true_residual(qllg_stag *S, int nrhs, const void *x, const void *b, double *out)
{
  if(ensure_links(S, QLLG_F64)) return -1;
  size_t vb = vec_bytes(S, QLLG_F64, nrhs);
  void *t = ws_get(S, WS_T64, vb), *v = ws_get(S, WS_V64, vb);
  if(!t || !v) return -1;
  if(apply_normal(S, QLLG_F64, QLLG_F64, nrhs, x, v, t, NULL, NULL, NULL, NULL)) return -1;
  /* t = b - t */
  if(qllg_k_axpby(QLLG_F64, t, QLLG_F64, b, NULL, -1.0, NULL, 1.0, S->g.Vh, 3, nrhs, NULL))
    return -1;
  double *dn = &S->sc->tmp[0];
  if(qllg_k_norm2(QLLG_F64, t, S->g.Vh, 3, nrhs, dn, &S->rb)) return -1;
  double num[QLLG_MAXRHS], den[QLLG_MAXRHS];
  if(qllg_d2h(num, dn, sizeof(double)*nrhs)) return -1;
  if(qllg_k_norm2(QLLG_F64, b, S->g.Vh, 3, nrhs, dn, &S->rb)) return -1;
  if(qllg_d2h(den, dn, sizeof(double)*nrhs)) return -1;
  for(int i=0; i<nrhs; i++) out[i] = den[i] > 0 ? num[i]/den[i] : 0;
  return 0;
}

/* info->true_rsq after a solve on FP64 vectors.  A mixed solve stops every
 * rhs on a reliable update, whose FP64 residual b - A x64 is that of the
 * returned x (left in rsq by the residual kernel), so only the FP64 solve
 * recomputes it */
static int
fill_true_rsq(qllg_stag *S, int mode, int nrhs, const void *x, const void *b, qllg_solve_info *info)
{
  if(mode == QLLG_SOLVE_MIXED_SINGLE || mode == QLLG_SOLVE_MIXED_HALF) {
    for(int i=0; i<nrhs; i++) info->true_rsq[i] = info->rsq[i];
    return 0;
  }
  return true_residual(S, nrhs, x, b, info->true_rsq);
}

/* mixed-precision reliable-update CG on FP64 device vectors x64, b (even
 * sites, nrhs rhs): sloppy vectors in ps storage (p, v, Ap, r) and px
 * (solution increment), links in pl */
static int
cg_mixed(qllg_stag *S, int ps, int px, int pl, int nrhs, void *x64, const void *b,
         const double mass[], double rsq, int maxits, double delta, int guess)
{
  if(ensure_links(S, pl) || ensure_links(S, QLLG_F64)) return -1;
  /* p, v: Dslash operands in ps; r and the solution increment in FP32 */
  size_t vs = vec_bytes(S, ps, nrhs), vx = vec_bytes(S, QLLG_F32, nrhs);
  size_t v64 = vec_bytes(S, QLLG_F64, nrhs);
  void *rs = ws_get(S, WS_R, vx), *p = ws_get(S, WS_P, vs);
  void *v = ws_get(S, WS_V, vs), *xs = ws_get(S, WS_X, vx);
  void *r64 = ws_get(S, WS_R64, v64), *t64 = ws_get(S, WS_T64, v64), *w64 = ws_get(S, WS_V64, v64);
  if(!rs || !p || !v || !xs || !r64 || !t64 || !w64) return -1;
  (void)px;
  memset(S->hsc, 0, sizeof(qllg_cg_scalars));
  for(int i=0; i<nrhs; i++) {
    S->hsc->mass2[i] = mass[i]*mass[i];
    S->hsc->rsq_stop[i] = rsq;
  }
  S->hsc->maxits = maxits;
  S->hsc->loop_limit = maxits + 2;
  S->hsc->delta2 = delta*delta;
  if(push_scalars(S)) return -1;
  int Vh = S->g.Vh;
  qllg_cg_scalars *sc = S->sc;
  if(guess) {
    /* x64 holds an initial guess: start from r = b - A x64 (FP64) */
    if(apply_normal(S, QLLG_F64, QLLG_F64, nrhs, x64, w64, t64, NULL, NULL, NULL, NULL) ||
       qllg_k_mcg_init_guess(ps, r64, xs, rs, p, b, t64, Vh, nrhs, sc, &S->rb)) return -1;
  } else if(qllg_k_mcg_init(QLLG_F32, ps, x64, r64, xs, rs, p, b, Vh, nrhs, sc, &S->rb)) {
    return -1;
  }
  iter_ctx c;
  memset(&c, 0, sizeof(c));
  c.mixed = 1;
  c.ps = ps; c.pl = pl; c.nrhs = nrhs;
  c.reortho = qllg_get_param("reortho") != 0;
  c.x = xs; c.r = rs; c.p = p; c.v = v;
  c.x64 = x64; c.r64 = r64; c.t64 = t64; c.w64 = w64;
  c.b = b;
  if(qllg_get_param("ru_df") != 0 && qllg_get_param("ru_compact") != 0) {
    if(ensure_links(S, QLLG_DF) || !(c.xdf = ws_get(S, WS_XDF, v64))) return -1;
  }
  if(run_loop(S, &c, maxits)) return -1;
  if(pull_scalars(S)) return -1;
  count_graph_trips(S);
  int its = 0;
  for(int i=0; i<nrhs; i++) if(S->hsc->iters[i] > its) its = S->hsc->iters[i];
  return its;
}

/* ---------------------------------------------- continuous batching */
/* A batch is the FP32 mixed CG (FP64 reliable updates) over all
 * QLLG_MAXRHS columns of the operator's workspaces.  Columns are admitted
 * (x = 0, r = b, own mass and tolerance) and retired one by one between
 * chunks; a chunk is one launch of the graph-captured iteration loop with a
 * trip limit, so the columns already running never stop for an admission.
 * Everything is asynchronous on the library stream except retire, which
 * waits for its copy. */

size_t
qllg_batch_bytes(const qllg_stag *S)
{
  const int n = QLLG_MAXRHS;
  /* rs, p, v, xs in FP32; r64, t64, w64, x64, b in FP64 (and the
   * double-float copy of x64 for the intermediate reliable updates); one
   * column of staging */
  const int ndf = qllg_get_param("ru_df") != 0 && qllg_get_param("ru_compact") != 0;
  return 4*vec_bytes(S, QLLG_F32, n) + (5 + ndf)*vec_bytes(S, QLLG_F64, n) + 48*(size_t)S->g.Vh;
}

int
qllg_batch_init(qllg_stag *S, int maxits)
{
  const int n = QLLG_MAXRHS;
  if(ensure_links(S, QLLG_F32) || ensure_links(S, QLLG_F64)) return -1;
  size_t vx = vec_bytes(S, QLLG_F32, n), v64 = vec_bytes(S, QLLG_F64, n);
  iter_ctx *c = &S->bctx;
  memset(c, 0, sizeof(*c));
  c->mixed = 1;
  c->ps = QLLG_F32;
  c->pl = f32_links(S);
  c->nrhs = n;
  c->reortho = qllg_get_param("reortho") != 0;
  c->r = ws_get(S, WS_R, vx);
  c->p = ws_get(S, WS_P, vx);
  c->v = ws_get(S, WS_V, vx);
  c->x = ws_get(S, WS_X, vx);
  c->r64 = ws_get(S, WS_R64, v64);
  c->t64 = ws_get(S, WS_T64, v64);
  c->w64 = ws_get(S, WS_V64, v64);
  c->x64 = ws_get(S, WS_X64, v64);
  c->b = ws_get(S, WS_B, v64);
  if(!c->r || !c->p || !c->v || !c->x || !c->r64 || !c->t64 || !c->w64 || !c->x64 || !c->b)
    return -1;
  if(qllg_get_param("ru_df") != 0 && qllg_get_param("ru_compact") != 0) {
    if(ensure_links(S, QLLG_DF) || !(c->xdf = ws_get(S, WS_XDF, v64))) return -1;
  }
  if(!S->bstage && !(S->bstage = qllg_dmalloc(48*(size_t)S->g.Vh))) return -1;
  if(!S->bev && qllg_check_cuda(cudaEventCreateWithFlags(&S->bev, cudaEventDisableTiming),
                                "batch event")) return -1;
  void *zero[] = {c->r, c->p, c->v, c->x};
  for(int i=0; i<4; i++)
    if(qllg_check_cuda(cudaMemsetAsync(zero[i], 0, vx, qllg_stream()), "batch clear")) return -1;
  void *zero64[] = {c->r64, c->t64, c->w64, c->x64, (void *)c->b};
  for(int i=0; i<5; i++)
    if(qllg_check_cuda(cudaMemsetAsync(zero64[i], 0, v64, qllg_stream()), "batch clear")) return -1;
  double delta = qllg_get_param("reliable_delta_single");
  memset(S->hsc, 0, sizeof(qllg_cg_scalars));
  S->hsc->maxits = maxits;
  S->hsc->delta2 = delta*delta;
  S->hsc->done = 1;
  S->hsc->no_ru = 1;
  if(push_scalars(S)) return -1;
  /* one iteration with every column idle (every launch returns at once)
   * loads the loop body's kernels before the graph is captured */
  if(issue_iteration(S, c)) return -1;
  S->batch_on = 1;
  return 0;
}

/* columns cols[i] take right-hand side src[i] (host, [Vh][6] FP64, the
 * even sites) with mass mass[i] and stopping |r|/|b| < tol[i] */
int
qllg_batch_admit(qllg_stag *S, int ncol, const int cols[], const double mass[], const double tol[],
                 const double *const src[])
{
  if(!S->batch_on) { qllg_set_error("batch_admit: batch not initialised"); return -1; }
  const int Vh = S->g.Vh;
  iter_ctx *c = &S->bctx;
  qllg_admit_args ad;
  memset(&ad, 0, sizeof(ad));
  for(int i=0; i<ncol; i++) {
    int col = cols[i];
    if(col < 0 || col >= QLLG_MAXRHS) { qllg_set_error("batch_admit: column %d", col); return -1; }
    if(qllg_h2d(S->bstage, src[i], 48*(size_t)Vh)) return -1;
    if(qllg_k_column_from_aos((void *)c->b, S->bstage, Vh, QLLG_MAXRHS, col)) return -1;
    ad.mask[col] = 1;
    ad.mass2[col] = mass[i]*mass[i];
    ad.tol2[col] = tol[i]*tol[i];
  }
  return qllg_k_mcg_admit(QLLG_F32, c->x64, c->r64, c->x, c->r, c->p, c->b, Vh, QLLG_MAXRHS, S->sc,
                          &ad, &S->rb);
}

/* at most iters more iterations of every running column; then the scalars
 * are copied back and the chunk's event recorded */
int
qllg_batch_launch(qllg_stag *S, int iters)
{
  if(!S->batch_on) { qllg_set_error("batch_launch: batch not initialised"); return -1; }
  if(qllg_k_chunk_limit(&S->sc->loops, &S->sc->loop_limit, iters)) return -1;
  if(qllg_get_param("graph") != 0 && !qllg_timing_on()) {
    cudaGraphExec_t exec = loop_graph(S, &S->bctx);
    if(!exec) return -1;
    if(qllg_check_cuda(cudaGraphLaunch(exec, qllg_stream()), "batch graph launch")) return -1;
  } else {
    for(int i=0; i<iters; i++) if(issue_iteration(S, &S->bctx)) return -1;
  }
  if(qllg_check_cuda(cudaMemcpyAsync(S->hsc, S->sc, sizeof(qllg_cg_scalars),
                                     cudaMemcpyDeviceToHost, qllg_stream()), "batch scalars"))
    return -1;
  return qllg_check_cuda(cudaEventRecord(S->bev, qllg_stream()), "batch event");
}

/* 1 when the last chunk (and its scalar copy) has finished, 0 while it runs */
int
qllg_batch_poll(qllg_stag *S)
{
  cudaError_t e = cudaEventQuery(S->bev);
  if(e == cudaSuccess) return 1;
  if(e == cudaErrorNotReady) return 0;
  return qllg_check_cuda(e, "batch poll") ? -1 : 0;
}

/* the scalars as of the last finished chunk (per column: active, iters,
 * rsq, bsq, nru) */
const qllg_cg_scalars *
qllg_batch_scalars(const qllg_stag *S)
{
  return S->hsc;
}

/* copy column col's FP64 solution to out (host, [Vh][6]); waits for it */
int
qllg_batch_retire(qllg_stag *S, int col, double *out)
{
  const int Vh = S->g.Vh;
  if(qllg_k_column_to_aos(S->bctx.x64, S->bstage, Vh, QLLG_MAXRHS, col)) return -1;
  return qllg_d2h(out, S->bstage, 48*(size_t)Vh);
}

static int
valid_nrhs(int nrhs)
{
  return nrhs == 1 || nrhs == 2 || nrhs == 4 || nrhs == 8 || nrhs == 16;
}

/* nrhs padded to the kernel batch sizes; padding rhs have b = 0 and start
 * inactive */
static int
pad_nrhs(int nrhs)
{
  int n = 1;
  while(n < nrhs) n *= 2;
  return n;
}

static int
solve_dev(qllg_stag *S, int nrhs, void *x, const void *b, const double mass[], double rsq,
          int maxits, int mode, qllg_solve_info *info)
{
  if(!valid_nrhs(nrhs)) { qllg_set_error("solve: nrhs %d not in {1,2,4,8,16}", nrhs); return -1; }
  if(rsq < 0) rsq = -rsq;
  cudaEventRecord(S->ev0, qllg_stream());
  int its;
  switch(mode) {
  case QLLG_SOLVE_DOUBLE:
    its = cg_plain(S, QLLG_F64, nrhs, x, b, mass, rsq, maxits);
    break;
  case QLLG_SOLVE_SINGLE:
    its = cg_plain(S, QLLG_F32, nrhs, x, b, mass, rsq, maxits);
    break;
  case QLLG_SOLVE_MIXED_HALF: {
    /* half_split: 0 16-bit Dslash operands and links, 1 16-bit links with
     * FP32 operands, 2 FP32 links with 16-bit operands */
    const int split = (int)qllg_get_param("half_split");
    const int ps = split == 1 ? QLLG_F32 : QLLG_I16, pl = split == 2 ? QLLG_F32 : QLLG_I16;
    its = cg_mixed(S, ps, QLLG_F32, pl, nrhs, x, b, mass, rsq, maxits,
                   qllg_get_param(split == 1 ? "reliable_delta_single" : "reliable_delta"), 0);
    break;
  }
  case QLLG_SOLVE_MIXED_SINGLE:
    its = cg_mixed(S, QLLG_F32, QLLG_F32, f32_links(S), nrhs, x, b, mass, rsq, maxits,
                   qllg_get_param("reliable_delta_single"), 0);
    break;
  default:
    qllg_set_error("solve: unknown mode %d", mode);
    return -1;
  }
  cudaEventRecord(S->ev1, qllg_stream());
  if(its < 0) return -1;
  if(info) {
    memset(info, 0, sizeof(*info));
    cudaEventSynchronize(S->ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, S->ev0, S->ev1);
    info->seconds = ms*1e-3;
    info->total_iters = its;
    for(int i=0; i<nrhs; i++) {
      info->iters[i] = S->hsc->iters[i];
      info->rsq[i] = S->hsc->bsq[i] > 0 ? S->hsc->rsq[i]/S->hsc->bsq[i] : 0;
      info->reliable_updates += S->hsc->nru[i];
    }
  }
  return its;
}

int
qllg_stag_solve_device(qllg_stag *S, int nrhs, void *x_dev, const void *b_dev,
                       const double mass[], double rsq, int maxits, int mode,
                       qllg_solve_info *info)
{
  if(S->master != QLLG_F64 && mode != QLLG_SOLVE_SINGLE) {
    qllg_set_error("solve_device: a float operator supports QLLG_SOLVE_SINGLE only");
    return -1;
  }
  if(mode == QLLG_SOLVE_SINGLE) {
    /* device API vectors are FP64: convert around an FP32 solve */
    size_t v32 = vec_bytes(S, QLLG_F32, nrhs);
    void *b32 = ws_get(S, WS_B, v32), *x32 = ws_get(S, WS_OUT, v32);
    if(!b32 || !x32) return -1;
    if(qllg_k_spinor_convert(QLLG_F32, b32, QLLG_F64, b_dev, S->g.Vh, 3, nrhs, NULL)) return -1;
    int its = solve_dev(S, nrhs, x32, b32, mass, rsq, maxits, mode, info);
    if(its < 0) return -1;
    if(qllg_k_spinor_convert(QLLG_F64, x_dev, QLLG_F32, x32, S->g.Vh, 3, nrhs, NULL)) return -1;
    return its;
  }
  int its = solve_dev(S, nrhs, x_dev, b_dev, mass, rsq, maxits, mode, info);
  if(its >= 0 && info && S->master == QLLG_F64) {
    if(fill_true_rsq(S, mode, nrhs, x_dev, b_dev, info)) return -1;
  }
  return its;
}

void *
qllg_stag_vec_alloc(qllg_stag *S, int nrhs)
{
  return qllg_dmalloc(vec_bytes(S, QLLG_F64, nrhs));
}

void
qllg_stag_vec_free(void *v)
{
  qllg_sync();
  qllg_dfree(v);
}

/* host arrays [V][6] of the operator's precision, even half */
static int
vec_upload(qllg_stag *S, int prec, void *v_dev, int nrhs, void *const h[], int dbl)
{
  int Vh = S->g.Vh;
  size_t blk = (dbl ? 8 : 4)*6*(size_t)Vh;
  char *stage = qllg_stage(blk*nrhs);
  if(!stage) return -1;
  for(int r=0; r<nrhs; r++) if(qllg_h2d(stage + blk*r, h[r], blk)) return -1;
  return qllg_k_spinor_from_aos(prec, v_dev, stage, dbl, Vh, 3, nrhs, 6*(size_t)Vh);
}

static int
vec_download(qllg_stag *S, int prec, const void *v_dev, int nrhs, void *const h[], int dbl)
{
  int Vh = S->g.Vh;
  size_t blk = (dbl ? 8 : 4)*6*(size_t)Vh;
  char *stage = qllg_stage(blk*nrhs);
  if(!stage) return -1;
  if(qllg_k_spinor_to_aos(prec, v_dev, stage, dbl, Vh, 3, nrhs, 6*(size_t)Vh)) return -1;
  for(int r=0; r<nrhs; r++)
    if(qllg_d2h_async(h[r], stage + blk*r, blk)) return -1;
  return qllg_sync();
}

int
qllg_stag_vec_upload(qllg_stag *S, void *v_dev, int nrhs, void *const h[])
{
  return vec_upload(S, QLLG_F64, v_dev, nrhs, h, S->master == QLLG_F64);
}

int
qllg_stag_vec_download(qllg_stag *S, const void *v_dev, int nrhs, void *const h[])
{
  return vec_download(S, QLLG_F64, v_dev, nrhs, h, S->master == QLLG_F64);
}

/* host-array solve; post_scale: x *= mass (solve2's scaling) when set */
static int
stag_solve_host(qllg_stag *S, int nrhs, void *const x[], void *const b[], const double mass[],
                double rsq, int maxits, int mode, qllg_solve_info *info, int post_scale,
                const double *scale_real)
{
  if(nrhs < 1 || nrhs > QLLG_MAXRHS) { qllg_set_error("solve: nrhs %d", nrhs); return -1; }
  int n = pad_nrhs(nrhs);
  int dbl = S->master == QLLG_F64;
  int prec = (mode == QLLG_SOLVE_SINGLE) ? QLLG_F32 : QLLG_F64;
  if(!dbl && mode != QLLG_SOLVE_SINGLE) {
    qllg_set_error("solve: a float operator supports QLLG_SOLVE_SINGLE only");
    return -1;
  }
  size_t vb = vec_bytes(S, prec, n);
  void *bd = ws_get(S, WS_B, vb), *xd = ws_get(S, WS_OUT, vb);
  if(!bd || !xd) return -1;
  void *hb[QLLG_MAXRHS];
  double m[QLLG_MAXRHS];
  for(int r=0; r<n; r++) { hb[r] = b[r < nrhs ? r : 0]; m[r] = mass[r < nrhs ? r : 0]; }
  if(vec_upload(S, prec, bd, n, hb, dbl)) return -1;
  if(n > nrhs) {   /* zero the padding rhs: they start inactive */
    double zero[QLLG_MAXRHS], one[QLLG_MAXRHS];
    for(int r=0; r<n; r++) { zero[r] = 0; one[r] = r < nrhs ? 1 : 0; }
    double *dcoef = S->sc->tmp;
    if(qllg_h2d(dcoef, one, sizeof(double)*n)) return -1;
    if(qllg_k_axpby(prec, bd, prec, bd, NULL, 0.0, dcoef, 0.0, S->g.Vh, 3, n, NULL)) return -1;
    (void)zero;
  }
  int its = solve_dev(S, n, xd, bd, m, rsq, maxits, mode, info);
  if(its < 0) return -1;
  if(info && dbl && prec == QLLG_F64) {
    if(fill_true_rsq(S, mode, n, xd, bd, info)) return -1;
  }
  if(post_scale) {
    double sc[QLLG_MAXRHS];
    for(int r=0; r<n; r++) sc[r] = scale_real[r < nrhs ? r : 0];
    double *dcoef = S->sc->tmp;
    if(qllg_h2d(dcoef, sc, sizeof(double)*n)) return -1;
    if(qllg_k_axpby(prec, xd, prec, xd, NULL, 0.0, dcoef, 0.0, S->g.Vh, 3, n, NULL)) return -1;
  }
  void *hx[QLLG_MAXRHS];
  char *scratch = NULL;
  for(int r=0; r<n; r++) hx[r] = r < nrhs ? x[r] : NULL;
  if(n > nrhs) {
    scratch = malloc((dbl ? 8 : 4)*6*(size_t)S->g.Vh);
    for(int r=nrhs; r<n; r++) hx[r] = scratch;
  }
  int rc = vec_download(S, prec, xd, n, hx, dbl);
  free(scratch);
  return rc ? -1 : its;
}

int
qllg_stag_solve(qllg_stag *S, int nrhs, void *const x[], void *const b[], const double mass[],
                double rsq, int maxits, int mode, qllg_solve_info *info)
{
  return stag_solve_host(S, nrhs, x, b, mass, rsq, maxits, mode, info, 0, NULL);
}

/* out = D in on the output parity, device vectors of nrhs rhs in the
 * library layout of precision prec (0 FP64, 1 FP32, 2 16-bit) */
int
qllg_stag_dslash_device(qllg_stag *S, int prec, int nrhs, int out_parity, void *out_dev,
                        const void *in_dev)
{
  if(!valid_nrhs(nrhs)) { qllg_set_error("dslash_device: nrhs %d", nrhs); return -1; }
  if(prec < 0 || prec > 4) { qllg_set_error("dslash_device: precision %d", prec); return -1; }
  /* 4: double-float spinors and links, the reliable-update kernel over
   * every rhs */
  if(prec == QLLG_DF)
    return dslash_half_x(S, QLLG_DF, QLLG_DF, out_parity, nrhs, in_dev, NULL, out_dev, 0, NULL, 0, 1,
                         NULL, NULL, NULL, NULL, 1, 0);
  /* 3: FP32 spinors with the reconstruct-12 links */
  return dslash_half(S, prec == 3 ? QLLG_F32 : prec, prec, out_parity, nrhs, in_dev, NULL, out_dev,
                     0, NULL, 0, 1, NULL, NULL, NULL, NULL);
}

/* out = D in as qllg_stag_dslash_device, plus |out|^2 of each rhs into
 * norm2_dev, without allocating any device memory: the grid reduction runs
 * in the fixed scratch of k_noalloc.cu instead of a workspace, and links
 * that do not exist yet in precision prec are refused rather than derived
 * (deriving them allocates).  For callers with a fixed device-memory budget
 * (a serving loop that admits solves against HBM) or with other streams in
 * flight that a device-synchronising cudaMalloc/cudaFree would stall.
 * The scratch's address and the kernels the call launches were resolved
 * and loaded when S's links of precision prec were made (noalloc_preload).
 * Calls that overlap in time share the scratch and race. */
int
qllg_stag_dslash_norm2_noalloc(qllg_stag *S, int prec, int nrhs, int out_parity,
                               void *out_dev, const void *in_dev, double *norm2_dev)
{
  if(!S || !out_dev || !in_dev || !norm2_dev) {
    qllg_set_error("dslash_norm2_noalloc: null argument");
    return -1;
  }
  if(!valid_nrhs(nrhs) || nrhs > QLLG_MAXRHS) {
    qllg_set_error("dslash_norm2_noalloc: nrhs %d not in {1,2,4,8,16} (the fixed scratch holds "
                   "partial sums of at most %d rhs)", nrhs, QLLG_MAXRHS);
    return -1;
  }
  if(prec < 0 || prec > 2) { qllg_set_error("dslash_norm2_noalloc: precision %d", prec); return -1; }
  if(out_parity != 0 && out_parity != 1) {
    qllg_set_error("dslash_norm2_noalloc: parity %d", out_parity);
    return -1;
  }
  if(!S->links[prec]) {
    qllg_set_error("dslash_norm2_noalloc: links of precision %d not created yet (creating them "
                   "allocates; one qllg_stag_dslash_device call of that precision does it)", prec);
    return -1;
  }
  qllg_redbuf rb;
  if(qllg_noalloc_redbuf(&rb)) return -1;
  /* the last-block counter must start at zero (the last block also leaves
   * it at zero); the partials are written before they are read and the
   * norms are stored, not accumulated */
  if(qllg_check_cuda(cudaMemsetAsync(rb.counter, 0, sizeof(unsigned), qllg_stream()),
                     "dslash_norm2_noalloc: counter clear")) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = S->g;
  A.out_parity = out_parity;
  A.nrhs = nrhs;
  A.nslots = S->nslots;
  A.fb = S->fb;
  A.links = S->links[prec];
  A.lscale = S->lscale;
  A.in = in_dev;
  A.out = out_dev;
  A.mode = 0;
  A.b = 1;
  A.norm_out = norm2_dev;
  A.rb = &rb;
  A.no_tune = 1;              /* tuning would allocate a side buffer */
  return qllg_k_stag_dslash(prec, prec, &A);
}

/* 1 when the operator's last solve ran as one persistent launch */
int
qllg_stag_last_solve_persistent(const qllg_stag *S)
{
  return S ? S->used_persistent : 0;
}

/* bytes of a device vector of nrhs rhs in precision prec (one parity) */
size_t
qllg_stag_vec_bytes(const qllg_stag *S, int prec, int nrhs)
{
  /* prec 3 of qllg_stag_dslash_device (reconstruct-12 links) has FP32
   * spinors; an unknown precision has no vector (0 bytes) */
  if(prec == 3) prec = QLLG_F32;
  if(prec < 0 || (prec > 2 && prec != QLLG_DF) || nrhs < 0) return 0;
  return vec_bytes(S, prec, nrhs);
}

int
qllg_stag_nbr_table(const int dims[4], int parity, int slot, int *host_out)
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return -1;
  int *d = qllg_dmalloc(sizeof(int)*g.Vh);
  if(!d) return -1;
  int rc = qllg_k_stag_nbr_table(&g, parity, slot, d);
  if(!rc) rc = qllg_d2h(host_out, d, sizeof(int)*g.Vh);
  qllg_dfree(d);
  return rc;
}

/* ------------------------------------------------- multishift CG */

/* cgmsSolveT (lib/cgms.c:6-179) with Aop = the normal operator of mass0,
 * on device fields: in (single rhs), out (n fields back to back) */
static int
cgms_run(qllg_stag *S, int prec, void *out, const void *in, const double shifts[], int n,
         double mass0, double rsqin, int itnlim)
{
  if(n < 1 || n > QLLG_MAXSHIFT) { qllg_set_error("cgms: %d shifts (1..%d)", n, QLLG_MAXSHIFT); return -1; }
  if(ensure_links(S, prec)) return -1;
  size_t vb = vec_bytes(S, prec, 1);
  void *r = ws_get(S, WS_R, vb), *Ap = ws_get(S, WS_AP, vb), *v = ws_get(S, WS_V, vb);
  void *ps = ws_get(S, WS_PS, vb*n);
  if(!r || !Ap || !v || !ps) return -1;
  int Vh = S->g.Vh;
  qllg_cgms_scalars *cs = S->cs, *h = S->hcs;
  if(qllg_k_norm2(prec, in, Vh, 3, 1, &cs->pkp, &S->rb)) return -1;
  double insq;
  if(qllg_d2h(&insq, &cs->pkp, sizeof(double))) return -1;
  if(qllg_k_zero(prec, out, Vh*n, 3, 1)) return -1;
  if(insq == 0) return qllg_sync() ? -1 : 0;
  memset(h, 0, sizeof(*h));
  h->n = n;
  for(int i=0; i<n; i++) {
    h->shifts[i] = shifts[i];
    h->zo[i] = h->z[i] = 1;
    h->bo[i] = -1;
    h->a[i] = 0;
    h->s[i] = 1;
  }
  h->rsqstop = rsqin*insq;
  h->rsq = insq;
  h->mass2 = mass0*mass0;
  h->itnlim = itnlim;
  if(qllg_check_cuda(cudaMemcpyAsync(cs, h, sizeof(*h), cudaMemcpyHostToDevice, qllg_stream()),
                     "push cgms scalars")) return -1;
  if(qllg_k_copy(prec, r, in, Vh, 3, 1)) return -1;
  for(int i=0; i<n; i++)
    if(qllg_k_copy(prec, (char *)ps + vb*i, r, Vh, 3, 1)) return -1;
  int batch = 8;
  for(;;) {
    for(int it=0; it<batch; it++) {
      if(qllg_k_cgms_pre(cs)) return -1;
      if(dslash_half(S, prec, prec, 1, 1, ps, NULL, v, 0, NULL, 0, 1, &cs->vnorm, NULL, NULL,
                     &cs->done)) return -1;
      if(dslash_half(S, prec, prec, 0, 1, v, ps, Ap, 2, &cs->mass2, 0, -1, NULL, &cs->pnorm,
                     NULL, &cs->done)) return -1;
      if(qllg_k_cgms_coef(cs)) return -1;
      if(qllg_k_cgms_update_xr(prec, out, r, ps, Ap, Vh, cs, &S->rb)) return -1;
      if(qllg_k_cgms_update_p(prec, ps, r, Vh, cs)) return -1;
    }
    int d;
    if(qllg_check_cuda(cudaMemcpyAsync(&h->done, &cs->done, sizeof(int), cudaMemcpyDeviceToHost,
                                       qllg_stream()), "pull done") || qllg_sync()) return -1;
    d = h->done;
    if(d) break;
    if(batch < 64) batch *= 2;
  }
  if(qllg_check_cuda(cudaMemcpyAsync(h, cs, sizeof(*h), cudaMemcpyDeviceToHost, qllg_stream()),
                     "pull cgms scalars") || qllg_sync()) return -1;
  return h->iteration;
}

/* host wrapper: in = y (even half), out[i] = x[i] (even half), optional
 * scaling by scale[i] as solveMulti2 does */
static int
cgms_host(qllg_stag *S, void *const x[], const void *y, const double shifts[], int n,
          double mass0, double rsq, int itnlim, const double *scale)
{
  int dbl = S->master == QLLG_F64;
  int prec = S->master;
  size_t vb = vec_bytes(S, prec, 1);
  if(n < 1 || n > QLLG_MAXSHIFT) { qllg_set_error("cgms: %d shifts (1..%d)", n, QLLG_MAXSHIFT); return -1; }
  void *b = ws_get(S, WS_B, vb), *out = ws_get(S, WS_OUT, vb*n);
  if(!b || !out) return -1;
  void *ya[1] = {(void *)y};
  if(vec_upload(S, prec, b, 1, ya, dbl)) return -1;
  int its = cgms_run(S, prec, out, b, shifts, n, mass0, rsq, itnlim);
  if(its < 0) return -1;
  for(int i=0; i<n; i++) {
    void *oi = (char *)out + vb*i;
    if(scale && qllg_k_axpby(prec, oi, prec, oi, NULL, 0.0, NULL, scale[i], S->g.Vh, 3, 1, NULL))
      return -1;
    void *xa[1] = {x[i]};
    if(vec_download(S, prec, oi, 1, xa, dbl)) return -1;
  }
  return its;
}

/* ------------------------------------------- foreign layouts (QDP, MILC) */
/* The embedding pattern of the reference (embedqop.c:193-258) repacks a
 * QOP/QDP code's double-stored links and vectors on the host (packM/packV,
 * qopstag.c:123-196: a site reordering and a matrix transpose) before
 * createStaggeredSolver.  Here the caller hands its arrays as they are:
 * foreign site s is QLL site perm[s] (NULL: the same order, as MILC's
 * even-first order is for one rank), matrices row-major when row_major;
 * the reordering and transpose run on the GPU.  fat[8]/lng[8] are the
 * double-stored slots in createStaggeredLinks order. */
static int *
perm_upload(const int *perm, int V)
{
  if(!perm) return NULL;
  int *d = qllg_dmalloc(sizeof(int)*(size_t)V);
  if(d && qllg_h2d(d, perm, sizeof(int)*(size_t)V)) { qllg_dfree(d); return NULL; }
  return d;
}

qllg_stag *
qllg_stag_create_foreign(const int dims[4], double *const fat[8], double *const lng[8],
                         const int *perm, int row_major)
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return NULL;
  const int nslots = lng ? 16 : 8;
  const size_t hb = 8*18*(size_t)g.V, per = qllg_link_bytes(QLLG_F64)*(size_t)g.V;
  int *dperm = perm_upload(perm, g.V);
  double *in = qllg_dmalloc(hb), *qll = qllg_dmalloc(hb);
  char *links = qllg_dmalloc(per*nslots);
  qllg_stag *S = NULL;
  if((perm && !dperm) || !in || !qll || !links) goto out;
  for(int s=0; s<nslots; s++) {
    const double *h = (nslots == 16) ? ((s & 1) ? lng[s/2] : fat[s/2]) : fat[s];
    if(!h) { qllg_set_error("foreign links: slot %d is NULL", s); goto out; }
    if(qllg_h2d(in, h, hb) || qllg_k_aos_from_foreign(qll, in, dperm, g.V, 18, row_major) ||
       qllg_k_link_from_aos(QLLG_F64, links + per*s, NULL, qll, 1, g.V)) goto out;
  }
  if(qllg_sync()) goto out;
  S = qllg_stag_alloc(dims, nslots, QLLG_F64);
  if(S) { qllg_stag_attach_links(S, QLLG_F64, links); links = NULL; }
out:
  qllg_sync();
  qllg_dfree(dperm);
  qllg_dfree(in);
  qllg_dfree(qll);
  qllg_dfree(links);
  return S;
}

/* device FP64 vector of nrhs rhs (even sites) <-> host arrays [V][6] in the
 * foreign site order (upload reads their even sites, download writes all
 * sites, zero at the odd ones) */
int
qllg_stag_vec_upload_foreign(qllg_stag *S, void *v_dev, int nrhs, void *const h[],
                             const int *perm)
{
  const int V = S->g.V;
  const size_t hb = 48*(size_t)V;
  int *dperm = perm_upload(perm, V);
  double *in = qllg_dmalloc(hb), *qll = qllg_dmalloc(hb*nrhs);
  int rc = -1;
  if((perm && !dperm) || !in || !qll) goto out;
  for(int r=0; r<nrhs; r++)
    if(qllg_h2d(in, h[r], hb) || qllg_k_aos_from_foreign(qll + 6*(size_t)V*r, in, dperm, V, 6, 0))
      goto out;
  /* the even half of each reordered block, rhs blocks 6V reals apart */
  rc = qllg_k_spinor_from_aos(QLLG_F64, v_dev, qll, 1, S->g.Vh, 3, nrhs, 6*(size_t)V);
out:
  qllg_sync();
  qllg_dfree(dperm);
  qllg_dfree(in);
  qllg_dfree(qll);
  return rc;
}

int
qllg_stag_vec_download_foreign(qllg_stag *S, const void *v_dev, int nrhs, void *const h[],
                               const int *perm)
{
  const int V = S->g.V;
  const size_t hb = 48*(size_t)V;
  int *dperm = perm_upload(perm, V);
  double *out = qllg_dmalloc(hb), *qll = qllg_dmalloc(hb*nrhs);
  int rc = -1;
  if((perm && !dperm) || !out || !qll) goto out;
  /* odd sites of the reordered blocks are zero, as the solvers leave them */
  if(qllg_check_cuda(cudaMemsetAsync(qll, 0, hb*nrhs, qllg_stream()), "clear")) goto out;
  if(qllg_k_spinor_to_aos(QLLG_F64, v_dev, qll, 1, S->g.Vh, 3, nrhs, 6*(size_t)V)) goto out;
  for(int r=0; r<nrhs; r++)
    if(qllg_k_aos_to_foreign(out, qll + 6*(size_t)V*r, dperm, V, 6) || qllg_d2h(h[r], out, hb))
      goto out;
  rc = 0;
out:
  qllg_sync();
  qllg_dfree(dperm);
  qllg_dfree(out);
  qllg_dfree(qll);
  return rc;
}

/* ------------------------------------------------ multi-rhs multishift */
/* cgmsSolveT (lib/cgms.c:6-179) for nr rhs at once in FP32 (vectors) with
 * FP64 recurrences per rhs column: bf the sources [3][Vh][nr] FP32, out n
 * solution fields of the same shape back to back, shifts relative to the
 * base m0^2 (shifts[0] = 0 for the base system itself); stops each column
 * at |r|^2 < rsq |b|^2.  Returns the largest iteration count. */
static int
mcgms_run(qllg_stag *S, int pl, int nr, void *out, const void *bf, const double shifts[], int n,
          double mass0, double rsq, int itnlim)
{
  const int Vh = S->g.Vh;
  const size_t vb = vec_bytes(S, QLLG_F32, nr);
  if(ensure_links(S, pl)) return -1;
  void *r = ws_get(S, WS_R, vb), *Ap = ws_get(S, WS_AP, vb), *v = ws_get(S, WS_V, vb);
  if(!r || !Ap || !v) return -1;
  if(!S->mcs && !(S->mcs = qllg_dmalloc(sizeof(qllg_mcgms_scalars)))) return -1;
  qllg_mcgms_scalars *h = malloc(sizeof(qllg_mcgms_scalars));
  void *ps = qllg_dmalloc(vb*n);
  double bn[QLLG_MAXRHS];
  int rc = -1;
  if(!h || !ps) goto out;
  if(qllg_k_norm2(QLLG_F32, bf, Vh, 3, nr, S->sc->tmp, &S->rb) ||
     qllg_d2h(bn, S->sc->tmp, sizeof(double)*nr)) goto out;
  memset(h, 0, sizeof(*h));
  h->n = n;
  h->nr = nr;
  h->itnlim = itnlim;
  for(int i=0; i<n; i++) h->shifts[i] = shifts[i];
  int any = 0;
  for(int q=0; q<nr; q++) {
    h->mass2[q] = mass0*mass0;
    h->rsq[q] = bn[q];
    h->rsqstop[q] = rsq*bn[q];
    h->active[q] = bn[q] > 0;
    any |= h->active[q];
    for(int i=0; i<n; i++) { h->zo[q][i] = h->z[q][i] = 1; h->bo[q][i] = -1; h->a[q][i] = 0; }
  }
  h->done = !any;
  if(qllg_check_cuda(cudaMemcpyAsync(S->mcs, h, sizeof(*h), cudaMemcpyHostToDevice, qllg_stream()),
                     "push multishift scalars")) goto out;
  if(qllg_check_cuda(cudaMemsetAsync(out, 0, vb*n, qllg_stream()), "clear") ||
     qllg_k_copy(QLLG_F32, r, bf, Vh, 3, nr)) goto out;
  for(int i=0; i<n; i++) if(qllg_k_copy(QLLG_F32, (char *)ps + vb*i, bf, Vh, 3, nr)) goto out;
  for(int batch=8;;) {
    for(int it=0; it<batch; it++) {
      qllg_mcgms_scalars *m = S->mcs;
      if(qllg_k_mcgms_pre(m) ||
         dslash_half(S, QLLG_F32, pl, 1, nr, ps, NULL, v, 0, NULL, 0, 1, m->vnorm, NULL, m->active,
                     &m->done) ||
         dslash_half(S, QLLG_F32, pl, 0, nr, v, ps, Ap, 2, m->mass2, 0, -1, NULL, m->pnorm,
                     m->active, &m->done) ||
         qllg_k_mcgms_coef(m) ||
         qllg_k_mcgms_update_xr(out, r, ps, Ap, Vh, nr, vb, m, &S->rb) ||
         qllg_k_mcgms_update_p(ps, r, Vh, nr, vb, m)) goto out;
    }
    if(qllg_d2h(&h->done, &S->mcs->done, sizeof(int))) goto out;
    if(h->done) break;
    if(batch < 64) batch *= 2;
  }
  if(qllg_d2h(h, S->mcs, sizeof(*h))) goto out;
  rc = 0;
  for(int q=0; q<nr; q++) if(h->iteration[q] > rc) rc = h->iteration[q];
out:
  qllg_sync();
  qllg_dfree(ps);
  free(h);
  return rc;
}

/* For every rhs r and shift k: (m^2 + shift_k - D_eo D_oe) x[r*nshift + k]
 * = b[r] on the even sites, stopping at |r_k|^2 < rsq |b_r|^2.
 *  - QLLG_SOLVE_DOUBLE: the reference's multishift CG (cgmsSolveT,
 *    lib/cgms.c:6-179) in FP64, all shifts of one rhs from one Krylov
 *    space, one rhs after the other (solveMulti2 per rhs);
 *  - QLLG_SOLVE_MIXED_SINGLE: first the same recurrence for up to 16 rhs
 *    at once in FP32 vectors (one multi-rhs Dslash per half iteration for
 *    all of them, FP64 recurrences per rhs), to about FP32 accuracy; then
 *    every (rhs, shift) pair from that first solution to the requested
 *    FP64 true residual, as a column of the 16-wide FP32 mixed CG with FP64
 *    reliable updates (pairs in order of shift, so a launch holds pairs of
 *    similar iteration counts).
 * Host arrays [V][6] FP64 (the even half is read and written).  iters and
 * true_rsq (|b - A_k x|^2/|b|^2 in FP64) are per pair, optional. */
int
qllg_stag_solve_multishift(qllg_stag *S, int nrhs, void *const x[], void *const b[], double mass,
                           int nshift, const double shifts[], double rsq, int maxits, int mode,
                           int iters[], double true_rsq[])
{
  if(S->master != QLLG_F64) { qllg_set_error("multishift: needs an FP64 operator"); return -1; }
  if(nrhs < 1 || nshift < 1 || nshift > QLLG_MAXSHIFT) {
    qllg_set_error("multishift: %d rhs, %d shifts (1..%d)", nrhs, nshift, QLLG_MAXSHIFT);
    return -1;
  }
  for(int k=0; k<nshift; k++)
    if(!(mass*mass + shifts[k] > 0)) { qllg_set_error("multishift: shift %d", k); return -1; }
  if(rsq < 0) rsq = -rsq;
  const int Vh = S->g.Vh;
  const size_t vb1 = vec_bytes(S, QLLG_F64, 1);
  int maxit_seen = 0;
  if(mode == QLLG_SOLVE_DOUBLE) {
    /* cgmsSolveT iterates on its first system and takes the others as
     * offsets from it (shift 0 is the base, lib/cgms.c): the smallest
     * shift, the slowest system, goes first and the others relative to it */
    int order[QLLG_MAXSHIFT], kmin = 0;
    for(int k=1; k<nshift; k++) if(shifts[k] < shifts[kmin]) kmin = k;
    double rel[QLLG_MAXSHIFT];
    order[0] = kmin;
    for(int k=0, j=1; k<nshift; k++) if(k != kmin) order[j++] = k;
    for(int j=0; j<nshift; j++) rel[j] = shifts[order[j]] - shifts[kmin];
    const double mass0 = sqrt(mass*mass + shifts[kmin]);
    void *xs[QLLG_MAXSHIFT];
    for(int r=0; r<nrhs; r++) {
      for(int j=0; j<nshift; j++) xs[j] = x[r*nshift + order[j]];
      int its = cgms_host(S, xs, b[r], rel, nshift, mass0, rsq, maxits, NULL);
      if(its < 0) return -1;
      if(its > maxit_seen) maxit_seen = its;
      /* cgms_host leaves b in WS_B and the n solutions in WS_OUT */
      for(int j=0; j<nshift; j++) {
        int k = order[j];
        if(iters) iters[r*nshift + k] = its;
        if(!true_rsq) continue;
        double m2 = mass*mass + shifts[k];
        if(qllg_h2d(S->sc->mass2, &m2, sizeof(double))) return -1;
        if(true_residual(S, 1, (char *)S->ws[WS_OUT] + vb1*j, S->ws[WS_B],
                         &true_rsq[r*nshift + k])) return -1;
      }
    }
    return maxit_seen;
  }
  if(mode != QLLG_SOLVE_MIXED_SINGLE) {
    qllg_set_error("multishift: mode %d (QLLG_SOLVE_DOUBLE or QLLG_SOLVE_MIXED_SINGLE)", mode);
    return -1;
  }
  /* 1. the reference's multishift recurrence for up to 16 rhs at once, in
   *    FP32 vectors (FP64 recurrences): a first solution of every pair,
   *    good to about FP32 accuracy, from one Krylov space per rhs.  The
   *    base system is the smallest shift (cgmsSolveT takes the others as
   *    offsets from its first). */
  int order[QLLG_MAXSHIFT], pos[QLLG_MAXSHIFT], kmin = 0;
  for(int k=1; k<nshift; k++) if(shifts[k] < shifts[kmin]) kmin = k;
  double rel[QLLG_MAXSHIFT];
  order[0] = kmin;
  for(int k=0, j=1; k<nshift; k++) if(k != kmin) order[j++] = k;
  for(int j=0; j<nshift; j++) { rel[j] = shifts[order[j]] - shifts[kmin]; pos[order[j]] = j; }
  const double mass0 = sqrt(mass*mass + shifts[kmin]);
  const int pl = f32_links(S);
  const double rsq_guess = rsq > qllg_get_param("multishift_guess_rsq") ? rsq
                                                                       : qllg_get_param("multishift_guess_rsq");
  const int ngroup = (nrhs + QLLG_MAXRHS - 1)/QLLG_MAXRHS;
  void **gb = calloc(ngroup, sizeof(void *)), **gx = calloc(ngroup, sizeof(void *));
  int *gits = calloc(ngroup, sizeof(int));
  void *stage = qllg_stage(48*(size_t)Vh), *bf = NULL;
  int rc = -1;
  if(!gb || !gx || !gits || !stage) goto done;
  for(int g=0; g<ngroup; g++) {
    const int g0 = g*QLLG_MAXRHS, nreal = nrhs - g0 < QLLG_MAXRHS ? nrhs - g0 : QLLG_MAXRHS;
    const int nr = pad_nrhs(nreal);
    gb[g] = qllg_dmalloc(vec_bytes(S, QLLG_F64, nr));
    gx[g] = qllg_dmalloc(vec_bytes(S, QLLG_F32, nr)*nshift);
    bf = qllg_dmalloc(vec_bytes(S, QLLG_F32, nr));
    if(!gb[g] || !gx[g] || !bf) goto done;
    if(qllg_check_cuda(cudaMemsetAsync(gb[g], 0, vec_bytes(S, QLLG_F64, nr), qllg_stream()), "clear"))
      goto done;
    for(int j=0; j<nreal; j++)
      if(qllg_h2d(stage, b[g0 + j], 48*(size_t)Vh) ||
         qllg_k_column_from_aos(gb[g], stage, Vh, nr, j)) goto done;
    if(qllg_k_spinor_convert(QLLG_F32, bf, QLLG_F64, gb[g], Vh, 3, nr, NULL)) goto done;
    gits[g] = mcgms_run(S, pl, nr, gx[g], bf, rel, nshift, mass0, rsq_guess, maxits);
    qllg_sync();
    qllg_dfree(bf);
    bf = NULL;
    if(gits[g] < 0) goto done;
  }
  /* 2. every pair to the requested FP64 true residual: the FP32 mixed CG
   *    with reliable updates, started from its first solution, 16 pairs per
   *    launch in order of shift */
  {
    const int npair = nrhs*nshift;
    size_t vb = vec_bytes(S, QLLG_F64, QLLG_MAXRHS);
    void *bd = ws_get(S, WS_B, vb), *xd = ws_get(S, WS_OUT, vb);
    if(!bd || !xd) goto done;
    const double delta = qllg_get_param("reliable_delta_single");
    for(int p0=0; p0<npair; p0+=QLLG_MAXRHS) {
      int n = npair - p0 < QLLG_MAXRHS ? npair - p0 : QLLG_MAXRHS;
      int nc = pad_nrhs(n);
      double m[QLLG_MAXRHS], tr[QLLG_MAXRHS];
      if(qllg_check_cuda(cudaMemsetAsync(bd, 0, vec_bytes(S, QLLG_F64, nc), qllg_stream()), "clear") ||
         qllg_check_cuda(cudaMemsetAsync(xd, 0, vec_bytes(S, QLLG_F64, nc), qllg_stream()), "clear"))
        goto done;
      for(int j=0; j<nc; j++) {
        int pr = p0 + (j < n ? j : 0), k = pr / nrhs, r = pr % nrhs;
        m[j] = sqrt(mass*mass + shifts[k]);
        if(j >= n) continue;            /* padding: b = 0, starts inactive */
        const int g = r/QLLG_MAXRHS, jr = r % QLLG_MAXRHS;
        const int nr = pad_nrhs(nrhs - g*QLLG_MAXRHS < QLLG_MAXRHS ? nrhs - g*QLLG_MAXRHS : QLLG_MAXRHS);
        const char *guess = (const char *)gx[g] + vec_bytes(S, QLLG_F32, nr)*pos[k];
        if(qllg_k_column_copy(QLLG_F64, bd, nc, j, QLLG_F64, gb[g], nr, jr, Vh) ||
           qllg_k_column_copy(QLLG_F64, xd, nc, j, QLLG_F32, guess, nr, jr, Vh)) goto done;
      }
      int its = cg_mixed(S, QLLG_F32, QLLG_F32, pl, nc, xd, bd, m, rsq, maxits, delta, 1);
      if(its < 0) goto done;
      int rits[QLLG_MAXRHS];
      for(int j=0; j<nc; j++) rits[j] = S->hsc->iters[j];
      if(true_rsq && true_residual(S, nc, xd, bd, tr)) goto done;
      for(int j=0; j<n; j++) {
        int pr = p0 + j, k = pr / nrhs, r = pr % nrhs;
        if(qllg_k_column_to_aos(xd, stage, Vh, nc, j) ||
           qllg_d2h(x[r*nshift + k], stage, 48*(size_t)Vh)) goto done;
        const int total = gits[r/QLLG_MAXRHS] + rits[j];
        if(iters) iters[r*nshift + k] = total;
        if(total > maxit_seen) maxit_seen = total;
        if(true_rsq) true_rsq[r*nshift + k] = tr[j];
      }
    }
  }
  rc = maxit_seen;
done:
  qllg_sync();
  if(bf) qllg_dfree(bf);
  for(int g=0; gb && g<ngroup; g++) qllg_dfree(gb[g]);
  for(int g=0; gx && g<ngroup; g++) qllg_dfree(gx[g]);
  free(gb);
  free(gx);
  free(gits);
  return rc;
}

/* createStaggeredLinksFb (lib/stagDslash.c:464-519): only the forward
 * links u[2mu] (and u3[2mu]) are read and held; the backward links
 * -U^dagger(x-mu) and -U3^dagger(x-3mu) are applied on the fly as
 * dslashFb2T does (V_vmeq_xMap_times_xVp, lib/vla.c:1368-1393), so the
 * resident links take half the memory of the double-stored form */

static qllg_stag *
stag_create_fb(const int dims[4], void *const u[8], void *const u3[8], int dbl)
{
  qllg_geom g;
  if(qllg_runtime_init() || qllg_geom_from_dims(&g, dims)) return NULL;
  /* single-stored: the forward slots [fat mu, long mu] (or [fat mu]) only;
   * the kernels make the backward links from them */
  int nslots = u3 ? 16 : 8, stored = nslots/2, prec = dbl ? QLLG_F64 : QLLG_F32;
  size_t per = qllg_link_bytes(prec)*(size_t)g.V, hb = (dbl ? 8 : 4)*18*(size_t)g.V;
  char *links = qllg_dmalloc(per*stored);
  void *stage = qllg_stage(hb);
  if(!links || !stage) { qllg_dfree(links); return NULL; }
  for(int mu=0; mu<4; mu++) {
    for(int nk=0; nk<(u3 ? 2 : 1); nk++) {
      const int fs = u3 ? 2*mu + nk : mu;
      const void *h = nk ? u3[2*mu] : u[2*mu];
      if(!h || qllg_h2d(stage, h, hb) ||
         qllg_k_link_from_aos(prec, links + per*fs, NULL, stage, dbl, g.V)) {
        qllg_sync();
        qllg_dfree(links);
        return NULL;
      }
    }
  }
  if(qllg_sync()) { qllg_dfree(links); return NULL; }
  qllg_stag *S = qllg_stag_alloc(dims, nslots, prec);
  if(!S) { qllg_dfree(links); return NULL; }
  S->fb = 1;
  qllg_stag_attach_links(S, prec, links);
  return S;
}

/* ------------------------------------------------- QLL drop-in layer */

/* private block behind StaggeredLinks.t: the Transporter records the
 * reference fills, then the device operator; t points at its start */
typedef struct {
  char t[16][sizeof(TransporterD)];
  qllg_stag *S;
  int own;          /* destroy S with this link set */
  int parity;       /* -1 all, 0 even, 1 odd */
} links_priv;

static int
sub_parity(const char *sub)
{
  return (sub && sub[0] == 'e') ? 0 : ((sub && sub[0] == 'o') ? 1 : -1);
}

static const char *
parity_sub(int p)
{
  return p == 0 ? "even" : (p == 1 ? "odd" : "all");
}

#define DEFINE_STAG_DROPIN(S_, real, DBL)                                          \
static void                                                                       \
links_fill##S_(StaggeredLinks##S_ *sl, Layout *l, real *u[], real *u3[], char *sub,\
               qllg_stag *S, int own, int fb)                                     \
{                                                                                 \
  links_priv *pv = calloc(1, sizeof(links_priv));                                 \
  pv->S = S;                                                                      \
  pv->own = own;                                                                  \
  pv->parity = sub_parity(sub);                                                   \
  int n = S ? S->nslots : (u3 ? 16 : 8);                                          \
  Transporter##S_ *t = (Transporter##S_ *)pv->t;                                  \
  for(int i=0; i<n; i++) {                                                        \
    t[i].u = u3 ? ((i & 1) ? u3[i/2] : u[i/2]) : u[i];                            \
    t[i].nelem = 6;                                                               \
    t[i].nc = 3;                                                                  \
    layoutSubset(&t[i].sub, l, sub);                                              \
    t[i].backward = 0;                                                            \
  }                                                                               \
  sl->t = t;                                                                      \
  sl->n = n;                                                                      \
  sl->massFac = (pv->parity >= 0) ? 0 : 1;                                        \
  sl->fb = fb;                                                                    \
}                                                                                 \
                                                                                  \
static qllg_stag *                                                                \
links_op##S_(StaggeredLinks##S_ *sl)                                              \
{                                                                                 \
  return sl && sl->t ? ((links_priv *)(void *)sl->t)->S : NULL;                   \
}                                                                                 \
                                                                                  \
void                                                                              \
createStaggeredLinks##S_(StaggeredLinks##S_ *sl, Layout *l, real *u[], real *u3[],\
                         char *sub)                                               \
{                                                                                 \
  qllg_geom g;                                                                    \
  memset(sl, 0, sizeof(*sl));                                                     \
  if(qllg_geom_from_layout(&g, l)) return;                                        \
  qllg_stag *S = DBL ? qllg_stag_create(g.L, (double *const *)u, (double *const *)u3) \
                     : qllg_stag_create_f(g.L, (float *const *)u, (float *const *)u3); \
  if(!S) return;                                                                  \
  links_fill##S_(sl, l, u, u3, sub, S, 1, 0);                                     \
}                                                                                 \
                                                                                  \
void                                                                              \
createStaggeredLinksFb##S_(StaggeredLinks##S_ *sl, Layout *l, real *u[], real *u3[],\
                           char *sub)                                             \
{                                                                                 \
  qllg_geom g;                                                                    \
  memset(sl, 0, sizeof(*sl));                                                     \
  if(qllg_geom_from_layout(&g, l)) return;                                        \
  qllg_stag *S = stag_create_fb(g.L, (void *const *)u, (void *const *)u3, DBL);   \
  if(!S) return;                                                                  \
  links_fill##S_(sl, l, u, u3, sub, S, 1, 1);                                     \
}                                                                                 \
                                                                                  \
void                                                                              \
freeStaggeredLinks##S_(StaggeredLinks##S_ *sl)                                    \
{                                                                                 \
  if(!sl || !sl->t) return;                                                       \
  links_priv *pv = (links_priv *)(void *)sl->t;                                   \
  if(pv->own) qllg_stag_destroy(pv->S);                                           \
  free(pv);                                                                       \
  sl->t = NULL;                                                                   \
}                                                                                 \
                                                                                  \
void                                                                              \
dslash2##S_(StaggeredLinks##S_ *d, real *x, real mass, real *y)                   \
{                                                                                 \
  qllg_stag *S = links_op##S_(d);                                                 \
  if(!S) { qllg_set_error("dslash2: links not created"); return; }               \
  mass *= d->massFac;                                                             \
  links_priv *pv = (links_priv *)(void *)d->t;                                    \
  qllg_stag_dslash(S, x, (double)mass, y, parity_sub(pv->parity));                \
}                                                                                 \
                                                                                  \
void                                                                              \
createStaggeredSolver##S_(StaggeredSolver##S_ *ss, Layout *l, real *u[],          \
                          real *u3[], char *sub)                                  \
{                                                                                 \
  (void)sub;                                                                      \
  memset(ss, 0, sizeof(*ss));                                                     \
  qllg_geom g;                                                                    \
  if(qllg_geom_from_layout(&g, l)) return;                                        \
  qllg_stag *S = DBL ? qllg_stag_create(g.L, (double *const *)u, (double *const *)u3) \
                     : qllg_stag_create_f(g.L, (float *const *)u, (float *const *)u3); \
  if(!S) return;                                                                  \
  links_fill##S_(&ss->sle, l, u, u3, "even", S, 1, 0);                            \
  links_fill##S_(&ss->slo, l, u, u3, "odd", S, 0, 0);                             \
  ss->v = NULL;                                                                   \
  cglsInit##S_(&ss->cgls, 6*l->nEvenOuter);                                       \
  layoutSubset(&ss->sube, l, "even");                                             \
  layoutSubset(&ss->subo, l, "odd");                                              \
  ss->noscale = 0;                                                                \
}                                                                                 \
                                                                                  \
void                                                                              \
freeStaggeredSolver##S_(StaggeredSolver##S_ *ss)                                  \
{                                                                                 \
  cglsFree##S_(&ss->cgls);                                                        \
  freeStaggeredLinks##S_(&ss->slo);                                               \
  freeStaggeredLinks##S_(&ss->sle);                                               \
}                                                                                 \
                                                                                  \
int                                                                               \
solve2##S_(StaggeredSolver##S_ *ss, real *x, real mass, real *y, double rsq,      \
           int maxits, char *sub)                                                 \
{                                                                                 \
  (void)sub;                                                                      \
  qllg_stag *S = links_op##S_(&ss->sle);                                          \
  if(!S) { qllg_set_error("solve2: solver not created"); return -1; }             \
  ss->mass = mass;                                                                \
  if(rsq < 0) { ss->cgls.verbose = 3; rsq = -rsq; }                               \
  double m = ss->mass, sc = (double)mass;                                         \
  void *xa[1] = {x}, *ya[1] = {y};                                                \
  /* the reference's precision, or (solve2_mixed, D only) FP32 iterations      \
   * with FP64 reliable updates to the same true residual */                      \
  int mode = DBL ? QLLG_SOLVE_DOUBLE : QLLG_SOLVE_SINGLE;                         \
  if(DBL && qllg_get_param("solve2_mixed") != 0) mode = QLLG_SOLVE_MIXED_SINGLE;  \
  int its = stag_solve_host(S, 1, xa, ya, &m, rsq, maxits, mode, NULL,            \
                            !ss->noscale, &sc);                                   \
  ss->its = its;                                                                  \
  return its;                                                                     \
}                                                                                 \
                                                                                  \
int                                                                               \
solveMulti2##S_(StaggeredSolver##S_ *ss, real *x[], double masses[], int nmasses, \
                real *y, double rsq, int maxits, char *sub)                       \
{                                                                                 \
  (void)sub;                                                                      \
  qllg_stag *S = links_op##S_(&ss->sle);                                          \
  if(!S) { qllg_set_error("solveMulti2: solver not created"); return -1; }        \
  if(nmasses < 1 || nmasses > QLLG_MAXSHIFT) {                                    \
    qllg_set_error("solveMulti2: %d masses (1..%d)", nmasses, QLLG_MAXSHIFT);     \
    return -1;                                                                    \
  }                                                                               \
  ss->mass = masses[0];                                                           \
  if(rsq < 0) { ss->cgls.verbose = 3; rsq = -rsq; }                               \
  double m2[QLLG_MAXSHIFT], sc[QLLG_MAXSHIFT];                                    \
  for(int i=0; i<nmasses; i++) {                                                  \
    m2[i] = masses[i]*masses[i] - masses[0]*masses[0];                            \
    sc[i] = (double)(real)masses[i];                                              \
  }                                                                               \
  int its = cgms_host(S, (void *const *)x, y, m2, nmasses, masses[0], rsq, maxits,\
                      ss->noscale ? NULL : sc);                                   \
  ss->its = its;                                                                  \
  return its;                                                                     \
}                                                                                 \
                                                                                  \
int                                                                               \
solveMulti##S_(real *x[], real *u[8], real *u3[8], double masses[], int nmasses,  \
               real *y, double rsq, char *sub)                                    \
{                                                                                 \
  Layout *l = qllg_current_layout();                                              \
  if(!l) { qllg_set_error("solveMulti: call stagDslashSetup first"); return -1; } \
  StaggeredSolver##S_ ss;                                                         \
  createStaggeredSolver##S_(&ss, l, u, u3, sub);                                  \
  if(!ss.sle.t) return -1;                                                        \
  int its = solveMulti2##S_(&ss, x, masses, nmasses, y, rsq, 1000000, sub);       \
  freeStaggeredSolver##S_(&ss);                                                   \
  return its;                                                                     \
}                                                                                 \
                                                                                  \
int                                                                               \
cgmsSolve##S_(Cgls##S_ *cgls, real *x[], real *b, double shifts[], int nshifts,   \
              Linop##S_ *Aop, void *Aargs, Linop##S_ *Mop, void *Margs,           \
              double rsqs[], int itnlim)                                          \
{                                                                                 \
  (void)cgls; (void)Margs;                                                        \
  if(Aop != stagLinop##S_ || Mop) {                                               \
    qllg_set_error("cgmsSolve: the operator must be stagLinop with no preconditioner"); \
    return -1;                                                                    \
  }                                                                               \
  StaggeredSolver##S_ *ss = (StaggeredSolver##S_ *)Aargs;                         \
  qllg_stag *S = links_op##S_(&ss->sle);                                          \
  if(!S) { qllg_set_error("cgmsSolve: solver not created"); return -1; }          \
  return cgms_host(S, (void *const *)x, b, shifts, nshifts, ss->mass, rsqs[0],    \
                   itnlim, NULL);                                                 \
}                                                                                 \
                                                                                  \
int                                                                               \
solve##S_(real *x, real *u[8], real *u3[8], real mass, real *y, double rsq,       \
          char *sub)                                                              \
{                                                                                 \
  Layout *l = qllg_current_layout();                                              \
  if(!l) { qllg_set_error("solve: call stagDslashSetup first"); return -1; }      \
  StaggeredSolver##S_ ss;                                                         \
  createStaggeredSolver##S_(&ss, l, u, u3, sub);                                  \
  if(!ss.sle.t) return -1;                                                        \
  int its = solve2##S_(&ss, x, mass, y, rsq, 1000000, sub);                       \
  freeStaggeredSolver##S_(&ss);                                                   \
  return its;                                                                     \
}                                                                                 \
                                                                                  \
void                                                                              \
cglsInit##S_(Cgls##S_ *cgls, int nelem)                                           \
{                                                                                 \
  memset(cgls, 0, sizeof(*cgls));                                                 \
  cgls->nelem = nelem;                                                            \
}                                                                                 \
                                                                                  \
void                                                                              \
cglsFree##S_(Cgls##S_ *cgls)                                                      \
{                                                                                 \
  (void)cgls;                                                                     \
}                                                                                 \
                                                                                  \
void                                                                              \
stagLinop##S_(real *Ax, real *x, LinopInfo *li, void *args, ThreadCtx *TC)        \
{                                                                                 \
  (void)Ax; (void)x; (void)li; (void)args; (void)TC;                              \
  qllg_set_error("stagLinop runs inside cgSolve/cgmsSolve only");                 \
}                                                                                 \
                                                                                  \
int                                                                               \
cgSolve##S_(Cgls##S_ *cgls, real *x, real *b, Linop##S_ *Aop, void *Aargs,        \
            Linop##S_ *Mop, void *Margs, double rsq, int itnlim)                  \
{                                                                                 \
  (void)cgls; (void)Margs;                                                        \
  if(Aop != stagLinop##S_ || Mop) {                                               \
    qllg_set_error("cgSolve: the operator must be stagLinop with no preconditioner"); \
    return -1;                                                                    \
  }                                                                               \
  StaggeredSolver##S_ *ss = (StaggeredSolver##S_ *)Aargs;                         \
  qllg_stag *S = links_op##S_(&ss->sle);                                          \
  if(!S) { qllg_set_error("cgSolve: solver not created"); return -1; }            \
  double m = ss->mass;                                                            \
  void *xa[1] = {x}, *ba[1] = {b};                                                \
  return stag_solve_host(S, 1, xa, ba, &m, rsq, itnlim,                           \
                         DBL ? QLLG_SOLVE_DOUBLE : QLLG_SOLVE_SINGLE, NULL, 0, NULL); \
}

DEFINE_STAG_DROPIN(D, double, 1)
DEFINE_STAG_DROPIN(F, float, 0)
