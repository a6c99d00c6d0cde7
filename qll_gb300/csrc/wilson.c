/*
 * wilson.c -- the Wilson operator on the GPU: resident links,
 * wilsonDslash (lib/wilsonDslash.c:272-285), the reference's wilsonSolve
 * (:318-364) and the even-odd preconditioned normal-equation solver.
 *
 * Conventions of the reference: x = (4+m) y - sum_mu [(1-g_mu) u_2mu(x)
 * y(x+mu) + (1+g_mu) u_2mu+1(x) y(x-mu)] with caller-supplied backward links
 * (testwilson.c uses +U(x-mu)^dagger); the e/o subsets drop the mass term;
 * sign is ignored.
 *
 * Normal-equation solver (no counterpart in the reference, whose
 * wilsonSolve is not a valid CG for the Wilson matrix): with a = 4+m and W
 * the massless half-Dslash, the Schur complement on even sites is
 * S = a - W_eo W_oe / a, S^dagger = g5 S g5, and CG runs on
 * S^dagger S x = S^dagger b (CGNR).  Precision modes: FP64 throughout, or
 * FP32 iterations with FP64 reliable updates (x accumulated in FP64, the
 * residual periodically recomputed from the FP64 operator).
 */
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

enum { WW_X, WW_R, WW_P, WW_AP, WW_S, WW_V, WW_B, WW_X64, WW_R64, WW_T64, WW_S64, WW_V64,
       WW_XDF, WW_IO, WW_CTL, WW_N };

#define WGRAPHS 4

struct qllg_wilson {
  qllg_geom g;
  int master;
  void *links[QLLG_NLINKP];  /* by precision (FP64, FP32, double-float): [8][9][V] */
  qllg_redbuf rb;
  qllg_cg_scalars *sc, *hsc;
  void *ws[WW_N];
  size_t ws_bytes[WW_N];
  cudaEvent_t ev0, ev1;
  /* captured CGNR loops, by what their launches bake in */
  struct { long key[7]; cudaGraphExec_t exec; int body, ifbody; } graphs[WGRAPHS];
  int ngraph_next;
  int cap_ifbody;        /* while capturing: kernels of the reliable-update block */
};

static void wgraphs_drop(qllg_wilson *W);

static void *
wws(qllg_wilson *W, int id, size_t bytes)
{
  if(bytes <= W->ws_bytes[id]) return W->ws[id];
  /* captured loops hold the old buffer's address */
  wgraphs_drop(W);
  if(W->ws[id]) { qllg_sync(); qllg_dfree(W->ws[id]); }
  W->ws[id] = qllg_dmalloc(bytes);
  W->ws_bytes[id] = W->ws[id] ? bytes : 0;
  return W->ws[id];
}

static size_t
wvec(const qllg_wilson *W, int prec)
{
  return qllg_spinor_bytes(prec, 12)*(size_t)W->g.Vh;
}

static int
wlinks(qllg_wilson *W, int prec)
{
  if(W->links[prec]) return 0;
  if(W->master != QLLG_F64) { qllg_set_error("Wilson operator from float links has no FP64 copy"); return -1; }
  size_t per = qllg_link_bytes(prec)*(size_t)W->g.V;
  if(!(W->links[prec] = qllg_dmalloc(per*8))) return -1;
  for(int s=0; s<8; s++)
    if(qllg_k_link_convert(prec, (char *)W->links[prec] + per*s, NULL,
                           (const double *)W->links[QLLG_F64] + (size_t)s*18*W->g.V, W->g.V))
      return -1;
  return 0;
}

void
qllg_wilson_destroy(qllg_wilson *W)
{
  if(!W) return;
  qllg_sync();
  for(int p=0; p<QLLG_NLINKP; p++) qllg_dfree(W->links[p]);
  qllg_dfree(W->sc);
  if(W->hsc) cudaFreeHost(W->hsc);
  qllg_redbuf_free(&W->rb);
  for(int i=0; i<WW_N; i++) qllg_dfree(W->ws[i]);
  for(int i=0; i<WGRAPHS; i++) if(W->graphs[i].exec) cudaGraphExecDestroy(W->graphs[i].exec);
  if(W->ev0) cudaEventDestroy(W->ev0);
  if(W->ev1) cudaEventDestroy(W->ev1);
  free(W);
}

static qllg_wilson *
wilson_create(const int dims[4], void *const u[8], int dbl)
{
  if(qllg_runtime_init()) return NULL;
  qllg_wilson *W = calloc(1, sizeof(qllg_wilson));
  if(qllg_geom_from_dims(&W->g, dims)) { free(W); return NULL; }
  W->master = dbl ? QLLG_F64 : QLLG_F32;
  if(qllg_redbuf_init(&W->rb)) goto fail;
  if(!(W->sc = qllg_dmalloc(sizeof(qllg_cg_scalars)))) goto fail;
  if(qllg_check_cuda(cudaMallocHost((void **)&W->hsc, sizeof(qllg_cg_scalars)), "cudaMallocHost"))
    goto fail;
  cudaEventCreate(&W->ev0);
  cudaEventCreate(&W->ev1);
  {
    int prec = W->master;
    size_t per = qllg_link_bytes(prec)*(size_t)W->g.V;
    size_t hb = (dbl ? 8 : 4)*18*(size_t)W->g.V;
    void *st = qllg_stage(hb);
    if(!(W->links[prec] = qllg_dmalloc(per*8)) || !st) goto fail;
    for(int s=0; s<8; s++) {
      if(!u[s]) { qllg_set_error("Wilson link %d is NULL", s); goto fail; }
      if(qllg_h2d(st, u[s], hb) ||
         qllg_k_link_from_aos(prec, (char *)W->links[prec] + per*s, NULL, st, dbl, W->g.V))
        goto fail;
    }
    if(qllg_sync()) goto fail;
  }
  return W;
fail:
  qllg_wilson_destroy(W);
  return NULL;
}

qllg_wilson *
qllg_wilson_create(const int dims[4], double *const u[8])
{
  return wilson_create(dims, (void *const *)u, 1);
}

qllg_wilson *
qllg_wilson_create_f(const int dims[4], float *const u[8])
{
  return wilson_create(dims, (void *const *)u, 0);
}

/* one half-Dslash; with active_eq, only the rhs whose flag equals it */
static int
whalf_eq(qllg_wilson *W, int prec, int out_parity, const void *in, const void *self, void *out,
         int mode, double a0, double b, double *norm_out, double *norm_self, const int *active,
         int active_eq, const int *done, int dag)
{
  if(wlinks(W, prec)) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = W->g;
  A.out_parity = out_parity;
  A.nrhs = 1;
  A.nslots = 8;
  A.links = W->links[prec];
  A.in = in;
  A.self = self;
  A.out = out;
  A.mode = mode;
  A.a0 = a0;
  A.b = b;
  A.norm_out = norm_out;
  A.norm_self = norm_self;
  A.active = active;
  A.active_eq = active_eq;
  A.done = done;
  A.rb = &W->rb;
  A.dag = dag;
  qllg_tm_begin("wilson_dslash");
  int rc = qllg_k_wilson_dslash(prec, prec, &A);
  qllg_tm_end();
  return rc;
}

static int
whalf(qllg_wilson *W, int prec, int out_parity, const void *in, const void *self, void *out,
      int mode, double a0, double b, double *norm_out, double *norm_self, const int *active,
      const int *done, int dag)
{
  return whalf_eq(W, prec, out_parity, in, self, out, mode, a0, b, norm_out, norm_self, active, 0,
                  done, dag);
}

/* out = W in on the output parity (the massless hop term of wilsonDslash,
 * lib/wilsonDslash.c:21-179), device vectors in the library layout
 * ([12][Vh] complex) of precision prec (0 FP64, 1 FP32) */
int
qllg_wilson_dslash_device(qllg_wilson *W, int prec, int out_parity, void *out_dev,
                          const void *in_dev)
{
  if(!W || !out_dev || !in_dev) { qllg_set_error("wilson_dslash_device: null argument"); return -1; }
  if(prec != QLLG_F64 && prec != QLLG_F32) {
    qllg_set_error("wilson_dslash_device: precision %d", prec);
    return -1;
  }
  if(out_parity != 0 && out_parity != 1) {
    qllg_set_error("wilson_dslash_device: parity %d", out_parity);
    return -1;
  }
  return whalf(W, prec, out_parity, in_dev, NULL, out_dev, 0, 0, 1, NULL, NULL, NULL, NULL, 0);
}

/* bytes of one parity of a Wilson device vector in precision prec */
size_t
qllg_wilson_vec_bytes(const qllg_wilson *W, int prec)
{
  return (prec == QLLG_F64 || prec == QLLG_F32) ? wvec(W, prec) : 0;
}

static int
wup(qllg_wilson *W, int prec, void *dev, const void *host, int dbl, int site0)
{
  int Vh = W->g.Vh;
  size_t bytes = (dbl ? 8 : 4)*24*(size_t)Vh;
  void *st = qllg_stage(bytes);
  if(!st || qllg_h2d(st, (const char *)host + (dbl ? 8 : 4)*24*(size_t)site0, bytes)) return -1;
  return qllg_k_spinor_from_aos(prec, dev, st, dbl, Vh, 12, 1, 0);
}

static int
wdown(qllg_wilson *W, int prec, const void *dev, void *host, int dbl, int site0)
{
  int Vh = W->g.Vh;
  size_t bytes = (dbl ? 8 : 4)*24*(size_t)Vh;
  void *st = qllg_stage(bytes);
  if(!st || qllg_k_spinor_to_aos(prec, dev, st, dbl, Vh, 12, 1, 0)) return -1;
  return qllg_d2h((char *)host + (dbl ? 8 : 4)*24*(size_t)site0, st, bytes);
}

/* x = mass'*y + W y on the sites of sub (wilsonDslash with the mass
 * already combined as massFac*(4+m)); dag applies g5 D g5 */
int
qllg_wilson_dslash(qllg_wilson *W, void *x, double massp, const void *y, const char *sub, int dag)
{
  int prec = W->master, dbl = prec == QLLG_F64;
  int Vh = W->g.Vh;
  size_t vb = wvec(W, prec);
  char *io = wws(W, WW_IO, 4*vb);
  if(!io) return -1;
  void *ye = io, *yo = io + vb, *xe = io + 2*vb, *xo = io + 3*vb;
  int doe = !(sub && sub[0] == 'o'), doo = !(sub && sub[0] == 'e');
  if((doe && wup(W, prec, yo, y, dbl, Vh)) || (doo && wup(W, prec, ye, y, dbl, 0))) return -1;
  int m = (doe && doo && massp != 0) ? 1 : 0;
  if(doe && whalf(W, prec, 0, yo, m ? ye : NULL, xe, m, massp, 1, NULL, NULL, NULL, NULL, dag))
    return -1;
  if(doo && whalf(W, prec, 1, ye, m ? yo : NULL, xo, m, massp, 1, NULL, NULL, NULL, NULL, dag))
    return -1;
  if(doe && wdown(W, prec, xe, x, dbl, 0)) return -1;
  if(doo && wdown(W, prec, xo, x, dbl, Vh)) return -1;
  return 0;
}

/* ------------------------------------------- reference wilsonSolve */

static int
wpush(qllg_wilson *W)
{
  return qllg_check_cuda(cudaMemcpyAsync(W->sc, W->hsc, sizeof(qllg_cg_scalars),
                                         cudaMemcpyHostToDevice, qllg_stream()), "push scalars");
}

static int
wpull(qllg_wilson *W, int all)
{
  size_t n = all ? sizeof(qllg_cg_scalars) : sizeof(int);
  void *h = all ? (void *)W->hsc : (void *)&W->hsc->done;
  void *d = all ? (void *)W->sc : (void *)&W->sc->done;
  if(qllg_check_cuda(cudaMemcpyAsync(h, d, n, cudaMemcpyDeviceToHost, qllg_stream()), "pull"))
    return -1;
  return qllg_sync();
}

/* cgSolveT with the Wilson dslashp2 (lib/wilsonDslash.c:287-316): A x =
 * m^2 x - W_e W_o x, <x,Ax> = m^2|x|^2 + |W_o x|^2 over all 24 reals */
static int
wilson_ref_cg(qllg_wilson *W, void *x, const void *b, double mass, double rsq, int maxits)
{
  int prec = W->master;
  size_t vb = wvec(W, prec);
  void *r = wws(W, WW_R, vb), *p = wws(W, WW_P, vb), *Ap = wws(W, WW_AP, vb), *v = wws(W, WW_V, vb);
  if(!r || !p || !Ap || !v) return -1;
  memset(W->hsc, 0, sizeof(qllg_cg_scalars));
  W->hsc->mass2[0] = mass*mass;
  W->hsc->rsq_stop[0] = rsq;
  W->hsc->maxits = maxits;
  if(wpush(W)) return -1;
  int Vh = W->g.Vh;
  qllg_cg_scalars *sc = W->sc;
  if(qllg_k_cg_init(prec, x, r, p, b, Vh, 12, 1, sc, &W->rb)) return -1;
  int issued = 0, batch = 8;
  while(issued < maxits) {
    int k = maxits - issued < batch ? maxits - issued : batch;
    for(int it=0; it<k; it++) {
      if(qllg_k_cg_update_p(prec, p, r, Vh, 12, 1, sc)) return -1;
      if(whalf(W, prec, 1, p, NULL, v, 0, 0, 1, sc->vnorm, NULL, sc->active, &sc->done, 0))
        return -1;
      /* Ap = m^2 p - W_e v, with |p|^2 */
      if(whalf(W, prec, 0, v, p, Ap, 2, mass*mass, -1, NULL, sc->pnorm, sc->active, &sc->done, 0))
        return -1;
      if(qllg_k_cg_update_xr(prec, x, r, p, Ap, Vh, 12, 1, sc, &W->rb)) return -1;
    }
    issued += k;
    if(wpull(W, 0)) return -1;
    if(W->hsc->done) break;
    if(batch < 64) batch *= 2;
  }
  if(wpull(W, 1)) return -1;
  return W->hsc->iters[0];
}

/* ---------------------------------------------------- CGNR on S */

/* out = S in (dag: S^dagger); tmp: odd scratch; |out|^2 into norm */
static int
apply_schur_eq(qllg_wilson *W, int prec, const void *in, void *out, void *tmp, double a, int dag,
               double *norm, const int *active, int eq, const int *done)
{
  if(whalf_eq(W, prec, 1, in, NULL, tmp, 0, 0, 1, NULL, NULL, active, eq, done, dag)) return -1;
  return whalf_eq(W, prec, 0, tmp, in, out, 2, a, -1.0/a, norm, NULL, active, eq, done, dag);
}

static int
apply_schur(qllg_wilson *W, int prec, const void *in, void *out, void *tmp, double a, int dag,
            double *norm, const int *active, const int *done)
{
  return apply_schur_eq(W, prec, in, out, tmp, a, dag, norm, active, 0, done);
}

/* what one CGNR iteration launches */
typedef struct {
  int ps;
  double a;
  void *xs, *r, *p, *Ap, *Sp, *v;
  void *x64, *r64, *bp, *s64, *vv64, *t64, *xdf;
} witer;

/* the reliable update of the mixed CGNR when one is flagged (every launch
 * returns at once otherwise): x64 += x, t = S^+ S x64 (intermediate ones in
 * double-float on request, the final candidates in FP64), r64 = b' - t and
 * r = r64 rounded, with |r|^2 and beta for the p update that follows */
static int
wilson_ru_block(qllg_wilson *W, const witer *c)
{
  qllg_cg_scalars *sc = W->sc;
  const int Vh = W->g.Vh, ps = c->ps;
  const double a = c->a;
  if(qllg_k_mcg_accum(ps, c->x64, c->xs, Vh, 12, 1, sc)) return -1;
  /* the double-float pass reuses s64, vv64 and t64 (same size); t
   * goes back to FP64 in place */
  if(c->xdf && (qllg_k_spinor_df(1, c->xdf, c->x64, Vh, 12, 1, sc->ru, 1, &sc->no_ru) ||
                apply_schur_eq(W, QLLG_DF, c->xdf, c->s64, c->vv64, a, 0, NULL, sc->ru, 1,
                               &sc->no_ru) ||
                apply_schur_eq(W, QLLG_DF, c->s64, c->t64, c->vv64, a, 1, NULL, sc->ru, 1,
                               &sc->no_ru) ||
                qllg_k_spinor_df(0, c->t64, c->t64, Vh, 12, 1, sc->ru, 1, &sc->no_ru)))
    return -1;
  const int eq = c->xdf ? 2 : 0;
  if(apply_schur_eq(W, QLLG_F64, c->x64, c->s64, c->vv64, a, 0, NULL, sc->ru, eq, &sc->no_ru) ||
     apply_schur_eq(W, QLLG_F64, c->s64, c->t64, c->vv64, a, 1, NULL, sc->ru, eq, &sc->no_ru))
    return -1;
  return qllg_k_mcg_residual(ps, c->r64, c->r, c->bp, c->t64, Vh, 12, 1, 1, sc, &W->rb);
}

/* the last half Dslash of an FP32 iteration fused with the CG update:
 * Ap = a Sp - W_eo^dagger v / a stays in registers, x += alpha p,
 * r -= alpha Ap and |r|^2, then the iteration's bookkeeping; cond: the
 * graph conditional the last block sets when an update is flagged */
static int
whalf_update(qllg_wilson *W, const witer *c, unsigned long long cond)
{
  if(wlinks(W, QLLG_F32)) return -1;
  qllg_stag_args A;
  memset(&A, 0, sizeof(A));
  A.g = W->g;
  A.out_parity = 0;
  A.nrhs = 1;
  A.nslots = 8;
  A.links = W->links[QLLG_F32];
  A.in = c->v;
  A.self = c->Sp;
  A.mode = 4;
  A.a0 = c->a;
  A.b = -1.0/c->a;
  A.active = W->sc->active;
  A.done = &W->sc->done;
  A.rb = &W->rb;
  A.dag = 1;
  A.x = c->xs;
  A.r = c->r;
  A.pvec = c->p;
  A.sc = W->sc;
  A.cond = cond;
  qllg_tm_begin("wilson_dslash");
  int rc = qllg_k_wilson_dslash(QLLG_F32, QLLG_F32, &A);
  qllg_tm_end();
  return rc;
}

/* one iteration of the CGNR on S^dagger S (the standard-form CG update,
 * with the FP32 mode's reliable update of the flagged rhs); every launch
 * returns at once when the solve is done, the reliable-update ones when
 * no update is flagged.  FP32: the CG update runs in the epilogue of the
 * last half Dslash (parameter wilson_fused_update) */
static int
wilson_iteration(qllg_wilson *W, const witer *c)
{
  qllg_cg_scalars *sc = W->sc;
  const int Vh = W->g.Vh, ps = c->ps;
  const double a = c->a;
  const int fused = ps == QLLG_F32 && qllg_get_param("wilson_fused_update") != 0;
  /* in a captured loop the reliable-update block is the body of a
   * conditional IF node, taken only in the iterations that flag one */
  const int cond = ps != QLLG_F64 && qllg_capturing() && qllg_get_param("graph_ru_if") != 0;
  unsigned long long h = 0;
  if(cond && qllg_capture_cond(&h)) return -1;
  if(apply_schur(W, ps, c->p, c->Sp, c->v, a, 0, sc->pnorm, sc->active, &sc->done)) return -1;
  if(fused) {
    if(whalf(W, ps, 1, c->Sp, NULL, c->v, 0, 0, 1, NULL, NULL, sc->active, &sc->done, 1) ||
       whalf_update(W, c, h)) return -1;
  } else {
    if(apply_schur(W, ps, c->Sp, c->Ap, c->v, a, 1, NULL, sc->active, &sc->done)) return -1;
    if(qllg_k_scg_update_xr(ps, ps, c->xs, c->r, c->p, c->Ap, Vh, 12, 1, sc, &W->rb)) return -1;
    if(cond && qllg_k_ru_cond(h, &sc->no_ru, &sc->ru_trips)) return -1;
  }
  if(ps != QLLG_F64) {
    unsigned long long n1 = 0;
    if(cond) {
      if(qllg_capture_if_begin(h)) return -1;
      n1 = qllg_launch_count();
    }
    if(wilson_ru_block(W, c)) return -1;
    if(cond) {
      W->cap_ifbody = (int)(qllg_launch_count() - n1);
      if(qllg_capture_if_end()) return -1;
    }
  }
  return qllg_k_scg_update_p(ps, c->p, c->r, Vh, 12, 1, sc);
}

static void
wgraphs_drop(qllg_wilson *W)
{
  for(int i=0; i<WGRAPHS; i++) {
    if(W->graphs[i].exec) cudaGraphExecDestroy(W->graphs[i].exec);
    W->graphs[i].exec = NULL;
  }
}

/* a CUDA graph whose conditional WHILE node repeats one captured CGNR
 * iteration until the done flag is set or the trip cap is reached (the
 * staggered solver's loop_graph, for the Wilson iteration); cached by what
 * the launches bake in: precision, a = 4 + m, the solution buffers */
static cudaGraphExec_t
wilson_graph(qllg_wilson *W, const witer *c, int *body_out, int *ifbody_out)
{
  long abits;
  memcpy(&abits, &c->a, sizeof(abits));
  long key[7] = {c->ps, abits, (long)c->xs, (long)c->x64, (long)c->xdf, (long)c->bp,
                 (qllg_get_param("graph_ru_if") != 0) + 2*(qllg_get_param("wilson_fused_update") != 0)};
  for(int i=0; i<WGRAPHS; i++)
    if(W->graphs[i].exec && !memcmp(W->graphs[i].key, key, sizeof(key))) {
      *body_out = W->graphs[i].body;
      *ifbody_out = W->graphs[i].ifbody;
      return W->graphs[i].exec;
    }
  W->cap_ifbody = 0;
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
    int rc = wilson_iteration(W, c);
    rc |= qllg_k_loop_cond((unsigned long long)h, &W->sc->done, &W->sc->loops,
                           &W->sc->loop_limit);
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
    int i = W->ngraph_next;
    W->ngraph_next = (i + 1) % WGRAPHS;
    if(W->graphs[i].exec) cudaGraphExecDestroy(W->graphs[i].exec);
    memcpy(W->graphs[i].key, key, sizeof(key));
    W->graphs[i].exec = exec;
    W->graphs[i].body = all - W->cap_ifbody;
    W->graphs[i].ifbody = W->cap_ifbody;
    *body_out = all - W->cap_ifbody;
    *ifbody_out = W->cap_ifbody;
  }
  return exec;
fail:
  if(qllg_capturing()) qllg_capture_end(np.conditional.phGraph_out[0]);
  if(g) cudaGraphDestroy(g);
  return NULL;
}

int qllg_timing_on(void);

/* the FP32 iterations as persistent launches (k_wilson.cu), each running
 * until a reliable update is flagged; the host takes the update with the
 * FP64 kernels, forms p and launches again */
static int
wilson_persistent_loop(qllg_wilson *W, const witer *c, int maxits)
{
  unsigned *ctl = wws(W, WW_CTL, 4*sizeof(unsigned));
  if(!ctl || wlinks(W, QLLG_F32)) return -1;
  if(qllg_check_cuda(cudaMemsetAsync(ctl, 0, 4*sizeof(unsigned), qllg_stream()),
                     "persistent CGNR: control words")) return -1;
  qllg_wcgp_args a;
  memset(&a, 0, sizeof(a));
  a.g = W->g;
  a.links = W->links[QLLG_F32];
  a.x = c->xs; a.r = c->r; a.p = c->p; a.Sp = c->Sp; a.v = c->v;
  a.sc = W->sc;
  a.a = c->a;
  a.partial = W->rb.partial;
  a.partial_len = 2*QLLG_MAXRHS*(size_t)W->rb.maxblocks;
  a.bar = ctl;
  a.err = (int *)(ctl + 2);
  a.poll_limit = (long long)qllg_get_param("wait_polls");
  a.extra = (int)qllg_get_param("cg_barrier_extra");
  a.trips = maxits + 2;
  for(int launch = 0; launch <= maxits + 2; launch++) {
    int grid = 0, err = 0;
    if(qllg_k_wilson_cgnr_persistent(&a, &grid) ||
       qllg_check_cuda(cudaMemcpyAsync(&err, ctl + 2, sizeof(int), cudaMemcpyDeviceToHost,
                                       qllg_stream()), "persistent CGNR: error flag") ||
       wpull(W, 1)) return -1;
    if(err) {
      qllg_set_error("persistent CGNR: a grid barrier wait ran out (%lld polls)", a.poll_limit);
      return -1;
    }
    if(W->hsc->done || W->hsc->no_ru) break;
    if(wilson_ru_block(W, c) ||
       qllg_k_scg_update_p(QLLG_F32, c->p, c->r, W->g.Vh, 12, 1, W->sc)) return -1;
  }
  if(wpull(W, 1)) return -1;
  return W->hsc->iters[0];
}

static int
wilson_cgnr(qllg_wilson *W, void *x64, const void *b64, double mass, double rsq, int maxits,
            int mode)
{
  double a = 4 + mass;
  size_t v64 = wvec(W, QLLG_F64);
  void *bp = wws(W, WW_B, v64), *s64 = wws(W, WW_S64, v64), *vv64 = wws(W, WW_V64, v64);
  void *t64 = wws(W, WW_T64, v64), *r64 = wws(W, WW_R64, v64);
  if(!bp || !s64 || !vv64 || !t64 || !r64) return -1;
  int Vh = W->g.Vh;
  /* b' = S^dagger b in FP64 */
  if(apply_schur(W, QLLG_F64, b64, bp, vv64, a, 1, NULL, NULL, NULL)) return -1;
  int ps = (mode == QLLG_SOLVE_DOUBLE) ? QLLG_F64 : QLLG_F32;
  size_t vs = wvec(W, ps);
  void *xs = (ps == QLLG_F64) ? x64 : wws(W, WW_X, vs);
  void *r = wws(W, WW_R, vs), *p = wws(W, WW_P, vs), *Ap = wws(W, WW_AP, vs);
  void *Sp = wws(W, WW_S, vs), *v = wws(W, WW_V, vs);
  if(!xs || !r || !p || !Ap || !Sp || !v) return -1;
  /* the FP32 iterations as persistent launches on small lattices */
  const int persist = ps == QLLG_F32 && qllg_get_param("wilson_persistent") != 0 && !qllg_timing_on() &&
                      (double)Vh <= qllg_get_param("wilson_persistent_max");
  /* intermediate reliable updates (ru 1) in double-float (wilson_ru_df 1,
   * or 2 with the persistent iterations): S^+ S x in the FP32 pipes at
   * about 44-bit precision; the final one (ru 2), whose residual may end
   * the solve, in FP64 */
  void *xdf = NULL;
  const double rdf = qllg_get_param("wilson_ru_df");
  if(ps != QLLG_F64 && (rdf == 1 || (rdf == 2 && persist)) &&
     (wlinks(W, QLLG_DF) || !(xdf = wws(W, WW_XDF, wvec(W, QLLG_DF))))) return -1;
  memset(W->hsc, 0, sizeof(qllg_cg_scalars));
  W->hsc->rsq_stop[0] = rsq;
  W->hsc->maxits = maxits;
  W->hsc->loop_limit = maxits + 2;
  const double delta = qllg_get_param("wilson_delta");
  W->hsc->delta2 = (ps == QLLG_F64) ? 0 : delta*delta;
  if(wpush(W)) return -1;
  qllg_cg_scalars *sc = W->sc;
  if(qllg_k_scg_init(ps, ps, xs, r, p, bp, ps == QLLG_F64 ? NULL : x64,
                     ps == QLLG_F64 ? NULL : r64, Vh, 12, 1, sc, &W->rb)) return -1;
  witer c = {ps, a, xs, r, p, Ap, Sp, v, x64, r64, bp, s64, vv64, t64, xdf};
  if(persist) return wilson_persistent_loop(W, &c, maxits);
  if(qllg_get_param("graph") != 0 && !qllg_timing_on()) {
    /* one iteration launched directly first (every kernel of the body is
     * then loaded before the capture), then the rest as one graph launch */
    if(wilson_iteration(W, &c)) return -1;
    int body = 0, ifbody = 0;
    cudaGraphExec_t exec = wilson_graph(W, &c, &body, &ifbody);
    if(!exec || qllg_check_cuda(cudaGraphLaunch(exec, qllg_stream()), "graph launch")) return -1;
    if(wpull(W, 1)) return -1;
    qllg_launch_adjust((long long)body*W->hsc->loops + (long long)ifbody*W->hsc->ru_trips);
    return W->hsc->iters[0];
  }
  int issued = 0, batch = 8;
  while(issued < maxits) {
    int k = maxits - issued < batch ? maxits - issued : batch;
    for(int it=0; it<k; it++) if(wilson_iteration(W, &c)) return -1;
    issued += k;
    if(wpull(W, 0)) return -1;
    if(W->hsc->done) break;
    if(batch < 64) batch *= 2;
  }
  if(wpull(W, 1)) return -1;
  return W->hsc->iters[0];
}

/* native: solve S x = b_e by CGNR; x, b host [V][24] (even half) */
int
qllg_wilson_solve(qllg_wilson *W, void *x, const void *b, double mass, double rsq, int maxits,
                  int mode, qllg_solve_info *info)
{
  if(W->master != QLLG_F64) { qllg_set_error("wilson_solve: needs an FP64 operator"); return -1; }
  if(mode != QLLG_SOLVE_DOUBLE && mode != QLLG_SOLVE_MIXED_SINGLE) {
    qllg_set_error("wilson_solve: mode %d (DOUBLE or MIXED_SINGLE)", mode);
    return -1;
  }
  if(rsq < 0) rsq = -rsq;
  size_t v64 = wvec(W, QLLG_F64);
  void *bd = wws(W, WW_IO, 2*v64);
  if(!bd) return -1;
  void *xd = (char *)bd + v64;
  if(wup(W, QLLG_F64, bd, b, 1, 0)) return -1;
  cudaEventRecord(W->ev0, qllg_stream());
  int its = wilson_cgnr(W, xd, bd, mass, rsq, maxits, mode);
  cudaEventRecord(W->ev1, qllg_stream());
  if(its < 0) return -1;
  if(info) {
    memset(info, 0, sizeof(*info));
    cudaEventSynchronize(W->ev1);
    float ms = 0;
    cudaEventElapsedTime(&ms, W->ev0, W->ev1);
    info->seconds = ms*1e-3;
    info->iters[0] = its;
    info->total_iters = its;
    info->reliable_updates = W->hsc->nru[0];
    info->rsq[0] = W->hsc->bsq[0] > 0 ? W->hsc->rsq[0]/W->hsc->bsq[0] : 0;
    /* true residual of S x = b in FP64 */
    void *t = wws(W, WW_T64, v64), *vv = wws(W, WW_V64, v64);
    double a = 4 + mass;
    if(!t || !vv || apply_schur(W, QLLG_F64, xd, t, vv, a, 0, NULL, NULL, NULL)) return -1;
    if(qllg_k_axpby(QLLG_F64, t, QLLG_F64, bd, NULL, -1.0, NULL, 1.0, W->g.Vh, 12, 1, NULL)) return -1;
    double *dn = W->sc->tmp, num, den;
    if(qllg_k_norm2(QLLG_F64, t, W->g.Vh, 12, 1, dn, &W->rb) || qllg_d2h(&num, dn, 8)) return -1;
    if(qllg_k_norm2(QLLG_F64, bd, W->g.Vh, 12, 1, dn, &W->rb) || qllg_d2h(&den, dn, 8)) return -1;
    info->true_rsq[0] = den > 0 ? num/den : 0;
  }
  if(wdown(W, QLLG_F64, xd, x, 1, 0)) return -1;
  return its;
}

/* ------------------------------------------------- drop-in layer */

typedef struct {
  char t[8][sizeof(TransporterD)];
  qllg_wilson *W;
  int own;
  int parity;
} wlinks_priv;

static int
wsub_parity(const char *sub)
{
  return (sub && sub[0] == 'e') ? 0 : ((sub && sub[0] == 'o') ? 1 : -1);
}

#define DEFINE_WILSON_DROPIN(S_, real, DBL)                                       \
static void                                                                       \
wfill##S_(WilsonLinks##S_ *sl, Layout *l, real *u[], char *sub, qllg_wilson *W, int own) \
{                                                                                 \
  wlinks_priv *pv = calloc(1, sizeof(wlinks_priv));                               \
  pv->W = W;                                                                      \
  pv->own = own;                                                                  \
  pv->parity = wsub_parity(sub);                                                  \
  Transporter##S_ *t = (Transporter##S_ *)pv->t;                                  \
  for(int i=0; i<8; i++) {                                                        \
    t[i].u = u[i];                                                                \
    t[i].nelem = 24;                                                              \
    t[i].nc = 3;                                                                  \
    layoutSubset(&t[i].sub, l, sub);                                              \
  }                                                                               \
  sl->t = t;                                                                      \
  sl->n = 8;                                                                      \
  sl->massFac = pv->parity >= 0 ? 0 : 1;                                          \
  sl->fb = 0;                                                                     \
}                                                                                 \
                                                                                  \
void                                                                              \
createWilsonLinks##S_(WilsonLinks##S_ *sl, Layout *l, real *u[], char *sub)       \
{                                                                                 \
  memset(sl, 0, sizeof(*sl));                                                     \
  qllg_geom g;                                                                    \
  if(qllg_geom_from_layout(&g, l)) return;                                        \
  qllg_wilson *W = wilson_create(g.L, (void *const *)u, DBL);                     \
  if(W) wfill##S_(sl, l, u, sub, W, 1);                                           \
}                                                                                 \
                                                                                  \
void                                                                              \
freeWilsonLinks##S_(WilsonLinks##S_ *sl)                                          \
{                                                                                 \
  if(!sl || !sl->t) return;                                                       \
  wlinks_priv *pv = (wlinks_priv *)(void *)sl->t;                                 \
  if(pv->own) qllg_wilson_destroy(pv->W);                                         \
  free(pv);                                                                       \
  sl->t = NULL;                                                                   \
}                                                                                 \
                                                                                  \
void                                                                              \
wilsonDslash##S_(WilsonLinks##S_ *d, real *x, real mass, int sign, real *y)       \
{                                                                                 \
  (void)sign;                                                                     \
  if(!d || !d->t) { qllg_set_error("wilsonDslash: links not created"); return; }  \
  wlinks_priv *pv = (wlinks_priv *)(void *)d->t;                                  \
  mass = d->massFac*(4 + mass);                                                   \
  qllg_wilson_dslash(pv->W, x, (double)mass, y,                                   \
                     pv->parity == 0 ? "even" : (pv->parity == 1 ? "odd" : "all"), 0); \
}                                                                                 \
                                                                                  \
void                                                                              \
createWilsonSolver##S_(WilsonSolver##S_ *ss, Layout *l, real *u[], char *sub)     \
{                                                                                 \
  (void)sub;                                                                      \
  memset(ss, 0, sizeof(*ss));                                                     \
  qllg_geom g;                                                                    \
  if(qllg_geom_from_layout(&g, l)) return;                                        \
  qllg_wilson *W = wilson_create(g.L, (void *const *)u, DBL);                     \
  if(!W) return;                                                                  \
  wfill##S_(&ss->sle, l, u, "even", W, 1);                                        \
  wfill##S_(&ss->slo, l, u, "odd", W, 0);                                         \
  cglsInit##S_(&ss->cgls, 24*l->nEvenOuter);                                      \
  layoutSubset(&ss->sube, l, "even");                                             \
  layoutSubset(&ss->subo, l, "odd");                                              \
}                                                                                 \
                                                                                  \
void                                                                              \
freeWilsonSolver##S_(WilsonSolver##S_ *ss)                                        \
{                                                                                 \
  freeWilsonLinks##S_(&ss->slo);                                                  \
  freeWilsonLinks##S_(&ss->sle);                                                  \
}                                                                                 \
                                                                                  \
int                                                                               \
wilsonSolve##S_(WilsonSolver##S_ *ss, real *x, real mass, real *y, double rsq,    \
                int maxits, char *sub)                                            \
{                                                                                 \
  (void)sub;                                                                      \
  if(!ss->sle.t) { qllg_set_error("wilsonSolve: solver not created"); return -1; }\
  qllg_wilson *W = ((wlinks_priv *)(void *)ss->sle.t)->W;                         \
  ss->mass = mass;                                                                \
  if(rsq < 0) { ss->cgls.verbose = 3; rsq = -rsq; }                               \
  int prec = W->master;                                                           \
  size_t vb = wvec(W, prec);                                                      \
  char *io = wws(W, WW_IO, 2*vb);                                                 \
  if(!io) return -1;                                                              \
  if(wup(W, prec, io, y, DBL, 0)) return -1;                                      \
  int its = wilson_ref_cg(W, io + vb, io, ss->mass, rsq, maxits);                 \
  ss->its = its;                                                                  \
  if(its < 0) return -1;                                                          \
  if(!ss->noscale &&                                                              \
     qllg_k_axpby(prec, io + vb, prec, io + vb, NULL, 0.0, NULL, (double)mass,    \
                  W->g.Vh, 12, 1, NULL)) return -1;                               \
  if(wdown(W, prec, io + vb, x, DBL, 0)) return -1;                               \
  return its;                                                                     \
}                                                                                 \
                                                                                  \
int                                                                               \
wilsonSolveMulti##S_(WilsonSolver##S_ *ss, real *x[], double masses[], int nmasses,\
                     real *y, double rsq, int maxits, char *sub)                  \
{                                                                                 \
  (void)ss; (void)x; (void)masses; (void)nmasses; (void)y; (void)rsq;             \
  (void)maxits; (void)sub;                                                        \
  qllg_set_error("wilsonSolveMulti: not available (the reference's body is disabled)"); \
  return -1;                                                                      \
}

DEFINE_WILSON_DROPIN(D, double, 1)
DEFINE_WILSON_DROPIN(F, float, 0)
