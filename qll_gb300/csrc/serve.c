/*
 * serve.c -- a solve-request loop over resident lattices with continuous
 * batching.
 *
 * The reference has no serving layer: its solvers are called one at a time
 * (solve2 / solveMulti2, lib/stagDslash.c:600-657).  Here a server keeps the
 * links of several lattices resident, takes solve requests (lattice, mass,
 * shifts, tolerance, source) as they arrive and runs them as columns of
 * 16-wide mixed-precision batches (stag.c, qllg_batch_*):
 *
 *  - a request with n shifts occupies n columns, column k solving
 *    (m^2 + shift_k - D_eo D_oe) x_k = b, i.e. mass sqrt(m^2 + shift_k);
 *  - batches advance in chunks (one graph launch of at most `chunk`
 *    iterations each); between two chunks of a batch its finished columns
 *    are retired and queued requests are admitted into free columns, while
 *    the other columns carry on where they were (continuous batching);
 *  - every batch has its own CUDA stream, so batches of different lattices
 *    (and several batches of one lattice) run concurrently;
 *  - a new batch (its workspaces) is created only while the device bytes of
 *    the resident links plus all batches stay within the HBM budget; idle
 *    batches are released when the budget is short.
 *
 * A column's arithmetic never involves another column (per-rhs scalars,
 * per-rhs reductions in a fixed order, a fixed grid for the fixed width),
 * so a request gives bitwise the same solution whichever requests run
 * beside it and whenever it was admitted.
 *
 * One host thread drives a server (qllg_server_step); nothing here blocks
 * except the copy of a finished solution to the caller's buffer.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

#define NCOL QLLG_MAXRHS
#define MAXLAT 16
#define MAXBATCH 64

/* a request ends DONE when every shift met its tolerance, FAILED when one
 * did not (a source or solution that is not a number, or the iteration
 * limit); either way its columns are freed and its batch-mates go on */
enum { REQ_QUEUED = 0, REQ_RUNNING = 1, REQ_DONE = 2, REQ_FAILED = 3 };

typedef struct {
  int lattice, ncol, state, batch, left, failed;
  double mass[NCOL], tol;
  const double *src;
  double *out[NCOL];
  int iters[NCOL];
  double true_rsq[NCOL];
  double t_submit, t_start, t_done;
} req_t;

typedef struct {
  qllg_stag *S;            /* shares the lattice operator's links */
  int lattice;
  cudaStream_t st;
  int running;             /* a chunk is in flight */
  int col_req[NCOL];       /* request in each column, -1 when free */
  int col_k[NCOL];         /* which of the request's shifts */
  int nfree;
  size_t bytes;
} batch_t;

struct qllg_server {
  size_t budget, used;
  int chunk, maxits, maxb;
  int nlat;
  struct { qllg_stag *S; size_t bytes; int nbatch; } lat[MAXLAT];
  batch_t b[MAXBATCH];
  int nb;
  req_t *req;
  int nreq, cap, first_open;
  long long admitted_cols, chunks;
};

static double
now_s(void)
{
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9*t.tv_nsec;
}

qllg_server *
qllg_server_create(size_t hbm_budget, int chunk_iters, int max_batches_per_lattice)
{
  if(qllg_runtime_init()) return NULL;
  if(chunk_iters < 1 || max_batches_per_lattice < 1) {
    qllg_set_error("server_create: chunk %d, batches per lattice %d", chunk_iters,
                   max_batches_per_lattice);
    return NULL;
  }
  qllg_server *V = calloc(1, sizeof(qllg_server));
  if(!V) { qllg_set_error("server_create: out of host memory"); return NULL; }
  V->budget = hbm_budget;
  V->chunk = chunk_iters;
  V->maxits = 20000;
  V->maxb = max_batches_per_lattice;
  return V;
}

int
qllg_server_add_lattice(qllg_server *V, qllg_stag *S)
{
  if(V->nlat == MAXLAT) { qllg_set_error("server: more than %d lattices", MAXLAT); return -1; }
  /* the batches run FP32 Dslashes and double-float/FP64 reliable updates
   * on these links: make them resident now and count them */
  qllg_stag *probe = qllg_stag_share(S);
  if(!probe) return -1;
  qllg_stag_destroy(probe);
  size_t bytes = qllg_stag_device_bytes(S);
  if(V->used + bytes > V->budget) {
    qllg_set_error("server: lattice needs %zu bytes, %zu of the %zu-byte budget left", bytes,
                   V->budget - V->used, V->budget);
    return -1;
  }
  V->lat[V->nlat].S = S;
  V->lat[V->nlat].bytes = bytes;
  V->lat[V->nlat].nbatch = 0;
  V->used += bytes;
  return V->nlat++;
}

int
qllg_server_submit(qllg_server *V, int lattice, double mass, int nshift, const double *shifts,
                   double tol, const double *src, double *const out[])
{
  if(lattice < 0 || lattice >= V->nlat) { qllg_set_error("submit: lattice %d", lattice); return -1; }
  int n = nshift < 1 ? 1 : nshift;
  if(n > NCOL) { qllg_set_error("submit: %d shifts (at most %d)", nshift, NCOL); return -1; }
  if(!(tol > 0) || !src || !out) { qllg_set_error("submit: tolerance or buffers"); return -1; }
  for(int k=0; k<n; k++) {
    double m2 = mass*mass + (nshift >= 1 ? shifts[k] : 0);
    if(!(m2 > 0)) { qllg_set_error("submit: shift %d gives m^2 = %g", k, m2); return -1; }
    if(!out[k]) { qllg_set_error("submit: output %d is NULL", k); return -1; }
  }
  if(V->nreq == V->cap) {
    int cap = V->cap ? 2*V->cap : 256;
    req_t *r = realloc(V->req, sizeof(req_t)*cap);
    if(!r) { qllg_set_error("submit: out of host memory"); return -1; }
    V->req = r;
    V->cap = cap;
  }
  req_t *R = &V->req[V->nreq];
  memset(R, 0, sizeof(*R));
  R->lattice = lattice;
  R->ncol = n;
  R->state = REQ_QUEUED;
  R->batch = -1;
  R->tol = tol;
  R->src = src;
  for(int k=0; k<n; k++) {
    R->mass[k] = sqrt(mass*mass + (nshift >= 1 ? shifts[k] : 0));
    R->out[k] = out[k];
  }
  R->t_submit = now_s();
  return V->nreq++;
}

static void
batch_free(qllg_server *V, int i)
{
  batch_t *B = &V->b[i];
  if(B->st) cudaStreamSynchronize(B->st);
  qllg_stag_destroy(B->S);
  if(B->st) cudaStreamDestroy(B->st);
  V->used -= B->bytes;
  V->lat[B->lattice].nbatch--;
  V->b[i] = V->b[--V->nb];
  /* requests point at batches by index: fix the moved one's */
  for(int r=V->first_open; r<V->nreq; r++)
    if(V->req[r].state == REQ_RUNNING && V->req[r].batch == V->nb) V->req[r].batch = i;
}

/* a new batch for lattice l within the budget (releasing idle batches if
 * that makes room): its index, -1 at the batch-count limits, -3 when the
 * budget has no room, -2 on an error */
static int
batch_new(qllg_server *V, int l)
{
  if(V->nb == MAXBATCH || V->lat[l].nbatch >= V->maxb) return -1;
  qllg_stag *S = V->lat[l].S;
  size_t need = qllg_batch_bytes(S) + (size_t)(1 << 20);
  for(int i=0; i<V->nb && V->used + need > V->budget; ) {
    if(!V->b[i].running && V->b[i].nfree == NCOL) { batch_free(V, i); continue; }
    i++;
  }
  if(V->used + need > V->budget) return -3;
  batch_t *B = &V->b[V->nb];
  memset(B, 0, sizeof(*B));
  B->lattice = l;
  if(qllg_check_cuda(cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking), "batch stream"))
    return -2;
  cudaStream_t old = qllg_stream_swap(B->st);
  B->S = qllg_stag_share(S);
  int rc = B->S ? qllg_batch_init(B->S, V->maxits) : -1;
  qllg_stream_swap(old);
  if(rc) {
    qllg_stag_destroy(B->S);
    cudaStreamDestroy(B->st);
    return -2;
  }
  B->bytes = qllg_stag_device_bytes(B->S);
  for(int c=0; c<NCOL; c++) B->col_req[c] = -1;
  B->nfree = NCOL;
  V->used += B->bytes;
  V->lat[l].nbatch++;
  return V->nb++;
}

/* retire the finished columns of batch i; returns requests completed */
static int
batch_harvest(qllg_server *V, int i)
{
  batch_t *B = &V->b[i];
  const qllg_cg_scalars *h = qllg_batch_scalars(B->S);
  int done = 0;
  for(int c=0; c<NCOL; c++) {
    int r = B->col_req[c];
    if(r < 0 || h->active[c]) continue;
    req_t *R = &V->req[r];
    int k = B->col_k[c];
    if(qllg_batch_retire(B->S, c, R->out[k])) return -1;
    R->iters[k] = h->iters[c];
    /* |b|^2 is 0 only for a zero source (x = 0 is exact); a source that is
     * not a number leaves NaN here */
    R->true_rsq[k] = h->bsq[c] > 0 || h->bsq[c] != h->bsq[c] ? h->rsq[c]/h->bsq[c] : 0;
    if(!(R->true_rsq[k] < R->tol*R->tol)) R->failed = 1;
    B->col_req[c] = -1;
    B->nfree++;
    if(--R->left == 0) {
      R->state = R->failed ? REQ_FAILED : REQ_DONE;
      R->t_done = now_s();
      done++;
    }
  }
  return done;
}

static int
admit(qllg_server *V, int r, int i)
{
  batch_t *B = &V->b[i];
  req_t *R = &V->req[r];
  int cols[NCOL];
  double tol[NCOL];
  const double *src[NCOL];
  int n = 0;
  for(int c=0; c<NCOL && n < R->ncol; c++) {
    if(B->col_req[c] >= 0) continue;
    cols[n] = c;
    tol[n] = R->tol;
    src[n] = R->src;
    B->col_req[c] = r;
    B->col_k[c] = n;
    n++;
  }
  B->nfree -= n;
  R->left = n;
  R->batch = i;
  R->state = REQ_RUNNING;
  R->t_start = now_s();
  V->admitted_cols += n;
  return qllg_batch_admit(B->S, n, cols, R->mass, tol, src);
}

int
qllg_server_step(qllg_server *V)
{
  cudaStream_t old = qllg_stream_swap(qllg_stream());
  int completed = 0, rc = 0;
  /* 1. finished chunks: retire finished columns */
  for(int i=0; i<V->nb; i++) {
    batch_t *B = &V->b[i];
    if(!B->running) continue;
    qllg_stream_swap(B->st);
    int p = qllg_batch_poll(B->S);
    if(p < 0) { rc = -1; goto out; }
    if(!p) continue;
    B->running = 0;
    int d = batch_harvest(V, i);
    if(d < 0) { rc = -1; goto out; }
    completed += d;
  }
  /* 2. admission, oldest request first.  A lattice whose oldest queued
   * request cannot be placed now admits nothing later this pass; and once
   * a request waits for HBM, other lattices admit nothing more until it is
   * placed, so their batches drain and can be released for it. */
  {
    int blocked[MAXLAT] = {0};
    int starving = -1;
    while(V->first_open < V->nreq && V->req[V->first_open].state >= REQ_DONE) V->first_open++;
    for(int r=V->first_open; r<V->nreq; r++) {
      req_t *R = &V->req[r];
      if(R->state != REQ_QUEUED || blocked[R->lattice]) continue;
      if(starving >= 0 && R->lattice != starving) continue;
      int target = -1, waiting = 0;
      for(int i=0; i<V->nb; i++) {
        batch_t *B = &V->b[i];
        if(B->lattice != R->lattice || B->nfree < R->ncol) continue;
        if(B->running) { waiting = 1; continue; }
        /* the fullest batch that fits keeps the others free for wide requests */
        if(target < 0 || B->nfree < V->b[target].nfree) target = i;
      }
      if(target < 0 && !waiting) {
        qllg_stream_swap(old);
        target = batch_new(V, R->lattice);
        if(target == -2) { rc = -1; goto out; }
        if(target == -3 && starving < 0) starving = R->lattice;
      }
      if(target < 0) { blocked[R->lattice] = 1; continue; }
      qllg_stream_swap(V->b[target].st);
      if(admit(V, r, target)) { rc = -1; goto out; }
    }
  }
  /* 3. next chunk of every batch with work */
  for(int i=0; i<V->nb; i++) {
    batch_t *B = &V->b[i];
    if(B->running || B->nfree == NCOL) continue;
    qllg_stream_swap(B->st);
    if(qllg_batch_launch(B->S, V->chunk)) { rc = -1; goto out; }
    B->running = 1;
    V->chunks++;
  }
out:
  qllg_stream_swap(old);
  return rc ? -1 : completed;
}

int
qllg_server_pending(const qllg_server *V)
{
  int n = 0;
  for(int r=V->first_open; r<V->nreq; r++) n += V->req[r].state < REQ_DONE;
  return n;
}

int
qllg_server_request(const qllg_server *V, int id, qllg_request_info *info)
{
  if(id < 0 || id >= V->nreq) { qllg_set_error("server_request: id %d", id); return -1; }
  const req_t *R = &V->req[id];
  memset(info, 0, sizeof(*info));
  info->status = R->state;
  info->ncol = R->ncol;
  for(int k=0; k<R->ncol; k++) {
    info->iters[k] = R->iters[k];
    info->true_rsq[k] = R->true_rsq[k];
  }
  if(R->state != REQ_QUEUED) info->seconds_queued = R->t_start - R->t_submit;
  if(R->state >= REQ_DONE) info->seconds_total = R->t_done - R->t_submit;
  return 0;
}

int
qllg_server_stats(const qllg_server *V, qllg_server_info *info)
{
  memset(info, 0, sizeof(*info));
  info->budget_bytes = V->budget;
  info->used_bytes = V->used;
  info->batches = V->nb;
  for(int i=0; i<V->nb; i++) info->busy_columns += NCOL - V->b[i].nfree;
  info->requests = V->nreq;
  info->pending = qllg_server_pending(V);
  info->admitted_columns = V->admitted_cols;
  info->chunks = V->chunks;
  return 0;
}

void
qllg_server_destroy(qllg_server *V)
{
  if(!V) return;
  while(V->nb) batch_free(V, V->nb - 1);
  free(V->req);
  free(V);
}
