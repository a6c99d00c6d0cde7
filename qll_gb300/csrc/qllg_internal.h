/*
 * qllg_internal.h -- internal interface between the C host code of
 * libqll_gb300 and its CUDA kernels (kernel launchers are extern "C").
 *
 * Device data layout (all fields are split by parity; a parity block holds
 * Vh = V/2 sites numbered as the reference's VLEN=1 layoutIndex does:
 * lexicographic with x0 fastest, halved):
 *
 *  - spinor, FP64/FP32, nrhs right-hand sides: component-major
 *    [3 colours][Vh sites][nrhs] of double2/float2 (re,im), so consecutive
 *    threads (rhs fastest, then site) read consecutive 8/16-byte words;
 *  - spinor, 16-bit: [Vh sites][nrhs] of int4 = six int16 (colour re/im,
 *    fixed point, full scale 32767) plus the float scale max|component|:
 *    one 128-bit load per site and rhs;
 *  - Wilson spinor: as above with 12 colour-spin components (FP64/FP32
 *    component-major [12][Vh][nrhs]);
 *  - 3x3 link field slot s, FP64/FP32: [9 complex entries][V sites] of
 *    double2/float2, entry k = 3*column + row (the reference's column-major
 *    Mat3, lib/vla.c:9-11), sites in full-lattice order (even block then odd
 *    block);
 *  - link field, 16-bit: [V sites] x (int4, int4, int) = 18 int16 fixed
 *    point with one float scale per slot.
 */
#ifndef QLLG_INTERNAL_H
#define QLLG_INTERNAL_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QLLG_MAXRHS 16

typedef struct {
  int L[4];   /* physical extents, all even and >= 4 */
  int V;      /* sites */
  int Vh;     /* sites per parity */
} qllg_geom;

enum { QLLG_F64 = 0, QLLG_F32 = 1, QLLG_I16 = 2,
       QLLG_F32R = 3,     /* links only: FP32 in 16-byte vectors, Naik slots as
                             two rows + a per-site sign (reconstruct-12) */
       QLLG_DF = 4 };     /* double-float: each real as the unevaluated sum of
                             two floats (hi, lo), same bytes as FP64; the
                             reliable-update Dslash computes in it with FP32
                             instructions */
#define QLLG_NLINKP 5

/* ------------------------------------------------------------ geometry */
struct Layout_s;
int qllg_geom_from_dims(qllg_geom *g, const int dims[4]);
void *qllg_stage(size_t bytes);          /* shared device staging buffer */
void qllg_stage_release(void);
/* bytes of one site and rhs of a spinor with ncomp complex components */
static inline size_t qllg_spinor_bytes(int prec, int ncomp) {
  return (prec == QLLG_F64 || prec == QLLG_DF) ? 16u*ncomp : (prec == QLLG_F32 ? 8u*ncomp : 16u);
}
static inline size_t qllg_link_bytes(int prec) {
  return (prec == QLLG_F64 || prec == QLLG_DF) ? 144u : (prec == QLLG_F32 ? 72u : 36u);
}

/* ------------------------------------------------------------ runtime */
int   qllg_runtime_init(void);                 /* 0 ok */
cudaStream_t qllg_stream(void);                /* current library stream */
void  qllg_set_error(const char *fmt, ...);
cudaStream_t qllg_stream_swap(cudaStream_t s);
void qllg_launch_adjust(long long n);
/* autotuner registry (tune.c): the variant chosen for a launch shape */
int  qllg_tune_lookup(const char *key);
void qllg_tune_store(const char *key, int choice, int ncand, const float *ms,
                     const char *const *names);
int   qllg_check_cuda(cudaError_t e, const char *what);   /* 0 ok */
void *qllg_dmalloc(size_t bytes);              /* NULL + error on failure */
void  qllg_dfree(void *p);
/* host <-> device copies on the library stream: at least 1 MiB between
   page-locked host memory and device memory, 16-byte aligned, runs on the
   SMs (qllg_k_copy16); anything else on a copy engine.  qllg_d2h waits for
   the copy, qllg_d2h_async does not */
int   qllg_h2d(void *d, const void *h, size_t bytes);
int   qllg_d2h(void *h, const void *d, size_t bytes);
int   qllg_d2h_async(void *h, const void *d, size_t bytes);
int   qllg_k_copy16(void *dst, const void *src, size_t bytes);
int   qllg_sync(void);
int   qllg_num_sms(void);
/* CUDA graph capture of library launches (graph bodies) */
int   qllg_capturing(void);
int   qllg_capture_begin(cudaGraph_t body);
int   qllg_capture_end(cudaGraph_t body);
/* a conditional IF block inside a capture: the handle (default 0 at each
 * launch of the captured graph), then the node, whose body takes the
 * launches up to qllg_capture_if_end */
int   qllg_capture_cond(unsigned long long *handle);
int   qllg_capture_if_begin(unsigned long long handle);
int   qllg_capture_if_end(void);
/* last kernel of a graph-loop body: keep looping while work remains */
int   qllg_k_loop_cond(unsigned long long handle, int *done, int *loops, const int *limit);
/* the IF condition of a captured reliable-update block: set when *no_ru is
 * clear, counting the times in *trips */
int   qllg_k_ru_cond(unsigned long long handle, const int *no_ru, int *trips);
/* after a kernel launch: count it and check the launch error */
int   qllg_launched(const char *what);
double qllg_get_param(const char *name);

/* reduction workspace: block partials + completion counter + results */
typedef struct {
  double *partial;     /* [maxblocks][2*QLLG_MAXRHS] */
  unsigned *counter;
  int maxblocks;
} qllg_redbuf;
int  qllg_redbuf_init(qllg_redbuf *rb);
void qllg_redbuf_free(qllg_redbuf *rb);
/* a redbuf over the fixed file-scope scratch of k_noalloc.cu (no
 * allocation; the first call on a device looks up its address) */
#define QLLG_NOALLOC_MAXBLOCKS 1024
int  qllg_noalloc_redbuf(qllg_redbuf *rb);

/* ----------------------------------------------------- field transfers */
/* stage: nrhs blocks of the reference's VLEN=1 host layout, each
 * [nsites][2*ncomp] reals (double when stage_is_double, else float), already
 * copied to device memory; converted to/from the device layout of prec.
 * rhs_stride: reals between consecutive rhs blocks of stage. */
int qllg_k_spinor_from_aos(int prec, void *dev, const void *stage, int stage_is_double,
                           int nsites, int ncomp, int nrhs, size_t rhs_stride);
int qllg_k_spinor_to_aos(int prec, const void *dev, void *stage, int stage_is_double,
                         int nsites, int ncomp, int nrhs, size_t rhs_stride);
/* y = convert(x) between precisions for the active rhs (active may be NULL) */
int qllg_k_spinor_convert(int prec_out, void *out, int prec_in, const void *in,
                          int nsites, int ncomp, int nrhs, const int *active);
/* links: stage [V][18] reals (device copy of host data) -> device slot */
int qllg_k_link_from_aos(int prec, void *dev, float *scale_dev, const void *stage,
                         int stage_is_double, int V);
/* device slot (FP64 or FP32 layout) -> [V][18] reals stage */
int qllg_k_link_to_aos(int prec, const void *dev, void *stage, int stage_is_double, int V);
/* convert a device FP64 link slot to prec (FP32 or I16) */
int qllg_k_link_convert(int prec, void *out, float *scale_dev, const double *in, int V);
/* one FP64 slot [9][V] into the reconstruct-12 format at out: a fat slot as
 * [4][V] float4 + [V] float2; a Naik slot (naik != 0) as rows 0 and 1, [3][V]
 * float4, with bit `bit` of signs[site] the sign that rebuilds row 2;
 * *bad is set when a Naik link is not a real multiple of an SU(3) matrix
 * (rows 0, 1 do not determine row 2 within FP32 rounding) */
/* FP64 spinor columns -> double-float (to_df 1) or back (0, may run in
 * place), for the rhs whose active[] entry is eq (any nonzero one when eq
 * is 0, all when active is NULL); nothing when *skip */
int qllg_k_spinor_df(int to_df, void *out, const void *in, int nsites, int ncomp, int nrhs,
                     const int *active, int eq, const int *skip);
int qllg_k_link_to_f32r(void *out, const double *in, int V, int naik, unsigned char *signs,
                        int bit, int *bad);

/* ----------------------------------------------------- staggered Dslash */
typedef struct {
  qllg_geom g;
  int out_parity;        /* parity of the output sites */
  int nrhs;              /* 1,2,4,8,16 */
  int nslots;            /* 16 (fat+Naik) or 8 (one-hop only) */
  const void *links;     /* device link store, prec_link */
  const float *lscale;   /* per slot scale (I16 links) */
  const void *in;        /* input spinor block of the opposite parity */
  const void *self;      /* same-parity input for the epilogue or NULL */
  void *out;
  /* epilogue mode 0: out = acc
   *          mode 1: acc starts at a0*self, out = acc (dslash2 mass term)
   *          mode 2: out = a[rhs]*self + b*acc (a NULL: a0) */
  int mode;
  const double *a;       /* device [nrhs] or NULL */
  double a0, b;
  double *norm_out;      /* device [nrhs]: |out|^2, or NULL */
  double *norm_self;     /* device [nrhs]: |self|^2, or NULL */
  const int *active;     /* device [nrhs] mask or NULL */
  const int *done;       /* device flag: skip everything when nonzero */
  qllg_redbuf *rb;        /* host struct; the launcher copies its device
                            pointers into partial/counter below */
  double *partial;        /* device block partials (from rb) */
  unsigned *counter;      /* device last-block counter (from rb) */
  int compact;           /* threads over (site, flagged rhs of active) only;
                            modes 0 and 2, no norms */
  int active_eq;         /* compact: flagged means active[r] == active_eq
                            (any nonzero entry when 0) */
  int one_path;          /* multi-rhs Dslash: always the slot loop with the
                            active checks (one code path) */
  int no_tune;           /* caller must not allocate: no autotuning */
  long long wait_cycles; /* bulk-copy pipeline: clock cycles a wait takes
                            before it gives up with an error */
  int wait_test;         /* bulk-copy pipeline, tests only: the producer
                            issues no copy, so the consumers' waits run out */
  int preload;           /* load every launch shape's kernel of these
                            precisions and slot count (each launcher's
                            occupancy query loads its kernel) and launch
                            nothing; nrhs and the pointers are ignored */
  int fb;                /* single-stored links: forward slots only, [nslots/2][9][V];
                            backward links made from them in the kernel */
  int dag;               /* Wilson only: gamma5 D gamma5 (projector signs flipped) */
  /* mode 3 (staggered CG, fused): Ap = a[rhs]*self - acc stays in registers,
   * then x += alpha self, r -= alpha Ap with alpha = 1/(a pnorm + vnorm) and
   * |r|^2 reduced; the last block does the iteration's bookkeeping (mixed:
   * reliable-update flags).  x is FP64 for FP64 spinors, else FP32; r has
   * the spinor precision. */
  void *x, *r;
  struct qllg_cg_scalars_s *sc;
  int mixed;
  /* mode 4 (Wilson standard-form CG, fused): Ap = a0*self + b*acc stays in
   * registers, then x += alpha pvec, r -= alpha Ap with alpha = rsq/pnorm
   * and |r|^2 reduced; the last block does the iteration's bookkeeping
   * (cg_finish_std) and, when cond is a graph conditional handle, sets it
   * to "a reliable update is flagged".  FP32 spinors, x and r FP32. */
  const void *pvec;
  unsigned long long cond;
} qllg_stag_args;
int qllg_k_stag_dslash(int prec_spinor, int prec_link, const qllg_stag_args *a);

/* Wilson half-Dslash with the same argument block (nslots = 8, spinors of
 * 12 colour-spin components, FP64 or FP32) */
int qllg_k_wilson_dslash(int prec_spinor, int prec_link, const qllg_stag_args *a);

/* neighbour index of slot s for every output site of a parity, written as
 * the full-lattice QLL site index (for the bit-exact table check) */
int qllg_k_stag_nbr_table(const qllg_geom *g, int parity, int slot, int *dev_out);

/* ------------------------------------------------------- CG kernels */
/* scalars live on the device, per rhs (QLLG_MAXRHS each) */
typedef struct qllg_cg_scalars_s {
  double rsq[QLLG_MAXRHS];      /* current |r|^2 */
  double rsq_stop[QLLG_MAXRHS]; /* stopping threshold */
  double bsq[QLLG_MAXRHS];
  double pnorm[QLLG_MAXRHS];    /* |p|^2 (even) */
  double vnorm[QLLG_MAXRHS];    /* |D_oe p|^2 (odd) */
  double mass2[QLLG_MAXRHS];    /* m^2 of the operator of each rhs */
  double alpha[QLLG_MAXRHS];
  double tmp[QLLG_MAXRHS];
  double maxr2[QLLG_MAXRHS];    /* |r|^2 at the last reliable update */
  double prev[QLLG_MAXRHS];     /* |r|^2 before the current iteration */
  double delta2;                /* reliable-update threshold, squared */
  int active[QLLG_MAXRHS];
  int iters[QLLG_MAXRHS];
  double orth_re[QLLG_MAXRHS];  /* <r,p>/|r|^2 after a reliable update */
  double orth_im[QLLG_MAXRHS];
  int ru[QLLG_MAXRHS];          /* rhs that take a reliable update now: 1 an
                                   intermediate one, 2 a final candidate */
  int nru[QLLG_MAXRHS];         /* reliable updates taken per rhs */
  int maxits;
  int done;                     /* all rhs inactive */
  int no_ru;                    /* no rhs takes a reliable update now */
  int count;                    /* iterations issued */
  int loops;                    /* graph-loop trips (safety cap) */
  int loop_limit;
  int ru_trips;                 /* graph-loop trips that took the reliable-update block */
} qllg_cg_scalars;

/* makeU's Gram-Schmidt (lib/vla.c:1635-1665) on device sites [s0, s1) of
 * nc x nc complex matrices, 2 nc^2 reals a site (nc <= 3) */
int qllg_k_make_u(int prec, void *m, int nc, size_t s0, size_t s1);

/* ------------------------------------------- persistent Wilson CGNR */
/* one cooperative launch runs FP32 iterations of the mixed Wilson CGNR
 * (k_wilson.cu) until a reliable update is flagged, the solve is done or
 * `trips` iterations ran; the scalars (sc, one rhs) must hold the solve's
 * state, p the current direction.  partial: partial_len doubles (at least
 * two per block); bar: two control words and err one, zeroed before the
 * first launch */
typedef struct {
  qllg_geom g;
  const void *links;
  void *x, *r, *p, *Sp, *v;
  struct qllg_cg_scalars_s *sc;
  double a;
  double *partial;
  size_t partial_len;
  unsigned *bar;
  int *err;
  long long poll_limit;
  int extra;
  int trips;
} qllg_wcgp_args;
int qllg_k_wilson_cgnr_persistent(const qllg_wcgp_args *a, int *grid_out);

/* ---------------------------------------------------- persistent CG */
/* one cooperative launch runs the CG loop (k_cgp.cu) on a small lattice:
 * FP64 iterations (mixed 0), or FP32 iterations with FP64 reliable updates
 * (mixed 1); x, r, p, v in the iteration precision, x64, r64, w64 and b
 * in FP64.  The scalars (sc) must hold an initialised solve (cg_init or
 * mcg_init); on return they hold the result.  partial: at least
 * qllg_cgp_partial_bytes(grid) bytes; bar: two unsigned words, zero at
 * rest; err: set to 1 when a barrier wait ran out after poll_limit polls
 * (extra: arrivals expected beyond the grid, nonzero only to make the
 * waits run out in a test) */
typedef struct {
  qllg_geom g;
  int nslots, fb, mixed, reortho, nrhs;
  const void *links, *links64;
  const float *lscale;
  void *x, *r, *p, *v, *x64, *r64, *w64;
  void *p2;                 /* a second buffer the size of p */
  const void *b;
  struct qllg_cg_scalars_s *sc;
  double *partial;
  unsigned *bar;
  int *err;
  long long poll_limit;
  int extra, trips;
} qllg_cgp_args;
int qllg_k_cg_persistent(const qllg_cgp_args *a, int *grid_out);
size_t qllg_cgp_partial_bytes(int grid);

/* ------------------------------------------ mixed-precision CG kernels */
/* start: r64 = b, x64 = 0, rs = b (sloppy prec ps), xs = 0 (prec px),
 * p = 0; bsq = rsq = maxr2 = |b|^2; rsq_stop *= bsq */
int qllg_k_mcg_init(int px, int ps, void *x64, void *r64, void *xs, void *rs, void *p,
                    const void *b, int nsites, int nrhs, qllg_cg_scalars *s,
                    qllg_redbuf *rb);
/* continuous batching on an operator (stag.c): a fixed-width FP32 mixed
 * CG whose columns are admitted and retired between chunks */
struct qllg_stag;
struct qllg_stag *qllg_stag_share(struct qllg_stag *S);
size_t qllg_batch_bytes(const struct qllg_stag *S);
int qllg_batch_init(struct qllg_stag *S, int maxits);
int qllg_batch_admit(struct qllg_stag *S, int ncol, const int cols[], const double mass[],
                     const double tol[], const double *const src[]);
int qllg_batch_launch(struct qllg_stag *S, int iters);
int qllg_batch_poll(struct qllg_stag *S);
int qllg_batch_retire(struct qllg_stag *S, int col, double *out);
const qllg_cg_scalars *qllg_batch_scalars(const struct qllg_stag *S);
/* mixed CG from an initial guess: x64 holds it, t64 = A x64 (FP64);
 * r64 = b - t64, rs = r64, xs = p = 0, fresh scalars with rsq_stop scaled
 * by |b|^2 */
int qllg_k_mcg_init_guess(int ps, void *r64, void *xs, void *rs, void *p, const void *b,
                          const void *t64, int nsites, int nrhs, qllg_cg_scalars *s,
                          qllg_redbuf *rb);
/* admission of right-hand sides into columns of a running mixed batch */
typedef struct {
  int mask[QLLG_MAXRHS];        /* columns admitted now */
  double mass2[QLLG_MAXRHS];    /* their m^2 */
  double tol2[QLLG_MAXRHS];     /* their stopping |r|^2/|b|^2 */
} qllg_admit_args;
int qllg_k_mcg_admit(int ps, void *x64, void *r64, void *xs, void *rs, void *p, const void *b,
                     int nsites, int nrhs, qllg_cg_scalars *s, const qllg_admit_args *ad,
                     qllg_redbuf *rb);
/* foreign site order / row-major matrices <-> the reference's order, FP64
 * [V][n] device arrays (foreign site s is QLL site perm[s]) */
int qllg_k_aos_from_foreign(double *out, const double *in, const int *perm, int V, int n,
                            int transpose);
int qllg_k_aos_to_foreign(double *out, const double *in, const int *perm, int V, int n);
/* one column of an FP64 [3][nsites][nrhs] device vector <-> a contiguous
 * [nsites][6] device array */
int qllg_k_column_from_aos(void *dev, const double *stage, int nsites, int nrhs, int col);
int qllg_k_column_to_aos(const void *dev, double *stage, int nsites, int nrhs, int col);
/* column jd of a [3][nsites][nd] field of precision pd = column js of a
 * [3][nsites][ns] field of precision ps (FP64/FP32) */
int qllg_k_column_copy(int pd, void *dst, int nd, int jd, int ps, const void *src, int ns, int js,
                       int nsites);
/* *limit = *loops + n on the stream (the next graph launch runs at most n
 * more trips) */
int qllg_k_chunk_limit(int *loops, int *limit, int n);
/* sloppy step: xs += a p, rs -= a Ap, |rs|^2; flags rhs for a reliable
 * update when |rs|^2 < delta2*maxr2, when |rs|^2 < rsq_stop, or at maxits */
int qllg_k_mcg_update(int px, int ps, void *xs, void *rs, const void *p, const void *Ap,
                      int nsites, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb);
/* sloppy p += rs/rsq */
int qllg_k_mcg_update_p(int ps, void *p, const void *rs, int nsites, int nrhs,
                        qllg_cg_scalars *s);
/* reliable update, part 1: x64 += xs, xs = 0 for the flagged rhs */
int qllg_k_mcg_accum(int px, void *x64, void *xs, int nsites, int ncomp, int nrhs,
                     qllg_cg_scalars *s);
/* part 2 (after t64 = A x64): r64 = b - t64, rs = r64, |r64|^2; retires
 * converged rhs and clears the flags; standard_form also resets the
 * direction coefficient to |r64|^2/prev (standard-form CG) */
int qllg_k_mcg_residual(int ps, void *r64, void *rs, const void *b, const void *t64,
                        int nsites, int ncomp, int nrhs, int standard_form,
                        qllg_cg_scalars *s, qllg_redbuf *rb);

/* r = b, x = 0, p = 0; bsq = rsq = |b|^2; rsq_stop *= bsq (rsq_stop holds
 * the relative tolerance on entry); rhs with b = 0 start inactive */
int qllg_k_cg_init(int prec, void *x, void *r, void *p, const void *b,
                   int nsites, int ncomp, int nrhs, qllg_cg_scalars *s,
                   qllg_redbuf *rb);
/* x += alpha p, r -= alpha Ap with alpha = 1/(m^2 pnorm + vnorm);
 * rsq = |r|^2; deactivate converged rhs and set done */
int qllg_k_cg_update_xr(int prec, void *x, void *r, const void *p, const void *Ap,
                        int nsites, int ncomp, int nrhs, qllg_cg_scalars *s,
                        qllg_redbuf *rb);
/* p = p + (1/rsq) r for active rhs */
int qllg_k_cg_update_p(int prec, void *p, const void *r, int nsites, int ncomp,
                       int nrhs, qllg_cg_scalars *s);
/* the same for staggered fields, fused with pnorm = |p|^2 of the new p
 * (r in VecPrec of prec) */
int qllg_k_cg_update_p_norm(int prec, void *p, const void *r, int nsites, int nrhs,
                            qllg_cg_scalars *s, qllg_redbuf *rb);
/* rsq = |r|^2 etc for start-up: out[rhs] = |x|^2 */
int qllg_k_norm2(int prec, const void *x, int nsites, int ncomp, int nrhs, double *out,
                 qllg_redbuf *rb);
/* y = a*y + b*x (per-rhs device coefficient arrays, or the scalar when the
 * pointer is NULL; a == 0 does not read y), precisions of y and x may differ */
int qllg_k_axpby(int py, void *y, int px, const void *x, const double *a, double a0,
                 const double *b, double b0, int nsites, int ncomp, int nrhs,
                 const int *active);
/* y = y + (bsign*b) x, rounded like X_veq_X_plus_r_times_X */
int qllg_k_xpay(int prec, void *y, const void *x, const double *b, double b0, double bsign,
                int nsites, int ncomp, int nrhs, const int *active);
int qllg_k_zero(int prec, void *x, int nsites, int ncomp, int nrhs);
int qllg_k_copy(int prec, void *y, const void *x, int nsites, int ncomp, int nrhs);

/* ------------------------------------------ standard-form CG kernels */
/* x += alpha p, r -= alpha Ap with alpha = rsq/pnorm (pnorm = <p,Ap>
 * from the operator), then prev = rsq, rsq = |r|^2, alpha[] = rsq/prev (the
 * next direction coefficient); retires converged rhs.  With
 * s->delta2 > 0 (mixed precision: x in px, r/p/Ap in ps) rhs are flagged
 * for a reliable update instead of retiring, as in qllg_k_mcg_update. */
int qllg_k_scg_update_xr(int px, int ps, void *x, void *r, const void *p, const void *Ap,
                         int nsites, int ncomp, int nrhs, qllg_cg_scalars *s,
                         qllg_redbuf *rb);
/* p = r + alpha[] p for active rhs */
int qllg_k_scg_update_p(int prec, void *p, const void *r, int nsites, int ncomp, int nrhs,
                        qllg_cg_scalars *s);
/* start of the standard-form CG: x = 0, r = b, p = b (precision prec,
 * converted from the FP64 b), rsq = bsq = maxr2 = |b|^2, rsq_stop *= bsq;
 * x64/r64 (FP64) set to 0 and b when not NULL */
int qllg_k_scg_init(int px, int ps, void *x, void *r, void *p, const void *b64,
                    void *x64, void *r64, int nsites, int ncomp, int nrhs,
                    qllg_cg_scalars *s, qllg_redbuf *rb);

/* after a reliable update (flagged rhs): restore the orthogonality of the
 * search direction to the new residual, p -= (<r,p>/|r|^2) r */
int qllg_k_mcg_reortho(int ps, void *p, const void *rs, int nsites, int nrhs,
                       qllg_cg_scalars *s, qllg_redbuf *rb);

/* ------------------------------------------------ matrix fields */
/* full-lattice 3x3 fields [9][V] of prec (F64/F32):
 * out = op(A)(x) op(B)(x + len*mu) (len 0: no shift), kind 0: A B,
 * 1: A B^dagger, 2: A^dagger B; acc adds to out */
int qllg_k_mat_mul(int prec, void *out, const void *A, const void *B, const qllg_geom *g,
                   int kind, int mu, int len, int acc);
/* out(x) = sgn * in(x + len*mu), or its adjoint when adj */
int qllg_k_mat_shift(int prec, void *out, const void *in, const qllg_geom *g, int mu, int len,
                     int adj, double sgn);
/* out = a*out + c*in over nreal reals (a = 0 does not read out) */
int qllg_k_mat_axpy(int prec, void *out, const void *in, double a, double c, size_t nreal);
/* out = out + c*in, X_vpeq_r_times_X */
int qllg_k_mat_peq(int prec, void *out, const void *in, double c, size_t nreal);
/* sum_x Re tr[(U_i(x)U_j(x+i))^dagger U_j(x)U_i(x+j)] into *out */
int qllg_k_plaq(int prec, const void *ui, const void *uj, const qllg_geom *g, int i, int j,
                double *out, qllg_redbuf *rb);

/* ------------------------------------------- host-layout (AoS) fields */
/* fields in the reference's host layout [V][nelem] on the device */
int qllg_k_aos_shift(int prec, void *out, const void *in, int nelem, const qllg_geom *g,
                     int mu, int len);
/* out(x) += U(x) in(x + len*mu) column by column (nelem = 6*columns), U [V][18] */
int qllg_k_aos_transport(int prec, void *out, const void *u, const void *in, int nelem,
                         const qllg_geom *g, int mu, int len);
/* sum of squares (sq = 1) or of values over sites [s0, s1) */
int qllg_k_aos_sum(int prec, const void *x, int nelem, int s0, int s1, int sq, double *out,
                   qllg_redbuf *rb);

/* ------------------------------------------------- multishift CG */
#define QLLG_MAXSHIFT 64
/* cgmsSolveT's scalar state (lib/cgms.c:12-17), kept on the GPU */
typedef struct {
  double a[QLLG_MAXSHIFT], b[QLLG_MAXSHIFT], s[QLLG_MAXSHIFT], bo[QLLG_MAXSHIFT];
  double z[QLLG_MAXSHIFT], zo[QLLG_MAXSHIFT], zn[QLLG_MAXSHIFT], shifts[QLLG_MAXSHIFT];
  double rsq, oldrsq, rsqstop, pkp;
  double mass2;                 /* m_0^2 of the operator */
  double pnorm, vnorm;          /* |p_0|^2, |D_oe p_0|^2 from the Dslash pair */
  int n, iteration, itnlim, done;
} qllg_cgms_scalars;

/* multishift CG for up to QLLG_MAXRHS right-hand sides at once (the same
 * shifts for all): cgmsSolveT's recurrences per rhs column, FP64 */
typedef struct {
  double a[QLLG_MAXRHS][QLLG_MAXSHIFT], b[QLLG_MAXRHS][QLLG_MAXSHIFT];
  double bo[QLLG_MAXRHS][QLLG_MAXSHIFT], z[QLLG_MAXRHS][QLLG_MAXSHIFT];
  double zo[QLLG_MAXRHS][QLLG_MAXSHIFT], zn[QLLG_MAXRHS][QLLG_MAXSHIFT];
  double shifts[QLLG_MAXSHIFT];
  double mass2[QLLG_MAXRHS];    /* m_0^2 per column (the Dslash epilogue's a[]) */
  double rsq[QLLG_MAXRHS], oldrsq[QLLG_MAXRHS], rsqstop[QLLG_MAXRHS];
  double pnorm[QLLG_MAXRHS], vnorm[QLLG_MAXRHS], tmp[QLLG_MAXRHS];
  int active[QLLG_MAXRHS], iteration[QLLG_MAXRHS];
  int n, nr, itnlim, done;
} qllg_mcgms_scalars;
int qllg_k_mcgms_pre(qllg_mcgms_scalars *s);
int qllg_k_mcgms_coef(qllg_mcgms_scalars *s);
/* FP32 fields of nr rhs, the n shift fields back to back (stride fs bytes):
 * out_i += b_i p_i, r -= b_0 Ap, |r|^2 per rhs, stop test, a_i */
int qllg_k_mcgms_update_xr(void *out, void *r, const void *ps, const void *Ap, int nsites, int nr,
                           size_t fs, qllg_mcgms_scalars *s, qllg_redbuf *rb);
int qllg_k_mcgms_update_p(void *ps, const void *r, int nsites, int nr, size_t fs,
                          qllg_mcgms_scalars *s);
/* start of an iteration: shift (bo,zo,z) <- (b,z,zn) after the first one;
 * oldrsq = rsq */
int qllg_k_cgms_pre(qllg_cgms_scalars *s);
/* pkp, b, zn of lib/cgms.c:71-89 (one thread); stops on pkp <= 0 */
int qllg_k_cgms_coef(qllg_cgms_scalars *s);
/* out_i += b_i s_i p_i, r -= b_0 s_0 Ap, rsq = |r|^2, stop test, a_i
 * (lib/cgms.c:91-135); ps and out hold n single-rhs fields back to back */
int qllg_k_cgms_update_xr(int prec, void *out, void *r, const void *ps, const void *Ap,
                          int nsites, qllg_cgms_scalars *s, qllg_redbuf *rb);
/* p_0 = a_0 p_0 + r, p_i = a_i p_i + zn_i r (lib/cgms.c:137-161) */
int qllg_k_cgms_update_p(int prec, void *ps, const void *r, int nsites,
                         qllg_cgms_scalars *s);

#ifdef __cplusplus
}
#endif
#endif
