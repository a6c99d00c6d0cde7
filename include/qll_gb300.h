/*
 * qll_gb300.h -- native API of libqll_gb300, beside the QLL drop-in API of
 * qll.h.  These entry points have no counterpart in the reference; they
 * expose what the GPU adds: several lattices at once (the reference keeps
 * one geometry in process-global tables, lib/stagDslash.c:715-719), many
 * right-hand sides per solve, mixed-precision solvers, status codes and a
 * caller-chosen CUDA stream.
 *
 * Conventions: every int-returning call returns a negative value on failure
 * and leaves a message in qllg_last_error(); nothing in the library calls
 * exit().  Host arrays use the layout of qll.h (one lane, [site][nelem],
 * even sites first).  Links of a staggered operator are 8 (one-hop) or 16
 * (one-hop and Naik) slots; slot s = 4*mu + 2*backward + naik (with Naik) or
 * 2*mu + backward (without), i.e. the order of createStaggeredLinks.
 */
#ifndef QLLG_QLL_GB300_H
#define QLLG_QLL_GB300_H

#include "qll.h"

#ifdef __cplusplus
extern "C" {
#endif

const char *qllg_last_error(void);
void qllg_clear_error(void);
const char *qllg_version(void);
/* CUDA device and stream: the library launches all work on one stream,
 * created at first use; qllg_set_stream hands it a cudaStream_t instead */
int qllg_init(void);
int qllg_set_stream(void *cuda_stream);
void *qllg_get_stream(void);

/* ----------------------------------------------------- input generator */
/* SU(3) links U_mu(x) = exp(i eps H), H traceless Hermitian with Gaussian
 * entries from a counter-based SplitMix64 keyed by (seed, site, mu,
 * entry), optionally times the staggered phases
 * eta_mu(x) = (-1)^(x_0+...+x_{mu-1}); u[mu] are [V][18] host arrays */
int qllg_gen_gauge(const int dims[4], unsigned long long seed, double eps,
                   int ks_phases, double *u[4]);
/* Gaussian reals (unit variance) on the sites of sub ("even", "odd",
 * "all"), nelem per site, zero elsewhere */
int qllg_gen_source(const int dims[4], unsigned long long seed, int nelem,
                    const char *sub, double *v);
/* asqtad coefficients: 5/8, -1/16, 1/64, -1/384, -1/16, -1/24 */
void qllg_asqtad_coeffs(Fat7Coeffs *c);

/* ---------------------------------------------- staggered operator */
typedef struct qllg_stag qllg_stag;

enum {
  QLLG_SOLVE_DOUBLE = 0,        /* FP64 everywhere (the reference's D path) */
  QLLG_SOLVE_SINGLE = 1,        /* FP32 everywhere (the reference's F path) */
  QLLG_SOLVE_MIXED_HALF = 2,    /* 16-bit storage, FP32 arithmetic, FP64
                                   reliable updates */
  QLLG_SOLVE_MIXED_SINGLE = 3   /* FP32 sloppy, FP64 reliable updates */
};

typedef struct {
  int iters[16];          /* iterations per right-hand side */
  double rsq[16];         /* final |r|^2/|b|^2 of the solver's recurrence */
  double true_rsq[16];    /* |b - A x|^2/|b|^2 in FP64 for the returned x:
                             recomputed after an FP64 solve; for the mixed
                             modes the residual of the final reliable update,
                             which every rhs ends on (r = b - A x in FP64) */
  int reliable_updates;
  int total_iters;        /* iterations of the batch (max over rhs) */
  double seconds;         /* device time of the solve */
} qllg_solve_info;

/* links: fat[8], lng[8] host arrays [V][18]; slot 2i of the reference's
 * createStaggeredLinks is fat[i], slot 2i+1 is lng[i]; lng NULL means no
 * Naik term.  The links are copied to the GPU. */
qllg_stag *qllg_stag_create(const int dims[4], double *const fat[8], double *const lng[8]);
qllg_stag *qllg_stag_create_f(const int dims[4], float *const fat[8], float *const lng[8]);
void qllg_stag_destroy(qllg_stag *S);
size_t qllg_stag_device_bytes(const qllg_stag *S);
int qllg_stag_nslots(const qllg_stag *S);
/* copy the FP64 link slots back to host arrays [V][18] (out[nslots]) */
int qllg_stag_get_links(qllg_stag *S, double *const out[16]);

/* x = mass*y + D y on the sites of sub (dslash2 semantics; "even"/"odd"
 * ignore the mass); host arrays [V][6] of the precision of the operator */
int qllg_stag_dslash(qllg_stag *S, void *x, double mass, const void *y, const char *sub);

/* solve (m_r^2 - D_eo D_oe) x_r = b_r on even sites for nrhs right-hand
 * sides (nrhs <= 16) in the requested precision mode; host arrays of
 * [V][6] reals of the operator's precision (only the even half is read and
 * written); stops when |r|^2 < rsq |b|^2 or after maxits iterations. */
int qllg_stag_solve(qllg_stag *S, int nrhs, void *const x[], void *const b[],
                    const double mass[], double rsq, int maxits, int mode,
                    qllg_solve_info *info);
/* the same with device buffers: b and x are FP64 device arrays in the
 * library's multi-rhs layout ([3][Vh][nrhs] double2), inputs resident */
int qllg_stag_solve_device(qllg_stag *S, int nrhs, void *x_dev, const void *b_dev,
                           const double mass[], double rsq, int maxits, int mode,
                           qllg_solve_info *info);
/* embedding codes' layouts (the QDP/QOP pattern of embedqop.c:193-258,
 * whose packM/packV repack on the host, qopstag.c:123-196): the caller's
 * arrays as they are, reordered and transposed on the GPU.  Foreign site s
 * is QLL site perm[s] (perm NULL: the same order, as MILC's even-first
 * order is for one rank); links [V][18] row-major (entry 3*row + col) when
 * row_major, else column-major; fat[8]/lng[8] double-stored slots in
 * createStaggeredLinks order.  Vectors: FP64 [V][6] host arrays in the
 * foreign order, of which upload reads the even sites and download writes
 * all sites (zero at the odd ones); the device side is the even-site
 * multi-rhs layout of qllg_stag_vec_alloc. */
qllg_stag *qllg_stag_create_foreign(const int dims[4], double *const fat[8], double *const lng[8],
                                    const int *perm, int row_major);
int qllg_stag_vec_upload_foreign(qllg_stag *S, void *v_dev, int nrhs, void *const h[],
                                 const int *perm);
int qllg_stag_vec_download_foreign(qllg_stag *S, const void *v_dev, int nrhs, void *const h[],
                                   const int *perm);
/* multi-rhs multishift solve (solveMulti2 of lib/stagDslash.c:625-657 for
 * many rhs): for every rhs r and shift k, (m^2 + shift_k - D_eo D_oe)
 * x[r*nshift + k] = b[r] on the even sites, each to |r|^2 < rsq |b|^2.
 * QLLG_SOLVE_DOUBLE runs the reference's FP64 multishift CG per rhs;
 * QLLG_SOLVE_MIXED_SINGLE runs the multishift recurrence for up to 16 rhs
 * at once in FP32 vectors (FP64 recurrences) to |r|^2 < max(rsq,
 * "multishift_guess_rsq") |b|^2, then takes every (rhs, shift) pair from
 * there to rsq with the FP32 mixed CG and FP64 reliable updates, 16 pairs a
 * launch.  Host arrays [V][6] FP64; iters (both stages) and true_rsq (FP64
 * |b - A_k x|^2/|b|^2) per pair, may be NULL.  Returns the largest
 * iteration count. */
int qllg_stag_solve_multishift(qllg_stag *S, int nrhs, void *const x[], void *const b[],
                               double mass, int nshift, const double shifts[], double rsq,
                               int maxits, int mode, int iters[], double true_rsq[]);
/* allocate / free a device even-site FP64 vector of nrhs rhs and fill it
 * from host arrays (or copy it back) */
void *qllg_stag_vec_alloc(qllg_stag *S, int nrhs);
void qllg_stag_vec_free(void *v);
int qllg_stag_vec_upload(qllg_stag *S, void *v_dev, int nrhs, void *const h[]);
int qllg_stag_vec_download(qllg_stag *S, const void *v_dev, int nrhs, void *const h[]);

/* the half Dslash out = D in (output sites of out_parity) on device vectors
 * of nrhs rhs, precision prec (0 FP64, 1 FP32, 2 16-bit, 3 FP32 with the
 * reconstruct-12 links, 4 double-float: each real a (hi, lo) pair of floats
 * in the FP64 layout, the arithmetic of the mixed solver's reliable
 * updates) in the library layout; links of that precision are derived from
 * FP64 on first use */
int qllg_stag_dslash_device(qllg_stag *S, int prec, int nrhs, int out_parity, void *out_dev,
                            const void *in_dev);

/* No counterpart in the reference (QLL takes its work memory from myalloc,
 * lib/common.c:10, e.g. per call in cgmsSolve, lib/cgms.c:43).  The same
 * half Dslash as qllg_stag_dslash_device, plus |out|^2 of each rhs written to the device
 * array norm2_dev[nrhs], and no device memory allocated by the call: the
 * grid reduction uses a fixed file-scope __device__ scratch of 262,400 B
 * (partials of up to 1024 blocks x 16 rhs), and links not yet created in
 * precision prec are refused, not derived.  It is for callers that cannot
 * allocate: a serving loop holding a fixed HBM budget for admitted solves,
 * or one whose concurrent streams a device-synchronising cudaMalloc/cudaFree
 * would stall.  Limits: nrhs in {1,2,4,8,16}; anything else, or links of
 * prec missing, returns -1 with qllg_last_error() saying why.  The set-up
 * happens when the operator's links of precision prec are made (at create
 * time for the precision the operator was created in, else at the first
 * call that derives them, e.g. one qllg_stag_dslash_device of that
 * precision): the scratch's address is looked up (cudaGetSymbolAddress with
 * that device current) and every kernel the call can launch is loaded, so
 * that CUDA's lazy module loading allocates nothing during the call itself.
 * The address is kept for the life of the process; do not use the library
 * across a cudaDeviceReset.  The scratch is one per device, so calls that
 * overlap in time (other host threads, other streams) race: serialise
 * them. */
int qllg_stag_dslash_norm2_noalloc(qllg_stag *S, int prec, int nrhs, int out_parity,
                                   void *out_dev, const void *in_dev, double *norm2_dev);
size_t qllg_stag_vec_bytes(const qllg_stag *S, int prec, int nrhs);
/* 1 when the last solve on S ran as one persistent cooperative launch
 * (parameter "persistent"), 0 when it ran the multi-launch loop */
int qllg_stag_last_solve_persistent(const qllg_stag *S);
/* 1 when the mixed FP32 solves of S use reconstruct-12 links: the 8 Naik
 * slots held as rows 0 and 1 (48 of 72 bytes) and row 2 rebuilt in the
 * kernel as s conj(r0 x r1)/|r0|, which holds for a real multiple of an
 * SU(3) matrix (the three-link Naik products of SU(3) links).  Derived on
 * first use when the "links_recon12" parameter is on and every Naik link
 * passes the check; 0 otherwise (plain FP32 links). */
int qllg_stag_recon12(qllg_stag *S);

/* neighbour table of slot s for the output sites of a parity, as QLL site
 * indices (host int[V/2]); the GPU computes it with the Dslash kernel's own
 * index arithmetic */
int qllg_stag_nbr_table(const int dims[4], int parity, int slot, int *host_out);

/* ------------------------------------------ link preparation (GPU) */
/* fat7/asqtad smearing of thin links u (and ulong for the Naik term, NULL
 * = u), host [V][18] FP64 arrays (smearFat7 of lib/gauge.c:264-416) */
int qllg_smear_fat7(const int dims[4], double *const fl[4], double *const ll[4],
                    const Fat7Coeffs *coef, double *const u[4], double *const ulong_[4]);
/* thin links -> fat7 -> the 16 slots (with -F^dagger(x-mu), -L^dagger(x-3mu)
 * backward links) of a resident FP64 operator, built on the GPU */
qllg_stag *qllg_stag_create_asqtad(const int dims[4], double *const thin[4],
                                   const Fat7Coeffs *coef);
/* the same with the links single-stored: the 8 forward slots only (half
 * the memory); the Dslash kernels make the backward links -F^dagger(x-mu),
 * -L^dagger(x-3mu) on the fly, with bitwise the same products */
qllg_stag *qllg_stag_create_asqtad_fb(const int dims[4], double *const thin[4],
                                      const Fat7Coeffs *coef);
/* the six plaquettes of gaugePlaq (normalised by 3V) */
int qllg_plaq(const int dims[4], double *const u[4], double plaqs[6]);

/* -------------------------------------------------- Wilson operator */
typedef struct qllg_wilson qllg_wilson;
/* u[8]: slot 2mu forward link, 2mu+1 backward link (host [V][18]) */
qllg_wilson *qllg_wilson_create(const int dims[4], double *const u[8]);
qllg_wilson *qllg_wilson_create_f(const int dims[4], float *const u[8]);
void qllg_wilson_destroy(qllg_wilson *W);
/* x = massp*y + W y on sub (massp already massFac*(4+m)); dag: g5 W g5 */
int qllg_wilson_dslash(qllg_wilson *W, void *x, double massp, const void *y, const char *sub,
                       int dag);
/* the massless Wilson hop term of one parity, out = W in on the output
 * sites of out_parity, on device vectors in the library layout ([12][Vh]
 * complex, FP64 or FP32 by prec 0 or 1; qllg_wilson_vec_bytes gives the
 * size); links of that precision are derived from FP64 on first use */
int qllg_wilson_dslash_device(qllg_wilson *W, int prec, int out_parity, void *out_dev,
                              const void *in_dev);
size_t qllg_wilson_vec_bytes(const qllg_wilson *W, int prec);
/* even-odd normal-equation solve of the Schur complement
 * S = (4+m) - W_eo W_oe/(4+m): CG on S^dagger S x = S^dagger b, stopping at
 * |r|^2 < rsq |S^dagger b|^2; mode QLLG_SOLVE_DOUBLE or
 * QLLG_SOLVE_MIXED_SINGLE; x, b host [V][24] FP64, even half; info->true_rsq
 * is |b - S x|^2/|b|^2 in FP64.  The iterations run as one CUDA-graph
 * launch (parameter "graph"; kernel timing on: a host-polled loop) */
int qllg_wilson_solve(qllg_wilson *W, void *x, const void *b, double mass, double rsq,
                      int maxits, int mode, qllg_solve_info *info);

/* ------------------------------------------------------------ serving */
/* No counterpart in the reference (its solvers run one call at a time).
 * A server keeps the links of several lattices resident and runs solve
 * requests as they arrive, with continuous batching: a request with n
 * shifts occupies n columns of a 16-column FP32 mixed-precision batch
 * (FP64 reliable updates; column k solves (m^2 + shift_k - D_eo D_oe) x_k
 * = b); batches advance in chunks of chunk_iters iterations, and between
 * two chunks finished columns are retired and queued requests admitted into
 * free columns while the others continue.  Each batch has its own stream,
 * so batches overlap on the device.  New batches are created only within
 * hbm_budget bytes (resident links plus batch workspaces; idle batches are
 * released when it is short).  A request's solution is bitwise the same
 * whichever requests run beside it.  One host thread drives a server. */
typedef struct qllg_server qllg_server;

typedef struct {
  int status;              /* 0 queued, 1 running, 2 done, 3 failed: a shift
                              ended without meeting the tolerance (a source
                              that is not a number, or the iteration limit) */
  int ncol;                /* shifts (columns) of the request */
  int iters[16];           /* iterations per shift */
  double true_rsq[16];     /* |b - A x|^2/|b|^2 per shift, FP64 */
  double seconds_queued;   /* submit -> admission (host clock) */
  double seconds_total;    /* submit -> solution copied out */
} qllg_request_info;

typedef struct {
  size_t budget_bytes, used_bytes;
  int batches, busy_columns, requests, pending;
  long long admitted_columns, chunks;
} qllg_server_info;

qllg_server *qllg_server_create(size_t hbm_budget, int chunk_iters, int max_batches_per_lattice);
/* a resident operator (not owned; it must outlive the server); returns
 * the lattice id */
int qllg_server_add_lattice(qllg_server *V, qllg_stag *S);
/* src: host [V/2][6] FP64 source on the even sites; out[k]: host [V/2][6]
 * FP64 solution of shift k (nshift <= 0: one solve at mass), written when
 * the request completes.  Both must stay valid until then.  Stops at
 * |b - A x| < tol |b|.  Returns the request id. */
int qllg_server_submit(qllg_server *V, int lattice, double mass, int nshift, const double *shifts,
                       double tol, const double *src, double *const out[]);
/* one scheduling pass (retire, admit, launch); never waits for the GPU.
 * Returns the number of requests completed (done or failed) in this pass,
 * or -1 with qllg_last_error() set.  A failure while creating a batch (a
 * device allocation) leaves the queued requests queued: a later step
 * admits them. */
int qllg_server_step(qllg_server *V);
int qllg_server_pending(const qllg_server *V);
int qllg_server_request(const qllg_server *V, int id, qllg_request_info *info);
int qllg_server_stats(const qllg_server *V, qllg_server_info *info);
void qllg_server_destroy(qllg_server *V);

/* solver parameters (name, default):
 *  "reliable_delta" (0.1, 16-bit mixed mode),
 *  "reliable_delta_single" (0.01, FP32 mixed mode of the staggered CG) and
 *    "wilson_delta" (0.001, the Wilson CGNR's FP32 mode): a reliable update
 *    when |r| falls by this factor;
 *  "half_split" (2: the 16-bit mixed mode stores the Dslash operands in 16
 *    bits and keeps FP32 links; 1: 16-bit links and FP32 operands; 0: both
 *    in 16 bits),
 *  "reortho" (1), "graph" (1: the solver loop as one CUDA-graph launch),
 *    "poll" (8: first batch of host-polled iterations);
 *  "persistent" (1: on small lattices the whole CG loop as one cooperative
 *    launch, for FP64 solves and FP32 mixed solves with FP64 reliable
 *    updates), "persistent_max" (65536: ... when even sites x rhs is at most
 *    this), "wait_polls" (2e7: polls, about 64 ns apart, a grid-barrier
 *    wait of the persistent CG takes before the solve fails with an error
 *    instead of hanging), "cg_barrier_extra" (0: arrivals its barriers
 *    expect beyond the grid; nonzero only to make the waits run out in a
 *    test); "fail_alloc_at" (0: off; n: the library's device allocation
 *    number n, counted by qllg_device_alloc_count, fails as cudaMalloc
 *    would, for tests of the failure paths); "bulk_wait_test" (0; 1: the
 *    bulk-copy Dslash issues no copies, so that its consumers' waits run
 *    out: a test of that error path);
 *  "ru_compact" (1: reliable updates over the flagged rhs only), "ru_df" (1:
 *    intermediate reliable updates in double-float, final ones in FP64),
 *    "df_blocks" (3: register cap of the double-float kernel);
 *  "dslash_mr" (1: multi-rhs Dslash kernels), "dslash_vec4" (1: 16-byte
 *    loads of rhs pairs), "dslash_split" (1: a slot loop without the active
 *    checks when every rhs of a launch is active);
 *  "autotune" (1: time the Dslash launch shapes of each new shape and keep
 *    the fastest), "dslash_tile" (1) and "dslash_bulk" (1): the staged and
 *    the bulk-copy candidates may be chosen, "dslash_pipe" (1) and
 *    "dslash_tma" (1): the per-warp cp.async and tensor-copy pipeline
 *    candidates may be chosen; "dslash_variant" (-1: autotuned;
 *    0-23 forces a candidate where it applies, qllg_autotune_report names
 *    them);
 *  "wilson_persistent" (1: the FP32 Wilson CGNR on a lattice of at most
 *    "wilson_persistent_max" (4194304) even sites runs its iterations as
 *    persistent cooperative launches, each until a reliable update is
 *    flagged, which the host then takes with the FP64 kernels),
 *  "wilson_fused_update" (1: the FP32 iterations of the Wilson CGNR run
 *    the CG update in the epilogue of their last half Dslash; 0: a separate
 *    update kernel),
 *  "graph_ru_if" (1: in the graph-captured mixed solver loops the
 *    reliable-update launches are the body of a conditional IF node, taken
 *    only in the iterations that flag an update; 0: they are launched every
 *    iteration and return at once when nothing is flagged),
 *  "host_copy_sm" (1: copies of at least 1 MiB between page-locked host
 *    arrays and the device, such as the sources and solutions of the
 *    host-array solves, run on the SMs through the arrays' mapped device
 *    addresses instead of on a copy engine; 0: copy engine always),
 *  "links_recon12" (0; 1: reconstruct-12 Naik links in the FP32 solves),
 *  "solve2_mixed" (0; 1: the drop-in solve2D runs FP32 iterations with FP64
 *    reliable updates, to the same true residual, instead of the reference's
 *    FP64 CG);
 *  "multishift_guess_rsq" (1e-10: the mixed multishift's first stage
 *    stops at |r|^2 < this |b|^2), "wilson_c3" (0; 1: three threads per site
 *    in small one-rhs FP32 Wilson launches), "wilson_ru_df" (2: the
 *    Wilson mixed CGNR's intermediate reliable updates in double-float
 *    with the persistent iterations; 1: always; 0: never),
 *    "wilson_df_c3" (1: three threads per site in the small double-float
 *    Wilson launches), "wilson_f64_c3" (0: the same for the FP64 ones),
 *    "wilson_f64_dir2" (1: two threads per site, split by direction, in the
 *    small one-rhs FP64 Wilson launches), "wilson_f32_dir2" (0: the same for
 *    the FP32 ones).
 * Returns -1 for an unknown name. */
int qllg_set_param(const char *name, double value);
double qllg_get_param(const char *name);

/* the autotuner's choices so far, one line per launch shape ("key: chosen
 * | variant time, ..."); returns the number of shapes */
int qllg_autotune_report(char *buf, size_t len);

/* kernel timing: when enabled, launches of the named kernel family are
 * bracketed by CUDA events on the library stream; read returns the count
 * and total milliseconds since the last reset.  Families:
 * "stag_dslash_<f64|f32|i16>_n<nrhs>" (half Dslash), "stag_cg_fused_<...>_n<nrhs>"
 * (D_eo with the fused CG update), "wilson_dslash" */
void qllg_timing_enable(int on);
/* number of kernels the library has launched since load */
unsigned long long qllg_launch_count(void);
/* number of device allocations (cudaMalloc) the library has made since
 * load */
unsigned long long qllg_device_alloc_count(void);
void qllg_timing_reset(void);
int qllg_timing_read(const char *name, int *count, double *ms);

#ifdef __cplusplus
}
#endif
#endif
