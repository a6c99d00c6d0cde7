/*
 * runtime.c -- device context of libqll_gb300: one CUDA stream per
 * process (replaceable by the caller), device allocation with error
 * reporting, a reusable device staging buffer for host transfers, and the
 * last-error string behind qllg_last_error().
 *
 * The reference library never reports errors (it calls exit(), e.g.
 * lib/common.c:22-25, lib/layout.c:49,63); this library never exits: every
 * failing call records a message here and returns a failure value.
 */
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "qllg_internal.h"
#include "qll_gb300.h"

static char g_err[1024];
static int g_inited = 0;
static int g_nsm = 0;
static cudaStream_t g_stream = 0;
static int g_own_stream = 0;

void
qllg_set_error(const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  if(getenv("QLLG_VERBOSE")) fprintf(stderr, "qll_gb300: %s\n", g_err);
}

const char *
qllg_last_error(void)
{
  return g_err;
}

void
qllg_clear_error(void)
{
  g_err[0] = 0;
}

int
qllg_check_cuda(cudaError_t e, const char *what)
{
  if(e == cudaSuccess) return 0;
  qllg_set_error("%s: %s", what, cudaGetErrorString(e));
  return -1;
}

static unsigned long long g_launches = 0;

int
qllg_launched(const char *what)
{
  g_launches++;
  return qllg_check_cuda(cudaGetLastError(), what);
}

unsigned long long
qllg_launch_count(void)
{
  return g_launches;
}

/* kernels launched through a CUDA graph: the capture counted the body once
 * without running it (-body), each executed trip runs it (+body per trip) */
void
qllg_launch_adjust(long long n)
{
  g_launches += (unsigned long long)n;
}

int
qllg_runtime_init(void)
{
  if(g_inited) return 0;
  int n = 0;
  if(qllg_check_cuda(cudaGetDeviceCount(&n), "cudaGetDeviceCount")) return -1;
  if(n < 1) { qllg_set_error("no CUDA device"); return -1; }
  int dev = 0;
  if(qllg_check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return -1;
  if(qllg_check_cuda(cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev),
                     "cudaDeviceGetAttribute")) return -1;
  if(!g_stream) {
    if(qllg_check_cuda(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking),
                       "cudaStreamCreate")) return -1;
    g_own_stream = 1;
  }
  g_inited = 1;
  return 0;
}

int
qllg_num_sms(void)
{
  if(!g_nsm) qllg_runtime_init();
  return g_nsm ? g_nsm : 1;
}

/* while a CUDA graph body is being captured, launches go to the capture
 * stream instead of the library stream */
static cudaStream_t g_cap = 0;
static int g_capturing = 0;
static cudaStream_t g_cap_if = 0;   /* capture of a conditional IF body inside g_cap's */
static int g_nested = 0;

cudaStream_t
qllg_stream(void)
{
  return g_capturing ? (g_nested ? g_cap_if : g_cap) : g_stream;
}

int
qllg_capturing(void)
{
  return g_capturing;
}

int
qllg_capture_begin(cudaGraph_t body)
{
  if(!g_cap && qllg_check_cuda(cudaStreamCreateWithFlags(&g_cap, cudaStreamNonBlocking),
                               "capture stream")) return -1;
  if(qllg_check_cuda(cudaStreamBeginCaptureToGraph(g_cap, body, NULL, NULL, 0,
                                                   cudaStreamCaptureModeRelaxed),
                     "begin capture")) return -1;
  g_capturing = 1;
  return 0;
}

int
qllg_capture_end(cudaGraph_t body)
{
  cudaGraph_t out = body;
  int rc = qllg_capture_if_end();
  g_capturing = 0;
  return qllg_check_cuda(cudaStreamEndCapture(g_cap, &out), "end capture") || rc;
}

/* inside a capture: a conditional handle of the graph being captured,
 * reset to 0 at each launch of that graph (a kernel sets it) */
int
qllg_capture_cond(unsigned long long *handle)
{
  enum cudaStreamCaptureStatus st;
  cudaGraph_t g = NULL;
  cudaGraphConditionalHandle h;
  if(!g_capturing || g_nested) { qllg_set_error("conditional handle outside a capture"); return -1; }
  if(qllg_check_cuda(cudaStreamGetCaptureInfo(g_cap, &st, NULL, &g, NULL, NULL, NULL), "capture info") ||
     qllg_check_cuda(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault),
                     "conditional handle")) return -1;
  *handle = (unsigned long long)h;
  return 0;
}

/* inside a capture: an IF node on handle, after everything captured so far;
 * the launches up to qllg_capture_if_end are captured into its body, and
 * the capture goes on after the node */
int
qllg_capture_if_begin(unsigned long long handle)
{
  enum cudaStreamCaptureStatus st;
  cudaGraph_t g = NULL;
  const cudaGraphNode_t *deps = NULL;
  const cudaGraphEdgeData *edges = NULL;
  size_t nd = 0;
  cudaGraphNode_t node;
  struct cudaGraphNodeParams np;
  if(!g_capturing || g_nested) { qllg_set_error("conditional node outside a capture"); return -1; }
  if(!g_cap_if && qllg_check_cuda(cudaStreamCreateWithFlags(&g_cap_if, cudaStreamNonBlocking),
                                  "conditional capture stream")) return -1;
  if(qllg_check_cuda(cudaStreamGetCaptureInfo(g_cap, &st, NULL, &g, &deps, &edges, &nd), "capture info"))
    return -1;
  memset(&np, 0, sizeof(np));
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = (cudaGraphConditionalHandle)handle;
  np.conditional.type = cudaGraphCondTypeIf;
  np.conditional.size = 1;
  if(qllg_check_cuda(cudaGraphAddNode(&node, g, deps, edges, nd, &np), "conditional IF node") ||
     qllg_check_cuda(cudaStreamUpdateCaptureDependencies(g_cap, &node, NULL, 1,
                                                         cudaStreamSetCaptureDependencies),
                     "capture dependencies") ||
     qllg_check_cuda(cudaStreamBeginCaptureToGraph(g_cap_if, np.conditional.phGraph_out[0], NULL, NULL,
                                                   0, cudaStreamCaptureModeRelaxed),
                     "begin conditional capture")) return -1;
  g_nested = 1;
  return 0;
}

int
qllg_capture_if_end(void)
{
  cudaGraph_t out = NULL;
  if(!g_nested) return 0;
  g_nested = 0;
  return qllg_check_cuda(cudaStreamEndCapture(g_cap_if, &out), "end conditional capture");
}

int
qllg_set_stream(void *stream)
{
  if(qllg_runtime_init()) return -1;
  if(g_own_stream && g_stream) {
    cudaStreamSynchronize(g_stream);
    cudaStreamDestroy(g_stream);
    g_own_stream = 0;
  }
  g_stream = (cudaStream_t)stream;
  return 0;
}

/* make s the library stream for a while and return the previous one (the
 * server's batches each run on their own stream); unlike qllg_set_stream
 * this never destroys the library's own stream */
cudaStream_t
qllg_stream_swap(cudaStream_t s)
{
  cudaStream_t old = g_stream;
  g_stream = s;
  return old;
}

void *
qllg_get_stream(void)
{
  return (void *)g_stream;
}

/* device allocations made through qllg_dmalloc since load (every device
 * allocation of the library goes through it) */
static unsigned long long g_dallocs = 0;

unsigned long long
qllg_device_alloc_count(void)
{
  return g_dallocs;
}

void *
qllg_dmalloc(size_t bytes)
{
  if(qllg_runtime_init()) return NULL;
  void *p = NULL;
  if(bytes == 0) bytes = 16;
  g_dallocs++;
  /* a failure injected by tests (parameter fail_alloc_at): allocation
   * number n fails as cudaMalloc would, without touching the device */
  const double fail_at = qllg_get_param("fail_alloc_at");
  if(fail_at > 0 && (double)g_dallocs == fail_at) {
    qllg_set_error("cudaMalloc(%zu bytes): injected failure", bytes);
    return NULL;
  }
  cudaError_t e = cudaMalloc(&p, bytes);
  if(e != cudaSuccess) {
    qllg_set_error("cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    return NULL;
  }
  return p;
}

void
qllg_dfree(void *p)
{
  if(p) cudaFree(p);
}

/* the device address of host buffer h when it is page-locked memory mapped
   into the device's address space (cudaHostAlloc, cudaHostRegister), with
   the large, aligned transfers that the SM copy takes; NULL otherwise */
static void *
sm_copy_host(const void *d, const void *h, size_t bytes)
{
  if(bytes < ((size_t)1 << 20) || (((uintptr_t)d | (uintptr_t)h | (uintptr_t)bytes) & 15u) ||
     qllg_get_param("host_copy_sm") == 0) return NULL;
  struct cudaPointerAttributes at;
  if(cudaPointerGetAttributes(&at, h) != cudaSuccess) { cudaGetLastError(); return NULL; }
  if(at.type != cudaMemoryTypeHost || !at.devicePointer) return NULL;
  /* the attributes may describe the allocation's start or h itself */
  char *dp = (char *)at.devicePointer;
  if(at.hostPointer) dp += (const char *)h - (const char *)at.hostPointer;
  return ((uintptr_t)dp & 15u) ? NULL : dp;
}

int
qllg_h2d(void *d, const void *h, size_t bytes)
{
  const void *hd = sm_copy_host(d, h, bytes);
  if(hd) return qllg_k_copy16(d, hd, bytes);
  return qllg_check_cuda(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, g_stream),
                         "copy host to device");
}

int
qllg_d2h_async(void *h, const void *d, size_t bytes)
{
  void *hd = sm_copy_host(d, h, bytes);
  if(hd) return qllg_k_copy16(hd, d, bytes);
  return qllg_check_cuda(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, g_stream),
                         "copy device to host");
}

int
qllg_d2h(void *h, const void *d, size_t bytes)
{
  if(qllg_d2h_async(h, d, bytes)) return -1;
  return qllg_sync();
}

int
qllg_sync(void)
{
  return qllg_check_cuda(cudaStreamSynchronize(g_stream), "stream synchronize");
}

int
qllg_redbuf_init(qllg_redbuf *rb)
{
  rb->maxblocks = qllg_num_sms()*16;
  rb->partial = qllg_dmalloc(sizeof(double)*2*QLLG_MAXRHS*(size_t)rb->maxblocks);
  rb->counter = qllg_dmalloc(sizeof(unsigned)*4);
  if(!rb->partial || !rb->counter) { qllg_redbuf_free(rb); return -1; }
  return qllg_check_cuda(cudaMemsetAsync(rb->counter, 0, sizeof(unsigned)*4, g_stream),
                         "memset counter");
}

void
qllg_redbuf_free(qllg_redbuf *rb)
{
  qllg_dfree(rb->partial);
  qllg_dfree(rb->counter);
  rb->partial = NULL;
  rb->counter = NULL;
}

/* one growing device staging buffer for host<->device layout transposes */
static void *g_stage = NULL;
static size_t g_stage_bytes = 0;

void *
qllg_stage(size_t bytes)
{
  if(bytes <= g_stage_bytes) return g_stage;
  if(g_stage) { qllg_sync(); qllg_dfree(g_stage); }
  g_stage = qllg_dmalloc(bytes);
  g_stage_bytes = g_stage ? bytes : 0;
  return g_stage;
}

void
qllg_stage_release(void)
{
  if(g_stage) { qllg_sync(); qllg_dfree(g_stage); }
  g_stage = NULL;
  g_stage_bytes = 0;
}

int
qllg_init(void)
{
  return qllg_runtime_init();
}

const char *
qllg_version(void)
{
  return "qll_gb300 0.1 (sm_103a)";
}

/* tunable solver parameters (qllg_set_param) */
static struct { const char *name; double value; } g_params[] = {
  {"reliable_delta", 0.1},   /* 16-bit mixed mode: reliable update when
                                |r| < delta * |r at the last update| */
  {"reliable_delta_single", 0.01}, /* the same for the FP32 mixed mode: FP32
                                      sloppy iterations keep the CG recurrence
                                      over two decades (measured: 455
                                      iterations at 32^3x64, m=0.01, for 0.1
                                      and 0.01; 464 at 0.003, 623 at 0.001) */
  {"wilson_delta", 0.001},   /* the same for the Wilson CGNR's FP32 mode
                                (measured at 16^3x32, kappa 0.12: 52
                                iterations and the same true residual for
                                0.01 down to 0.0003; 9.6 ms per solve at
                                0.01, 9.0 at 0.003, 8.4 at 0.001: fewer
                                FP64 updates) */
  {"reortho", 1},            /* restore p orthogonal to r after a reliable update */
  {"half_split", 2},         /* MIXED_HALF solves: 0 16-bit Dslash operands and
                                links, 1 16-bit links with FP32 operands, 2 FP32
                                links with 16-bit operands.  At 32^3x64, m = 0.01,
                                16 rhs: 1382, 996 and 455 iterations (4.96, 2.81
                                and 1.30 s; FP32 operands and links: 455, 1.04 s):
                                the 16-bit links, one scale per slot, cost the
                                iterations, the 16-bit operands do not */
  {"graph", 1},              /* run solver iterations as one CUDA graph launch */
  {"persistent", 1},         /* small lattices: the whole CG loop in one cooperative
                                launch (FP64, or FP32 with FP64 reliable updates) */
  {"persistent_max", 65536}, /* ... when even sites x rhs is at most this */
  {"wait_polls", 2e7},       /* polls (about 64 ns apart) a grid-barrier wait takes
                                before it gives up with an error: about a second */
  {"bulk_wait_test", 0},     /* tests: the bulk-copy Dslash's producer issues no copy,
                                so its consumers' bounded waits run out */
  {"fail_alloc_at", 0},      /* tests: the library's device allocation number n
                                (qllg_device_alloc_count() + 1 = the next) fails
                                as cudaMalloc would; 0: off */
  {"cg_barrier_extra", 0},   /* arrivals a persistent-CG barrier expects beyond the
                                grid: nonzero only in a test that makes the waits
                                run out */
  {"poll", 8},               /* first batch of iterations between host checks */
  {"dslash_mr", 1},          /* multi-rhs Dslash: one thread per site and 4 rhs */
  {"ru_compact", 1},         /* reliable-update Dslash over the flagged rhs only */
  {"df_blocks", 3},          /* register cap of the double-float reliable-update
                                Dslash: resident blocks of 256 it must allow
                                (1 or 3; 32^3x64, 1 rhs: 0.47 and 0.41 ms,
                                the FP64 one 1.04 ms) */
  {"ru_df", 1},              /* intermediate reliable updates of the mixed CG in
                                double-float (FP32 pipes, about 48 bits); the
                                final ones, on which a rhs may stop, in FP64 */
  {"dslash_vec4", 1},        /* 16-byte loads of rhs pairs (FP32) */
  {"autotune", 1},           /* time the Dslash variants of a new launch shape */
  {"dslash_tile", 1},        /* allow the shared-memory-staged Dslash variant */
  {"dslash_bulk", 1},        /* allow the bulk-copy pipeline Dslash variant */
  {"dslash_pipe", 1},        /* allow the per-warp cp.async pipeline Dslash variants */
  {"dslash_tma", 1},         /* allow the per-warp tensor-copy (TMA) pipeline Dslash variants */
  {"wilson_persistent", 1},  /* FP32 Wilson CGNR with even sites up to
                                wilson_persistent_max: the iterations as persistent
                                cooperative launches, each until a reliable update
                                is flagged */
  {"wilson_persistent_max", 4194304}, /* ... (with double-float updates, against the
                                graph loop with FP64 ones: 16^3x32 4.8 against 7.6 ms,
                                24^3x48 24.1 against 27.7 ms, 32^3x64 71 against 76 ms) */
  {"wilson_fused_update", 1}, /* FP32 Wilson CGNR: the CG update (x, r, |r|^2 and the
                                iteration's bookkeeping) in the epilogue of the last
                                half Dslash of the iteration */
  {"graph_ru_if", 1},        /* graph-captured mixed solver loops: the reliable-update
                                launches sit in a conditional IF node taken only in
                                the iterations that flag an update (else they are
                                launched every iteration and return at once) */
  {"host_copy_sm", 1},       /* copies of at least 1 MiB between page-locked host
                                memory and the device run on the SMs instead of
                                a copy engine (805 MB on GB300 after a solve: 4 ms
                                against 35-90 ms) */
  {"solve2_mixed", 0},       /* solve2D (drop-in): FP32 iterations with FP64 reliable
                                updates instead of the reference's FP64 CG */
  {"wilson_f64_dir2", 1},    /* small one-rhs FP64 Wilson launches: two threads
                                per site, split by direction */
  {"wilson_f32_dir2", 0},    /* the same for the FP32 ones */
  {"wilson_f64_c3", 0},      /* the same for the FP64 launches (the reliable
                                updates of the mixed CGNR, and the FP64 CGNR) */
  {"wilson_c3", 0},          /* small one-rhs FP32 Wilson launches: three threads
                                per site, one per output colour (C2 at 16^3x32:
                                17.8 ms per mixed solve against 14.7 ms with one
                                thread per site, so off) */
  {"wilson_ru_df", 2},       /* intermediate reliable updates of the Wilson mixed
                                CGNR in double-float: 1 always, 2 with the
                                persistent iterations only (C2: 4.78 against 5.28
                                ms per solve), 0 never.  In the graph loop their
                                extra launches cost more than they save (updates
                                at each 10x fall of |r|: C2 15.1 against 14.8 ms,
                                32^3x64 139 against 128 ms) */
  {"wilson_df_c3", 1},       /* three threads per site in the small double-float
                                Wilson launches, whose one-thread kernel holds one
                                block of 256 threads per SM */
  {"dslash_split", 1},       /* multi-rhs Dslash: a slot loop without the active
                                checks for launches with every rhs active */
  {"dslash_variant", -1},    /* force a Dslash variant (0-23, qllg_autotune_report names
                                them); -1: autotuned */
  {"multishift_guess_rsq", 1e-10}, /* mixed multishift: the FP32 multishift CG
                                       goes to |r|^2 < this |b|^2 before the
                                       pairs are refined in FP64 (C3 at
                                       24^3x48: 0.73 s at 1e-9 and 1e-10,
                                       0.81 s at 1e-11, 0.85 s at 1e-12) */
  {"links_recon12", 0},      /* mixed FP32 solves: Naik links as two rows + sign
                                (measured slower: 1.40 against 0.93 ms per 16-rhs
                                half Dslash at 32^3x64, so off by default) */
};

int
qllg_set_param(const char *name, double value)
{
  for(size_t i=0; i<sizeof(g_params)/sizeof(g_params[0]); i++)
    if(!strcmp(g_params[i].name, name)) { g_params[i].value = value; return 0; }
  qllg_set_error("unknown parameter %s", name);
  return -1;
}

double
qllg_get_param(const char *name)
{
  for(size_t i=0; i<sizeof(g_params)/sizeof(g_params[0]); i++)
    if(!strcmp(g_params[i].name, name)) return g_params[i].value;
  return 0;
}
