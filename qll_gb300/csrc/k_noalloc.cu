// k_noalloc.cu -- fixed, statically sized reduction scratch for
// qllg_stag_dslash_norm2_noalloc, the one entry point of the library that
// allocates no device memory at all (see the declaration in qll_gb300.h).
//
// Callers that cannot allocate: a serving loop that admits solves against a
// fixed HBM budget has every byte of device memory accounted to admitted
// work, and a library allocation would either exceed that budget or fail in
// the middle of serving; and cudaMalloc/cudaFree may synchronise the whole
// device, which would stall the other streams' solves that such a loop keeps
// in flight.  Those callers need a call that adds nothing to the device
// footprint once the operator is set up.
//
// CUDA loads modules lazily by default: the first cudaGetSymbolAddress of
// the scratch loads it (262,400 B), and a kernel's first launch loads its
// code.  Both happen when an operator's links of a precision are made
// (noalloc_preload in stag.c), an allocating step anyway, so the
// no-allocation call itself only finds them there.
//
// The scratch is the block-partial array and last-block counter of the
// deterministic grid reduction (grid_reduce / grid_reduce_mr): partial
// sums of two quantities for up to QLLG_MAXRHS rhs per block, for at most
// QLLG_NOALLOC_MAXBLOCKS blocks (the launchers cap their grid at the
// redbuf's maxblocks), followed by the counter on its own 256-byte line.
// Size: 2*16*1024*8 B = 256 KiB of partials + 256 B = 262,400 B per device.
//
// The array is one per device and per process: calls that overlap in time
// (two host threads, or two streams whose launches can run concurrently)
// share it and race.  Callers serialise them, e.g. on one stream.
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

#define NOALLOC_PARTIAL_BYTES (sizeof(double)*2*QLLG_MAXRHS*(size_t)QLLG_NOALLOC_MAXBLOCKS)
#define NOALLOC_MAXDEV 64

static __device__ __align__(256) unsigned char noalloc_scratch[NOALLOC_PARTIAL_BYTES + 256];

// device address of the scratch, looked up once per device with that
// device current (at the first link set-up on it).  Kept for the life of
// the process: after cudaDeviceReset the module is reloaded and the
// address may move, so the library must not be used across a device reset.
static void *g_scratch_base[NOALLOC_MAXDEV];

extern "C" int
qllg_noalloc_redbuf(qllg_redbuf *rb)
{
  int dev = -1;
  if(qllg_check_cuda(cudaGetDevice(&dev), "no-alloc scratch: current device")) return -1;
  if(dev < 0 || dev >= NOALLOC_MAXDEV) {
    qllg_set_error("no-alloc scratch: device %d beyond the %d devices it is kept for", dev,
                   NOALLOC_MAXDEV);
    return -1;
  }
  if(!g_scratch_base[dev]) {
    void *p = NULL;
    if(qllg_check_cuda(cudaGetSymbolAddress(&p, noalloc_scratch),
                       "no-alloc scratch: symbol address")) return -1;
    g_scratch_base[dev] = p;
  }
  rb->partial = (double *)g_scratch_base[dev];
  rb->counter = (unsigned *)((char *)g_scratch_base[dev] + NOALLOC_PARTIAL_BYTES);
  rb->maxblocks = QLLG_NOALLOC_MAXBLOCKS;
  return 0;
}
