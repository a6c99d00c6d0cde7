/*
 * thread.h -- the ThreadCtx type of QLL's C API (drop-in for the
 * reference's include/thread.h:43-51).
 *
 * The reference runs each API call inside its own OpenMP region and hands
 * every thread a ThreadCtx; its Linop callbacks (include/solversP.h) take
 * one.  This library runs the work on the GPU from one host thread, so it
 * never creates a ThreadCtx itself, but the type stays layout-identical so
 * that code written against the reference compiles unchanged.
 */
#ifndef QLLG_THREAD_H
#define QLLG_THREAD_H

typedef struct {
  double **sum;
  int volatile *tbar;
  int tid;
  int nid;
  int tib;
  int n0, n1, d0;
} ThreadCtx;

#endif
