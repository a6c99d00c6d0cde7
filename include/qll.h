/*
 * qll.h -- QLL's public C API served by libqll_gb300 (drop-in for the
 * reference's include/qll.h:1-58).  Code written against the reference
 * includes this header instead and links -lqll_gb300 (and the CUDA
 * runtime, -lcudart); it needs no QMP.  Every symbol exists in a ..F
 * (float) and a ..D (double) variant.  Differences from the reference:
 * links live on the GPU (copied at create time), errors return a failure
 * value with the message in qllg_last_error() instead of calling exit(),
 * and the geometry is one process's whole lattice (no QMP ranks).
 */
#ifndef QLLG_QLL_H
#define QLLG_QLL_H

#include <stddef.h>
#include "layout.h"
#include "thread.h"
#include "solvers.h"

#ifdef __cplusplus
extern "C" {
#endif

/* lib/common.c:9-28: 64-byte aligned host allocation (exits on failure,
 * as the reference does) */
void *myalloc(size_t size);
/* lib/common.c:52-72: global sum over ranks; one rank here, so it leaves
 * x unchanged (TC may be NULL) */
void gsum(double *x, int n, ThreadCtx *TC);
/* lib/common.c:7 */
extern int myrank;

/* include/qll.h:7-15 */
typedef struct {
  double one_link;
  double three_staple;
  double five_staple;
  double seven_staple;
  double lepage;
  double naik;
} Fat7Coeffs;
#define FAT7COEFFS_ZERO (Fat7Coeffs){0,0,0,0,0,0}

#define real float
#define PR(x) x ## F
#include "qllP.h"
#undef real
#undef PR

#define real double
#define PR(x) x ## D
#include "qllP.h"
#undef real
#undef PR

#ifdef __cplusplus
}
#endif

#endif
