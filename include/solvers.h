/*
 * solvers.h -- QLL solver interface (drop-in for the reference's
 * include/solvers.h:1-18): LinopInfo and both precisions of solversP.h.
 */
#ifndef QLLG_SOLVERS_H
#define QLLG_SOLVERS_H

#include "thread.h"

#ifdef __cplusplus
extern "C" {
#endif

/* include/solvers.h:1-5 */
typedef struct {
  int adj;
  int wantAnorm2;
  double Anorm2;
} LinopInfo;
#define LINOP_INFO_DEFAULT {0,0,0}

#define real float
#define PR(x) x ## F
#include "solversP.h"
#undef real
#undef PR

#define real double
#define PR(x) x ## D
#include "solversP.h"
#undef real
#undef PR

#ifdef __cplusplus
}
#endif

#endif
