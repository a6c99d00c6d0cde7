/*
 * solversP.h -- per-precision solver declarations of QLL's C API, included
 * twice by solvers.h with `real` and `PR` defined (drop-in for the
 * reference's include/solversP.h:1-22).
 *
 * cgSolve and cgmsSolve run the whole Krylov loop on the GPU.  The operator
 * must be one this library provides (the staggered even-odd normal
 * operator, stagLinopD/F, with a StaggeredSolver as its argument); any other
 * callback is refused with -1 and a message in qllg_last_error(), since a
 * host callback cannot run inside the device loop.  Mop (preconditioner) is
 * accepted only as NULL, which is how every caller in the reference passes
 * it (lib/stagDslash.c:611,641; lib/wilsonDslash.c:352).
 */
typedef struct {
  real *r1;
  real *r2;
  real *z;
  real *p;
  real *Ap;
  real *Adr2;
  int nelem;
  int verbose;
  int indent;
} PR(Cgls);

typedef void (PR(Linop))(real *Ax, real *x, LinopInfo *li,
                         void *args, ThreadCtx *TC);

/* lib/cg.c:8-33: records nelem; allocates no host vectors (NULL members) */
void PR(cglsInit)(PR(Cgls) *cgls, int nelem);
void PR(cglsFree)(PR(Cgls) *cgls);
/* lib/cg.c:124-136 */
int PR(cgSolve)(PR(Cgls) *cgls, real *x, real *b, PR(Linop) *Aop, void *Aargs,
                PR(Linop) *Mop, void *Margs, double rsq, int itnlim);
/* lib/cgms.c:181-195 */
int PR(cgmsSolve)(PR(Cgls) *cgls, real *x[], real *b, double shifts[],
                  int nshifts, PR(Linop) *Aop, void *Aargs, PR(Linop) *Mop,
                  void *Margs, double rsqs[], int itnlim);
