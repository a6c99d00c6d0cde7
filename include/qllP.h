/*
 * qllP.h -- per-precision part of QLL's C API, included twice by qll.h
 * with `real` and `PR` defined (drop-in for the reference's
 * include/qllP.h:1-110, plus the entry points that the reference declares
 * in its internal include/common.h:50-60 and defines in lib/stagDslash.c).
 *
 * Semantics that differ from the reference are stated per function.
 * Common to all: arrays are host arrays in
 * the one-lane layout of layout.h; links are copied to GPU memory when the
 * link or solver object is created (the reference keeps the caller's
 * pointers and re-reads them on every call, lib/stagDslash.c:441-447), so a
 * caller that changes its host links afterwards re-creates the object.
 */

/* include/qllP.h:1-6 */
typedef struct {
  Layout *l;
  real *f;
  int nelem;
} PR(Field);

/* lib/field.c:3-63 */
void PR(fieldNew)(PR(Field) *f, Layout *l, int nelem);
void PR(fieldFree)(PR(Field) *f);
void PR(fieldSet)(PR(Field) *f, real *r, Layout *l, int nelem);
void PR(fieldZero)(PR(Field) *f, Subset *sub);
double PR(fieldSumElem)(PR(Field) *f, Subset *sub);
double PR(fieldNorm2)(PR(Field) *f, Subset *sub);

/* include/qllP.h:16-27 */
typedef struct {
  real *u;
  ShiftIndices si;
  int nelem;
  int nc;
  int td;
  ShiftBuf sb;
  Subset sub;
  int backward;
  real *dest;
  real *src;
} PR(Transporter);

/* lib/transporter.c:12-193: dest(x) (+)= u(x) src(neighbour); the
 * start/local/wait split runs the whole transport on the GPU in
 * transporterWaitT (StartT and LocalT only record the operands) */
void PR(transporterNew)(PR(Transporter) *t, real *u, ShiftIndices *si,
                        Subset *sub, int nelem, int nc);
void PR(transporterFree)(PR(Transporter) *t);
void PR(transporterStartT)(PR(Transporter) *t, real *dest, real *src,
                           int td, ThreadCtx *TC);
void PR(transporterLocalT)(PR(Transporter) *t, ThreadCtx *TC);
void PR(transporterWaitT)(PR(Transporter) *t, ThreadCtx *TC);
void PR(transporterDoT)(PR(Transporter) *t, real *dest, real *src, int td,
                        ThreadCtx *TC);
void PR(transporterDo)(PR(Transporter) *t, real *dest, real *src, int td);

/* lib/gauge.c:34-63, 114-183, 264-416 */
void PR(gaugeDoublestore)(PR(Field) *ua[], PR(Field) *u[], int dirs[], int lens[], int n);
void PR(gaugePlaq)(double plaqs[], PR(Field) *u[]);
void PR(smearFat7)(PR(Field) *fl[], PR(Field) *ll[], Fat7Coeffs *coef,
                   PR(Field) *u[], PR(Field) *uLong[]);

/* include/qllP.h:49-55 */
typedef struct {
  double massFac;
  PR(Transporter) *t;
  int n;
  int fb;
} PR(StaggeredLinks);

/* include/qllP.h:57-68 */
typedef struct {
  PR(StaggeredLinks) sle, slo;
  double mass;
  real *v;
  PR(Cgls) cgls;
  int its;
  int noscale;
  double flops;
  double secs;
  Subset sube, subo;
} PR(StaggeredSolver);

/* lib/stagDslash.c:788-875 (one rank: rg NULL or all ones) */
void PR(stagDslashSetup)(Layout *layout, int nd, int ls[], int rg[]);
/* lib/stagDslash.c:422-462, 464-519 */
void PR(createStaggeredLinks)(PR(StaggeredLinks) *sl, Layout *l,
                              real *u[], real *u3[], char *sub);
void PR(createStaggeredLinksFb)(PR(StaggeredLinks) *sl, Layout *l,
                                real *u[], real *u3[], char *sub);
void PR(freeStaggeredLinks)(PR(StaggeredLinks) *sl);
/* lib/stagDslash.c:531-544 */
void PR(dslash2)(PR(StaggeredLinks) *d, real *x, real mass, real *y);

/* lib/stagDslash.c:577-598 */
void PR(createStaggeredSolver)(PR(StaggeredSolver) *ss, Layout *l,
                               real *u[], real *u3[], char *sub);
void PR(freeStaggeredSolver)(PR(StaggeredSolver) *ss);
/* declared but never defined by the reference (include/qllP.h:71-74);
 * defined here as create solver, solve2 / solveMulti2, free */
int PR(solve)(real *x, real *u[8], real *u3[8], real mass, real *y,
              double rsq, char *sub);
int PR(solveMulti)(real *x[], real *u[8], real *u3[8], double masses[],
                   int nmasses, real *y, double rsq, char *sub);
/* lib/stagDslash.c:600-657 */
int PR(solve2)(PR(StaggeredSolver) *ss, real *x, real mass, real *y,
               double rsq, int maxits, char *sub);
int PR(solveMulti2)(PR(StaggeredSolver) *ss, real *x[], double masses[],
                    int nmasses, real *y, double rsq, int maxits, char *sub);

/* the staggered normal operator of a StaggeredSolver as a Linop for
 * cgSolve/cgmsSolve (the reference's static dslashp2,
 * lib/stagDslash.c:546-575); args is the StaggeredSolver */
void PR(stagLinop)(real *Ax, real *x, LinopInfo *li, void *args, ThreadCtx *TC);

/* lib/stagDslash.c:91-101, 721-749 */
void PR(shift)(real *x, real *y, int nelem, int dir, int len);
ShiftIndices *PR(getStaggeredSI)(int naik, char *sub);
ShiftIndices *PR(getShift)(int dir, int len, char *sub);
/* lib/stagDslash.c:659-713 (GPU event timers of dslash2) */
void PR(dslashResetTimer)(void);
void PR(dslashPrintTimer)(double scale);

/* include/qllP.h:76-81 */
typedef struct {
  double massFac;
  PR(Transporter) *t;
  int n;
  int fb;
} PR(WilsonLinks);

/* include/qllP.h:83-94 */
typedef struct {
  PR(WilsonLinks) sle, slo;
  double mass;
  real *v;
  PR(Cgls) cgls;
  int its;
  int noscale;
  double flops;
  double secs;
  Subset sube, subo;
} PR(WilsonSolver);

/* lib/wilsonDslash.c:181-202, 272-285 (sign ignored, as in the reference) */
void PR(createWilsonLinks)(PR(WilsonLinks) *sl, Layout *l, real *u[], char *sub);
void PR(freeWilsonLinks)(PR(WilsonLinks) *sl);
void PR(wilsonDslash)(PR(WilsonLinks) *d, real *x, real mass, int sign, real *y);
/* lib/wilsonDslash.c:318-364 */
void PR(createWilsonSolver)(PR(WilsonSolver) *ss, Layout *l, real *u[], char *sub);
void PR(freeWilsonSolver)(PR(WilsonSolver) *ss);
int PR(wilsonSolve)(PR(WilsonSolver) *ss, real *x, real mass, real *y,
                    double rsq, int maxits, char *sub);
/* declared by the reference (include/qllP.h:108) with its body disabled
 * (lib/wilsonDslash.c:366-400): always returns -1 here */
int PR(wilsonSolveMulti)(PR(WilsonSolver) *ss, real *x[], double masses[],
                         int nmasses, real *y, double rsq, int maxits, char *sub);
void PR(wilsonDslashResetTimer)(void);
void PR(wilsonDslashPrintTimer)(double scale);
