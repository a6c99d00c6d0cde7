/*
 * embed_solve.c -- a C program written against the drop-in headers only
 * (include/qll.h; the native qll_gb300.h just for the seeded generator),
 * the way an embedding code uses the reference library
 * (embedqop.c:193-258): set up the layout, build the asqtad links from
 * thin links with smearFat7, make the double-stored backward links with
 * shift and the negative adjoint, create a staggered solver and solve2 on
 * the even sites.  Built by the CPU tests (compiles and links against
 * -lqll_gb300) and run by a GPU test, which checks its output.
 *
 * Usage: embed_solve L0 L1 L2 L3 mass; prints "its <n> resid <|r|/|b|>".
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "qll.h"
#include "qll_gb300.h"
#include "vla.h"

/* the test programs' re-unitarisation entry points link too (QLL's
 * stress.c and fieldtest.c call makeU on their link fields) */
void (*const reunitarise_d)(double *, int, int, int) = makeUD;
void (*const reunitarise_f)(float *, int, int, int) = makeUF;

/* x = -y^dagger for every 3x3 matrix of a [V][18] field (column-major
 * complex entries, entry 3*column + row) */
static void
neg_adjoint(double *x, const double *y, int V)
{
  for(int s=0; s<V; s++)
    for(int c=0; c<3; c++)
      for(int r=0; r<3; r++) {
        const double *a = y + 18*(size_t)s + 2*(3*r + c);
        double *b = x + 18*(size_t)s + 2*(3*c + r);
        b[0] = -a[0];
        b[1] = a[1];
      }
}

int
main(int argc, char *argv[])
{
  if(argc < 6) { fprintf(stderr, "usage: embed_solve L0 L1 L2 L3 mass\n"); return 2; }
  int ls[4];
  for(int i=0; i<4; i++) ls[i] = atoi(argv[1 + i]);
  double mass = atof(argv[5]);
  Layout layout;
  memset(&layout, 0, sizeof(layout));
  layout.nranks = 1;
  layout.myrank = 0;
  stagDslashSetupD(&layout, 4, ls, NULL);
  int V = layout.nSites;
  if(V <= 0) { fprintf(stderr, "setup failed: %s\n", qllg_last_error()); return 1; }

  /* thin links with the staggered phases, then fat7 with the asqtad
   * coefficients (smearFat7, lib/gauge.c:264) */
  double *thin[4], *fat[4], *lng[4];
  FieldD tf[4], ff[4], lf[4], *tp[4], *fp[4], *lp[4];
  for(int mu=0; mu<4; mu++) {
    thin[mu] = malloc(sizeof(double)*18*V);
    fat[mu] = malloc(sizeof(double)*18*V);
    lng[mu] = malloc(sizeof(double)*18*V);
  }
  if(qllg_gen_gauge(ls, 1001, 0.3, 1, thin)) { fprintf(stderr, "%s\n", qllg_last_error()); return 1; }
  for(int mu=0; mu<4; mu++) {
    fieldSetD(&tf[mu], thin[mu], &layout, 18);
    fieldSetD(&ff[mu], fat[mu], &layout, 18);
    fieldSetD(&lf[mu], lng[mu], &layout, 18);
    tp[mu] = &tf[mu]; fp[mu] = &ff[mu]; lp[mu] = &lf[mu];
  }
  Fat7Coeffs coef = {5.0/8, -1.0/16, 1.0/64, -1.0/384, -1.0/16, -1.0/24};
  smearFat7D(fp, lp, &coef, tp, tp);

  /* double-stored links: u[2mu] = F_mu(x), u[2mu+1] = -F_mu(x-mu)^dagger;
   * the same with three hops for the Naik links (testdslash.c:219-243) */
  double *u[8], *u3[8], *tmp = malloc(sizeof(double)*18*V);
  for(int mu=0; mu<4; mu++) {
    u[2*mu] = fat[mu];
    u3[2*mu] = lng[mu];
    u[2*mu + 1] = malloc(sizeof(double)*18*V);
    u3[2*mu + 1] = malloc(sizeof(double)*18*V);
    shiftD(tmp, fat[mu], 18, -(mu + 1), 1);
    neg_adjoint(u[2*mu + 1], tmp, V);
    shiftD(tmp, lng[mu], 18, -(mu + 1), 3);
    neg_adjoint(u3[2*mu + 1], tmp, V);
  }

  StaggeredSolverD ss;
  createStaggeredSolverD(&ss, &layout, u, u3, "even");
  ss.noscale = 1;
  double *b = calloc(6*(size_t)V, sizeof(double)), *x = calloc(6*(size_t)V, sizeof(double));
  if(qllg_gen_source(ls, 2100, 6, "even", b)) { fprintf(stderr, "%s\n", qllg_last_error()); return 1; }
  int its = solve2D(&ss, x, mass, b, 1e-16, 5000, "even");
  if(its <= 0) { fprintf(stderr, "solve2D failed: %s\n", qllg_last_error()); return 1; }

  /* the true residual with the drop-in operator: r = b - (m^2 x - D_eo D_oe x),
   * from dslash2 on the odd then the even sites */
  StaggeredLinksD so, se;
  createStaggeredLinksD(&so, &layout, u, u3, "odd");
  createStaggeredLinksD(&se, &layout, u, u3, "even");
  double *v = calloc(6*(size_t)V, sizeof(double)), *w = calloc(6*(size_t)V, sizeof(double));
  dslash2D(&so, v, 0, x);
  dslash2D(&se, w, 0, v);
  double rr = 0, bb = 0;
  for(int i=0; i<6*V/2; i++) {
    double r = b[i] - (mass*mass*x[i] - w[i]);
    rr += r*r;
    bb += b[i]*b[i];
  }
  printf("its %d resid %.3e\n", its, sqrt(rr/bb));
  freeStaggeredLinksD(&so);
  freeStaggeredLinksD(&se);
  freeStaggeredSolverD(&ss);
  return 0;
}
