/*
 * ref_harnessP.h -- the per-precision entry points of ref_harness.c,
 * included once with REAL double and once with float.
 */

/* a field of nelem reals per site from the one-lane site order into this
 * build's layout (to_layout 1) or back (0) */
void
SFX(refh_convert)(REAL *dst, const REAL *src, int nelem, int to_layout)
{
  const int p = sizeof(REAL) == sizeof(double) ? 0 : 1;
  const int V = ls[0]*ls[1]*ls[2]*ls[3];
  const int vl = lay[p].nSitesInner;
  for(int s=0; s<V; s++) {
    int o, ln;
    site_slot(p, s, &o, &ln);
    for(int e=0; e<nelem; e++) {
      long k = ((long)o*nelem + e)*vl + ln;
      if(to_layout) dst[k] = src[(long)s*nelem + e];
      else dst[(long)s*nelem + e] = src[k];
    }
  }
}

/* defined in lib/stagDslash.c:522 and lib/wilsonDslash.c:263, not
 * declared in the reference's public headers */
void SFX(freeStaggeredLinks)(SFX(StaggeredLinks) *sl);
void SFX(freeWilsonLinks)(SFX(WilsonLinks) *sl);

/* x = dslash2 of the reference: m*y + sum of the 16 hops on the output
 * sites of sub ("all", "even", "odd"); u[2mu] forward fat links,
 * u[2mu+1] = -F_mu(x-mu)^dagger, u3 the same for the Naik links
 * (lib/stagDslash.c:422-462,531-544) */
void
SFX(refh_dslash)(REAL *x, REAL *u[8], REAL *u3[8], double mass, REAL *y, const char *sub)
{
  SFX(StaggeredLinks) sl;
  SFX(createStaggeredLinks)(&sl, LAYOUT, u, u3, (char *)sub);
  SFX(dslash2)(&sl, x, (REAL)mass, y);
  SFX(freeStaggeredLinks)(&sl);
}

/* solve2 (lib/stagDslash.c:600-623): (m^2 - D_eo D_oe) x = y on the even
 * sites to |r|^2 < rsq |y|^2; x scaled by m unless noscale */
int
SFX(refh_solve2)(REAL *x, REAL *u[8], REAL *u3[8], double mass, REAL *y, double rsq,
                 int maxits, int noscale)
{
  SFX(StaggeredSolver) ss;
  SFX(createStaggeredSolver)(&ss, LAYOUT, u, u3, "even");
  ss.noscale = noscale;
  int its = SFX(solve2)(&ss, x, (REAL)mass, y, rsq, maxits, "even");
  SFX(freeStaggeredSolver)(&ss);
  return its;
}

/* solveMulti2 (lib/stagDslash.c:625-657): the multishift CG, shifts
 * masses[i]^2 - masses[0]^2 */
int
SFX(refh_solveMulti2)(REAL *x[], REAL *u[8], REAL *u3[8], double masses[], int n, REAL *y,
                      double rsq, int maxits, int noscale)
{
  SFX(StaggeredSolver) ss;
  SFX(createStaggeredSolver)(&ss, LAYOUT, u, u3, "even");
  ss.noscale = noscale;
  int its = SFX(solveMulti2)(&ss, x, masses, n, y, rsq, maxits, "even");
  SFX(freeStaggeredSolver)(&ss);
  return its;
}

/* smearFat7 (lib/gauge.c:264-416) on thin links u[4] (forward only):
 * fat links fl[4] and, when ll is not NULL, Naik links ll[4]; coef in
 * the order one_link, three_staple, five_staple, seven_staple, lepage,
 * naik */
void
SFX(refh_smearFat7)(REAL *fl[4], REAL *ll[4], const double coef[6], REAL *u[4])
{
  Fat7Coeffs c = {coef[0], coef[1], coef[2], coef[3], coef[4], coef[5]};
  SFX(Field) F[4], Lg[4], U[4], *fp[4], *lp[4], *up[4];
  for(int i=0; i<4; i++) {
    SFX(fieldSet)(&F[i], fl[i], LAYOUT, 18);
    if(ll) SFX(fieldSet)(&Lg[i], ll[i], LAYOUT, 18);
    SFX(fieldSet)(&U[i], u[i], LAYOUT, 18);
    fp[i] = &F[i];
    lp[i] = &Lg[i];
    up[i] = &U[i];
  }
  SFX(smearFat7)(fp, ll ? lp : NULL, &c, up, up);
}

/* gaugePlaq (lib/gauge.c:133-183) */
void
SFX(refh_plaq)(double plaq[], REAL *u[4])
{
  SFX(Field) U[4], *up[4];
  for(int i=0; i<4; i++) {
    SFX(fieldSet)(&U[i], u[i], LAYOUT, 18);
    up[i] = &U[i];
  }
  SFX(gaugePlaq)(plaq, up);
}

/* x = wilsonDslash of the reference (lib/wilsonDslash.c:272-285): links
 * u[2mu] forward, u[2mu+1] backward (the caller's U_mu(x-mu)^dagger),
 * spinors of 24 reals per site */
void
SFX(refh_wilson_dslash)(REAL *x, REAL *u[8], double mass, int sign, REAL *y, const char *sub)
{
  SFX(WilsonLinks) wl;
  SFX(createWilsonLinks)(&wl, LAYOUT, u, (char *)sub);
  SFX(wilsonDslash)(&wl, x, (REAL)mass, sign, y);
  SFX(freeWilsonLinks)(&wl);
}

/* shift of lib/stagDslash.c:87-101 (declared in the reference's internal
 * include/common.h:51): x(site) = y(site + len*dir-hat), dir = +-(mu+1)
 * as in the reference's test programs (testdslash.c:219-242) */
void SFX(shift)(REAL *x, REAL *y, int nelem, int dir, int len);

void
SFX(refh_shift)(REAL *x, REAL *y, int nelem, int dir, int len)
{
  SFX(shift)(x, y, nelem, dir, len);
}

/* gaugeDoublestore (lib/gauge.c:34-63): ua[i] = shift of u[i] by
 * (dirs[i], lens[i]), then the adjoint of each 3x3 matrix */
void
SFX(refh_doublestore)(REAL *ua[], REAL *u[], int dirs[], int lens[], int n)
{
  SFX(Field) A[n], U[n], *ap[n], *up[n];
  for(int i=0; i<n; i++) {
    SFX(fieldSet)(&A[i], ua[i], LAYOUT, 18);
    SFX(fieldSet)(&U[i], u[i], LAYOUT, 18);
    ap[i] = &A[i];
    up[i] = &U[i];
  }
  SFX(gaugeDoublestore)(ap, up, dirs, lens, n);
}

/* makeU of lib/vla.c:1656-1665 (declared in the reference's internal
 * include/vla.h:85) on sites [0, n) of nc x nc matrices, 2 nc^2 reals a
 * site.  Site-local, so the one-lane build takes the array as it is. */
void SFX(makeU)(REAL *mm, int nc, int i0, int i1);

void
SFX(refh_makeU)(REAL *m, int nc, int n)
{
  SFX(makeU)(m, nc, 0, n);
}
