/*
 * layout.c -- QLL's layout functions for one rank and one lane
 * (lib/layout.c:5-217, lib/stagDslash.c:754-875), myalloc and gsum.
 *
 * The site numbering is the reference's layoutIndex with innerGeom = 1:
 * lexicographic index (x0 fastest) halved, even sites first.  The GPU
 * kernels compute the same numbering in closed form (kcommon.cuh), so this
 * file also owns the host-side neighbour tables that getShift and
 * getStaggeredSI return for API compatibility.
 */
#define _POSIX_C_SOURCE 200112L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

int myrank = 0;

void *
myalloc(size_t size)
{
  void *b = NULL;
  if(size == 0) size = 64;
  if(posix_memalign(&b, 64, size)) {
    /* the reference exits here too (lib/common.c:22-25) */
    fprintf(stderr, "myalloc(%zu) failed\n", size);
    exit(1);
  }
  return b;
}

void
gsum(double *x, int n, ThreadCtx *TC)
{
  (void)x; (void)n; (void)TC;   /* one rank, one host thread: nothing to add */
}

void
layoutSubset(Subset *s, Layout *l, char *sub)
{
  s->begin = 0;
  s->end = l->nSites;
  s->beginOuter = 0;
  s->endOuter = l->nSitesOuter;
  if(sub && sub[0] == 'e') {
    s->end = l->nEven;
    s->endOuter = l->nEvenOuter;
  } else if(sub && sub[0] == 'o') {
    s->begin = l->nOdd;
    s->beginOuter = l->nOddOuter;
  }
}

/* lib/layout.c:21-80 for innerGeom = 1 (no SIMD lanes, innerCb = 0) */
void
layoutSetup(Layout *l)
{
  int nd = l->nDim;
  l->outerGeom = myalloc(nd*sizeof(int));
  l->localGeom = myalloc(nd*sizeof(int));
  int pvol = 1, lvol = 1, ovol = 1;
  for(int i=0; i<nd; i++) {
    int rg = l->rankGeom ? l->rankGeom[i] : 1;
    int ig = l->innerGeom ? l->innerGeom[i] : 1;
    l->localGeom[i] = l->physGeom[i]/rg;
    l->outerGeom[i] = l->localGeom[i]/ig;
    pvol *= l->physGeom[i];
    lvol *= l->localGeom[i];
    ovol *= l->outerGeom[i];
  }
  l->physVol = pvol;
  l->nSites = lvol;
  l->nOdd = lvol/2;
  l->nEven = lvol - l->nOdd;
  l->nSitesOuter = ovol;
  l->nOddOuter = ovol/2;
  l->nEvenOuter = ovol - l->nOddOuter;
  l->nSitesInner = l->nSites/l->nSitesOuter;
  l->innerCb = 0;
  l->innerCbDir = 0;
}

void
layoutIndex(Layout *l, LayoutIndex *li, int coords[])
{
  int nd = l->nDim;
  int oi = 0, p = 0;
  for(int i=nd-1; i>=0; --i) oi = oi*l->outerGeom[i] + (coords[i] % l->outerGeom[i]);
  for(int i=0; i<nd; i++) p += coords[i];
  int oi2 = oi/2;
  if(p & 1) oi2 = (oi + l->nSitesOuter)/2;
  li->rank = 0;
  li->index = oi2;
}

void
layoutCoord(Layout *l, int coords[], LayoutIndex *li)
{
  int nd = l->nDim;
  int ii = li->index, p = 0;
  if(ii >= l->nEvenOuter) { ii -= l->nEvenOuter; p++; }
  ii *= 2;
  for(int i=0; i<nd; i++) {
    int k = ii % l->outerGeom[i];
    coords[i] = k;
    p += k;
    ii /= l->outerGeom[i];
  }
  if(p & 1) {
    for(int i=0; i<nd; i++) {
      coords[i]++;
      if(coords[i] >= l->outerGeom[i]) coords[i] = 0;
      else break;
    }
  }
}

void
layoutShift(Layout *l, LayoutIndex *li, LayoutIndex *li2, int disp[])
{
  int nd = l->nDim;
  int x[16];
  layoutCoord(l, x, li2);
  for(int i=0; i<nd; i++) x[i] = (x[i] + disp[i] + l->physGeom[i]) % l->physGeom[i];
  layoutIndex(l, li, x);
}

/* ------------------------------------------------------------ geometry */

/* the geometry of the last stagDslashSetup, as the reference keeps one
 * (lib/stagDslash.c:715-719); the native API takes dims explicitly */
static Layout *g_layout = NULL;
static int g_dims[4] = {0,0,0,0};

int
qllg_geom_from_dims(qllg_geom *g, const int dims[4])
{
  g->V = 1;
  for(int i=0; i<4; i++) {
    if(dims[i] < 4 || (dims[i] & 1)) {
      qllg_set_error("lattice extent %d of direction %d: every extent must be even and >= 4",
                     dims[i], i);
      return -1;
    }
    g->L[i] = dims[i];
    g->V *= dims[i];
  }
  g->Vh = g->V/2;
  return 0;
}

int
qllg_geom_from_layout(qllg_geom *g, const Layout *l)
{
  if(!l || l->nDim != 4) {
    qllg_set_error("layout: only 4-dimensional lattices are supported");
    return -1;
  }
  if(l->nSitesInner != 1) {
    qllg_set_error("layout: this library uses one lane per site (innerGeom = 1)");
    return -1;
  }
  return qllg_geom_from_dims(g, l->physGeom);
}

Layout *
qllg_current_layout(void)
{
  return g_layout;
}

static void
stag_setup(Layout *layout, int nd, int ls[], int rg0[])
{
  myrank = layout->myrank;
  if(nd != 4) {
    qllg_set_error("stagDslashSetup: nd = %d, only 4 is supported", nd);
    return;
  }
  if(rg0) for(int i=0; i<nd; i++) if(rg0[i] != 1) {
    qllg_set_error("stagDslashSetup: one rank only (rank geometry must be all ones)");
    return;
  }
  qllg_geom g;
  if(qllg_geom_from_dims(&g, ls)) return;
  layout->nDim = nd;
  layout->physGeom = malloc(nd*sizeof(int));
  layout->rankGeom = malloc(nd*sizeof(int));
  layout->innerGeom = malloc(nd*sizeof(int));
  for(int i=0; i<nd; i++) {
    layout->physGeom[i] = ls[i];
    layout->rankGeom[i] = 1;
    layout->innerGeom[i] = 1;
  }
  if(layout->nranks < 1) layout->nranks = 1;
  layoutSetup(layout);
  g_layout = layout;
  memcpy(g_dims, ls, sizeof(g_dims));
  qllg_runtime_init();
}

void stagDslashSetupD(Layout *layout, int nd, int ls[], int rg[]) { stag_setup(layout, nd, ls, rg); }
void stagDslashSetupF(Layout *layout, int nd, int ls[], int rg[]) { stag_setup(layout, nd, ls, rg); }

/* --------------------------------------------------- neighbour tables */

/* host tables of getShift/getStaggeredSI, built on first request per
 * (dims, displacement, parity) with the closed-form numbering */
typedef struct { int dims[4]; int disp[4]; int parity; ShiftIndices si; } shift_entry;
static shift_entry *g_shifts = NULL;
static int g_nshifts = 0;

static void
site_coord(const int L[4], int idx, int x[4])
{
  int V = L[0]*L[1]*L[2]*L[3];
  int p = idx >= V/2;
  int i = idx - p*(V/2);
  int X0h = L[0]/2;
  int x0h = i % X0h, r = i / X0h;
  x[1] = r % L[1]; r /= L[1];
  x[2] = r % L[2]; x[3] = r / L[2];
  x[0] = 2*x0h + ((p + x[1] + x[2] + x[3]) & 1);
}

static int
site_index(const int L[4], const int x[4])
{
  int V = L[0]*L[1]*L[2]*L[3];
  int lex = x[0] + L[0]*(x[1] + L[1]*(x[2] + L[2]*x[3]));
  int p = (x[0] + x[1] + x[2] + x[3]) & 1;
  return lex/2 + p*(V/2);
}

ShiftIndices *
qllg_shift_indices(const int dims[4], const int disp[4], int parity)
{
  for(int i=0; i<g_nshifts; i++) {
    shift_entry *e = &g_shifts[i];
    if(!memcmp(e->dims, dims, sizeof(e->dims)) && !memcmp(e->disp, disp, sizeof(e->disp))
       && e->parity == parity) return &e->si;
  }
  g_shifts = realloc(g_shifts, sizeof(shift_entry)*(g_nshifts + 1));
  shift_entry *e = &g_shifts[g_nshifts++];
  memset(e, 0, sizeof(*e));
  memcpy(e->dims, dims, sizeof(e->dims));
  memcpy(e->disp, disp, sizeof(e->disp));
  e->parity = parity;
  int V = dims[0]*dims[1]*dims[2]*dims[3];
  ShiftIndices *si = &e->si;
  si->disp = malloc(4*sizeof(int));
  memcpy(si->disp, disp, 4*sizeof(int));
  si->pidx = malloc(V*sizeof(int));
  si->sidx = malloc(V*sizeof(int));
  for(int i=0; i<V; i++) {
    int x[4], y[4];
    site_coord(dims, i, x);
    int p = (x[0] + x[1] + x[2] + x[3]) & 1;
    if(parity >= 0 && p != parity) { si->pidx[i] = si->sidx[i] = -1; continue; }
    for(int k=0; k<4; k++) y[k] = (x[k] - disp[k] + dims[k]) % dims[k];
    si->pidx[i] = si->sidx[i] = site_index(dims, y);
  }
  si->vv = V;
  return si;
}

static int
sub_parity(const char *sub)
{
  return (sub && sub[0] == 'e') ? 0 : ((sub && sub[0] == 'o') ? 1 : -1);
}

static ShiftIndices *
get_shift(int dir, int len, char *sub)
{
  if(!g_layout) { qllg_set_error("getShift: call stagDslashSetup first"); return NULL; }
  int disp[4] = {0,0,0,0};
  if(dir < 0 || dir > 3) { qllg_set_error("getShift: dir %d", dir); return NULL; }
  disp[dir] = -len;
  return qllg_shift_indices(g_dims, disp, sub_parity(sub));
}

ShiftIndices *getShiftD(int dir, int len, char *sub) { return get_shift(dir, len, sub); }
ShiftIndices *getShiftF(int dir, int len, char *sub) { return get_shift(dir, len, sub); }

/* getStaggeredSI (lib/stagDslash.c:721-733): the array of the slots of a
 * link set, in the slot order of createStaggeredLinks */
static ShiftIndices g_stagsi[2][3][16];

static ShiftIndices *
get_stag_si(int naik, char *sub)
{
  if(!g_layout) { qllg_set_error("getStaggeredSI: call stagDslashSetup first"); return NULL; }
  int par = sub_parity(sub);
  int n = naik ? 16 : 8;
  ShiftIndices *arr = g_stagsi[naik ? 1 : 0][par + 1];
  for(int s=0; s<n; s++) {
    int i = naik ? s/2 : s;
    int len = (naik && (s & 1)) ? 3 : 1;
    int disp[4] = {0,0,0,0};
    disp[i/2] = len*(2*(i & 1) - 1);
    arr[s] = *qllg_shift_indices(g_dims, disp, par);
  }
  return arr;
}

ShiftIndices *getStaggeredSID(int naik, char *sub) { return get_stag_si(naik, sub); }
ShiftIndices *getStaggeredSIF(int naik, char *sub) { return get_stag_si(naik, sub); }
