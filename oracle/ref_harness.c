/*
 * ref_harness.c -- C entry points (test infrastructure) over the
 * reference library compiled by ref_build.py, so that tests and the CPU
 * timing arm can call it through ctypes with plain arrays.  They drive the
 * reference API as its own test programs do (testdslash.c:158-330,
 * testwilson.c): one rank, Layout filled by stagDslashSetup, links and
 * vectors in the one-lane site order of layoutIndex (even sites first),
 * links column-major 3x3 complex ([site][18]).
 *
 * refh_setup(dims) must come first; it sets up both precisions.  The
 * reference keeps only pointers to the caller's links
 * (lib/stagDslash.c:441-447), so every call builds its link and solver
 * objects from the arrays it is given and releases them before returning.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <fcntl.h>
#include <omp.h>
#include <qmp.h>    /* layout.h uses its handle types */
#include "qll.h"

static Layout lay[2];          /* [0] double, [1] float */
static int ls[4];

/* the reference prints its geometry while setting up; keep stdout clean
 * for the programs that parse it */
static int
quiet_begin(void)
{
  fflush(stdout);
  int saved = dup(1);
  int nul = open("/dev/null", O_WRONLY);
  if(nul >= 0) { dup2(nul, 1); close(nul); }
  return saved;
}

static void
quiet_end(int saved)
{
  fflush(stdout);
  if(saved >= 0) { dup2(saved, 1); close(saved); }
}

int
refh_setup(const int dims[4])
{
  for(int i=0; i<4; i++) {
    if(dims[i] < 4 || (dims[i] & 1)) return -1;
    ls[i] = dims[i];
  }
  int q = quiet_begin();
  for(int p=0; p<2; p++) {
    memset(&lay[p], 0, sizeof(Layout));
    lay[p].nranks = 1;
    lay[p].myrank = 0;
    lay[p].nDim = 4;
    lay[p].physGeom = ls;
  }
  stagDslashSetupD(&lay[0], 4, ls, NULL);
  stagDslashSetupF(&lay[1], 4, ls, NULL);
  quiet_end(q);
  return 0;
}

/* the OpenMP thread count of the reference's parallel regions.  Its
 * smearFat7 is not deterministic with many threads on the smallest
 * lattices (4^4: a site range per thread of a few sites gives run-to-run
 * differences in some fat links), so parity runs use one thread. */
void
refh_set_threads(int n)
{
  if(n > 0) omp_set_num_threads(n);
}

int
refh_nsites(void)
{
  return lay[0].nSites;
}

/* SIMD lanes per vector of this build (1 for -DC1; -DC4 packs 4 sites) */
int
refh_vlen(void)
{
  return lay[0].nSitesInner;
}

/* position of one-lane site s (the order of layoutIndex with one lane:
 * even sites first, each parity lexicographic with x0 fastest, halved) in
 * this build's layout, whose arrays are [(outer*nelem + e)*VLEN + lane]
 * with layoutIndex's index = outer*VLEN + lane */
static void
site_slot(int p, int s, int *outer, int *lane)
{
  const Layout *l = &lay[p];
  int V = ls[0]*ls[1]*ls[2]*ls[3];
  int par = s >= V/2;
  int i = s - par*(V/2);
  int x[4];
  int x0h = i % (ls[0]/2), r = i / (ls[0]/2);
  x[1] = r % ls[1]; r /= ls[1];
  x[2] = r % ls[2]; x[3] = r / ls[2];
  x[0] = 2*x0h + ((par + x[1] + x[2] + x[3]) & 1);
  LayoutIndex li;
  layoutIndex((Layout *)l, &li, x);
  *outer = li.index / l->nSitesInner;
  *lane = li.index % l->nSitesInner;
}

#define REAL double
#define SFX(x) x ## D
#define LAYOUT (&lay[0])
#include "ref_harnessP.h"
#undef REAL
#undef SFX
#undef LAYOUT

#define REAL float
#define SFX(x) x ## F
#define LAYOUT (&lay[1])
#include "ref_harnessP.h"
#undef REAL
#undef SFX
#undef LAYOUT
