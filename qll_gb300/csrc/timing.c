/*
 * timing.c -- optional per-kernel-family timing with CUDA events on the
 * library stream (the GPU counterpart of the reference's rdtsc phase
 * timers, lib/stagDslash.c:103-108, 659-713).  Disabled by default; when
 * enabled, each timed launch is bracketed by an event pair, and pairs are
 * harvested (elapsed times summed per family) when the pool fills or on
 * read.
 */
#include <string.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

#define NPAIR 8192
#define NFAM 16

static int g_on = 0;
static cudaEvent_t g_ev[2*NPAIR];
static int g_ev_made = 0;
static int g_fam_of[NPAIR];
static int g_npair = 0;
static int g_open = -1;
static char g_fam_name[NFAM][32];
static int g_nfam = 0;
static int g_count[NFAM];
static double g_ms[NFAM];

static int
fam_id(const char *name)
{
  for(int i=0; i<g_nfam; i++) if(!strcmp(g_fam_name[i], name)) return i;
  if(g_nfam == NFAM) return -1;
  strncpy(g_fam_name[g_nfam], name, 31);
  g_count[g_nfam] = 0;
  g_ms[g_nfam] = 0;
  return g_nfam++;
}

static void
harvest(void)
{
  if(!g_npair) return;
  cudaEventSynchronize(g_ev[2*(g_npair-1)+1]);
  for(int k=0; k<g_npair; k++) {
    float ms = 0;
    if(cudaEventElapsedTime(&ms, g_ev[2*k], g_ev[2*k+1]) == cudaSuccess) {
      g_ms[g_fam_of[k]] += ms;
      g_count[g_fam_of[k]]++;
    }
  }
  g_npair = 0;
}

void
qllg_timing_enable(int on)
{
  if(on && !g_ev_made) {
    for(int i=0; i<2*NPAIR; i++) cudaEventCreate(&g_ev[i]);
    g_ev_made = 1;
  }
  g_on = on;
}

void
qllg_timing_reset(void)
{
  if(g_npair) harvest();
  for(int i=0; i<g_nfam; i++) { g_count[i] = 0; g_ms[i] = 0; }
}

int
qllg_timing_read(const char *name, int *count, double *ms)
{
  harvest();
  for(int i=0; i<g_nfam; i++) if(!strcmp(g_fam_name[i], name)) {
    *count = g_count[i];
    *ms = g_ms[i];
    return 0;
  }
  *count = 0;
  *ms = 0;
  return -1;
}

/* bracket one launch; no-ops unless enabled */
int qllg_capturing(void);

void
qllg_tm_begin(const char *name)
{
  if(!g_on || qllg_capturing()) return;
  if(g_npair == NPAIR) harvest();
  int f = fam_id(name);
  if(f < 0) return;
  g_fam_of[g_npair] = f;
  g_open = g_npair;
  cudaEventRecord(g_ev[2*g_npair], qllg_stream());
}

void
qllg_tm_end(void)
{
  if(!g_on || g_open < 0 || qllg_capturing()) return;
  cudaEventRecord(g_ev[2*g_open+1], qllg_stream());
  g_npair = g_open + 1;
  g_open = -1;
}

int
qllg_timing_on(void)
{
  return g_on;
}
