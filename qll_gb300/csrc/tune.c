/*
 * tune.c -- registry of the autotuner's choices.  A kernel launcher that
 * has variants (the multi-rhs Dslash: rhs per thread) times them the first
 * time it sees a launch shape and stores the fastest here under a key
 * naming the shape; later launches look it up.  qllg_autotune_report
 * lists the choices with the measured times.
 */
#include <stdio.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "qll_gb300.h"
#include "qllg_internal.h"

#define NTUNE 256
#define NCAND 24

static struct {
  char key[96];
  int choice, ncand;
  float ms[NCAND];
  const char *names[NCAND];
} g_tune[NTUNE];
static int g_ntune = 0;

int
qllg_tune_lookup(const char *key)
{
  for(int i=0; i<g_ntune; i++) if(!strcmp(g_tune[i].key, key)) return g_tune[i].choice;
  return -1;
}

void
qllg_tune_store(const char *key, int choice, int ncand, const float *ms, const char *const *names)
{
  int i = 0;
  while(i < g_ntune && strcmp(g_tune[i].key, key)) i++;
  if(i == NTUNE) return;              /* full: the shape is re-timed on next use */
  if(i == g_ntune) g_ntune++;
  snprintf(g_tune[i].key, sizeof(g_tune[i].key), "%s", key);
  g_tune[i].choice = choice;
  g_tune[i].ncand = ncand < NCAND ? ncand : NCAND;
  for(int c=0; c<g_tune[i].ncand; c++) {
    g_tune[i].ms[c] = ms[c];
    g_tune[i].names[c] = names[c];
  }
}

int
qllg_autotune_report(char *buf, size_t len)
{
  size_t n = 0;
  if(len) buf[0] = 0;
  for(int i=0; i<g_ntune && n < len; i++) {
    int w = snprintf(buf + n, len - n, "%s: %s", g_tune[i].key,
                     g_tune[i].names[g_tune[i].choice]);
    n += w > 0 ? (size_t)w : 0;
    for(int c=0; c<g_tune[i].ncand && n < len; c++) {
      if(g_tune[i].ms[c] < 0) continue;
      w = snprintf(buf + n, len - n, "%s %s %.4f ms", c ? "," : " |", g_tune[i].names[c],
                   g_tune[i].ms[c]);
      n += w > 0 ? (size_t)w : 0;
    }
    if(n < len) { w = snprintf(buf + n, len - n, "\n"); n += w > 0 ? (size_t)w : 0; }
  }
  return g_ntune;
}
