/*
 * oracle_gen.c -- test infrastructure: the seeded input generator of the
 * library (qll_gb300/csrc/gen_core.h, the same source) exported from the
 * oracle, so that CPU-only programs (the CPU timing arm of the benchmark,
 * CPU tests) make the same inputs without loading the GPU library.
 */
#include "../qll_gb300/csrc/gen_core.h"

static int
dims_ok(const int dims[4])
{
  for(int i=0; i<4; i++) if(dims[i] < 4 || (dims[i] & 1)) return 0;
  return 1;
}

int
or_gen_gauge(const int dims[4], unsigned long long seed, double eps, int ks, double *u[4])
{
  if(!dims_ok(dims)) return -1;
  gen_gauge_fill(dims, seed, eps, ks, u);
  return 0;
}

int
or_gen_source(const int dims[4], unsigned long long seed, int nelem, const char *sub, double *v)
{
  if(!dims_ok(dims)) return -1;
  gen_source_fill(dims, seed, nelem, sub, v);
  return 0;
}
