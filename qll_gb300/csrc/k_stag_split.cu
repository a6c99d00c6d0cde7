// k_stag_split.cu -- the asqtad half-Dslash with spinors and links in
// different storage, for the mixed solver's 16-bit split modes: FP32
// spinors with 16-bit links (one float scale per slot), and 16-bit spinors
// (per-site scale) with FP32 links; FP32 arithmetic in both.  Two launch
// shapes only, without autotuning: 16 slots and 16 rhs take the 4-rhs
// kernel's lean 64-register rolled shape (the one the FP32 pair chooses),
// everything else the one-thread-per-(site, rhs) kernel.
#include "k_stag.cuh"

namespace {

template <int PS, int PL, int NS>
int launch_split_ns(const qllg_stag_args *a)
{
  if(a->compact) {
    qllg_set_error("stag_dslash: no compacted launch for split precisions");
    return -1;
  }
  switch(a->nrhs) {
  case 1: return launch_plain<PS,PL,NS,1>(a);
  case 2: return launch_plain<PS,PL,NS,2>(a);
  case 4: return launch_plain<PS,PL,NS,4>(a);
  case 8: return launch_plain<PS,PL,NS,8>(a);
  case 16:
    if(NS == 16) return launch_mr<PS,PL,NS,16,4,8>(a);
    return launch_plain<PS,PL,NS,16>(a);
  }
  qllg_set_error("stag_dslash: nrhs %d not in {1,2,4,8,16}", a->nrhs);
  return -1;
}

template <int PS, int PL>
int launch_split(const qllg_stag_args *a)
{
  if(a->nslots == 16) return launch_split_ns<PS,PL,16>(a);
  if(a->nslots == 8) return launch_split_ns<PS,PL,8>(a);
  qllg_set_error("stag_dslash: nslots %d not 8 or 16", a->nslots);
  return -1;
}

} // namespace

extern "C" int
qllg_k_stag_dslash_split(int ps, int pl, const qllg_stag_args *a)
{
  if(ps == QLLG_F32 && pl == QLLG_I16) return launch_split<QLLG_F32, QLLG_I16>(a);
  if(ps == QLLG_I16 && pl == QLLG_F32) return launch_split<QLLG_I16, QLLG_F32>(a);
  qllg_set_error("stag_dslash: unsupported precision pair %d/%d", ps, pl);
  return -1;
}
