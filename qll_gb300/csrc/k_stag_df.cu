// k_stag_df.cu -- the double-float asqtad half-Dslash (kernels and
// launchers in k_stag.cuh): the compacted launch over the flagged rhs only,
// for the reliable updates of the mixed solver.  Links and spinors hold
// each real as a (hi, lo) pair of floats in the FP64 layout; the arithmetic
// is the dfl type of kcommon.cuh, on the FP32 pipes.
#include "k_stag.cuh"

namespace {

template <int NS, int MB>
int launch_df_nr(const qllg_stag_args *a)
{
  switch(a->nrhs) {
  case 1: return launch_compact<QLLG_DF,QLLG_DF,NS,1,MB>(a);
  case 2: return launch_compact<QLLG_DF,QLLG_DF,NS,2,MB>(a);
  case 4: return launch_compact<QLLG_DF,QLLG_DF,NS,4,MB>(a);
  case 8: return launch_compact<QLLG_DF,QLLG_DF,NS,8,MB>(a);
  case 16: return launch_compact<QLLG_DF,QLLG_DF,NS,16,MB>(a);
  }
  qllg_set_error("stag_dslash: nrhs %d not in {1,2,4,8,16}", a->nrhs);
  return -1;
}

} // namespace

extern "C" int
qllg_k_stag_dslash_df(const qllg_stag_args *a)
{
  if(!a->compact) {
    qllg_set_error("stag_dslash: double-float runs the compacted reliable-update launch only");
    return -1;
  }
  const int mb = (int)qllg_get_param("df_blocks");
  if(a->nslots == 16) return mb >= 3 ? launch_df_nr<16,3>(a) : launch_df_nr<16,1>(a);
  if(a->nslots == 8) return mb >= 3 ? launch_df_nr<8,3>(a) : launch_df_nr<8,1>(a);
  qllg_set_error("stag_dslash: nslots %d not 8 or 16", a->nslots);
  return -1;
}
