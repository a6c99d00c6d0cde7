// k_stag_f64_ns8.cu -- the FP64 asqtad half-Dslash with 8 slots (fat links
// only), split from k_stag_f64.cu.
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_f64_ns8(const qllg_stag_args *a)
{
  return launch_ns_only<QLLG_F64, QLLG_F64, 8>(a);
}
