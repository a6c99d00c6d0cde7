// k_stag_f64.cu -- the FP64 instantiations of the asqtad half-Dslash (kernels
// and launchers in k_stag.cuh): 16 slots here, 8 slots in k_stag_f64_ns8.cu
// (the two compile in parallel).
#include "k_stag.cuh"

extern "C" int qllg_k_stag_dslash_f64_ns8(const qllg_stag_args *a);

extern "C" int
qllg_k_stag_dslash_f64(const qllg_stag_args *a)
{
  if(a->nslots == 8) return qllg_k_stag_dslash_f64_ns8(a);
  return launch_ns_only<QLLG_F64, QLLG_F64, 16>(a);
}
