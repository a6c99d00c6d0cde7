// k_stag_i16.cu -- the 16-bit-storage instantiations of the asqtad half-Dslash (kernels
// and launchers in k_stag.cuh): 16 slots here, 8 slots in k_stag_i16_ns8.cu
// (the two compile in parallel).
#include "k_stag.cuh"

extern "C" int qllg_k_stag_dslash_i16_ns8(const qllg_stag_args *a);

extern "C" int
qllg_k_stag_dslash_i16(const qllg_stag_args *a)
{
  if(a->nslots == 8) return qllg_k_stag_dslash_i16_ns8(a);
  return launch_ns_only<QLLG_I16, QLLG_I16, 16>(a);
}
