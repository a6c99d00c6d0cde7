// k_stag_f32_ns8.cu -- the FP32 asqtad half-Dslash with 8 slots (fat links
// only), split from k_stag_f32.cu so that the two compile in parallel.
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_f32_ns8(const qllg_stag_args *a)
{
  return launch_ns_only<QLLG_F32, QLLG_F32, 8>(a);
}
