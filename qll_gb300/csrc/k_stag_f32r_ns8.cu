// k_stag_f32r_ns8.cu -- the FP32-spinor, reconstruct-12-link asqtad
// half-Dslash with 8 slots (fat links only), split from k_stag_f32r.cu.
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_f32r_ns8(const qllg_stag_args *a)
{
  return launch_ns_only<QLLG_F32, QLLG_F32R, 8>(a);
}
