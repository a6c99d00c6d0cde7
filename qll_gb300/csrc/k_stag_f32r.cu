// k_stag_f32r.cu -- the FP32-spinor, reconstruct-12-link instantiations of
// the asqtad half-Dslash (kernels and launchers in k_stag.cuh).
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_f32r(const qllg_stag_args *a)
{
  return launch_ns<QLLG_F32, QLLG_F32R>(a);
}
