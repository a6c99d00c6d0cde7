// k_stag_f64.cu -- the FP64 instantiations of the asqtad half-Dslash
// (kernels and launchers in k_stag.cuh).
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_f64(const qllg_stag_args *a)
{
  return launch_ns<QLLG_F64, QLLG_F64>(a);
}
