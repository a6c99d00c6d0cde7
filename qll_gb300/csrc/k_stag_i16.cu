// k_stag_i16.cu -- the 16-bit instantiations of the asqtad half-Dslash
// (kernels and launchers in k_stag.cuh).
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_i16(const qllg_stag_args *a)
{
  return launch_ns<QLLG_I16, QLLG_I16>(a);
}
