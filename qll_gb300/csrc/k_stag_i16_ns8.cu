// k_stag_i16_ns8.cu -- the 16-bit-storage asqtad half-Dslash with 8 slots (fat links
// only), split from k_stag_i16.cu.
#include "k_stag.cuh"

extern "C" int
qllg_k_stag_dslash_i16_ns8(const qllg_stag_args *a)
{
  return launch_ns_only<QLLG_I16, QLLG_I16, 8>(a);
}
