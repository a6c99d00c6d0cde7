// k_stag_f32.cu -- the FP32 instantiations of the asqtad half-Dslash
// (kernels and launchers in k_stag.cuh): 16 slots here, 8 slots (fat links
// only) in k_stag_f32_ns8.cu.
#include "k_stag.cuh"

extern "C" int qllg_k_stag_dslash_f32_ns8(const qllg_stag_args *a);

extern "C" int
qllg_k_stag_dslash_f32(const qllg_stag_args *a)
{
  if(a->nslots == 8) return qllg_k_stag_dslash_f32_ns8(a);
  return launch_ns_only<QLLG_F32, QLLG_F32, 16>(a);
}

// the bulk-copy pipeline's error flag (a bounded wait ran out): returns it
// and clears it when reset is set
extern "C" int
qllg_k_bulk_error(int reset)
{
  int v = 0;
  if(cudaMemcpyFromSymbol(&v, g_bulk_err, sizeof(int)) != cudaSuccess) return -1;
  if(reset && v) {
    const int z = 0;
    if(cudaMemcpyToSymbol(g_bulk_err, &z, sizeof(int)) != cudaSuccess) return -1;
  }
  return v;
}
