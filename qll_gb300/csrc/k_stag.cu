// k_stag.cu -- dispatch of the asqtad half-Dslash to the per-precision
// translation units, and the neighbour table the kernels' index arithmetic
// gives (for the bit-exactness test against the reference's tables).
#include "kcommon.cuh"

using namespace qk;

extern "C" int qllg_k_stag_dslash_f64(const qllg_stag_args *a);
extern "C" int qllg_k_stag_dslash_f32(const qllg_stag_args *a);
extern "C" int qllg_k_stag_dslash_i16(const qllg_stag_args *a);
extern "C" int qllg_k_stag_dslash_f32r(const qllg_stag_args *a);
extern "C" int qllg_k_stag_dslash_df(const qllg_stag_args *a);
extern "C" int qllg_k_stag_dslash_split(int ps, int pl, const qllg_stag_args *a);

namespace {

__global__ void
nbr_table(qllg_geom g, int p, int slot, int *out)
{
  const Geo G = make_geo(g);
  int i = blockIdx.x*blockDim.x + threadIdx.x;
  if(i >= G.Vh) return;
  int x[4];
  site_coords(G, p, i, x);
  int mu = slot/4, back = (slot/2) & 1, nk = slot & 1;
  int d = (nk ? 3 : 1)*(back ? -1 : 1);
  out[i] = (1 - p)*G.Vh + nbr_index(G, x, mu, d);
}

} // namespace

extern "C" int
qllg_k_stag_dslash(int ps, int pl, const qllg_stag_args *a)
{
  if(a->compact && (a->norm_out || a->norm_self || a->mode == 1 || a->mode == 3)) {
    qllg_set_error("stag_dslash: compacted launch takes modes 0 and 2 only, without norms");
    return -1;
  }
  if((a->norm_out || a->norm_self || a->mode == 3) && !a->rb) {
    qllg_set_error("stag_dslash: reduction requested without workspace");
    return -1;
  }
  if(ps == QLLG_F64 && pl == QLLG_F64) return qllg_k_stag_dslash_f64(a);
  if(ps == QLLG_F32 && pl == QLLG_F32) return qllg_k_stag_dslash_f32(a);
  if(ps == QLLG_I16 && pl == QLLG_I16) return qllg_k_stag_dslash_i16(a);
  if(ps == QLLG_F32 && pl == QLLG_F32R) return qllg_k_stag_dslash_f32r(a);
  if(ps == QLLG_DF && pl == QLLG_DF) return qllg_k_stag_dslash_df(a);
  if((ps == QLLG_F32 && pl == QLLG_I16) || (ps == QLLG_I16 && pl == QLLG_F32))
    return qllg_k_stag_dslash_split(ps, pl, a);
  qllg_set_error("stag_dslash: unsupported precision pair %d/%d", ps, pl);
  return -1;
}

extern "C" int
qllg_k_stag_nbr_table(const qllg_geom *g, int parity, int slot, int *dev_out)
{
  int n = g->Vh;
  nbr_table<<<(n + 255)/256, 256, 0, qllg_stream()>>>(*g, parity, slot, dev_out);
  return qllg_launched("nbr_table launch");
}
