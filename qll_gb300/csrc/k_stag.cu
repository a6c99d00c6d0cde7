// k_stag.cu -- asqtad staggered half-Dslash kernels (sm_103a).
//
// One thread per (output site, right-hand side), rhs fastest, so the nrhs
// threads of a site share every link load (a broadcast from L1) while the
// spinor loads stay coalesced.  Neighbours are computed in-kernel from the
// even-odd lexicographic site order (periodic in every direction), which
// replaces the reference's gather tables (lib/shifts.c:516-736) and halo
// exchange.  The slot order and the per-slot arithmetic follow dslash2T
// (lib/stagDslash.c:316-328) and PeqM3AtimesV3o (lib/vla0.c.lua:193-213):
// slot s = 4*mu + 2*backward + naik, acc += U_s(x) psi(x + d_s).
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kThreads = 256;

int qllg_mr_disabled() { return qllg_get_param("dslash_mr") == 0; }

template <int PS, int PL, int NS, int NR>
__global__ void __launch_bounds__(kThreads)
stag_dslash(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  __shared__ double shm[2*kThreads];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh * NR;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  double red[2] = {0.0, 0.0};
  const int rhs = threadIdx.x % NR;
  const bool act = !a.active || a.active[rhs];
  const T ca = (T)(a.a ? a.a[rhs] : a.a0);
  const T cb = (T)a.b;
  constexpr int PX = VecPrec<PS>::value;   // x and r of the fused CG epilogue
  T alpha = 0;
  if(a.mode == 3 && act)
    alpha = (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs]));
  if(!skip && act) {
    for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < total;
        t += (size_t)gridDim.x*blockDim.x) {
      const int site = (int)(t / NR);
      int x[4];
      site_coords(G, p, site, x);
      Cx<T> acc[3], self[3];
      if(a.self && a.mode == 1) SpinorIO<PS,3>::load(a.self, total, t, self);
      if(a.mode == 1) {
#pragma unroll
        for(int c=0; c<3; c++) { acc[c].r = ca*self[c].r; acc[c].i = ca*self[c].i; }
      } else {
#pragma unroll
        for(int c=0; c<3; c++) { acc[c].r = 0; acc[c].i = 0; }
      }
#pragma unroll
      for(int mu=0; mu<4; mu++) {
#pragma unroll
        for(int back=0; back<2; back++) {
#pragma unroll
          for(int nk=0; nk<(NS == 16 ? 2 : 1); nk++) {
            const int slot = (NS == 16) ? (4*mu + 2*back + nk) : (2*mu + back);
            const int d = (nk ? 3 : 1)*(back ? -1 : 1);
            const int k = nbr_index(G, x, mu, d);
            Cx<T> U[9], v[3];
            LinkIO<PL>::load(a.links, slot, V, loff + site, a.lscale, U);
            SpinorIO<PS,3>::load(a.in, total, (size_t)k*NR + rhs, v);
#pragma unroll
            for(int l=0; l<3; l++) {
#pragma unroll
              for(int j=0; j<3; j++) cmac(acc[j], U[3*l + j], v[l]);
            }
          }
        }
      }
      if(a.self && a.mode != 1) SpinorIO<PS,3>::load(a.self, total, t, self);
      Cx<T> out[3];
      if(a.mode == 3) {
        // Ap = m^2 p - D v; x += alpha p; r -= alpha Ap (cgSolveT, lib/cg.c:101-105)
        Cx<T> xv[3], rv[3];
        SpinorIO<PX,3>::load(a.x, total, t, xv);
        SpinorIO<PX,3>::load(a.r, total, t, rv);
#pragma unroll
        for(int c=0; c<3; c++) {
          T apr = fma(cb, acc[c].r, ca*self[c].r), api = fma(cb, acc[c].i, ca*self[c].i);
          xv[c].r = fma(alpha, self[c].r, xv[c].r); xv[c].i = fma(alpha, self[c].i, xv[c].i);
          rv[c].r = fma(-alpha, apr, rv[c].r); rv[c].i = fma(-alpha, api, rv[c].i);
          red[0] += (double)rv[c].r*rv[c].r + (double)rv[c].i*rv[c].i;
        }
        SpinorIO<PX,3>::store(a.x, total, t, xv);
        SpinorIO<PX,3>::store(a.r, total, t, rv);
        continue;
      }
      if(a.mode == 2) {
#pragma unroll
        for(int c=0; c<3; c++) {
          T sr = a.self ? ca*self[c].r : (T)0, si = a.self ? ca*self[c].i : (T)0;
          out[c].r = fma(cb, acc[c].r, sr);
          out[c].i = fma(cb, acc[c].i, si);
        }
      } else {
#pragma unroll
        for(int c=0; c<3; c++) out[c] = acc[c];
      }
      SpinorIO<PS,3>::store(a.out, total, t, out);
      if(a.norm_out) {
#pragma unroll
        for(int c=0; c<3; c++) red[0] += (double)out[c].r*out[c].r + (double)out[c].i*out[c].i;
      }
      if(a.norm_self && a.self) {
#pragma unroll
        for(int c=0; c<3; c++) red[1] += (double)self[c].r*self[c].r + (double)self[c].i*self[c].i;
      }
    }
  }
  if(a.mode == 3) {
    if(skip) return;   // uniform: the flag was set before this launch
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce<2>(red, NR, rhs, a.partial, a.counter, shm, res)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce<2>(red, NR, rhs, a.partial, a.counter, shm, res);
  }
}


// Multi-rhs variant: a thread owns one site and R consecutive right-hand
// sides, so each link is loaded and converted once per R rhs and the R
// accumulator sets give independent FMA chains.  Same epilogues as above.
template <int PS, int PL, int NS, int NR, int R>
__global__ void __launch_bounds__(kThreads)
stag_dslash_mr(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  constexpr int Q = NR/R;                       // threads per site
  constexpr int PX = VecPrec<PS>::value;
  __shared__ double shm[2*R*kThreads];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh * NR;
  const size_t nwork = (size_t)G.Vh * Q;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  const int q = threadIdx.x % Q;
  bool act[R];
  T ca[R], alpha[R];
  bool anyact = false;
  const T cb = (T)a.b;
#pragma unroll
  for(int j=0; j<R; j++) {
    const int rhs = q*R + j;
    act[j] = !a.active || a.active[rhs];
    anyact |= act[j];
    ca[j] = (T)(a.a ? a.a[rhs] : a.a0);
    alpha[j] = (a.mode == 3 && act[j])
      ? (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs])) : (T)0;
  }
  double red[2][R];
#pragma unroll
  for(int j=0; j<R; j++) { red[0][j] = 0; red[1][j] = 0; }
  if(!skip && anyact) {
    for(size_t w = (size_t)blockIdx.x*blockDim.x + threadIdx.x; w < nwork;
        w += (size_t)gridDim.x*blockDim.x) {
      const int site = (int)(w / Q);
      const size_t t0 = (size_t)site*NR + q*R;
      int x[4];
      site_coords(G, p, site, x);
      Cx<T> acc[R][3];
#pragma unroll
      for(int j=0; j<R; j++) {
        if(a.mode == 1 && a.self) {
          Cx<T> s[3];
          SpinorIO<PS,3>::load(a.self, total, t0 + j, s);
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = ca[j]*s[c].r; acc[j][c].i = ca[j]*s[c].i; }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = 0; acc[j][c].i = 0; }
        }
      }
#pragma unroll
      for(int mu=0; mu<4; mu++) {
#pragma unroll
        for(int back=0; back<2; back++) {
#pragma unroll
          for(int nk=0; nk<(NS == 16 ? 2 : 1); nk++) {
            const int slot = (NS == 16) ? (4*mu + 2*back + nk) : (2*mu + back);
            const int d = (nk ? 3 : 1)*(back ? -1 : 1);
            const size_t kb = (size_t)nbr_index(G, x, mu, d)*NR + q*R;
            Cx<T> U[9];
            LinkIO<PL>::load(a.links, slot, V, loff + site, a.lscale, U);
#pragma unroll
            for(int j=0; j<R; j++) {
              if(!act[j]) continue;
              Cx<T> v[3];
              SpinorIO<PS,3>::load(a.in, total, kb + j, v);
#pragma unroll
              for(int l=0; l<3; l++) {
#pragma unroll
                for(int c=0; c<3; c++) cmac(acc[j][c], U[3*l + c], v[l]);
              }
            }
          }
        }
      }
#pragma unroll
      for(int j=0; j<R; j++) {
        if(!act[j]) continue;
        const size_t t = t0 + j;
        Cx<T> self[3];
        if(a.self && a.mode != 1) SpinorIO<PS,3>::load(a.self, total, t, self);
        if(a.mode == 3) {
          Cx<T> xv[3], rv[3];
          SpinorIO<PX,3>::load(a.x, total, t, xv);
          SpinorIO<PX,3>::load(a.r, total, t, rv);
#pragma unroll
          for(int c=0; c<3; c++) {
            T apr = fma(cb, acc[j][c].r, ca[j]*self[c].r), api = fma(cb, acc[j][c].i, ca[j]*self[c].i);
            xv[c].r = fma(alpha[j], self[c].r, xv[c].r); xv[c].i = fma(alpha[j], self[c].i, xv[c].i);
            rv[c].r = fma(-alpha[j], apr, rv[c].r); rv[c].i = fma(-alpha[j], api, rv[c].i);
            red[0][j] += (double)rv[c].r*rv[c].r + (double)rv[c].i*rv[c].i;
          }
          SpinorIO<PX,3>::store(a.x, total, t, xv);
          SpinorIO<PX,3>::store(a.r, total, t, rv);
          continue;
        }
        Cx<T> out[3];
        if(a.mode == 2) {
#pragma unroll
          for(int c=0; c<3; c++) {
            T sr = a.self ? ca[j]*self[c].r : (T)0, si = a.self ? ca[j]*self[c].i : (T)0;
            out[c].r = fma(cb, acc[j][c].r, sr);
            out[c].i = fma(cb, acc[j][c].i, si);
          }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) out[c] = acc[j][c];
        }
        SpinorIO<PS,3>::store(a.out, total, t, out);
        if(a.norm_out) {
#pragma unroll
          for(int c=0; c<3; c++) red[0][j] += (double)out[c].r*out[c].r + (double)out[c].i*out[c].i;
        }
        if(a.norm_self && a.self) {
#pragma unroll
          for(int c=0; c<3; c++) red[1][j] += (double)self[c].r*self[c].r + (double)self[c].i*self[c].i;
        }
      }
    }
  }
  if(a.mode == 3) {
    if(skip) return;
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res);
  }
}

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

template <int PS, int PL, int NS, int NR, int R>
int launch_mr(const qllg_stag_args *a)
{
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash_mr<PS,PL,NS,NR,R>, kThreads, 0), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  size_t work = (size_t)a->g.Vh * (NR/R);
  size_t need = (work + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  stag_dslash_mr<PS,PL,NS,NR,R><<<grid, kThreads, 0, qllg_stream()>>>(A);
  return qllg_launched("stag_dslash_mr launch");
}

template <int PS, int PL, int NS, int NR>
int launch_t(const qllg_stag_args *a)
{
  if(NR >= 4 && !qllg_mr_disabled()) return launch_mr<PS,PL,NS,NR,(NR >= 4 ? 4 : 1)>(a);
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash<PS,PL,NS,NR>, kThreads, 0), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  size_t total = (size_t)a->g.Vh * NR;
  size_t need = (total + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  stag_dslash<PS,PL,NS,NR><<<grid, kThreads, 0, qllg_stream()>>>(A);
  return qllg_launched("stag_dslash launch");
}

template <int PS, int PL, int NS>
int launch_nr(const qllg_stag_args *a)
{
  switch(a->nrhs) {
  case 1: return launch_t<PS,PL,NS,1>(a);
  case 2: return launch_t<PS,PL,NS,2>(a);
  case 4: return launch_t<PS,PL,NS,4>(a);
  case 8: return launch_t<PS,PL,NS,8>(a);
  case 16: return launch_t<PS,PL,NS,16>(a);
  }
  qllg_set_error("stag_dslash: nrhs %d not in {1,2,4,8,16}", a->nrhs);
  return -1;
}

template <int PS, int PL>
int launch_ns(const qllg_stag_args *a)
{
  if(a->nslots == 16) return launch_nr<PS,PL,16>(a);
  if(a->nslots == 8) return launch_nr<PS,PL,8>(a);
  qllg_set_error("stag_dslash: nslots %d not 8 or 16", a->nslots);
  return -1;
}

} // namespace

extern "C" int
qllg_k_stag_dslash(int ps, int pl, const qllg_stag_args *a)
{
  if((a->norm_out || a->norm_self || a->mode == 3) && !a->rb) {
    qllg_set_error("stag_dslash: reduction requested without workspace");
    return -1;
  }
  if(ps == QLLG_F64 && pl == QLLG_F64) return launch_ns<QLLG_F64, QLLG_F64>(a);
  if(ps == QLLG_F32 && pl == QLLG_F32) return launch_ns<QLLG_F32, QLLG_F32>(a);
  if(ps == QLLG_I16 && pl == QLLG_I16) return launch_ns<QLLG_I16, QLLG_I16>(a);

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
