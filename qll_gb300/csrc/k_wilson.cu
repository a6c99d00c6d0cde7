// k_wilson.cu -- Wilson half-Dslash (sm_103a): per slot project the
// neighbour spinor to two spin components, multiply by the link, and
// reconstruct (the half-spinor form of lib/vlaw0.c.lua:545-652 with the
// DeGrand-Rossi gamma matrices of lib/Gamma.lua:5-26):
//   out = mode-dependent mass term - sum_mu [ (1 - g_mu) U_2mu(x) psi(x+mu)
//                                           + (1 + g_mu) U_2mu+1(x) psi(x-mu) ]
// dag = 1 flips the projector signs, which is gamma5 D gamma5.
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kThreads = 256;

// one nonzero per row of gamma_mu (DeGrand-Rossi): its column and phase
// (0:+1 1:+i 2:-1 3:-i); compile-time so the unrolled loops index registers
//   mu=0: cols 3,2,1,0 phases  i, i,-i,-i     mu=1: cols 3,2,1,0 phases -1,1,1,-1
//   mu=2: cols 2,3,0,1 phases  i,-i,-i, i     mu=3: cols 2,3,0,1 phases  1,1,1, 1
__device__ __forceinline__ constexpr int gcol(int mu, int row) {
  return mu < 2 ? 3 - row : (row ^ 2);
}
__device__ __forceinline__ constexpr int gph(int mu, int row) {
  return mu == 0 ? (row < 2 ? 1 : 3)
       : mu == 1 ? ((row == 0 || row == 3) ? 2 : 0)
       : mu == 2 ? ((row == 0 || row == 3) ? 1 : 3) : 0;
}

template <typename T>
__device__ __forceinline__ Cx<T> phase(const Cx<T> &z, int code) {
  Cx<T> r;
  switch(code & 3) {
  case 0: r = z; break;
  case 1: r.r = -z.i; r.i = z.r; break;
  case 2: r.r = -z.r; r.i = -z.i; break;
  default: r.r = z.i; r.i = -z.r; break;
  }
  return r;
}

// acc -= the eight hops of site `site` (coordinates x) of the output
// parity: per slot the neighbour spinor projected to two spin components,
// multiplied by the link and reconstructed (dag: gamma5 D gamma5)
template <int PS, int PL, int NR, typename T>
__device__ __forceinline__ void wilson_hops(const void *links, const float *lscale, const void *in, int dag,
                                            const Geo &G, size_t V, size_t loff, int site, const int x[4],
                                            int rhs, size_t total, Cx<T> acc[12])
{
#pragma unroll
  for(int mu=0; mu<4; mu++) {
#pragma unroll
    for(int back=0; back<2; back++) {
      // slot 2mu: (1 - g_mu) from x+mu; slot 2mu+1: (1 + g_mu) from x-mu
      const int sgn = (back ? 1 : -1)*(dag ? -1 : 1);
      const int k = nbr_index(G, x, mu, back ? -1 : 1);
      Cx<T> U[9], f[12];
      LinkIO<PL>::load(links, 2*mu + back, V, loff + site, lscale, U);
      SpinorIO<PS,12>::load(in, total, (size_t)k*NR + rhs, f);
#pragma unroll
      for(int hk=0; hk<2; hk++) {
        const int col = gcol(mu, hk);
        const int ph = gph(mu, hk) + (sgn < 0 ? 2 : 0);
        Cx<T> h[3], tt[3];
#pragma unroll
        for(int c=0; c<3; c++) {
          Cx<T> y = phase(f[3*col + c], ph);
          h[c].r = f[3*hk + c].r + y.r; h[c].i = f[3*hk + c].i + y.i;
          tt[c].r = 0; tt[c].i = 0;
        }
#pragma unroll
        for(int l=0; l<3; l++) {
#pragma unroll
          for(int j=0; j<3; j++) cmac(tt[j], U[3*l + j], h[l]);
        }
        // r_hk -= t; r_a -= sgn*phase_a*t for the lower row a fed by hk
#pragma unroll
        for(int c=0; c<3; c++) { acc[3*hk + c].r -= tt[c].r; acc[3*hk + c].i -= tt[c].i; }
#pragma unroll
        for(int ar=2; ar<4; ar++) {
          if(gcol(mu, ar) == hk) {
            const int pa = gph(mu, ar) + (sgn < 0 ? 0 : 2);   // minus sign folded in
#pragma unroll
            for(int c=0; c<3; c++) {
              Cx<T> y = phase(tt[c], pa);
              acc[3*ar + c].r += y.r; acc[3*ar + c].i += y.i;
            }
          }
        }
      }
    }
  }
}

// UPD: the body of mode 4 (FP32 only), a kernel of its own
// (wilson_dslash_upd) so that the fused update's registers do not cost
// the other launches occupancy
template <int PS, int PL, int NR, bool UPD>
__device__ __forceinline__ void wilson_dslash_body(const qllg_stag_args &a)
{
  typedef typename Calc<PS, PL>::T T;
  __shared__ double shm[2*kThreads];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh * NR;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  Acc<T> acc0, acc1;
  const int rhs = threadIdx.x % NR;
  const bool act = !a.active || (a.active[rhs] && (!a.active_eq || a.active[rhs] == a.active_eq));
  const T ca = (T)(a.a ? a.a[rhs] : a.a0);
  const T cb = (T)a.b;
  // mode 4: the step length of the fused x, r update (read before any
  // block's bookkeeping can change the scalars: the last block writes them
  // only after every block has reduced)
  static_assert(!UPD || (PS == QLLG_F32 && PL == QLLG_F32), "mode 4 is FP32 only");
  constexpr bool F4 = UPD;
  float alpha = 0;
  if constexpr (F4) if(a.mode == 4 && act && !skip) alpha = (float)(a.sc->rsq[rhs]/a.sc->pnorm[rhs]);
  if(!skip && act) {
    for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < total;
        t += (size_t)gridDim.x*blockDim.x) {
      const int site = (int)(t / NR);
      int x[4];
      site_coords(G, p, site, x);
      Cx<T> acc[12], self[12];
      if(a.self && a.mode == 1) SpinorIO<PS,12>::load(a.self, total, t, self);
#pragma unroll
      for(int c=0; c<12; c++) {
        if(a.mode == 1) { acc[c].r = ca*self[c].r; acc[c].i = ca*self[c].i; }
        else { acc[c].r = 0; acc[c].i = 0; }
      }
      wilson_hops<PS,PL,NR,T>(a.links, a.lscale, a.in, a.dag, G, V, loff, site, x, rhs, total, acc);
      if(a.self && a.mode != 1) SpinorIO<PS,12>::load(a.self, total, t, self);
      Cx<T> out[12];
#pragma unroll
      for(int c=0; c<12; c++) {
        if(a.mode == 2 || (UPD && a.mode == 4)) {
          T sr = a.self ? ca*self[c].r : (T)0, si = a.self ? ca*self[c].i : (T)0;
          out[c].r = kfma(cb, acc[c].r, sr); out[c].i = kfma(cb, acc[c].i, si);
        } else out[c] = acc[c];
      }
      if constexpr (F4) if(a.mode == 4) {
        // out is Ap: x += alpha p, r -= alpha Ap, |r|^2 (as scg_xr_k)
        Cx<T> xv[12], rv[12], pv[12];
        SpinorIO<PS,12>::load(a.x, total, t, xv);
        SpinorIO<PS,12>::load(a.r, total, t, rv);
        SpinorIO<PS,12>::load(a.pvec, total, t, pv);
#pragma unroll
        for(int c=0; c<12; c++) {
          xv[c].r = fma(alpha, pv[c].r, xv[c].r); xv[c].i = fma(alpha, pv[c].i, xv[c].i);
          rv[c].r = fma(-alpha, out[c].r, rv[c].r); rv[c].i = fma(-alpha, out[c].i, rv[c].i);
        }
        acc0.norm(rv);
        SpinorIO<PS,12>::store(a.x, total, t, xv);
        SpinorIO<PS,12>::store(a.r, total, t, rv);
        continue;
      }
      SpinorIO<PS,12>::store(a.out, total, t, out);
      if(a.norm_out) acc0.norm(out);
      if(a.norm_self && a.self) acc1.norm(self);
    }
  }
  if(F4 && a.mode == 4) {
    if(skip) return;                   // uniform: the solve is done
    double red1[1] = {acc0.get()};
    double *res1[1] = {a.sc->tmp};
    if(grid_reduce<1>(red1, NR, rhs, a.partial, a.counter, shm, res1)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        cg_finish_std(a.sc, NR);
        if(a.cond) {
          // the reliable-update block of a captured loop runs when flagged
          const int take = !a.sc->no_ru;
          if(take) a.sc->ru_trips++;
          cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond, take ? 1u : 0u);
        }
      }
    }
    return;
  }
  double red[2] = {acc0.get(), acc1.get()};
  if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce<2>(red, NR, rhs, a.partial, a.counter, shm, res);
  }
}

template <int PS, int PL, int NR>
__global__ void __launch_bounds__(kThreads)
wilson_dslash(qllg_stag_args a)
{
  wilson_dslash_body<PS,PL,NR,false>(a);
}

// mode 4, two blocks of 256 a SM (128 registers)
__global__ void __launch_bounds__(kThreads, 2)
wilson_dslash_upd(qllg_stag_args a)
{
  wilson_dslash_body<QLLG_F32,QLLG_F32,1,true>(a);
}

// ------------------------------------------ persistent CGNR iterations
// One cooperative launch runs the FP32 iterations of the mixed Wilson CGNR
// (the standard-form CG on S^dagger S of wilson.c, one rhs) until a
// reliable update is flagged, the solve is done or the trip cap is reached;
// the host then takes the update with the double-float and FP64 kernels and
// launches again.  On a small lattice (C2, 16^3x32: 65,536 even sites) the
// graph loop's half Dslashes are about 10 us of work each and the gaps
// between its kernel nodes cost as much again; at 32^3x64 the launch is
// still a few percent ahead.  The grid is the co-resident blocks at most,
// each walking its sites with a grid stride.  Per iteration:
//   v = W_oe p; Sp = a p - W_eo v / a with |Sp|^2; v = W_oe^+ Sp;
//   Ap = a Sp - W_eo^+ v / a, x += alpha p, r -= alpha Ap with |r|^2
//   (alpha = |r|^2/|Sp|^2); the bookkeeping of cg_finish_std; p = r + beta p
// with a grid barrier after each step.  Each reduction writes one partial
// per block, a barrier follows, and every block folds the partials in
// block order itself, so all blocks hold bitwise the same scalars.  The
// barrier is a counter and a generation word whose waits give up after
// poll_limit polls: the block sets the error word and returns, and so do
// the others at their next barrier.
struct WcgpArgs {
  qllg_geom g;
  const void *links;              // FP32 links
  void *x, *r, *p, *Sp, *v;       // FP32: x, r, p, S p (even sites), v (odd sites)
  qllg_cg_scalars *sc;
  double a;                       // 4 + m
  double *partial;                // [2][gridDim]
  unsigned *bar;                  // [0] arrivals, [1] generation
  int *err;                       // 1: a barrier wait ran out
  long long poll_limit;
  int extra;                      // barrier arrivals expected beyond the grid (tests)
  int trips;                      // iteration cap of this launch
};

__device__ bool wcg_barrier(const WcgpArgs &a)
{
  __shared__ int ok;
  __syncthreads();
  if(threadIdx.x == 0) {
    ok = 1;
    volatile unsigned *gen = a.bar + 1;
    const unsigned g = *gen;
    __threadfence();
    const unsigned want = gridDim.x + (unsigned)a.extra;
    if(atomicAdd(a.bar, 1u) == want - 1) {
      a.bar[0] = 0;
      __threadfence();
      atomicAdd(a.bar + 1, 1u);
    } else {
      long long n = 0;
      while(*gen == g) {
        if(++n > a.poll_limit || *(volatile int *)a.err) {
          atomicExch(a.err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// the grid's sum of val (one value a thread), the same in every block
__device__ bool wcg_sum(const WcgpArgs &a, double val, double &out, int &phase)
{
  __shared__ double buf[kThreads];
  __shared__ double res;
  buf[threadIdx.x] = val;
  __syncthreads();
  for(int w = kThreads/2; w > 0; w >>= 1) {
    if(threadIdx.x < w) buf[threadIdx.x] += buf[threadIdx.x + w];
    __syncthreads();
  }
  double *part = a.partial + (size_t)(phase & 1)*gridDim.x;
  if(threadIdx.x == 0) part[blockIdx.x] = buf[0];
  phase++;
  if(!wcg_barrier(a)) return false;
  if(threadIdx.x < 32) {
    double t = 0;
    for(int b = threadIdx.x; b < (int)gridDim.x; b += 32) t += ((volatile double *)part)[b];
#pragma unroll
    for(int o=16; o>0; o>>=1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if(threadIdx.x == 0) res = t;
  }
  __syncthreads();
  out = res;
  return true;
}

// out = W_oe^(dag) in on the odd sites (mode 0 of the half Dslash)
__device__ __forceinline__ void wcg_hop_odd(const WcgpArgs &a, const Geo &G, const void *in, int dag)
{
  const size_t V = (size_t)a.g.V, total = (size_t)G.Vh;
  for(size_t t = (size_t)blockIdx.x*kThreads + threadIdx.x; t < total; t += (size_t)gridDim.x*kThreads) {
    int x[4];
    site_coords(G, 1, (int)t, x);
    Cx<float> acc[12];
#pragma unroll
    for(int c=0; c<12; c++) { acc[c].r = 0; acc[c].i = 0; }
    wilson_hops<QLLG_F32,QLLG_F32,1,float>(a.links, NULL, in, dag, G, V, (size_t)G.Vh, (int)t, x, 0, total,
                                           acc);
    SpinorIO<QLLG_F32,12>::store(a.v, total, t, acc);
  }
}

__global__ void __launch_bounds__(kThreads, 2)
wilson_cgnr_persistent(WcgpArgs a)
{
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V, total = (size_t)G.Vh;
  const float ca = (float)a.a, cb = (float)(-1.0/a.a);
  __shared__ double s_rsq, s_pn, s_beta, s_maxr2, s_stop, s_delta2, s_prev;
  __shared__ int s_act, s_iters, s_maxits, s_ru, s_stop_loop;
  if(threadIdx.x == 0) {
    qllg_cg_scalars *sc = a.sc;
    s_rsq = sc->rsq[0]; s_pn = sc->pnorm[0]; s_beta = sc->alpha[0]; s_maxr2 = sc->maxr2[0];
    s_stop = sc->rsq_stop[0]; s_delta2 = sc->delta2; s_prev = sc->prev[0];
    s_act = sc->active[0] && !sc->done; s_iters = sc->iters[0]; s_maxits = sc->maxits;
    s_ru = 0; s_stop_loop = 0;
  }
  __syncthreads();
  int phase = 0, trip = 0;
  while(s_act && !s_stop_loop && trip < a.trips) {
    trip++;
    // v = W_oe p
    wcg_hop_odd(a, G, a.p, 0);
    if(!wcg_barrier(a)) return;
    // Sp = a p - W_eo v / a, |Sp|^2
    Acc<float> an;
    for(size_t t = (size_t)blockIdx.x*kThreads + threadIdx.x; t < total; t += (size_t)gridDim.x*kThreads) {
      int x[4];
      site_coords(G, 0, (int)t, x);
      Cx<float> acc[12], pv[12], o[12];
#pragma unroll
      for(int c=0; c<12; c++) { acc[c].r = 0; acc[c].i = 0; }
      wilson_hops<QLLG_F32,QLLG_F32,1,float>(a.links, NULL, a.v, 0, G, V, 0, (int)t, x, 0, total, acc);
      SpinorIO<QLLG_F32,12>::load(a.p, total, t, pv);
#pragma unroll
      for(int c=0; c<12; c++) { o[c].r = kfma(cb, acc[c].r, ca*pv[c].r); o[c].i = kfma(cb, acc[c].i, ca*pv[c].i); }
      SpinorIO<QLLG_F32,12>::store(a.Sp, total, t, o);
      an.norm(o);
    }
    double pn;
    if(!wcg_sum(a, an.get(), pn, phase)) return;
    // v = W_oe^+ Sp
    wcg_hop_odd(a, G, a.Sp, 1);
    if(!wcg_barrier(a)) return;
    // Ap = a Sp - W_eo^+ v / a; x += alpha p, r -= alpha Ap, |r|^2
    Acc<float> ar;
    {
      const float alpha = (float)(s_rsq/pn);
      for(size_t t = (size_t)blockIdx.x*kThreads + threadIdx.x; t < total; t += (size_t)gridDim.x*kThreads) {
        int x[4];
        site_coords(G, 0, (int)t, x);
        Cx<float> acc[12], sv[12], xv[12], rv[12], pv[12];
#pragma unroll
        for(int c=0; c<12; c++) { acc[c].r = 0; acc[c].i = 0; }
        wilson_hops<QLLG_F32,QLLG_F32,1,float>(a.links, NULL, a.v, 1, G, V, 0, (int)t, x, 0, total, acc);
        SpinorIO<QLLG_F32,12>::load(a.Sp, total, t, sv);
        SpinorIO<QLLG_F32,12>::load(a.x, total, t, xv);
        SpinorIO<QLLG_F32,12>::load(a.r, total, t, rv);
        SpinorIO<QLLG_F32,12>::load(a.p, total, t, pv);
#pragma unroll
        for(int c=0; c<12; c++) {
          const float apr = kfma(cb, acc[c].r, ca*sv[c].r), api = kfma(cb, acc[c].i, ca*sv[c].i);
          xv[c].r = fmaf(alpha, pv[c].r, xv[c].r); xv[c].i = fmaf(alpha, pv[c].i, xv[c].i);
          rv[c].r = fmaf(-alpha, apr, rv[c].r); rv[c].i = fmaf(-alpha, api, rv[c].i);
        }
        ar.norm(rv);
        SpinorIO<QLLG_F32,12>::store(a.x, total, t, xv);
        SpinorIO<QLLG_F32,12>::store(a.r, total, t, rv);
      }
    }
    double r2;
    if(!wcg_sum(a, ar.get(), r2, phase)) return;
    // cg_finish_std's bookkeeping (every block the same)
    if(threadIdx.x == 0) {
      s_pn = pn;
      s_iters++;
      s_prev = s_rsq;
      s_rsq = r2;
      s_beta = r2/s_prev;
      if(r2 < s_stop || s_iters >= s_maxits || !(r2 == r2)) s_ru = 2;
      else s_ru = r2 < s_delta2*s_maxr2 ? 1 : 0;
      s_stop_loop = s_ru != 0;       // the host takes the update, then p
    }
    __syncthreads();
    if(s_stop_loop) break;
    // p = r + beta p
    {
      const float beta = (float)s_beta;
      for(size_t t = (size_t)blockIdx.x*kThreads + threadIdx.x; t < total; t += (size_t)gridDim.x*kThreads) {
        Cx<float> pv[12], rv[12];
        SpinorIO<QLLG_F32,12>::load(a.p, total, t, pv);
        SpinorIO<QLLG_F32,12>::load(a.r, total, t, rv);
#pragma unroll
        for(int c=0; c<12; c++) { pv[c].r = fmaf(beta, pv[c].r, rv[c].r); pv[c].i = fmaf(beta, pv[c].i, rv[c].i); }
        SpinorIO<QLLG_F32,12>::store(a.p, total, t, pv);
      }
    }
    if(!wcg_barrier(a)) return;
  }
  if(blockIdx.x == 0 && threadIdx.x == 0) {
    qllg_cg_scalars *sc = a.sc;
    sc->rsq[0] = s_rsq; sc->prev[0] = s_prev; sc->alpha[0] = s_beta; sc->pnorm[0] = s_pn;
    sc->iters[0] = s_iters;
    sc->ru[0] = s_ru;
    sc->no_ru = s_ru == 0;
    sc->count += trip;
  }
}

int launch_wcgp(const WcgpArgs &a0, size_t partial_len, int *grid_out)
{
  static int per_sm = 0;
  if(!per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wilson_cgnr_persistent,
                                                                     kThreads, 0),
                       "persistent CGNR occupancy")) return -1;
    if(per_sm < 1) { qllg_set_error("persistent CGNR: no resident block"); return -1; }
  }
  size_t want = ((size_t)a0.g.Vh + kThreads - 1)/kThreads;
  const size_t cap = (size_t)qllg_num_sms()*per_sm;
  if(want > cap) want = cap;
  const int grid = want < 1 ? 1 : (int)want;
  *grid_out = grid;
  if(2*(size_t)grid > partial_len) {
    qllg_set_error("persistent CGNR: the reduction buffer is too small");
    return -1;
  }
  WcgpArgs a = a0;
  void *args[] = {&a};
  return qllg_check_cuda(cudaLaunchCooperativeKernel((const void *)wilson_cgnr_persistent, dim3(grid),
                                                     dim3(kThreads), args, 0, qllg_stream()),
                         "persistent CGNR launch") || qllg_launched("wilson_cgnr_persistent launch");
}

// Small one-rhs launches split by direction: a block is 64 sites and two
// halves of two warps; half 0 takes the x and y hops (slots 0-3), half 1
// the z and t hops (slots 4-7), each with wilson_dslash's arithmetic, and
// half 1 hands its partial sums to half 0 through shared memory, which adds
// them and finishes the site.  Twice the threads of the one-thread kernel
// with no repeated work (the FP64 launches are bound by the FP64 pipe, so
// the three-threads-per-colour form, which repeats the spin projections,
// is slower).  The two partial sums are added at the end, so the result
// differs from the one-thread kernel's in rounding only.
constexpr int kDir2Threads = 128;

template <int PS, int PL>
__global__ void __launch_bounds__(kDir2Threads, 3)
wilson_dslash_dir2(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  constexpr int SB = kDir2Threads/2;            // sites a block
  __shared__ double shm[2*kDir2Threads];
  __shared__ T part[24][SB];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  const int half = threadIdx.x / SB, ls = threadIdx.x % SB;
  Acc<T> acc0, acc1;
  const bool act = !a.active || (a.active[0] && (!a.active_eq || a.active[0] == a.active_eq));
  const T ca = (T)(a.a ? a.a[0] : a.a0);
  const T cb = (T)a.b;
  if(!skip && act) {
    for(size_t base = (size_t)blockIdx.x*SB; base < total; base += (size_t)gridDim.x*SB) {
      const size_t t = base + ls;
      const bool valid = t < total;
      Cx<T> acc[12], self[12];
#pragma unroll
      for(int c=0; c<12; c++) { acc[c].r = 0; acc[c].i = 0; }
      auto hops = [&](auto mu0) {
        constexpr int M0 = decltype(mu0)::value;
        int x[4];
        site_coords(G, p, (int)t, x);
#pragma unroll
        for(int mu=M0; mu<M0+2; mu++) {
#pragma unroll
          for(int back=0; back<2; back++) {
            const int sgn = (back ? 1 : -1)*(a.dag ? -1 : 1);
            const int k = nbr_index(G, x, mu, back ? -1 : 1);
            Cx<T> U[9], f[12];
            LinkIO<PL>::load(a.links, 2*mu + back, V, loff + t, a.lscale, U);
            SpinorIO<PS,12>::load(a.in, total, (size_t)k, f);
#pragma unroll
            for(int hk=0; hk<2; hk++) {
              const int col = gcol(mu, hk);
              const int ph = gph(mu, hk) + (sgn < 0 ? 2 : 0);
              Cx<T> h[3], tt[3];
#pragma unroll
              for(int c=0; c<3; c++) {
                Cx<T> y = phase(f[3*col + c], ph);
                h[c].r = f[3*hk + c].r + y.r; h[c].i = f[3*hk + c].i + y.i;
                tt[c].r = 0; tt[c].i = 0;
              }
#pragma unroll
              for(int l=0; l<3; l++) {
#pragma unroll
                for(int j=0; j<3; j++) cmac(tt[j], U[3*l + j], h[l]);
              }
#pragma unroll
              for(int c=0; c<3; c++) { acc[3*hk + c].r -= tt[c].r; acc[3*hk + c].i -= tt[c].i; }
#pragma unroll
              for(int ar=2; ar<4; ar++) {
                if(gcol(mu, ar) == hk) {
                  const int pa = gph(mu, ar) + (sgn < 0 ? 0 : 2);
#pragma unroll
                  for(int c=0; c<3; c++) {
                    Cx<T> y = phase(tt[c], pa);
                    acc[3*ar + c].r += y.r; acc[3*ar + c].i += y.i;
                  }
                }
              }
            }
          }
        }
      };
      if(valid) {
        if(half == 0) hops(std::integral_constant<int, 0>());
        else hops(std::integral_constant<int, 2>());
      }
      if(half == 1 && valid) {
#pragma unroll
        for(int c=0; c<12; c++) { part[2*c][ls] = acc[c].r; part[2*c + 1][ls] = acc[c].i; }
      }
      __syncthreads();
      if(half == 0 && valid) {
        if(a.self) SpinorIO<PS,12>::load(a.self, total, t, self);
        Cx<T> out[12];
#pragma unroll
        for(int c=0; c<12; c++) {
          Cx<T> s;
          s.r = acc[c].r + part[2*c][ls]; s.i = acc[c].i + part[2*c + 1][ls];
          if(a.mode == 1) {
            s.r = kfma(ca, self[c].r, s.r); s.i = kfma(ca, self[c].i, s.i);
            out[c] = s;
          } else if(a.mode == 2) {
            T sr = a.self ? ca*self[c].r : (T)0, si = a.self ? ca*self[c].i : (T)0;
            out[c].r = kfma(cb, s.r, sr); out[c].i = kfma(cb, s.i, si);
          } else out[c] = s;
        }
        SpinorIO<PS,12>::store(a.out, total, t, out);
        if(a.norm_out) acc0.norm(out);
        if(a.norm_self && a.self) acc1.norm(self);
      }
      __syncthreads();
    }
  }
  double red[2] = {acc0.get(), acc1.get()};
  if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce<2>(red, 1, 0, a.partial, a.counter, shm, res);
  }
}

// one component of a spinor, one row of a link (the layouts of SpinorIO and
// LinkIO: component-major spinors, [slot][9][V] links, entry 3*col + row)
template <int P, typename T>
__device__ __forceinline__ Cx<T> comp_load(const void *b, size_t stride, size_t idx, int c)
{
  Cx<T> z;
  if constexpr (P == QLLG_F64) {
    const double2 t = __ldg((const double2 *)b + c*stride + idx); z.r = (T)t.x; z.i = (T)t.y;
  } else if constexpr (P == QLLG_DF) {
    const float4 t = __ldg((const float4 *)b + c*stride + idx); z.r = dfl(t.x, t.y); z.i = dfl(t.z, t.w);
  } else {
    const float2 t = __ldg((const float2 *)b + c*stride + idx); z.r = (T)t.x; z.i = (T)t.y;
  }
  return z;
}
template <int P, typename T>
__device__ __forceinline__ void comp_store(void *b, size_t stride, size_t idx, int c, const Cx<T> &z)
{
  if constexpr (P == QLLG_F64) ((double2 *)b)[c*stride + idx] = make_double2((double)z.r, (double)z.i);
  else if constexpr (P == QLLG_DF) ((float4 *)b)[c*stride + idx] = make_float4(z.r.h, z.r.l, z.i.h, z.i.l);
  else ((float2 *)b)[c*stride + idx] = make_float2((float)z.r, (float)z.i);
}

// Small launches (one rhs, fewer sites than the GPU holds threads): three
// threads per site, one per output colour j.  Each loads the neighbour
// spinor (the three share it through L1), projects it, and applies row j
// of the link only, so the launch has three times the threads at a third
// of the registers.  The per-thread arithmetic follows wilson_dslash (the
// same projector, phase and reconstruction), restricted to colour j.
template <int PS, int PL>
__global__ void __launch_bounds__(kThreads)
wilson_dslash_c3(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  __shared__ double shm[2*kThreads];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh;                  // one rhs
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  Acc<T> acc0, acc1;
  const bool act = !a.active || (a.active[0] && (!a.active_eq || a.active[0] == a.active_eq));
  const T ca = (T)(a.a ? a.a[0] : a.a0);
  const T cb = (T)a.b;
  if(!skip && act) {
    for(size_t w = (size_t)blockIdx.x*blockDim.x + threadIdx.x; w < 3*total;
        w += (size_t)gridDim.x*blockDim.x) {
      const int site = (int)(w / 3), j = (int)(w % 3);
      int x[4];
      site_coords(G, p, site, x);
      Cx<T> acc[4], self[4];
#pragma unroll
      for(int sp=0; sp<4; sp++) {
        if(a.self && a.mode == 1) {
          self[sp] = comp_load<PS,T>(a.self, total, site, 3*sp + j);
          acc[sp].r = ca*self[sp].r; acc[sp].i = ca*self[sp].i;
        } else {
          acc[sp].r = 0; acc[sp].i = 0;
        }
      }
#pragma unroll
      for(int mu=0; mu<4; mu++) {
#pragma unroll
        for(int back=0; back<2; back++) {
          const int sgn = (back ? 1 : -1)*(a.dag ? -1 : 1);
          const int k = nbr_index(G, x, mu, back ? -1 : 1);
          const int slot = 2*mu + back;
          Cx<T> Ur[3], f[12];
#pragma unroll
          for(int l=0; l<3; l++)
            Ur[l] = comp_load<PL,T>(a.links, 0, (size_t)(slot*9 + 3*l + j)*V + loff + site, 0);
          SpinorIO<PS,12>::load(a.in, total, (size_t)k, f);
#pragma unroll
          for(int hk=0; hk<2; hk++) {
            const int col = gcol(mu, hk);
            const int ph = gph(mu, hk) + (sgn < 0 ? 2 : 0);
            Cx<T> h[3], tt;
#pragma unroll
            for(int c=0; c<3; c++) {
              Cx<T> y = phase(f[3*col + c], ph);
              h[c].r = f[3*hk + c].r + y.r; h[c].i = f[3*hk + c].i + y.i;
            }
            tt.r = 0; tt.i = 0;
#pragma unroll
            for(int l=0; l<3; l++) cmac(tt, Ur[l], h[l]);
            acc[hk].r -= tt.r; acc[hk].i -= tt.i;
#pragma unroll
            for(int ar=2; ar<4; ar++) {
              if(gcol(mu, ar) == hk) {
                const int pa = gph(mu, ar) + (sgn < 0 ? 0 : 2);
                Cx<T> y = phase(tt, pa);
                acc[ar].r += y.r; acc[ar].i += y.i;
              }
            }
          }
        }
      }
      if(a.self && a.mode != 1) {
#pragma unroll
        for(int sp=0; sp<4; sp++) self[sp] = comp_load<PS,T>(a.self, total, site, 3*sp + j);
      }
      Cx<T> out[4];
#pragma unroll
      for(int sp=0; sp<4; sp++) {
        if(a.mode == 2) {
          T sr = a.self ? ca*self[sp].r : (T)0, si = a.self ? ca*self[sp].i : (T)0;
          out[sp].r = kfma(cb, acc[sp].r, sr); out[sp].i = kfma(cb, acc[sp].i, si);
        } else out[sp] = acc[sp];
        comp_store<PS,T>(a.out, total, site, 3*sp + j, out[sp]);
      }
      if(a.norm_out) acc0.norm(out);
      if(a.norm_self && a.self) acc1.norm(self);
    }
  }
  double red[2] = {acc0.get(), acc1.get()};
  if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce<2>(red, 1, 0, a.partial, a.counter, shm, res);
  }
}

template <int PS, int PL>
int launch_c3(const qllg_stag_args *a)
{
  static int bps = 0;
  if(!bps) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &bps, wilson_dslash_c3<PS,PL>, kThreads, 0), "occupancy")) return -1;
    if(bps < 1) bps = 1;
  }
  size_t need = (3*(size_t)a->g.Vh + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*bps;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  wilson_dslash_c3<PS,PL><<<grid, kThreads, 0, qllg_stream()>>>(A);
  return qllg_launched("wilson_dslash_c3 launch");
}

template <int PS, int PL>
int launch_dir2(const qllg_stag_args *a)
{
  static int bps = 0;
  if(!bps) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &bps, wilson_dslash_dir2<PS,PL>, kDir2Threads, 0), "occupancy")) return -1;
    if(bps < 1) bps = 1;
  }
  size_t need = ((size_t)a->g.Vh + kDir2Threads/2 - 1)/(kDir2Threads/2);
  size_t maxg = (size_t)qllg_num_sms()*bps;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  wilson_dslash_dir2<PS,PL><<<grid, kDir2Threads, 0, qllg_stream()>>>(A);
  return qllg_launched("wilson_dslash_dir2 launch");
}

// mode 4: the FP32 one-rhs kernel with the fused CG update
int launch_upd(const qllg_stag_args *a)
{
  static int bps = 0;
  if(!bps) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &bps, wilson_dslash_upd, kThreads, 0), "occupancy")) return -1;
    if(bps < 1) bps = 1;
  }
  size_t need = ((size_t)a->g.Vh + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*bps;
  if(maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb->partial;
  A.counter = a->rb->counter;
  wilson_dslash_upd<<<grid, kThreads, 0, qllg_stream()>>>(A);
  return qllg_launched("wilson_dslash launch");
}

template <int PS, int PL, int NR>
int launch_t(const qllg_stag_args *a)
{
  // one rhs in FP64, fewer sites than the GPU's resident threads: two
  // threads per site, split by direction
  if(a->mode == 4 && (PS != QLLG_F32 || PL != QLLG_F32 || NR != 1 || !a->rb || !a->sc || !a->x || !a->r ||
                     !a->pvec)) {
    qllg_set_error("wilson_dslash: the fused CG update (mode 4) takes FP32, a reduction workspace and x, r, p");
    return -1;
  }
  if constexpr (NR == 1 && ((PS == QLLG_F64 && PL == QLLG_F64) || (PS == QLLG_F32 && PL == QLLG_F32))) {
    if(a->mode != 4 && qllg_get_param(PS == QLLG_F64 ? "wilson_f64_dir2" : "wilson_f32_dir2") != 0 &&
       (size_t)a->g.Vh < (size_t)qllg_num_sms()*1024)
      return launch_dir2<PS,PL>(a);
  }
  // one rhs, fewer sites than half the GPU's resident threads: three
  // threads per site (FP32 on request; double-float by default, whose
  // one-thread kernel holds one block of 256 threads per SM)
  if constexpr (NR == 1 && (PS == QLLG_F32 || PS == QLLG_DF || PS == QLLG_F64)) {
    const char *knob = PS == QLLG_DF ? "wilson_df_c3" : PS == QLLG_F64 ? "wilson_f64_c3" : "wilson_c3";
    if(a->mode != 4 && qllg_get_param(knob) != 0 && (size_t)a->g.Vh < (size_t)qllg_num_sms()*1024)
      return launch_c3<PS,PL>(a);
  }
  if constexpr (PS == QLLG_F32 && PL == QLLG_F32 && NR == 1)
    if(a->mode == 4) return launch_upd(a);
  static int bps = 0;
  if(!bps) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &bps, wilson_dslash<PS,PL,NR>, kThreads, 0), "occupancy")) return -1;
    if(bps < 1) bps = 1;
  }
  size_t total = (size_t)a->g.Vh * NR;
  size_t need = (total + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*bps;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  wilson_dslash<PS,PL,NR><<<grid, kThreads, 0, qllg_stream()>>>(A);
  return qllg_launched("wilson_dslash launch");
}

template <int PS, int PL>
int launch_nr(const qllg_stag_args *a)
{
  switch(a->nrhs) {
  case 1: return launch_t<PS,PL,1>(a);
  case 2: return launch_t<PS,PL,2>(a);
  case 4: return launch_t<PS,PL,4>(a);
  }
  qllg_set_error("wilson_dslash: nrhs %d not in {1,2,4}", a->nrhs);
  return -1;
}

} // namespace

extern "C" int
qllg_k_wilson_cgnr_persistent(const qllg_wcgp_args *h, int *grid_out)
{
  WcgpArgs a;
  memset(&a, 0, sizeof(a));
  a.g = h->g;
  a.links = h->links;
  a.x = h->x; a.r = h->r; a.p = h->p; a.Sp = h->Sp; a.v = h->v;
  a.sc = h->sc;
  a.a = h->a;
  a.partial = h->partial;
  a.bar = h->bar;
  a.err = h->err;
  a.poll_limit = h->poll_limit;
  a.extra = h->extra;
  a.trips = h->trips;
  return launch_wcgp(a, h->partial_len, grid_out);
}

extern "C" int
qllg_k_wilson_dslash(int ps, int pl, const qllg_stag_args *a)
{
  if((a->norm_out || a->norm_self) && !a->rb) {
    qllg_set_error("wilson_dslash: reduction requested without workspace");
    return -1;
  }
  if(ps == QLLG_F64 && pl == QLLG_F64) return launch_nr<QLLG_F64, QLLG_F64>(a);
  if(ps == QLLG_F32 && pl == QLLG_F32) return launch_nr<QLLG_F32, QLLG_F32>(a);
  // double-float (the reliable updates of the mixed CGNR): one rhs
  if(ps == QLLG_DF && pl == QLLG_DF && a->nrhs == 1) return launch_t<QLLG_DF, QLLG_DF, 1>(a);
  qllg_set_error("wilson_dslash: unsupported precision pair %d/%d (%d rhs)", ps, pl, a->nrhs);
  return -1;
}
