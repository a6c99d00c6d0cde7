// k_cgp.cu -- the persistent CG: one cooperative launch runs every
// iteration of a solve on a small lattice, where the multi-launch loop is
// bound by launch latency (8^4 is 2,048 even sites: a half Dslash there is
// a few microseconds of work against a few microseconds per launch).
//
// The iteration is cgSolveT's scaled form (lib/cg.c:77-115), as in the
// multi-launch solver (stag.c: cg_iteration): p += r/|r|^2 with |p|^2;
// v = D_oe p with |v|^2; Ap = m^2 p - D_eo v, a = 1/(m^2|p|^2 + |v|^2),
// x += a p, r -= a Ap with |r|^2.  In the mixed mode the iterations run on
// FP32 vectors and links and a right-hand side whose |r| fell by delta
// since its last reliable update (or that passed its target, hit maxits or
// is not a number) takes one: x64 += x, r64 = b - A x64 in FP64, r = r64,
// then p is re-orthogonalised to r (k_mixed.cu's kernels, in one pass).
//
// Every block runs the whole loop.  Each reduction writes one partial per
// block and quantity, a grid barrier follows, and every block then folds
// the partials in block order itself, so all blocks hold bitwise the same
// scalars without a second barrier.  Partials alternate between two
// buffers: a block can run at most one reduction ahead of another.
//
// The grid barrier is a counter and a generation word with bounded waits:
// a block that waits more than poll_limit polls (about a second by
// default) sets the error word and returns, and so, at their next
// barrier, do all the others; the host reports the error and the context
// stays usable.
#include "k_stag.cuh"

namespace {

constexpr int kPT = 256;          // threads per block
constexpr int kQmax = 2;          // reduced quantities per phase

struct CgpArgs {
  qllg_geom g;
  int nslots, fb, mixed, reortho;
  const void *links;              // links of the iterations: FP64, or FP32 (mixed)
  const void *links64;            // FP64 links of the reliable updates (mixed)
  const float *lscale;
  void *x, *r, *p, *v;            // iteration vectors (FP64, or FP32 when mixed)
  void *v2;                       // the second p buffer
  void *x64, *r64, *w64;          // mixed: FP64 solution, residual, odd temporary
  const void *b;                  // FP64 source
  qllg_cg_scalars *sc;
  double *partial;                // [2][gridDim][kQmax][QLLG_MAXRHS]
  unsigned *bar;                  // [0] arrivals, [1] generation
  int *err;                       // 1: a barrier wait ran out
  long long poll_limit;
  int extra;                      // barrier arrivals expected beyond the grid (tests)
  int trips;                      // iteration cap of this launch
};

// the block's view of the solver scalars (shared memory)
struct Sc {
  double rsq[QLLG_MAXRHS], stop[QLLG_MAXRHS], m2[QLLG_MAXRHS], maxr2[QLLG_MAXRHS];
  double pn[QLLG_MAXRHS], vn[QLLG_MAXRHS], red[kQmax][QLLG_MAXRHS];
  double delta2;
  int act[QLLG_MAXRHS], iters[QLLG_MAXRHS], ru[QLLG_MAXRHS], nru[QLLG_MAXRHS];
  int maxits, any, anyru, failed;
};

__device__ bool grid_barrier(const CgpArgs &a)
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

// per-rhs sums of Q quantities over the grid: each thread holds val[q]
// for its rhs ((threadIdx.x/4) % NR); the block folds them per rhs in
// thread order, writes one partial per (quantity, rhs), and after the
// barrier every block folds the partials of all blocks in block order into
// s.red.  false: a barrier wait ran out.
template <int Q, int NR>
__device__ bool grid_sum(const CgpArgs &a, Sc &s, const double (&val)[Q], int &phase)
{
  __shared__ double buf[Q][kPT];
#pragma unroll
  for(int q=0; q<Q; q++) buf[q][threadIdx.x] = val[q];
  __syncthreads();
  // block fold, a fixed tree: threads t and t + w hold the same rhs while
  // w is a multiple of 4*NR; the last four entries of a rhs are its lanes
  for(int w = kPT/2; w >= 4*NR; w >>= 1) {
    if(threadIdx.x < w) {
#pragma unroll
      for(int q=0; q<Q; q++) buf[q][threadIdx.x] += buf[q][threadIdx.x + w];
    }
    __syncthreads();
  }
  double *part = a.partial + (size_t)(phase & 1)*gridDim.x*kQmax*QLLG_MAXRHS;
  if(threadIdx.x < Q*NR) {
    const int q = threadIdx.x / NR, r = threadIdx.x % NR;
    const double t = (buf[q][4*r] + buf[q][4*r + 1]) + (buf[q][4*r + 2] + buf[q][4*r + 3]);
    part[((size_t)blockIdx.x*kQmax + q)*QLLG_MAXRHS + r] = t;
  }
  phase++;
  if(!grid_barrier(a)) return false;
  // fold of the blocks' partials: warp k takes the sums k, k + 8, ...; its
  // lanes read blocks lane, lane + 32, ... in order and a butterfly adds
  // the lanes, the same fixed order in every block
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for(int c = warp; c < Q*NR; c += kPT/32) {
    const int q = c / NR, r = c % NR;
    double t = 0;
    for(int b = lane; b < (int)gridDim.x; b += 32)
      t += ((volatile double *)part)[((size_t)b*kQmax + q)*QLLG_MAXRHS + r];
#pragma unroll
    for(int o=16; o>0; o>>=1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if(lane == 0) s.red[q][r] = t;
  }
  __syncthreads();
  return true;
}

// The hop sum of one (site, rhs) item on four lanes of a warp, lane mu
// taking the four slots of direction mu, then a butterfly over the four
// lanes: every lane ends with the full sum.  The input of the slots is
// in + beta*add (add NULL: in alone), formed at each neighbour as it is
// loaded, so that a p update needs no pass (and no barrier) of its own.
template <int PL, typename T, int NR>
__device__ __forceinline__ void hop_sum4(const qllg_stag_args &sa, const Geo &G, int p, int site, int rhs,
                                         const void *in, const void *add, T beta, Cx<T> acc[3])
{
  constexpr int PS = std::is_same<T, double>::value ? QLLG_F64 : QLLG_F32;
  const size_t V = (size_t)sa.g.V, total = (size_t)G.Vh*NR;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const int mu = threadIdx.x & 3;
  int x[4];
  site_coords(G, p, site, x);
#pragma unroll
  for(int c=0; c<3; c++) { acc[c].r = 0; acc[c].i = 0; }
#pragma unroll
  for(int back=0; back<2; back++) {
#pragma unroll
    for(int nk=0; nk<2; nk++) {
      if(nk && sa.nslots != 16) continue;
      const int d = (nk ? 3 : 1)*(back ? -1 : 1);
      const int k = nbr_index(G, x, mu, d);
      Cx<T> U[9], v[3];
      if(sa.nslots == 16)
        slot_link<PL,16>(sa, mu, back, nk, V, (size_t)G.Vh, loff, (size_t)site, (size_t)k, U);
      else
        slot_link<PL,8>(sa, mu, back, 0, V, (size_t)G.Vh, loff, (size_t)site, (size_t)k, U);
      SpinorIO<PS,3>::load(in, total, (size_t)k*NR + rhs, v);
      if(add) {
        Cx<T> w[3];
        SpinorIO<PS,3>::load(add, total, (size_t)k*NR + rhs, w);
#pragma unroll
        for(int c=0; c<3; c++) { v[c].r = fma(beta, w[c].r, v[c].r); v[c].i = fma(beta, w[c].i, v[c].i); }
      }
#pragma unroll
      for(int l=0; l<3; l++) {
#pragma unroll
        for(int j=0; j<3; j++) cmac(acc[j], U[3*l + j], v[l]);
      }
    }
  }
#pragma unroll
  for(int c=0; c<3; c++) {
#pragma unroll
    for(int o=1; o<4; o<<=1) {
      acc[c].r += __shfl_xor_sync(0xffffffffu, acc[c].r, o);
      acc[c].i += __shfl_xor_sync(0xffffffffu, acc[c].i, o);
    }
  }
}

// Items are (site, rhs) pairs, rhs fastest, four lanes each; a warp holds
// eight consecutive items and the grid stride is a multiple of eight, so a
// warp runs its loop trips together (the butterflies need every lane).
#define ITEM_LOOP(item, valid, n)                                                              \
  const size_t n##_round = ((size_t)(n) + 7)/8*8;                                              \
  for(size_t item##_ = ((size_t)blockIdx.x*kPT + threadIdx.x) >> 2; item##_ < n##_round;       \
      item##_ += ((size_t)gridDim.x*kPT) >> 2)                                                 \
    for(bool valid = item##_ < (size_t)(n), once_ = true; once_; once_ = false)                \
      for(size_t item = valid ? item##_ : (size_t)(n) - 1, once2_ = 1; once2_; once2_ = 0)

template <int NR, bool MIXED>
__global__ void __launch_bounds__(kPT)
cg_persistent(CgpArgs a)
{
  typedef typename std::conditional<MIXED, float, double>::type T;
  constexpr int P = MIXED ? QLLG_F32 : QLLG_F64;
  constexpr int PL = MIXED ? QLLG_F32 : QLLG_F64;
  __shared__ Sc s;
  const Geo G = make_geo(a.g);
  const size_t total = (size_t)G.Vh*NR;
  const int rhs = (threadIdx.x >> 2) % NR;
  const bool lead = (threadIdx.x & 3) == 0;
  qllg_stag_args sa;
  memset(&sa, 0, sizeof(sa));
  sa.g = a.g;
  sa.nslots = a.nslots;
  sa.fb = a.fb;
  sa.links = a.links;
  sa.lscale = a.lscale;
  qllg_stag_args sa64 = sa;
  sa64.links = a.links64;
  if(threadIdx.x == 0) {
    for(int q=0; q<NR; q++) {
      s.rsq[q] = a.sc->rsq[q]; s.stop[q] = a.sc->rsq_stop[q]; s.m2[q] = a.sc->mass2[q];
      s.maxr2[q] = a.sc->maxr2[q]; s.act[q] = a.sc->active[q]; s.iters[q] = a.sc->iters[q];
      s.nru[q] = a.sc->nru[q]; s.ru[q] = 0; s.pn[q] = 0; s.vn[q] = 0;
    }
    s.delta2 = a.sc->delta2;
    s.maxits = a.sc->maxits;
    s.failed = 0;
  }
  __syncthreads();
  // p is double-buffered: the p update of an iteration writes the other
  // buffer while the hop sums read the current one at the neighbours
  void *pb[2] = {a.p, a.v2};
  int cur = 0;
  int phase = 0, trip = 0;
  for(;;) {
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) any |= s.act[q];
      s.any = any;
    }
    __syncthreads();
    if(!s.any || trip >= a.trips) break;
    trip++;
    const bool act = s.act[rhs] != 0;
    void *pc = pb[cur], *pn = pb[cur ^ 1];
    const T beta = act ? (T)(1.0/s.rsq[rhs]) : (T)0;
    // p' = p + r/|r|^2 with |p'|^2 (even sites), and v = D_oe p' with |v|^2
    // (odd sites), p' formed at each neighbour from p and r
    {
      Acc<T> accp, accv;
      {
        // every lane of a warp runs every trip (the butterflies need them
        // all); the rhs that are done only skip their stores
        ITEM_LOOP(t, valid, total) {
          if(lead && valid && act) {
            Cx<T> pv[3], rv[3];
            SpinorIO<P,3>::load(pc, total, t, pv);
            SpinorIO<P,3>::load(a.r, total, t, rv);
#pragma unroll
            for(int c=0; c<3; c++) { pv[c].r = fma(beta, rv[c].r, pv[c].r); pv[c].i = fma(beta, rv[c].i, pv[c].i); }
            SpinorIO<P,3>::store(pn, total, t, pv);
            accp.norm(pv);
          }
          Cx<T> o[3];
          hop_sum4<PL,T,NR>(sa, G, 1, (int)(t/NR), rhs, pc, a.r, beta, o);
          if(lead && valid && act) {
            SpinorIO<P,3>::store(a.v, total, t, o);
            accv.norm(o);
          }
        }
      }
      const double val[2] = {accp.get(), accv.get()};
      if(!grid_sum<2,NR>(a, s, val, phase)) return;
      if(threadIdx.x < NR) { s.pn[threadIdx.x] = s.red[0][threadIdx.x]; s.vn[threadIdx.x] = s.red[1][threadIdx.x]; }
      __syncthreads();
    }
    cur ^= 1;
    pc = pb[cur];
    // Ap = m^2 p - D_eo v; x += a p, r -= a Ap with |r|^2
    {
      Acc<T> acc;
      {
        const T alpha = act ? (T)(1.0/(s.m2[rhs]*s.pn[rhs] + s.vn[rhs])) : (T)0;
        const T ca = (T)s.m2[rhs];
        ITEM_LOOP(t, valid, total) {
          Cx<T> hs[3];
          hop_sum4<PL,T,NR>(sa, G, 0, (int)(t/NR), rhs, a.v, NULL, (T)0, hs);
          if(lead && valid && act) {
            Cx<T> pv[3], xv[3], rv[3];
            SpinorIO<P,3>::load(pc, total, t, pv);
            SpinorIO<P,3>::load(a.x, total, t, xv);
            SpinorIO<P,3>::load(a.r, total, t, rv);
#pragma unroll
            for(int c=0; c<3; c++) {
              T apr = fma((T)-1, hs[c].r, ca*pv[c].r), api = fma((T)-1, hs[c].i, ca*pv[c].i);
              xv[c].r = fma(alpha, pv[c].r, xv[c].r); xv[c].i = fma(alpha, pv[c].i, xv[c].i);
              rv[c].r = fma(-alpha, apr, rv[c].r); rv[c].i = fma(-alpha, api, rv[c].i);
            }
            SpinorIO<P,3>::store(a.x, total, t, xv);
            SpinorIO<P,3>::store(a.r, total, t, rv);
            acc.norm(rv);
          }
        }
      }
      const double val[1] = {acc.get()};
      if(!grid_sum<1,NR>(a, s, val, phase)) return;
      if(threadIdx.x == 0) {
        int anyru = 0;
        for(int q=0; q<NR; q++) {
          s.ru[q] = 0;
          if(!s.act[q]) continue;
          const double r2 = s.red[0][q];
          s.iters[q]++;
          s.rsq[q] = r2;
          if(MIXED) {
            if(r2 < s.stop[q] || s.iters[q] >= s.maxits || !(r2 == r2)) s.ru[q] = 2;
            else if(r2 < s.delta2*s.maxr2[q]) s.ru[q] = 1;
            anyru |= s.ru[q];
          } else if(!(r2 >= s.stop[q] && s.iters[q] < s.maxits)) {
            s.act[q] = 0;
          }
        }
        s.anyru = anyru;
      }
      __syncthreads();
    }
    if(!MIXED || !s.anyru) continue;
    // reliable update of the flagged rhs: x64 += x, x = 0
    const bool fl = s.ru[rhs] != 0;
    if(fl) {
      ITEM_LOOP(t, valid, total) {
        if(lead && valid) {
          Cx<double> xv[3];
          Cx<float> sv[3], z[3];
          SpinorIO<QLLG_F64,3>::load(a.x64, total, t, xv);
          SpinorIO<QLLG_F32,3>::load(a.x, total, t, sv);
#pragma unroll
          for(int c=0; c<3; c++) { xv[c].r += sv[c].r; xv[c].i += sv[c].i; z[c].r = 0; z[c].i = 0; }
          SpinorIO<QLLG_F64,3>::store(a.x64, total, t, xv);
          SpinorIO<QLLG_F32,3>::store(a.x, total, t, z);
        }
      }
    }
    if(!grid_barrier(a)) return;
    // w64 = D_oe x64 (FP64)
    {
      ITEM_LOOP(t, valid, total) {
        Cx<double> o[3];
        hop_sum4<QLLG_F64,double,NR>(sa64, G, 1, (int)(t/NR), rhs, a.x64, NULL, 0.0, o);
        if(lead && valid && fl) SpinorIO<QLLG_F64,3>::store(a.w64, total, t, o);
      }
    }
    if(!grid_barrier(a)) return;
    // r64 = b - (m^2 x64 - D_eo w64), r = r64 in FP32, |r64|^2
    {
      double r2 = 0;
      {
        const double m2 = s.m2[rhs];
        ITEM_LOOP(t, valid, total) {
          Cx<double> hs[3];
          hop_sum4<QLLG_F64,double,NR>(sa64, G, 0, (int)(t/NR), rhs, a.w64, NULL, 0.0, hs);
          if(lead && valid && fl) {
            Cx<double> xv[3], bv[3];
            Cx<float> f[3];
            SpinorIO<QLLG_F64,3>::load(a.x64, total, t, xv);
            SpinorIO<QLLG_F64,3>::load(a.b, total, t, bv);
#pragma unroll
            for(int c=0; c<3; c++) {
              const double tr = fma(-1.0, hs[c].r, m2*xv[c].r), ti = fma(-1.0, hs[c].i, m2*xv[c].i);
              bv[c].r = bv[c].r - tr; bv[c].i = bv[c].i - ti;
              r2 += bv[c].r*bv[c].r + bv[c].i*bv[c].i;
              f[c].r = (float)bv[c].r; f[c].i = (float)bv[c].i;
            }
            SpinorIO<QLLG_F64,3>::store(a.r64, total, t, bv);
            SpinorIO<QLLG_F32,3>::store(a.r, total, t, f);
          }
        }
      }
      const double val[1] = {r2};
      if(!grid_sum<1,NR>(a, s, val, phase)) return;
      if(threadIdx.x == 0) {
        for(int q=0; q<NR; q++) {
          if(!s.ru[q]) continue;
          const double rr = s.red[0][q];
          s.rsq[q] = rr;
          s.maxr2[q] = rr;
          s.nru[q]++;
          if(!(rr >= s.stop[q] && s.iters[q] < s.maxits)) s.act[q] = 0;
        }
      }
      __syncthreads();
    }
    if(!a.reortho) continue;
    // p -= (<r,p>/|r|^2) r for the flagged rhs (FP32, as mcg_orth_dot_k and
    // mcg_orth_axpy_k), on the current p buffer
    {
      Acc<float> are, aim;
      if(fl) {
        ITEM_LOOP(t, valid, total) {
          if(lead && valid) {
            Cx<float> pv[3], rv[3];
            SpinorIO<QLLG_F32,3>::load(pc, total, t, pv);
            SpinorIO<QLLG_F32,3>::load(a.r, total, t, rv);
            float re = 0, im = 0;
#pragma unroll
            for(int c=0; c<3; c++) {
              re = fmaf(rv[c].r, pv[c].r, re); re = fmaf(rv[c].i, pv[c].i, re);
              im = fmaf(rv[c].r, pv[c].i, im); im = fmaf(-rv[c].i, pv[c].r, im);
            }
            are.add(re);
            aim.add(im);
          }
        }
      }
      const double val[2] = {are.get(), aim.get()};
      if(!grid_sum<2,NR>(a, s, val, phase)) return;
      if(fl) {
        const double r2 = s.rsq[rhs];
        const float cr = (float)(r2 > 0 ? s.red[0][rhs]/r2 : 0);
        const float ci = (float)(r2 > 0 ? s.red[1][rhs]/r2 : 0);
        ITEM_LOOP(t, valid, total) {
          if(lead && valid) {
            Cx<float> pv[3], rv[3];
            SpinorIO<QLLG_F32,3>::load(pc, total, t, pv);
            SpinorIO<QLLG_F32,3>::load(a.r, total, t, rv);
#pragma unroll
            for(int c=0; c<3; c++) {
              pv[c].r -= cr*rv[c].r - ci*rv[c].i;
              pv[c].i -= cr*rv[c].i + ci*rv[c].r;
            }
            SpinorIO<QLLG_F32,3>::store(pc, total, t, pv);
          }
        }
      }
    }
  }
  // the current p back where the caller keeps it (the double buffer may
  // end on the other one); the scalars to the host's struct (every block
  // holds the same)
  if(cur) {
    // every block's last p writes (a re-orthogonalisation ends without a
    // barrier) before any block copies
    if(!grid_barrier(a)) return;
    for(size_t t = (size_t)blockIdx.x*kPT + threadIdx.x; t < total; t += (size_t)gridDim.x*kPT) {
      Cx<T> pv[3];
      SpinorIO<P,3>::load(pb[1], total, t, pv);
      SpinorIO<P,3>::store(pb[0], total, t, pv);
    }
  }
  if(blockIdx.x == 0 && threadIdx.x == 0) {
    int any = 0;
    for(int q=0; q<NR; q++) {
      a.sc->rsq[q] = s.rsq[q]; a.sc->maxr2[q] = s.maxr2[q]; a.sc->active[q] = s.act[q];
      a.sc->iters[q] = s.iters[q]; a.sc->nru[q] = s.nru[q]; a.sc->pnorm[q] = s.pn[q];
      a.sc->vnorm[q] = s.vn[q];
      any |= s.act[q];
    }
    a.sc->done = !any;
    a.sc->count += trip;
  }
}

template <int NR, bool MIXED>
int launch_cgp(const CgpArgs &a0, int *grid_out)
{
  static int per_sm = 0;
  auto kern = cg_persistent<NR, MIXED>;
  if(!per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPT, 0),
                       "persistent CG occupancy")) return -1;
    if(per_sm < 1) { qllg_set_error("persistent CG: no resident block"); return -1; }
  }
  const size_t total = (size_t)a0.g.Vh*NR;
  size_t want = (4*total + kPT - 1)/kPT;          // four lanes per (site, rhs)
  // few blocks: the barriers and the partial folds cost per block
  const size_t cap = (size_t)qllg_num_sms()*per_sm;
  if(want > cap) want = cap;
  if(want > 128) want = 128;
  const int grid = want < 1 ? 1 : (int)want;
  *grid_out = grid;
  CgpArgs a = a0;
  void *args[] = {&a};
  return qllg_check_cuda(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kPT), args,
                                                     0, qllg_stream()),
                         "persistent CG launch") || qllg_launched("cg_persistent launch");
}

} // namespace

extern "C" int
qllg_k_cg_persistent(const qllg_cgp_args *h, int *grid_out)
{
  CgpArgs a;
  memset(&a, 0, sizeof(a));
  a.g = h->g;
  a.nslots = h->nslots;
  a.fb = h->fb;
  a.mixed = h->mixed;
  a.reortho = h->reortho;
  a.links = h->links;
  a.links64 = h->links64;
  a.lscale = h->lscale;
  a.x = h->x; a.r = h->r; a.p = h->p; a.v = h->v; a.v2 = h->p2;
  a.x64 = h->x64; a.r64 = h->r64; a.w64 = h->w64;
  a.b = h->b;
  a.sc = h->sc;
  a.partial = h->partial;
  a.bar = h->bar;
  a.err = h->err;
  a.poll_limit = h->poll_limit;
  a.extra = h->extra;
  a.trips = h->trips;
  if(h->mixed) {
    switch(h->nrhs) {
    case 1: return launch_cgp<1, true>(a, grid_out);
    case 2: return launch_cgp<2, true>(a, grid_out);
    case 4: return launch_cgp<4, true>(a, grid_out);
    case 8: return launch_cgp<8, true>(a, grid_out);
    case 16: return launch_cgp<16, true>(a, grid_out);
    }
  } else {
    switch(h->nrhs) {
    case 1: return launch_cgp<1, false>(a, grid_out);
    case 2: return launch_cgp<2, false>(a, grid_out);
    case 4: return launch_cgp<4, false>(a, grid_out);
    case 8: return launch_cgp<8, false>(a, grid_out);
    case 16: return launch_cgp<16, false>(a, grid_out);
    }
  }
  qllg_set_error("persistent CG: nrhs %d not in {1,2,4,8,16}", h->nrhs);
  return -1;
}

// bytes of the partial-sum buffer the persistent CG needs for `grid` blocks
extern "C" size_t
qllg_cgp_partial_bytes(int grid)
{
  return sizeof(double)*2*(size_t)grid*kQmax*QLLG_MAXRHS;
}
