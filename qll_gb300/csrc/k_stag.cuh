// k_stag.cuh -- asqtad staggered half-Dslash kernels and their launchers (sm_103a),
// included by one translation unit per precision (k_stag_f64.cu, k_stag_f32.cu,
// k_stag_i16.cu), which are compiled in parallel.
//
// One thread per (output site, right-hand side), rhs fastest, so the nrhs
// threads of a site share every link load (a broadcast from L1) while the
// spinor loads stay coalesced.  Neighbours are computed in-kernel from the
// even-odd lexicographic site order (periodic in every direction), which
// replaces the reference's gather tables (lib/shifts.c:516-736) and halo
// exchange.  The slot order and the per-slot arithmetic follow dslash2T
// (lib/stagDslash.c:316-328) and PeqM3AtimesV3o (lib/vla0.c.lua:193-213):
// slot s = 4*mu + 2*backward + naik, acc += U_s(x) psi(x + d_s).
#pragma once
#include <stdio.h>
#include <type_traits>
#include <cuda.h>                 // CUtensorMap (the encoder is reached through the runtime)
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kThreads = 256;

int qllg_mr_disabled() { return qllg_get_param("dslash_mr") == 0; }

// The link of one slot for output site `site` (parity p).  Double-stored
// operators keep all slots.  Single-stored ones (a.fb, createStaggeredLinksFb)
// keep the forward slots only, [NS/2][9][V], and a backward slot's link
// -U(y)^dagger is made here from the forward link at y = x - mu (or x - 3mu),
// the site whose spinor the slot reads (nb, of the other parity):
// entry 3l+c of -U^dagger is (-re, im) of entry 3c+l of U, so the products
// are bitwise those of the double-stored links (dslashFb2T and
// V_vmeq_xMap_times_xVp, lib/stagDslash.c:110-257, lib/vla.c:1368-1393).
// reconstruct-12 layout: stored slot s (fat, or Naik when NS == 16 and s
// is odd) starts at byte (s/2)*120V + (s&1)*72V (NS == 16) or 72V*s; the
// sign bytes follow all stored slots
__device__ __forceinline__ size_t f32r_base(int NS, int s, size_t V)
{
  return NS == 16 ? ((size_t)(s >> 1)*120 + (s & 1)*72)*V : (size_t)s*72*V;
}

template <int NS>
__device__ __forceinline__ void f32r_link(const qllg_stag_args &a, bool fb, int s, size_t V, size_t site,
                                          Cx<float> U[9])
{
  const char *base = (const char *)a.links + f32r_base(NS, s, V);
  if(NS == 16 && (s & 1)) {
    const int stored = fb ? NS/2 : NS;
    const unsigned char sg = __ldg((const unsigned char *)a.links + f32r_base(NS, stored, V) + site);
    LinkR::naik(base, V, site, (sg >> (s >> 1)) & 1, U);
  } else {
    LinkR::fat(base, V, site, U);
  }
}

// FB: 0 or 1 when the caller knows a.fb at compile time (no branch on it),
// -1 to read it at run time
template <int PL, int NS, int FB = -1, typename T>
__device__ __forceinline__ void slot_link(const qllg_stag_args &a, int mu, int back, int nk,
                                          size_t V, size_t Vh, size_t loff, size_t site, size_t nb,
                                          Cx<T> U[9])
{
  const int slot = (NS == 16) ? (4*mu + 2*back + nk) : (2*mu + back);
  const bool fb = FB < 0 ? a.fb != 0 : FB != 0;
  if constexpr (PL == QLLG_F32R) {
    const int fslot = (NS == 16) ? (2*mu + nk) : mu;
    if(!fb) { f32r_link<NS>(a, fb, slot, V, loff + site, U); return; }
    if(!back) { f32r_link<NS>(a, fb, fslot, V, loff + site, U); return; }
    Cx<T> F[9];
    f32r_link<NS>(a, fb, fslot, V, (Vh - loff) + nb, F);
#pragma unroll
    for(int l=0; l<3; l++)
#pragma unroll
      for(int c=0; c<3; c++) { U[3*l + c].r = -F[3*c + l].r; U[3*l + c].i = F[3*c + l].i; }
  } else {
    if(!fb) {
      LinkIO<PL>::load(a.links, slot, V, loff + site, a.lscale, U);
      return;
    }
    const int fslot = (NS == 16) ? (2*mu + nk) : mu;
    if(!back) {
      LinkIO<PL>::load(a.links, fslot, V, loff + site, a.lscale, U);
      return;
    }
    Cx<T> F[9];
    LinkIO<PL>::load(a.links, fslot, V, (Vh - loff) + nb, a.lscale, F);
#pragma unroll
    for(int l=0; l<3; l++)
#pragma unroll
      for(int c=0; c<3; c++) { U[3*l + c].r = -F[3*c + l].r; U[3*l + c].i = F[3*c + l].i; }
  }
}

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
  Acc<T> acc0, acc1;
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
            const int d = (nk ? 3 : 1)*(back ? -1 : 1);
            const int k = nbr_index(G, x, mu, d);
            Cx<T> U[9], v[3];
            slot_link<PL,NS>(a, mu, back, nk, V, (size_t)G.Vh, loff, (size_t)site, (size_t)k, U);
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
        }
        acc0.norm(rv);
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
      if(a.norm_out) acc0.norm(out);
      if(a.norm_self && a.self) acc1.norm(self);
    }
  }
  double red[2] = {acc0.get(), acc1.get()};
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


// Launch shapes of the multi-rhs kernel.  CFG 0: 256 threads, 2 blocks/SM
// (FP64: 1; 2 rhs/thread: 3) and the register cap that gives; 1: CFG 0 with
// the complex FMAs on packed FP32 pairs (cmac_f2).  The others are "lean":
// the per-rhs scalars and the norm sums in shared memory, for more resident
// warps at fewer registers.  2 and 3: 3 and 4 blocks/SM (80 and 64
// registers); 5 and 6: CFG 0 and lean CFG 0 with the slot loop software-
// pipelined one slot ahead; 7, 8 and 9: CFG 0 and lean CFG 3 and 2 with the
// direction loop rolled (a quarter of the code, and fewer loads hoisted);
// 14 and 15: lean and rolled in 128-thread blocks, 7 and 8 blocks/SM (72 and
// 64 registers).  (Candidates measured slower and dropped: 56 and 48
// registers, every slot loop rolled, 32-byte spinor loads, lean 2 rhs per
// thread.)
// 16 and 17: 8 and 15 with the rhs of a thread taken in interleaved pairs
// (thread q of a site holds rhs 2q, 2q+1, 2Q+2q, 2Q+2q+1 for Q threads per
// site instead of 4q..4q+3): the four threads of a site then read 64
// contiguous bytes (two whole 32-byte sectors) of a neighbour's colour
// vector per 16-byte load instead of four half sectors, halving the
// sectors the L1 moves for spinor loads.  (Also measured slower and
// dropped: 16 with packed FP32 FMAs, 1.3x the time of 8 at 32^3x64; 8 and
// 15 with the next slot's neighbour spinors and link rows prefetched into
// L1 by prefetch.global.L1, 1.6x.)
// 18-22: the per-warp asynchronous pipeline (FP32 links and spinors,
// double-stored links): each warp copies the links and neighbour spinors
// of its eight sites for a slot ST - 1 slots ahead with cp.async into a
// ring of ST shared-memory stages of its own, and computes the current
// slot from shared memory, so that no register holds a load in flight and
// a slot costs one wait instead of the two or three dependent load round
// trips of the register shapes.  128-thread blocks; (ST, blocks/SM):
// 18 (2, 6), 19 (3, 4), 20 (4, 3).  Dropped: the 3-stage ring at 5
// blocks/SM (102 registers) spilled and measured 1.03 ms at 32^3x64
// against 0.73 at 4 blocks; 19 and 20 with packed FP32 FMAs measured 0.75
// and 0.72 against 0.73 and 0.72 (fma.rn.f32x2 wants its operands as
// register pairs, and the complex MAC's v.r and v.i broadcast into pairs
// costs the moves that the halved FMA count saves).
// 23, 24 and 25: 18, 19 and 20 for single-stored links (a separate
// instantiation, so that the double-stored one carries no run-time branch
// on the link storage in its slot loop).
template <int PS, int R, int CFG> struct MrCfg {
  static constexpr int pc = CFG >= 23 ? CFG - 5 : CFG;          // the pipeline shape
  static constexpr bool fbp = CFG >= 23 && CFG <= 25;           // single-stored links
  static constexpr int pipe = (((CFG >= 18 && CFG <= 20) || fbp) && PS == QLLG_F32 && R == 4)
                              ? (pc == 18 ? 2 : pc == 20 ? 4 : 3) : 0;
  static constexpr int threads = (CFG == 14 || CFG == 15 || CFG == 17 || CFG >= 18) ? 128 : 256;
  static constexpr int minb = (CFG == 2 || CFG == 9) ? 3 :
                              (CFG == 3 || CFG == 8 || CFG == 16) ? 4 :
                              CFG == 14 ? 7 : (CFG == 15 || CFG == 17) ? 8 :
                              pc == 18 ? 6 : pc == 19 ? 4 : pc == 20 ? 3 :
                              (PS == QLLG_F64 ? 1 : (R <= 2 ? 3 : 2));
  static constexpr bool f2 = CFG == 1 && PS == QLLG_F32;
  static constexpr bool lean = CFG != 0 && CFG != 1 && CFG != 5 && CFG != 7 && !pipe;
  static constexpr bool pf = CFG == 5 || CFG == 6;
  static constexpr bool roll = CFG == 7 || CFG == 8 || CFG == 9 || CFG >= 14;   // direction loop rolled
  static constexpr bool pairs = (CFG == 16 || CFG == 17) && R == 4;
};

// Multi-rhs variant: a thread owns one site and R consecutive right-hand
// sides, so each link is loaded and converted once per R rhs and the R
// accumulator sets give independent FMA chains.  Same epilogues as above.
// one stage of the per-warp pipeline: the neighbour spinors of the warp's
// eight sites, [colour][site half e >> 2][pair half h][((e & 3) ^ h)][q] 16
// bytes, where lane 4e + q holds rhs 4q + 2h, 4q + 2h + 1 of site e: each
// copy instruction writes 512 contiguous bytes, the two halves of a
// 32-byte sector land in different banks, and a stage is read with
// conflict-free 16-byte loads; then the links, [entry][site] 8 bytes
constexpr int kPipeSpinor = 3*1024;
constexpr int kPipeStage = kPipeSpinor + 9*8*8;              // 3648

__device__ __forceinline__ void cp_async16_ca(unsigned s, const void *gmem)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8_ca(unsigned s, const void *gmem)
{
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait()
{
  asm volatile("cp.async.wait_group %0;\n" :: "n"(N) : "memory");
}

template <int PS, int PL, int NS, int NR, int R, bool V4, int CFG>
__global__ void __launch_bounds__(MrCfg<PS,R,CFG>::threads, MrCfg<PS,R,CFG>::minb)
stag_dslash_mr(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  constexpr int Q = NR/R;                       // threads per site
  constexpr int PX = VecPrec<PS>::value;
  constexpr bool F2 = MrCfg<PS,R,CFG>::f2;
  constexpr bool PF = MrCfg<PS,R,CFG>::pf;
  constexpr int TB = MrCfg<PS,R,CFG>::threads;
  constexpr bool LEAN = MrCfg<PS,R,CFG>::lean;
  constexpr int ST = MrCfg<PS,R,CFG>::pipe;
  constexpr bool PIPE = ST > 0 && PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16 && V4;
  extern __shared__ __align__(16) unsigned char dsm[];
  // the pipeline's ring takes the reduction's scratch once the slot loop is done
  __shared__ double shm_s[PIPE ? 1 : 2*R*TB];
  double *shm = PIPE ? reinterpret_cast<double *>(dsm) : shm_s;
  __shared__ T s_ca[LEAN ? NR : 1], s_alpha[LEAN ? NR : 1];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh * NR;
  const size_t nwork = (size_t)G.Vh * Q;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const bool skip = a.done && *(volatile const int *)a.done;
  const int q = threadIdx.x % Q;
  constexpr bool PAIRS = MrCfg<PS,R,CFG>::pairs;
  // the rhs held in slot j of this thread
  auto rix = [&](int j) -> int { return PAIRS ? (j >> 1)*2*Q + 2*q + (j & 1) : q*R + j; };
  bool act[R];
  T ca[R], alpha[R];
  bool anyact = false, allact = true;
  constexpr bool v4 = (R % 2 == 0) && V4 && PS == QLLG_F32;
  const T cb = (T)a.b;
  // every rhs of the launch active: the slot loop without the active
  // checks.  Chosen per launch, not per thread, so that a launch runs one
  // copy of the unrolled loop (two would compete for the instruction cache)
  bool allrhs = !a.one_path;
  if(a.active) for(int r=0; r<NR; r++) allrhs &= a.active[r] != 0;
#pragma unroll
  for(int j=0; j<R; j++) {
    const int rhs = rix(j);
    act[j] = !a.active || a.active[rhs];
    anyact |= act[j];
    allact &= act[j];
    if constexpr (!LEAN) {
      ca[j] = (T)(a.a ? a.a[rhs] : a.a0);
      alpha[j] = (a.mode == 3 && act[j])
        ? (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs])) : (T)0;
    }
  }
  // LEAN: the per-rhs scalars and the compensated norm sums live in shared
  // memory instead of registers (the sums in shm, [2][R][TB], until the
  // grid reduction takes it over)
  if constexpr (LEAN) {
    if(threadIdx.x < NR) {
      const int rhs = threadIdx.x;
      s_ca[rhs] = (T)(a.a ? a.a[rhs] : a.a0);
      s_alpha[rhs] = (a.mode == 3 && (!a.active || a.active[rhs]))
        ? (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs])) : (T)0;
    }
    __syncthreads();
  }
  auto cav = [&](int j) -> T { if constexpr (LEAN) return s_ca[rix(j)]; else return ca[j]; };
  auto alv = [&](int j) -> T { if constexpr (LEAN) return s_alpha[rix(j)]; else return alpha[j]; };
  Acc<T> acc0r[LEAN ? 1 : R], acc1r[LEAN ? 1 : R];
  Acc<T> *accs = reinterpret_cast<Acc<T> *>(shm);
  static_assert(sizeof(Acc<T>) <= sizeof(double), "norm sums in shm");
  if constexpr (LEAN) {
#pragma unroll
    for(int j=0; j<2*R; j++) accs[j*TB + threadIdx.x] = Acc<T>();
  }
  auto norm0 = [&](int j, const Cx<T> (&v)[3]) {
    if constexpr (LEAN) { Acc<T> t = accs[j*TB + threadIdx.x]; t.norm(v); accs[j*TB + threadIdx.x] = t; }
    else acc0r[j].norm(v);
  };
  auto norm1 = [&](int j, const Cx<T> (&v)[3]) {
    if constexpr (LEAN) { Acc<T> t = accs[(R + j)*TB + threadIdx.x]; t.norm(v); accs[(R + j)*TB + threadIdx.x] = t; }
    else acc1r[j].norm(v);
  };
  // the per-warp pipeline's issue pointer: the work item, slot and site
  // coordinates of the next slot to copy, and the ring stage it goes to
  const int lane = threadIdx.x & 31;
  const unsigned wring = (unsigned)__cvta_generic_to_shared(dsm) + (threadIdx.x >> 5)*(ST ? ST : 1)*kPipeStage;
  const unsigned char *wring_p = dsm + (threadIdx.x >> 5)*(ST ? ST : 1)*kPipeStage;
  // the issue pointer: this lane's work item and slot of the next slot to
  // copy; the byte offsets of the issue and the consume stages in the ring
  size_t iw = (size_t)blockIdx.x*blockDim.x + threadIdx.x;
  int isl = 0;
  unsigned ioff = 0, coff = 0;
  // the neighbours of the warp's eight sites for the sixteen slots of the
  // issue pointer's site group, [slot][site], after the ring: filled when
  // the issue pointer reaches a group, lane 4e + q taking the four slots of
  // direction q of site e; read by the copies of each slot
  int *wnb = reinterpret_cast<int *>(dsm + (TB/32)*(ST ? ST : 1)*kPipeStage) + (threadIdx.x >> 5)*8*NS;
  // lane L copies the 16-byte pieces b = L & 7 of the colour vectors of
  // sites L >> 3 and 4 + (L >> 3) (the neighbours come from the table), to
  // [colour][0 or 1][b & 1][(L >> 3) ^ (b & 1)][b >> 1], and link piece L
  // (and 32 + L): entry L >> 2 of sites 2(L & 3), 2(L & 3) + 1 of the group
  const unsigned dlane = ((lane & 1) << 8) + ((((lane >> 3) ^ (lane & 1)) << 2) << 4) + (((lane & 7) >> 1) << 4);
  const size_t cst = total*8;                   // bytes between colours
  const char *const isp0 = (const char *)a.in + (lane & 7)*16;
  const char *const isp1 = isp0 + cst, *const isp2 = isp1 + cst;
  const size_t lstride = (size_t)9*V*8;         // bytes between slots' link blocks
  const char *ilk = nullptr, *ilk8 = nullptr;   // this lane's link pieces of slot 0 of the group
  // single-stored links (createStaggeredLinksFb): a forward slot's block is
  // stored slot 2mu + naik; a backward slot reads the forward link of each
  // neighbour site, -F(y)^dagger, so its 72 entries are gathered one 8-byte
  // piece at a time (lane L: entries L >> 3, 4 + (L >> 3) and, for L < 8,
  // 8, of site L & 7) and the transpose and sign are applied when it is read
  constexpr bool fbl = MrCfg<PS,R,CFG>::fbp;
  auto pipe_issue = [&]() {
    if constexpr (PIPE) {
      if(iw < nwork) {
        if(isl == 0) {
          const int isite = (int)(iw / Q);
          const int e = lane >> 2, qd = lane & 3;
          int xs[4];
          site_coords(G, p, isite, xs);
#pragma unroll
          for(int k=0; k<4; k++)
            wnb[(4*qd + k)*8 + e] = nbr_index(G, xs, qd, (k & 1 ? 3 : 1)*(k & 2 ? -1 : 1));
          const float2 *lk = (const float2 *)a.links + loff + (size_t)(isite - e) + 2*qd;
          ilk = (const char *)(lk + (size_t)e*V);
          ilk8 = (const char *)(lk + 8*V);
          __syncwarp();
        }
        const unsigned n0 = (unsigned)wnb[isl*8 + (lane >> 3)], n1 = (unsigned)wnb[isl*8 + 4 + (lane >> 3)];
        const unsigned dst = wring + ioff + dlane;
        cp_async16_ca(dst, isp0 + (size_t)n0*(NR*8));
        cp_async16_ca(dst + 512, isp0 + (size_t)n1*(NR*8));
        cp_async16_ca(dst + 1024, isp1 + (size_t)n0*(NR*8));
        cp_async16_ca(dst + 1024 + 512, isp1 + (size_t)n1*(NR*8));
        cp_async16_ca(dst + 2048, isp2 + (size_t)n0*(NR*8));
        cp_async16_ca(dst + 2048 + 512, isp2 + (size_t)n1*(NR*8));
        const unsigned lbase = wring + ioff + kPipeSpinor;
        const int bk = (isl >> 1) & 1;
        const int lslot = fbl ? 2*(isl >> 2) + (isl & 1) : isl;
        if(!fbl || !bk) {
          const size_t so = (size_t)lslot*lstride;
          cp_async16_ca(lbase + lane*16, ilk + so);
          if(lane < 4) cp_async16_ca(lbase + 512 + lane*16, ilk8 + so);
        } else {
          const int e8 = lane & 7, k0 = lane >> 3;
          const unsigned nbe = (unsigned)wnb[isl*8 + e8];
          const char *f = (const char *)a.links +
                          ((size_t)lslot*9*V + (size_t)(G.Vh - (int)loff) + nbe)*8;
          cp_async8_ca(lbase + k0*64 + e8*8, f + (size_t)k0*V*8);
          cp_async8_ca(lbase + (4 + k0)*64 + e8*8, f + (size_t)(4 + k0)*V*8);
          if(lane < 8) cp_async8_ca(lbase + 8*64 + e8*8, f + (size_t)8*V*8);
        }
        if(++isl == NS) { isl = 0; iw += (size_t)gridDim.x*blockDim.x; }
      }
      cp_async_commit();
      ioff = ioff + kPipeStage == (unsigned)(ST*kPipeStage) ? 0u : ioff + kPipeStage;
    }
  };
  // the pipeline runs whole warps (its copies and shuffles are warp-wide):
  // a thread whose rhs are all inactive computes along and stores nothing
  if(!skip && (PIPE || anyact)) {
    if constexpr (PIPE) {
#pragma unroll
      for(int i=0; i<ST-1; i++) pipe_issue();
    }
    for(size_t w = (size_t)blockIdx.x*blockDim.x + threadIdx.x; w < nwork;
        w += (size_t)gridDim.x*blockDim.x) {
      const int site = (int)(w / Q);
      const size_t sb = (size_t)site*NR;
      int x[4];
      site_coords(G, p, site, x);
      Cx<T> acc[R][3];
#pragma unroll
      for(int j=0; j<R; j++) {
        if(a.mode == 1 && a.self) {
          Cx<T> s[3];
          SpinorIO<PS,3>::load(a.self, total, sb + rix(j), s);
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = cav(j)*s[c].r; acc[j][c].i = cav(j)*s[c].i; }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = 0; acc[j][c].i = 0; }
        }
      }
      // the 16 (or 8) slots.  With every rhs of the launch active (the
      // usual case) the unrolled slot loop has no branches, so the compiler
      // can move the loads of later slots ahead of the FMAs of earlier ones
      auto slots = [&](auto ck) {
        constexpr bool CK = decltype(ck)::value;     // check the active flags
        constexpr int UMU = MrCfg<PS,R,CFG>::roll ? 1 : 4;
#pragma unroll UMU
        for(int mu=0; mu<4; mu++) {
#pragma unroll
          for(int back=0; back<2; back++) {
#pragma unroll
            for(int nk=0; nk<(NS == 16 ? 2 : 1); nk++) {
              const int d = (nk ? 3 : 1)*(back ? -1 : 1);
              const size_t nb = (size_t)nbr_index(G, x, mu, d);
              const size_t kb = nb*NR;
              Cx<T> U[9];
              slot_link<PL,NS>(a, mu, back, nk, V, (size_t)G.Vh, loff, (size_t)site, nb, U);
              if constexpr (v4) {
                // two rhs per 16-byte load and colour
#pragma unroll
                for(int h=0; h<R/2; h++) {
                  if constexpr (CK) { if(!act[2*h] && !act[2*h + 1]) continue; }
                  Cx<T> v[2][3];
                  Spinor4<PS>::load_pair(a.in, total, kb + rix(2*h), v);
#pragma unroll
                  for(int jj=0; jj<2; jj++) {
#pragma unroll
                    for(int l=0; l<3; l++) {
#pragma unroll
                      for(int c=0; c<3; c++) {
                        if constexpr (F2) cmac_f2(acc[2*h + jj][c], U[3*l + c], v[jj][l]);
                        else cmac(acc[2*h + jj][c], U[3*l + c], v[jj][l]);
                      }
                    }
                  }
                }
              } else {
#pragma unroll
                for(int j=0; j<R; j++) {
                  if constexpr (CK) { if(!act[j]) continue; }
                  Cx<T> v[3];
                  SpinorIO<PS,3>::load(a.in, total, kb + rix(j), v);
#pragma unroll
                  for(int l=0; l<3; l++) {
#pragma unroll
                    for(int c=0; c<3; c++) cmac(acc[j][c], U[3*l + c], v[l]);
                  }
                }
              }
            }
          }
        }
      };
      // the per-warp pipeline: per slot, copy the slot ST - 1 ahead, wait
      // for this one, compute it from the ring.  The warp barriers order
      // the ring: every lane's copies are visible before the stage is
      // read, and every lane has read a stage before it is refilled
      auto pipe_slots = [&]() {
        if constexpr (PIPE) {
#pragma unroll 1
          for(int sl=0; sl<NS; sl++) {
            pipe_issue();
            cp_async_wait<ST - 1>();
            __syncwarp();
            const unsigned char *sb = wring_p + coff;
            Cx<T> U[9];
            const float2 *ls = (const float2 *)(sb + kPipeSpinor) + (lane >> 2);
            if(fbl && ((sl >> 1) & 1)) {
              // -F^dagger of the neighbour's forward link
#pragma unroll
              for(int l=0; l<3; l++)
#pragma unroll
                for(int c=0; c<3; c++) {
                  const float2 t = ls[8*(3*c + l)];
                  U[3*l + c].r = -t.x; U[3*l + c].i = t.y;
                }
            } else {
#pragma unroll
              for(int k=0; k<9; k++) { const float2 t = ls[8*k]; U[k].r = t.x; U[k].i = t.y; }
            }
#pragma unroll
            for(int h=0; h<R/2; h++) {
              Cx<T> v[2][3];
#pragma unroll
              for(int c=0; c<3; c++) {
                const float4 t = *(const float4 *)(sb + c*1024 + h*256 + ((lane >> 4) << 9) +
                                                   (((lane ^ (h << 2)) & 15) << 4));
                v[0][c].r = t.x; v[0][c].i = t.y; v[1][c].r = t.z; v[1][c].i = t.w;
              }
#pragma unroll
              for(int jj=0; jj<2; jj++) {
#pragma unroll
                for(int l=0; l<3; l++) {
#pragma unroll
                  for(int c=0; c<3; c++) {
                    if constexpr (F2) cmac_f2(acc[2*h + jj][c], U[3*l + c], v[jj][l]);
                    else cmac(acc[2*h + jj][c], U[3*l + c], v[jj][l]);
                  }
                }
              }
            }
            __syncwarp();
            coff = coff + kPipeStage == (unsigned)(ST*kPipeStage) ? 0u : coff + kPipeStage;
          }
        }
      };
      if constexpr (PIPE) {
        // inactive rhs are computed too (their sums are neither stored nor
        // reduced), so that one copy of the slot loop serves every launch
        pipe_slots();
      } else if constexpr (PF && v4) {
        // software pipeline, one slot ahead: the links and neighbour
        // spinors of slot s+1 are loaded before the FMAs of slot s.  The
        // run-time branch on a.fb in slot_link keeps the compiler from
        // hoisting loads further ahead than that
        constexpr int NSL = NS;
        auto load_slot = [&](int sl, Cx<T> (&U)[9], Cx<T> (&v)[R][3]) {
          const int mu = NS == 16 ? sl >> 2 : sl >> 1;
          const int back = NS == 16 ? (sl >> 1) & 1 : sl & 1;
          const int nk = NS == 16 ? sl & 1 : 0;
          const int d = (nk ? 3 : 1)*(back ? -1 : 1);
          const size_t nb = (size_t)nbr_index(G, x, mu, d);
          slot_link<PL,NS>(a, mu, back, nk, V, (size_t)G.Vh, loff, (size_t)site, nb, U);
#pragma unroll
          for(int h=0; h<R/2; h++) {
            Cx<T> w[2][3];
            Spinor4<PS>::load_pair(a.in, total, nb*NR + rix(2*h), w);
#pragma unroll
            for(int c=0; c<3; c++) { v[2*h][c] = w[0][c]; v[2*h + 1][c] = w[1][c]; }
          }
        };
        auto fma_slot = [&](const Cx<T> (&U)[9], const Cx<T> (&v)[R][3]) {
#pragma unroll
          for(int j=0; j<R; j++) {
#pragma unroll
            for(int l=0; l<3; l++) {
#pragma unroll
              for(int c=0; c<3; c++) {
                if constexpr (F2) cmac_f2(acc[j][c], U[3*l + c], v[j][l]);
                else cmac(acc[j][c], U[3*l + c], v[j][l]);
              }
            }
          }
        };
        if(allrhs) {
          Cx<T> U0[9], U1[9], v0[R][3], v1[R][3];
          load_slot(0, U0, v0);
#pragma unroll
          for(int sl=0; sl<NSL; sl+=2) {
            load_slot(sl + 1, U1, v1);
            fma_slot(U0, v0);
            if(sl + 2 < NSL) load_slot(sl + 2, U0, v0);
            fma_slot(U1, v1);
          }
        } else {
          slots(std::integral_constant<bool, true>());
        }
      } else {
        if(allrhs) slots(std::integral_constant<bool, false>());
        else slots(std::integral_constant<bool, true>());
      }
      // epilogue.  With v4 and all R rhs active, the R rhs of the site move
      // as 16-byte vectors (inactive rhs must keep their old values, so a
      // partly active group takes the per-rhs path)
      if constexpr (v4) {
        if(allact) {
          // per pair of rhs (one 16-byte vector per colour) to keep few
          // values live
#pragma unroll
          for(int h=0; h<R/2; h++) {
            Cx<T> sv[2][3];
            const size_t tp = sb + rix(2*h);
            if(a.self) Spinor4<PS>::load_pair(a.self, total, tp, sv);
            if(a.mode == 3) {
              Cx<T> xv[2][3], rv[2][3];
              Spinor4<PX>::load_pair(a.x, total, tp, xv);
              Spinor4<PX>::load_pair(a.r, total, tp, rv);
#pragma unroll
              for(int jj=0; jj<2; jj++) {
                const int j = 2*h + jj;
#pragma unroll
                for(int c=0; c<3; c++) {
                  T apr = fma(cb, acc[j][c].r, cav(j)*sv[jj][c].r);
                  T api = fma(cb, acc[j][c].i, cav(j)*sv[jj][c].i);
                  xv[jj][c].r = fma(alv(j), sv[jj][c].r, xv[jj][c].r);
                  xv[jj][c].i = fma(alv(j), sv[jj][c].i, xv[jj][c].i);
                  rv[jj][c].r = fma(-alv(j), apr, rv[jj][c].r);
                  rv[jj][c].i = fma(-alv(j), api, rv[jj][c].i);
                }
                norm0(j, rv[jj]);
              }
              Spinor4<PX>::store_pair(a.x, total, tp, xv);
              Spinor4<PX>::store_pair(a.r, total, tp, rv);
              continue;
            }
            Cx<T> ov[2][3];
#pragma unroll
            for(int jj=0; jj<2; jj++) {
              const int j = 2*h + jj;
#pragma unroll
              for(int c=0; c<3; c++) {
                if(a.mode == 2) {
                  T sr = a.self ? cav(j)*sv[jj][c].r : (T)0, si = a.self ? cav(j)*sv[jj][c].i : (T)0;
                  ov[jj][c].r = fma(cb, acc[j][c].r, sr);
                  ov[jj][c].i = fma(cb, acc[j][c].i, si);
                } else {
                  ov[jj][c] = acc[j][c];
                }
              }
              if(a.norm_out) norm0(j, ov[jj]);
              if(a.norm_self && a.self) norm1(j, sv[jj]);
            }
            Spinor4<PS>::store_pair(a.out, total, tp, ov);
          }
          continue;
        }
      }
#pragma unroll
      for(int j=0; j<R; j++) {
        if(!act[j]) continue;
        const size_t t = sb + rix(j);
        Cx<T> self[3];
        if(a.self && a.mode != 1) SpinorIO<PS,3>::load(a.self, total, t, self);
        if(a.mode == 3) {
          Cx<T> xv[3], rv[3];
          SpinorIO<PX,3>::load(a.x, total, t, xv);
          SpinorIO<PX,3>::load(a.r, total, t, rv);
#pragma unroll
          for(int c=0; c<3; c++) {
            T apr = fma(cb, acc[j][c].r, cav(j)*self[c].r), api = fma(cb, acc[j][c].i, cav(j)*self[c].i);
            xv[c].r = fma(alv(j), self[c].r, xv[c].r); xv[c].i = fma(alv(j), self[c].i, xv[c].i);
            rv[c].r = fma(-alv(j), apr, rv[c].r); rv[c].i = fma(-alv(j), api, rv[c].i);
          }
          norm0(j, rv);
          SpinorIO<PX,3>::store(a.x, total, t, xv);
          SpinorIO<PX,3>::store(a.r, total, t, rv);
          continue;
        }
        Cx<T> out[3];
        if(a.mode == 2) {
#pragma unroll
          for(int c=0; c<3; c++) {
            T sr = a.self ? cav(j)*self[c].r : (T)0, si = a.self ? cav(j)*self[c].i : (T)0;
            out[c].r = fma(cb, acc[j][c].r, sr);
            out[c].i = fma(cb, acc[j][c].i, si);
          }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) out[c] = acc[j][c];
        }
        SpinorIO<PS,3>::store(a.out, total, t, out);
        if(a.norm_out) norm0(j, out);
        if(a.norm_self && a.self) norm1(j, self);
      }
    }
  }
  if constexpr (PIPE) {
    cp_async_wait<0>();              // only empty groups are left
    __syncthreads();                 // the reduction reuses the ring
  }
  double red[2][R];
  if constexpr (LEAN) {
#pragma unroll
    for(int j=0; j<R; j++) {
      red[0][j] = accs[j*TB + threadIdx.x].get();
      red[1][j] = accs[(R + j)*TB + threadIdx.x].get();
    }
    __syncthreads();                 // the grid reduction reuses shm
  } else {
#pragma unroll
    for(int j=0; j<R; j++) { red[0][j] = acc0r[j].get(); red[1][j] = acc1r[j].get(); }
  }
  if(a.mode == 3) {
    if(skip) return;
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, 0, PAIRS)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, 0, PAIRS);
  }
}

// Compacted variant for sparse masks (the FP64 reliable update of the
// mixed solver, where one or a few rhs of the batch are flagged at a time):
// work item w maps to (site, k-th flagged rhs), so the cost follows the
// number of flagged rhs instead of running whole warps at the FP64 rate for
// one of their lanes.  Modes 0 and 2 without norms.
template <int PS, int PL, int NS, int NR, int MINB = 1>
__global__ void __launch_bounds__(kThreads, MINB)
stag_dslash_compact(qllg_stag_args a)
{
  typedef typename Calc<PS, PL>::T T;
  __shared__ int list[NR];
  __shared__ int nact_s;
  if(a.done && *(volatile const int *)a.done) return;      // uniform
  if(threadIdx.x == 0) {
    int n = 0;
    for(int r=0; r<NR; r++)
      if(!a.active || (a.active[r] && (!a.active_eq || a.active[r] == a.active_eq))) list[n++] = r;
    nact_s = n;
  }
  __syncthreads();
  const int nact = nact_s;
  if(!nact) return;
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh * NR;
  const size_t nwork = (size_t)G.Vh * nact;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const T cb = (T)a.b;
  for(size_t w = (size_t)blockIdx.x*blockDim.x + threadIdx.x; w < nwork;
      w += (size_t)gridDim.x*blockDim.x) {
    const int site = (int)(w / nact);
    const int rhs = list[w % nact];
    const size_t t = (size_t)site*NR + rhs;
    int x[4];
    site_coords(G, p, site, x);
    Cx<T> acc[3];
#pragma unroll
    for(int c=0; c<3; c++) { acc[c].r = 0; acc[c].i = 0; }
    // double-float: one slot is about 600 instructions, so the slot loops
    // stay rolled (16 unrolled slots would not fit the instruction cache)
    constexpr int UMU = PS == QLLG_DF ? 1 : 4, UB = PS == QLLG_DF ? 1 : 2;
#pragma unroll UMU
    for(int mu=0; mu<4; mu++) {
#pragma unroll UB
      for(int back=0; back<2; back++) {
#pragma unroll UB
        for(int nk=0; nk<(NS == 16 ? 2 : 1); nk++) {
          const int d = (nk ? 3 : 1)*(back ? -1 : 1);
          const int k = nbr_index(G, x, mu, d);
          Cx<T> U[9], v[3];
          slot_link<PL,NS>(a, mu, back, nk, V, (size_t)G.Vh, loff, (size_t)site, (size_t)k, U);
          SpinorIO<PS,3>::load(a.in, total, (size_t)k*NR + rhs, v);
#pragma unroll
          for(int l=0; l<3; l++) {
#pragma unroll
            for(int j=0; j<3; j++) cmac(acc[j], U[3*l + j], v[l]);
          }
        }
      }
    }
    Cx<T> out[3];
    if(a.mode == 2) {
      const T ca = (T)(a.a ? a.a[rhs] : a.a0);
      Cx<T> self[3];
      if(a.self) SpinorIO<PS,3>::load(a.self, total, t, self);
#pragma unroll
      for(int c=0; c<3; c++) {
        T sr = a.self ? ca*self[c].r : (T)0, si = a.self ? ca*self[c].i : (T)0;
        out[c].r = kfma(cb, acc[c].r, sr);
        out[c].i = kfma(cb, acc[c].i, si);
      }
    } else {
#pragma unroll
      for(int c=0; c<3; c++) out[c] = acc[c];
    }
    SpinorIO<PS,3>::store(a.out, total, t, out);
  }
}

// MINB: resident blocks per SM the compiler must allow (a register cap)
template <int PS, int PL, int NS, int NR, int MINB = 1>
int launch_compact(const qllg_stag_args *a)
{
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash_compact<PS,PL,NS,NR,MINB>, kThreads, 0), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  if(a->preload) return 0;
  // sized for one flagged rhs: with more, the grid-stride loop takes them
  size_t need = ((size_t)a->g.Vh + kThreads - 1)/kThreads;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  stag_dslash_compact<PS,PL,NS,NR,MINB><<<grid, kThreads, 0, qllg_stream()>>>(*a);
  return qllg_launched("stag_dslash_compact launch");
}

// 16-byte vector access to the spinor buffers is allowed when every base
// pointer the kernel touches is 16-byte aligned (per-colour strides and the
// 4-rhs offsets keep that alignment)
bool vec4_ok(const qllg_stag_args *a)
{
  const void *ptrs[5] = {a->in, a->self, a->out, a->x, a->r};
  for(int i=0; i<5; i++) if(((uintptr_t)ptrs[i] & 15u) != 0) return false;
  return true;
}

// CFG 0 falls back to per-rhs loads when the buffers are not 16-byte
// aligned; the other launch shapes are 16-byte only (variant_ok checks)
template <int PS, int PL, int NS, int NR, int R, int CFG = 0>
int launch_mr(const qllg_stag_args *a)
{
  constexpr int TB = MrCfg<PS,R,CFG>::threads;
  const bool v4 = CFG != 0 ||
                  ((R % 2 == 0) && PS == QLLG_F32 && qllg_get_param("dslash_vec4") != 0 && vec4_ok(a));
  auto kern = [](bool vec) {
    if constexpr (CFG == 0) return vec ? stag_dslash_mr<PS,PL,NS,NR,R,true,0> : stag_dslash_mr<PS,PL,NS,NR,R,false,0>;
    else { (void)vec; return stag_dslash_mr<PS,PL,NS,NR,R,true,CFG>; }
  };
  // the per-warp pipeline's ring: dynamic shared memory
  constexpr int ST = MrCfg<PS,R,CFG>::pipe;
  constexpr size_t DSM = (ST && PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16)
                         ? (size_t)(TB/32)*(ST*kPipeStage + 8*NS*sizeof(int)) : 0;
  static int blocks_per_sm[2] = {0, 0};
  for(int k=0; k<2; k++) {
    // a preload loads both access widths of CFG 0
    const bool vk = a->preload ? (CFG != 0 || k == 1) : v4;
    if(!a->preload && k) break;
    if(!blocks_per_sm[vk]) {
      if(DSM > 48*1024 && qllg_check_cuda(cudaFuncSetAttribute(kern(vk),
           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DSM), "shared memory")) return -1;
      if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
           &blocks_per_sm[vk], kern(vk), TB, DSM), "occupancy")) return -1;
      if(blocks_per_sm[vk] < 1) blocks_per_sm[vk] = 1;
    }
  }
  if(a->preload) return 0;
  size_t work = (size_t)a->g.Vh * (NR/R);
  size_t need = (work + TB - 1)/TB;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm[v4];
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  A.one_path = qllg_get_param("dslash_split") == 0;
  kern(v4)<<<grid, TB, DSM, qllg_stream()>>>(A);
  return qllg_launched("stag_dslash_mr launch");
}

template <int PS, int PL, int NS, int NR>
int launch_plain(const qllg_stag_args *a)
{
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash<PS,PL,NS,NR>, kThreads, 0), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  if(a->preload) return 0;
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

// ------------------------------------------------ shared-memory staging
// FP32, 16 slots, 16 rhs: a block takes tiles of 64 consecutive output sites
// (4 threads per site, 4 rhs each) and walks the 16 slots with a 3-stage
// pipeline of asynchronous copies (cp.async.cg, 16 bytes, L1 bypassed): while
// slot n is computed from shared memory, the links and neighbour spinors of
// slots n+1 and n+2 are in flight, without holding registers.  The copies
// are fully coalesced (a site's 16 rhs of one colour are 128 contiguous
// bytes; a tile's link row is 512 contiguous bytes).  In shared memory a
// (colour, site) segment is padded to 144 bytes so that the 16-byte reads of
// 8 lanes hit distinct banks.  Needs Vh a multiple of 64 and 16-byte aligned
// spinor buffers (the launcher checks).
constexpr int kTileSites = 64;
constexpr int kTileStages = 3;
constexpr int kSpSeg = 144;                                  // bytes per (colour, site)
constexpr int kSpStage = 3*kTileSites*kSpSeg;                // 27648
constexpr int kLkStage = 9*kTileSites*8;                     // 4608
constexpr int kStageBytes = kSpStage + kLkStage;             // 32256
constexpr int kTileSmem = kTileStages*kStageBytes;           // 96768

__device__ __forceinline__ void cp16(void *smem, const void *gmem)
{
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait()
{
  asm volatile("cp.async.wait_group %0;\n" :: "n"(N) : "memory");
}

template <int NR_>
__global__ void __launch_bounds__(kThreads, 2)
stag_dslash_tile(qllg_stag_args a)
{
  extern __shared__ __align__(16) unsigned char smem[];
  typedef float T;
  constexpr int NR = 16, R = 4, PX = QLLG_F32;
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh*NR;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const int tid = threadIdx.x;
  const int q = tid & 3, i = tid >> 2;            // compute role: site i of the tile, rhs 4q..4q+3
  bool act[R], allact = true, anyact = false, blockact = !a.active;
  T ca[R], alpha[R];
  const T cb = (T)a.b;
#pragma unroll
  for(int j=0; j<R; j++) {
    const int rhs = q*R + j;
    act[j] = !a.active || a.active[rhs];
    allact &= act[j];
    anyact |= act[j];
    ca[j] = (T)(a.a ? a.a[rhs] : a.a0);
    alpha[j] = (a.mode == 3 && act[j])
      ? (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs])) : (T)0;
  }
  if(a.active) for(int r=0; r<NR; r++) blockact |= a.active[r] != 0;
  const bool skip = (a.done && *(volatile const int *)a.done) || !blockact;   // uniform
  Acc<T> acc0[R], acc1[R];
  if(!skip) {
    const int ntiles = G.Vh/kTileSites;
    const int mytiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x)/(int)gridDim.x + 1 : 0;
    const size_t cstride = total*8;                 // bytes between colours of a spinor
    // copy role: sites tid/8 and tid/8 + 32 of the tile, 16-byte part tid%8
    const int csite = tid >> 3, cpart = tid & 7;
    int xc[2][4], xn[2][4];                         // copy-site coordinates, this and next tile
    // the links and neighbour spinors of one slot of one tile, into stage st
    // (called with compile-time slots from the unrolled loop below)
    auto issue_slot = [&](int slot, int tile, const int (&xs)[2][4], int st) {
      const int mu = slot >> 2, back = (slot >> 1) & 1, nk = slot & 1;
      const int d = (nk ? 3 : 1)*(back ? -1 : 1);
      unsigned char *base = smem + st*kStageBytes;
#pragma unroll
      for(int hh=0; hh<2; hh++) {
        const char *src = (const char *)a.in + (size_t)nbr_index(G, xs[hh], mu, d)*(NR*8) + cpart*16;
        unsigned char *dst = base + (csite + 32*hh)*kSpSeg + cpart*16;
#pragma unroll
        for(int c=0; c<3; c++) cp16(dst + c*kTileSites*kSpSeg, src + c*cstride);
      }
      const char *lk = (const char *)a.links + (((size_t)slot*9)*V + loff + (size_t)tile*kTileSites)*8;
      for(int ch=tid; ch<9*32; ch+=kThreads) {
        const int k = ch >> 5, part = ch & 31;
        cp16(base + kSpStage + k*512 + part*16, lk + (size_t)k*V*8 + part*16);
      }
    };
    if(mytiles > 0) {
      site_coords(G, p, (int)blockIdx.x*kTileSites + csite, xc[0]);
      site_coords(G, p, (int)blockIdx.x*kTileSites + csite + 32, xc[1]);
      issue_slot(0, blockIdx.x, xc, 0);
      cp_commit();
      issue_slot(1, blockIdx.x, xc, 1);
      cp_commit();
    }
    Cx<T> acc[R][3];
    int st = 0, st2 = 2;                            // stages of the current step and of step + 2
    for(int lt=0; lt<mytiles; lt++) {
      const int tile = (int)blockIdx.x + lt*(int)gridDim.x;
      const bool more = lt + 1 < mytiles;
      const size_t t0 = ((size_t)tile*kTileSites + i)*NR + q*R;
#pragma unroll
      for(int slot=0; slot<16; slot++) {
        // one barrier per step: after it, step n's copies are visible and
        // every thread is done with step n-1, whose stage is the one step
        // n+2 fills
        cp_wait<1>();
        __syncthreads();
        if(slot < 14) {
          issue_slot(slot + 2, tile, xc, st2);
        } else if(more) {
          if(slot == 14) {
            site_coords(G, p, (tile + (int)gridDim.x)*kTileSites + csite, xn[0]);
            site_coords(G, p, (tile + (int)gridDim.x)*kTileSites + csite + 32, xn[1]);
          }
          issue_slot(slot - 14, tile + (int)gridDim.x, xn, st2);
        }
        cp_commit();
        st2 = st2 == kTileStages - 1 ? 0 : st2 + 1;
        if(slot == 0) {
#pragma unroll
          for(int j=0; j<R; j++) {
            if(a.mode == 1 && a.self) {
              Cx<T> sv[3];
              SpinorIO<QLLG_F32,3>::load(a.self, total, t0 + j, sv);
#pragma unroll
              for(int c=0; c<3; c++) { acc[j][c].r = ca[j]*sv[c].r; acc[j][c].i = ca[j]*sv[c].i; }
            } else {
#pragma unroll
              for(int c=0; c<3; c++) { acc[j][c].r = 0; acc[j][c].i = 0; }
            }
          }
        }
        if(anyact) {
          const unsigned char *base = smem + st*kStageBytes;
          Cx<T> U[9];
          const float2 *lk = (const float2 *)(base + kSpStage);
#pragma unroll
          for(int k=0; k<9; k++) { float2 u = lk[k*kTileSites + i]; U[k].r = u.x; U[k].i = u.y; }
#pragma unroll
          for(int h=0; h<R/2; h++) {
            if(!act[2*h] && !act[2*h + 1]) continue;
            Cx<T> v[2][3];
#pragma unroll
            for(int c=0; c<3; c++) {
              float4 w = *(const float4 *)(base + (c*kTileSites + i)*kSpSeg + q*32 + h*16);
              v[0][c].r = w.x; v[0][c].i = w.y; v[1][c].r = w.z; v[1][c].i = w.w;
            }
#pragma unroll
            for(int jj=0; jj<2; jj++)
#pragma unroll
              for(int l=0; l<3; l++)
#pragma unroll
                for(int c=0; c<3; c++) cmac(acc[2*h + jj][c], U[3*l + c], v[jj][l]);
          }
        }
        if(slot == 15 && anyact) {
          // epilogue of the tile's site (as the 16-byte path of stag_dslash_mr)
          if(allact) {
#pragma unroll
            for(int h=0; h<R/2; h++) {
              Cx<T> sv[2][3];
              if(a.self) Spinor4<QLLG_F32>::load_half(a.self, total, t0, h, sv);
              if(a.mode == 3) {
                Cx<T> xv[2][3], rv[2][3];
                Spinor4<PX>::load_half(a.x, total, t0, h, xv);
                Spinor4<PX>::load_half(a.r, total, t0, h, rv);
#pragma unroll
                for(int jj=0; jj<2; jj++) {
                  const int j = 2*h + jj;
#pragma unroll
                  for(int c=0; c<3; c++) {
                    T apr = fma(cb, acc[j][c].r, ca[j]*sv[jj][c].r);
                    T api = fma(cb, acc[j][c].i, ca[j]*sv[jj][c].i);
                    xv[jj][c].r = fma(alpha[j], sv[jj][c].r, xv[jj][c].r);
                    xv[jj][c].i = fma(alpha[j], sv[jj][c].i, xv[jj][c].i);
                    rv[jj][c].r = fma(-alpha[j], apr, rv[jj][c].r);
                    rv[jj][c].i = fma(-alpha[j], api, rv[jj][c].i);
                  }
                  acc0[j].norm(rv[jj]);
                }
                Spinor4<PX>::store_half(a.x, total, t0, h, xv);
                Spinor4<PX>::store_half(a.r, total, t0, h, rv);
                continue;
              }
              Cx<T> ov[2][3];
#pragma unroll
              for(int jj=0; jj<2; jj++) {
                const int j = 2*h + jj;
#pragma unroll
                for(int c=0; c<3; c++) {
                  if(a.mode == 2) {
                    T sr = a.self ? ca[j]*sv[jj][c].r : (T)0, si = a.self ? ca[j]*sv[jj][c].i : (T)0;
                    ov[jj][c].r = fma(cb, acc[j][c].r, sr);
                    ov[jj][c].i = fma(cb, acc[j][c].i, si);
                  } else {
                    ov[jj][c] = acc[j][c];
                  }
                }
                if(a.norm_out) acc0[j].norm(ov[jj]);
                if(a.norm_self && a.self) acc1[j].norm(sv[jj]);
              }
              Spinor4<QLLG_F32>::store_half(a.out, total, t0, h, ov);
            }
          } else {
#pragma unroll
            for(int j=0; j<R; j++) {
              if(!act[j]) continue;
              const size_t t = t0 + j;
              Cx<T> self[3];
              if(a.self && a.mode != 1) SpinorIO<QLLG_F32,3>::load(a.self, total, t, self);
              if(a.mode == 3) {
                Cx<T> xv[3], rv[3];
                SpinorIO<PX,3>::load(a.x, total, t, xv);
                SpinorIO<PX,3>::load(a.r, total, t, rv);
#pragma unroll
                for(int c=0; c<3; c++) {
                  T apr = fma(cb, acc[j][c].r, ca[j]*self[c].r), api = fma(cb, acc[j][c].i, ca[j]*self[c].i);
                  xv[c].r = fma(alpha[j], self[c].r, xv[c].r); xv[c].i = fma(alpha[j], self[c].i, xv[c].i);
                  rv[c].r = fma(-alpha[j], apr, rv[c].r); rv[c].i = fma(-alpha[j], api, rv[c].i);
                }
                acc0[j].norm(rv);
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
              SpinorIO<QLLG_F32,3>::store(a.out, total, t, out);
              if(a.norm_out) acc0[j].norm(out);
              if(a.norm_self && a.self) acc1[j].norm(self);
            }
          }
        }
        st = st == kTileStages - 1 ? 0 : st + 1;
      }
      if(more) {
#pragma unroll
        for(int hh=0; hh<2; hh++)
#pragma unroll
          for(int k=0; k<4; k++) xc[hh][k] = xn[hh][k];
      }
    }
    cp_wait<0>();
    __syncthreads();
  }
  double red[2][R];
#pragma unroll
  for(int j=0; j<R; j++) { red[0][j] = acc0[j].get(); red[1][j] = acc1[j].get(); }
  double *shm = (double *)smem;                   // the pipeline is drained: reuse its buffer
  if(a.mode == 3) {
    if(skip) return;
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce_mr<2,R>(red, NR, 4, a.partial, a.counter, shm, res)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce_mr<2,R>(red, NR, 4, a.partial, a.counter, shm, res);
  }
}

template <int NR_>
int launch_tile(const qllg_stag_args *a)
{
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaFuncSetAttribute(stag_dslash_tile<NR_>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            kTileSmem), "tile smem") ||
       qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash_tile<NR_>, kThreads, kTileSmem), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  if(a->preload) return 0;
  size_t ntiles = (size_t)a->g.Vh/kTileSites;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(ntiles < maxg ? ntiles : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  stag_dslash_tile<NR_><<<grid, kThreads, kTileSmem, qllg_stream()>>>(A);
  return qllg_launched("stag_dslash_tile launch");
}

#include "k_stag_bulk.cuh"
#include "k_stag_tma.cuh"

// variants of one launch shape, in the order the autotuner tries them:
// 0 = 4 rhs per thread, 1 = 2 rhs per thread, 2 = one thread per (site,
// rhs), 3 = shared-memory staging (FP32, 16 slots, 16 rhs only); FP32
// spinors at 16 rhs with 16-byte access also the 4-rhs kernel's other
// launch shapes (MrCfg 1, 2, 3, 5, 6, 7, 8, 9, 14, 15, 16, 17 as variants
// 4-10 and 12-16), 17-19 the per-warp cp.async pipeline (MrCfg 18-20:
// FP32 links too, double-stored, Vh a multiple of 8), and 20-21 the
// per-warp tensor-copy pipeline (k_stag_tma.cuh, 3 and 4 stages; the same
// conditions), 22-23 the same in one-warp blocks and 11 = the bulk-copy pipeline (FP32 links and
// spinors, 16 slots, 16 rhs, k_stag_bulk.cuh)
constexpr int kNumVariants = 24;
const char *const kVariantName[kNumVariants] = {"4 rhs/thread", "2 rhs/thread", "1 rhs/thread",
                                                "smem-staged 4 rhs/thread", "4 rhs/thread packed FMA",
                                                "4 rhs/thread lean 80 regs", "4 rhs/thread lean 64 regs",
                                                "4 rhs/thread prefetch", "4 rhs/thread lean prefetch",
                                                "4 rhs/thread rolled", "4 rhs/thread lean 64 regs rolled",
                                                "bulk-copy pipeline", "4 rhs/thread lean 80 regs rolled",
                                                "4 rhs/thread lean 72 regs rolled (128 threads)",
                                                "4 rhs/thread lean 64 regs rolled (128 threads)",
                                                "4 rhs/thread lean 64 regs rolled, paired rhs",
                                                "4 rhs/thread lean 64 regs rolled (128 threads), paired rhs",
                                                "warp pipeline, 2 stages", "warp pipeline, 3 stages",
                                                "warp pipeline, 4 stages", "warp tensor-copy pipeline, 3 stages",
                                                "warp tensor-copy pipeline, 4 stages",
                                                "one-warp tensor-copy pipeline, 3 stages",
                                                "one-warp tensor-copy pipeline, 4 stages"};

template <int PS, int PL, int NS, int NR>
bool variant_ok(const qllg_stag_args *a, int v)
{
  if(v == 0) return NR >= 4;
  if(v == 1) return NR >= 2;
  if(v == 2) return true;
  if(v == 11)
    return PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16 && !a->fb &&
           a->g.Vh % kBkSites == 0 && vec4_ok(a) && qllg_get_param("dslash_bulk") != 0;
  if(v >= 20)
    return PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16 && tma_ok(a) && vec4_ok(a) &&
           qllg_get_param("dslash_tma") != 0;
  if(v >= 17)
    return PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16 &&
           a->g.Vh % 8 == 0 && ((uintptr_t)a->links & 15u) == 0 && vec4_ok(a) &&
           qllg_get_param("dslash_vec4") != 0 && qllg_get_param("dslash_pipe") != 0;
  if(v >= 4)
    return PS == QLLG_F32 && NR == 16 && vec4_ok(a) && qllg_get_param("dslash_vec4") != 0;
  return PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16 && !a->fb &&
         a->g.Vh % kTileSites == 0 && vec4_ok(a) && qllg_get_param("dslash_tile") != 0;
}

template <int PS, int PL, int NS, int NR>
int launch_variant(const qllg_stag_args *a, int v)
{
  if(!variant_ok<PS,PL,NS,NR>(a, v)) v = NR >= 4 ? 0 : (NR >= 2 ? 1 : 2);
  if constexpr (PS == QLLG_F32 && PL == QLLG_F32 && NS == 16 && NR == 16) {
    if(v == 3) return launch_tile<NR>(a);
    if(v == 11) return launch_bulk<NR>(a);
    if(v == 20) return launch_tma<NR,3,4,4>(a);
    if(v == 21) return launch_tma<NR,4,3,4>(a);
    if(v == 22) return launch_tma<NR,3,16,1>(a);
    if(v == 23) return launch_tma<NR,4,13,1>(a);
  }
  if constexpr (PS == QLLG_F32 && NR == 16) {
    if(v >= 4) {
      switch(v) {
      case 4: return launch_mr<PS,PL,NS,NR,4,1>(a);
      case 5: return launch_mr<PS,PL,NS,NR,4,2>(a);
      case 6: return launch_mr<PS,PL,NS,NR,4,3>(a);
      case 7: return launch_mr<PS,PL,NS,NR,4,5>(a);
      case 8: return launch_mr<PS,PL,NS,NR,4,6>(a);
      case 9: return launch_mr<PS,PL,NS,NR,4,7>(a);
      case 10: return launch_mr<PS,PL,NS,NR,4,8>(a);
      case 12: return launch_mr<PS,PL,NS,NR,4,9>(a);
      case 13: return launch_mr<PS,PL,NS,NR,4,14>(a);
      case 14: return launch_mr<PS,PL,NS,NR,4,15>(a);
      case 15: return launch_mr<PS,PL,NS,NR,4,16>(a);
      case 16: return launch_mr<PS,PL,NS,NR,4,17>(a);
      case 17: return a->fb ? launch_mr<PS,PL,NS,NR,4,23>(a) : launch_mr<PS,PL,NS,NR,4,18>(a);
      case 18: return a->fb ? launch_mr<PS,PL,NS,NR,4,24>(a) : launch_mr<PS,PL,NS,NR,4,19>(a);
      default: return a->fb ? launch_mr<PS,PL,NS,NR,4,25>(a) : launch_mr<PS,PL,NS,NR,4,20>(a);
      }
    }
  }
  if constexpr (NR >= 4) { if(v == 0) return launch_mr<PS,PL,NS,NR,4>(a); }
  if constexpr (NR >= 2) { if(v == 1) return launch_mr<PS,PL,NS,NR,2>(a); }
  return launch_plain<PS,PL,NS,NR>(a);
}

// Autotuner: the first launch of a shape (precisions, slots, rhs, lattice)
// times each variant on a side output buffer (mode 0, no reductions, every
// rhs active: the same Dslash work the solvers do) and keeps the fastest
// in the registry; later launches of that shape use it, in every mode but
// the fused CG update (mode 3), which is timed the same way (every rhs
// active) on copies of its x, r and scalars under a key of its own.
// All variants give bitwise the same Dslash output; only the order of the
// per-rhs reductions differs between them.  No tuning during a stream
// capture or for callers that must not allocate: they use a tuned choice
// if one exists, else variant 0.
template <int PS, int PL, int NS, int NR>
int tuned_variant(const qllg_stag_args *a)
{
  if(NR < 2 || qllg_mr_disabled()) return 2;
  const int force = (int)qllg_get_param("dslash_variant");
  if(force >= 0 && force < kNumVariants && variant_ok<PS,PL,NS,NR>(a, force)) return force;
  // the fused CG launch (mode 3: its epilogue reads and writes x and r) is
  // tuned on its own: its best launch shape differs from the plain one's
  const bool fused = a->mode == 3;
  char key[96];
  snprintf(key, sizeof(key), "stag_dslash%s p%d/%d s%d%s n%d V%d (%d %d %d %d)", fused ? " fused" : "",
           PS, PL, NS, a->fb ? "fb" : "", NR, a->g.V, a->g.L[0], a->g.L[1], a->g.L[2], a->g.L[3]);
  int v = qllg_tune_lookup(key);
  if(v >= 0) return v;
  const int first = NR >= 4 ? 0 : 1;
  if(a->no_tune || qllg_capturing() || qllg_get_param("autotune") == 0) return first;
  qllg_stag_args T = *a;
  void *scratch[3] = {NULL, NULL, NULL};
  if(fused) {
    // the same launch on copies of x, r and the CG scalars.  The kernel
    // reads and writes x and r in VecPrec<PS> (FP32 for 16-bit operands)
    const size_t xb = qllg_spinor_bytes(VecPrec<PS>::value, 3)*(size_t)a->g.Vh*NR;
    const size_t sizes[3] = {xb, xb, sizeof(qllg_cg_scalars)};
    const void *src[3] = {a->x, a->r, a->sc};
    for(int i=0; i<3; i++) {
      scratch[i] = qllg_dmalloc(sizes[i]);
      if(!scratch[i] || qllg_check_cuda(cudaMemcpyAsync(scratch[i], src[i], sizes[i],
                                                         cudaMemcpyDeviceToDevice, qllg_stream()),
                                        "tune copy")) {
        for(int k=0; k<=i; k++) qllg_dfree(scratch[k]);
        return -1;
      }
    }
    T.x = scratch[0];
    T.r = scratch[1];
    T.sc = (qllg_cg_scalars *)scratch[2];
    T.done = NULL;
    // every rhs active, as for the plain launch: a first launch with few
    // active columns (a serving batch filling up) would favour shapes that
    // are slow once the batch is full
    T.active = NULL;
  } else {
    T.mode = 0;
    T.self = NULL;
    T.norm_out = T.norm_self = NULL;
    T.active = NULL;
    T.done = NULL;
    T.x = T.r = NULL;
    T.sc = NULL;
    T.rb = NULL;
    T.compact = 0;
    T.out = scratch[0] = qllg_dmalloc(qllg_spinor_bytes(PS, 3)*(size_t)a->g.Vh*NR);
    if(!T.out) return -1;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms[kNumVariants];
  for(int c=0; c<kNumVariants; c++) ms[c] = -1;
  int best = first, rc = 0;
  for(int c=first; c<kNumVariants && !rc; c++) {
    if(!variant_ok<PS,PL,NS,NR>(&T, c)) continue;
    // the fastest of five timed launches after a warm one: candidates are
    // often within a few percent, and the minimum is steadier than a mean
    rc |= launch_variant<PS,PL,NS,NR>(&T, c);                 // warm
    ms[c] = -1;
    for(int k=0; k<5 && !rc; k++) {
      cudaEventRecord(e0, qllg_stream());
      rc |= launch_variant<PS,PL,NS,NR>(&T, c);
      cudaEventRecord(e1, qllg_stream());
      cudaEventSynchronize(e1);
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      if(ms[c] < 0 || t < ms[c]) ms[c] = t;
    }
    if(ms[c] >= 0 && (ms[best] < 0 || ms[c] < ms[best])) best = c;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  qllg_sync();
  for(int i=0; i<3; i++) qllg_dfree(scratch[i]);
  if(rc) return -1;
  qllg_tune_store(key, best, kNumVariants, ms, kVariantName);
  return best;
}

template <int PS, int PL, int NS, int NR>
int launch_t(const qllg_stag_args *a)
{
  if(a->preload) {
    // every launch shape the dispatch can reach for this rhs count
    for(int v=0; v<kNumVariants; v++) if(launch_variant<PS,PL,NS,NR>(a, v)) return -1;
    return launch_compact<PS,PL,NS,NR>(a);
  }
  if(a->compact) return launch_compact<PS,PL,NS,NR>(a);
  int v = tuned_variant<PS,PL,NS,NR>(a);
  if(v < 0) return -1;
  return launch_variant<PS,PL,NS,NR>(a, v);
}

template <int PS, int PL, int NS>
int launch_nr(const qllg_stag_args *a)
{
  if(a->preload)
    return launch_t<PS,PL,NS,1>(a) || launch_t<PS,PL,NS,2>(a) || launch_t<PS,PL,NS,4>(a) ||
           launch_t<PS,PL,NS,8>(a) || launch_t<PS,PL,NS,16>(a) ? -1 : 0;
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

// one slot count only (the FP32 instantiations are split by slot count
// over two translation units, which compile in parallel)
template <int PS, int PL, int NS>
int launch_ns_only(const qllg_stag_args *a)
{
  if(a->nslots == NS) return launch_nr<PS,PL,NS>(a);
  qllg_set_error("stag_dslash: nslots %d not 8 or 16", a->nslots);
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
