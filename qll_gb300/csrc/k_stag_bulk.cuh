// k_stag_bulk.cuh -- the 16-rhs FP32 asqtad half-Dslash as a warp-specialised
// bulk-copy pipeline (sm_90 and later: cp.async.bulk, mbarrier), included
// by k_stag.cuh.
//
// A block is 8 consumer warps (64 consecutive output sites x 4 groups of 4
// rhs, as the 4-rhs kernel) and one producer warp.  For each tile of 64
// sites the producer walks the 16 slots: it computes the tile's neighbour
// sites for the slot and copies, with cp.async.bulk, the slot's link rows
// (9 entries x 64 sites, 512 contiguous bytes each) and the neighbour
// spinors (per colour, each run of consecutive neighbour sites as one copy
// of 128-byte site blocks: 16 rhs x 8 bytes) into one stage of a ring in
// shared memory.  A "full" mbarrier per stage completes on the copies'
// transaction bytes; the consumers wait on it, read links and spinors from
// shared memory, and release the stage through an "empty" mbarrier.  The
// consumers issue no global loads in the slot loop and compute no neighbour
// indices; the ring keeps kBkStages slots of copies in flight per block
// without holding registers.
//
// Every wait is bounded: the pipeline's waits by the library's wait limit
// (parameter wait_polls, about a second by default), after which the wait
// records an error in g_bulk_err, stops the pipeline and lets the block
// finish; the producer first waits for its copies in flight to land, with
// a fixed limit of 2e9 clock cycles whatever the pipeline's own, so that
// no copy lands in the shared memory of a block that has left.  A broken
// launch returns garbage with an error, not a hang.
#pragma once

// (included inside k_stag.cuh's anonymous namespace)
constexpr int kBkSites = 64;
constexpr int kBkCons = 4*kBkSites;                 // consumer threads
constexpr int kBkThreads = kBkCons + 32;            // + the producer warp
constexpr int kBkStages = 3;
constexpr int kBkLk = 9*kBkSites*8;                 // link rows of a slot: 4608 B
constexpr int kBkSpC = kBkSites*128;                // one colour of the spinors: 8192 B
constexpr int kBkStage = kBkLk + 3*kBkSpC;          // 29184 B (a multiple of 128)
constexpr int kBkSmem = kBkStages*kBkStage + 2*kBkStages*8;
constexpr long long kBkWait = 2000000000ll;         // clock64 cycles the drain waits at most

__device__ int g_bulk_err;                          // nonzero: a wait ran out

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, unsigned bytes)
{
  asm volatile("{\n\t.reg .b64 st;\n\t"
               "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
               :: "r"(smem_addr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b)
{
  asm volatile("{\n\t.reg .b64 st;\n\t"
               "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}"
               :: "r"(smem_addr(b)) : "memory");
}
// wait for the completion of the phase of parity ph; false when it has not
// completed within `limit` clock64 cycles
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned ph, long long limit)
{
  const unsigned a = smem_addr(b);
  const long long t0 = clock64();
  while(true) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(a), "r"(ph) : "memory");
    if(ok) return true;
    if(clock64() - t0 > limit) return false;
  }
}
// global -> shared bulk copy (16-byte aligned ends, size a multiple of 16)
// completing on mbarrier b
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *b)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(b)) : "memory");
}

// FP32 spinors and links (double-stored), 16 slots, 16 rhs; modes 0-3 and
// the norms as stag_dslash_mr.  Needs Vh a multiple of 64 and 16-byte
// aligned spinor buffers (the launcher checks).
template <int NR_>
__global__ void __launch_bounds__(kBkThreads, 2)
stag_dslash_bulk(qllg_stag_args a)
{
  extern __shared__ __align__(16) unsigned char smem[];   // 16-byte copies, 8-byte barriers
  typedef float T;
  constexpr int NR = 16, R = 4, Q = 4, PS = QLLG_F32, PX = QLLG_F32;
  uint64_t *full = (uint64_t *)(smem + kBkStages*kBkStage);
  uint64_t *empty = full + kBkStages;
  __shared__ T s_ca[NR], s_alpha[NR];
  const Geo G = make_geo(a.g);
  const size_t V = (size_t)a.g.V;
  const size_t total = (size_t)G.Vh*NR;
  const int p = a.out_parity;
  const size_t loff = p ? (size_t)G.Vh : 0;
  const int tid = threadIdx.x;
  const bool producer = tid >= kBkCons;
  const int lane = tid & 31;
  const int ntiles = G.Vh/kBkSites;
  const bool skip = a.done && *(volatile const int *)a.done;     // uniform
  if(tid == 0) {
    for(int s=0; s<kBkStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kBkCons/32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if(tid < NR) {
    const int rhs = tid;
    s_ca[rhs] = (T)(a.a ? a.a[rhs] : a.a0);
    s_alpha[rhs] = (a.mode == 3 && (!a.active || a.active[rhs]))
      ? (T)(1.0/(a.sc->mass2[rhs]*a.sc->pnorm[rhs] + a.sc->vnorm[rhs])) : (T)0;
  }
  __syncthreads();
  const T cb = (T)a.b;
  Acc<T> acc0[R], acc1[R];
  bool ok = true;
  if(!skip && producer) {
    // ------------------------------------------------------------ producer
    unsigned cnt = 0;
    // a test of the waits' error path: the producer issues nothing (so no
    // copy is ever in flight) and the consumers' first waits run out
    if(a.wait_test) ok = false;
    for(int tile=blockIdx.x; tile<ntiles && ok; tile+=gridDim.x) {
      const int site0 = tile*kBkSites;
      int x0[4], x1[4];
      site_coords(G, p, site0 + lane, x0);
      site_coords(G, p, site0 + 32 + lane, x1);
#pragma unroll 1
      for(int sl=0; sl<16; sl++, cnt++) {
        const int st = cnt % kBkStages;
        const unsigned use = cnt/kBkStages;
        // every lane waits (each takes the barrier's acquire); the outcome
        // is made warp-uniform so that the shuffles below stay converged
        if(use > 0 && !__all_sync(0xffffffffu, mbar_wait(&empty[st], (use - 1) & 1, a.wait_cycles))) {
          ok = false;
          break;
        }
        const int mu = sl >> 2, back = (sl >> 1) & 1, nk = sl & 1;
        const int d = (nk ? 3 : 1)*(back ? -1 : 1);
        const int nb0 = nbr_index(G, x0, mu, d), nb1 = nbr_index(G, x1, mu, d);
        // runs of consecutive neighbour sites: site i starts one unless
        // nb[i] == nb[i-1] + 1
        const int up0 = __shfl_up_sync(0xffffffffu, nb0, 1);
        const int up1 = __shfl_up_sync(0xffffffffu, nb1, 1);
        const int last0 = __shfl_sync(0xffffffffu, nb0, 31);
        const bool st0 = lane == 0 || nb0 != up0 + 1;
        const bool st1 = lane == 0 ? nb1 != last0 + 1 : nb1 != up1 + 1;
        const unsigned m0 = __ballot_sync(0xffffffffu, st0), m1 = __ballot_sync(0xffffffffu, st1);
        const unsigned long long starts = (unsigned long long)m0 | ((unsigned long long)m1 << 32);
        unsigned char *stage = smem + st*kBkStage;
        if(lane == 0) mbar_expect_tx(&full[st], kBkStage);
        __syncwarp();
        if(lane < 9) {
          const char *src = (const char *)a.links +
                            (((size_t)sl*9 + lane)*V + loff + (size_t)site0)*8;
          bulk_load(stage + lane*kBkSites*8, src, kBkSites*8, &full[st]);
        }
#pragma unroll
        for(int hh=0; hh<2; hh++) {
          const int i = lane + 32*hh;
          if(!((starts >> i) & 1ull)) continue;
          // the run goes to the next start (or the end of the tile)
          const unsigned long long after = i == 63 ? 0ull : (starts >> (i + 1));
          const int len = after ? __ffsll((long long)after) : kBkSites - i;
          const int nb = hh ? nb1 : nb0;
#pragma unroll
          for(int c=0; c<3; c++) {
            const char *src = (const char *)a.in + ((size_t)c*total + (size_t)nb*NR)*8;
            bulk_load(stage + kBkLk + c*kBkSpC + i*128, src, (unsigned)len*128, &full[st]);
          }
        }
      }
    }
    if(!ok) {
      atomicExch(&g_bulk_err, 1);
      // let the copies already issued (the last kBkStages uses) land before
      // the block moves on: this wait keeps the long fixed limit, whatever
      // the pipeline's own (a copy in flight lands within microseconds)
      for(unsigned c = cnt > kBkStages ? cnt - kBkStages : 0; c < cnt; c++)
        mbar_wait(&full[c % kBkStages], (c/kBkStages) & 1, kBkWait);
    }
  } else if(!skip) {
    // ----------------------------------------------------------- consumers
    // thread (site i of the tile, rhs group q: rhs 4q..4q+3 = 16-byte chunks
    // 2q, 2q+1 of the site's 128 bytes).  Odd sites take the two chunks in
    // the other order (sw), so that the 8 lanes of a 16-byte access phase
    // (2 sites) hit distinct banks: accumulator pair L holds rhs pair
    // L ^ sw.  The index changes nothing in the sums of any rhs.
    const int i = tid >> 2, q = tid & 3, sw = i & 1;
    unsigned actm = 0;                   // bit jp: rhs q*R + jp active
#pragma unroll
    for(int jp=0; jp<R; jp++) if(!a.active || a.active[q*R + jp]) actm |= 1u << jp;
    const bool allact = actm == (1u << R) - 1;
    unsigned cnt = 0;
    for(int tile=blockIdx.x; tile<ntiles && ok; tile+=gridDim.x) {
      const int site = tile*kBkSites + i;
      const size_t t0 = (size_t)site*NR + q*R;
      Cx<T> acc[R][3];
#pragma unroll
      for(int j=0; j<R; j++) {
        const int jp = j ^ (2*sw);
        if(a.mode == 1 && a.self) {
          Cx<T> s[3];
          SpinorIO<PS,3>::load(a.self, total, t0 + jp, s);
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = s_ca[q*R + jp]*s[c].r; acc[j][c].i = s_ca[q*R + jp]*s[c].i; }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) { acc[j][c].r = 0; acc[j][c].i = 0; }
        }
      }
#pragma unroll 1
      for(int sl=0; sl<16; sl++, cnt++) {
        const int st = cnt % kBkStages;
        if(!__all_sync(0xffffffffu, mbar_wait(&full[st], (cnt/kBkStages) & 1, a.wait_cycles))) { ok = false; break; }
        const unsigned char *stage = smem + st*kBkStage;
        Cx<T> U[9];
#pragma unroll
        for(int e=0; e<9; e++) {
          const float2 w = *(const float2 *)(stage + e*kBkSites*8 + i*8);
          U[e].r = w.x; U[e].i = w.y;
        }
#pragma unroll
        for(int L=0; L<2; L++) {
          const int h = L ^ sw;
          Cx<T> v[2][3];
#pragma unroll
          for(int c=0; c<3; c++) {
            const float4 w = *(const float4 *)(stage + kBkLk + c*kBkSpC + i*128 + q*32 + h*16);
            v[0][c].r = w.x; v[0][c].i = w.y; v[1][c].r = w.z; v[1][c].i = w.w;
          }
#pragma unroll
          for(int jj=0; jj<2; jj++) {
#pragma unroll
            for(int l=0; l<3; l++) {
#pragma unroll
              for(int c=0; c<3; c++) cmac(acc[2*L + jj][c], U[3*l + c], v[jj][l]);
            }
          }
        }
        __syncwarp();
        if(lane == 0) mbar_arrive(&empty[st]);
      }
      if(!ok) break;
      // epilogue, as stag_dslash_mr's (accumulator j is rhs q*R + (j ^ 2sw))
#pragma unroll
      for(int j=0; j<R; j++) {
        const int jp = j ^ (2*sw);
        if(!allact && !((actm >> jp) & 1)) continue;
        const size_t t = t0 + jp;
        const T ca = s_ca[q*R + jp], alpha = s_alpha[q*R + jp];
        Cx<T> self[3];
        if(a.self && a.mode != 1) SpinorIO<PS,3>::load(a.self, total, t, self);
        if(a.mode == 3) {
          Cx<T> xv[3], rv[3];
          SpinorIO<PX,3>::load(a.x, total, t, xv);
          SpinorIO<PX,3>::load(a.r, total, t, rv);
#pragma unroll
          for(int c=0; c<3; c++) {
            T apr = fma(cb, acc[j][c].r, ca*self[c].r), api = fma(cb, acc[j][c].i, ca*self[c].i);
            xv[c].r = fma(alpha, self[c].r, xv[c].r); xv[c].i = fma(alpha, self[c].i, xv[c].i);
            rv[c].r = fma(-alpha, apr, rv[c].r); rv[c].i = fma(-alpha, api, rv[c].i);
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
            T sr = a.self ? ca*self[c].r : (T)0, si = a.self ? ca*self[c].i : (T)0;
            out[c].r = fma(cb, acc[j][c].r, sr);
            out[c].i = fma(cb, acc[j][c].i, si);
          }
        } else {
#pragma unroll
          for(int c=0; c<3; c++) out[c] = acc[j][c];
        }
        SpinorIO<PS,3>::store(a.out, total, t, out);
        if(a.norm_out) acc0[j].norm(out);
        if(a.norm_self && a.self) acc1[j].norm(self);
      }
    }
    if(!ok) atomicExch(&g_bulk_err, 1);
  }
  // the norm sums per rhs of the thread (accumulator j holds rhs j ^ 2sw)
  const int swr = producer ? 0 : ((tid >> 2) & 1);
  double red[2][R];
#pragma unroll
  for(int jp=0; jp<R; jp++) {
    red[0][jp] = swr ? acc0[jp ^ 2].get() : acc0[jp].get();
    red[1][jp] = swr ? acc1[jp ^ 2].get() : acc1[jp].get();
  }
  __syncthreads();                  // the ring is idle: the reduction reuses it
  double *shm = (double *)smem;
  if(a.mode == 3) {
    if(skip) return;
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, kBkCons)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, kBkCons);
  }
}

template <int NR_>
int launch_bulk(const qllg_stag_args *a)
{
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaFuncSetAttribute(stag_dslash_bulk<NR_>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            kBkSmem), "bulk smem") ||
       qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash_bulk<NR_>, kBkThreads, kBkSmem), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  if(a->preload) return 0;
  size_t ntiles = (size_t)a->g.Vh/kBkSites;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(ntiles < maxg ? ntiles : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  // the pipeline's waits give up after the library's wait limit (polls of
  // about 64 ns, so about 100 clock cycles each)
  A.wait_cycles = (long long)(qllg_get_param("wait_polls")*100.0);
  A.wait_test = qllg_get_param("bulk_wait_test") != 0;
  stag_dslash_bulk<NR_><<<grid, kBkThreads, kBkSmem, qllg_stream()>>>(A);
  return qllg_launched("stag_dslash_bulk launch");
}
