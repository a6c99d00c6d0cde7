// k_stag_tma.cuh -- the 16-rhs FP32 asqtad half-Dslash with one tensor-copy
// pipeline per warp (sm_100 and later: cp.async.bulk.tensor with
// tile::gather4, mbarrier), included by k_stag.cuh after k_stag_bulk.cuh,
// whose mbarrier helpers, wait limits and error flag it shares.
//
// A warp owns 8 consecutive output sites at a time (4 threads a site, 4 rhs a
// thread, as the 4-rhs kernel) and a ring of ST stages in shared memory.  For
// the slot ST - 1 ahead of the one it computes, lane 0 issues seven tensor
// copies that complete on the stage's mbarrier:
// - six gather4 loads of the neighbour spinors: per colour, two loads of four
//   128-byte rows (one site's 16 rhs) at row coordinates colour*Vh +
//   neighbour, so that any neighbour pattern (wrap-around included) is the
//   same two loads;
// - one tiled load of the slot's link block, 9 entries x 8 sites (576 bytes).
// The lanes then wait on the current slot's barrier and compute from shared
// memory.  No lane issues a global load in the slot loop, and the copies take
// no load/store-unit instructions: the L1 data pipe carries the shared-memory
// reads only.  Odd sites take their two 16-byte chunks in the other order (as
// in the bulk-copy kernel), so that the 8 lanes of an access phase, two sites,
// hit distinct banks.
//
// With one warp per block (W = 1) the group index comes from blockIdx alone,
// so the first site's coordinates and its neighbour in each slot are
// block-uniform values, which the copies take as operands directly: when the
// eight neighbours of a slot are consecutive sites (every slot but the
// x-direction ones at a row's end, when the row holds a whole number of
// groups) the slot's spinors are one tiled 3-D copy of 3 x 8 rows instead of
// six gathers.  (With four warps a block, each copy's operands come from
// per-lane registers, and the issuing lane pays for moving them into
// uniform registers: about 120 instructions a slot.)
//
// Waits are bounded as in the bulk-copy kernel: a wait that runs out records
// an error in g_bulk_err and stops the warp's pipeline; the warp then lets the
// copies it has issued land (each wait bounded by the fixed drain limit) and
// skips its stores, so a broken launch returns garbage with an error, not a
// hang.
#pragma once

// (included inside k_stag.cuh's anonymous namespace)
constexpr int kTmSp = 3*8*128;                  // spinor rows of a stage: 3072 B
constexpr int kTmLk = 9*8*8;                    // link block of a stage: 576 B
constexpr int kTmLkPad = 640;                   // link stages 128-byte aligned

// per block of W warps: [warp][stage] spinor rows, [warp][stage] link
// blocks, [warp][stage] barriers, [warp] tables of the neighbours' spinor
// rows ([slot][colour][site]: colour*Vh + neighbour), the per-rhs scalars,
// and room for the norm reduction (2 x 4 rhs doubles a thread)
template <int ST, int W> struct TmaLayout {
  static constexpr int sp = 0;
  static constexpr int lk = W*ST*kTmSp;
  static constexpr int bar = lk + W*ST*kTmLkPad;
  static constexpr int nbt = (bar + W*ST*8 + 127)/128*128;   // read as 16-byte vectors
  static constexpr int scal = nbt + W*16*3*8*4;
  static constexpr int end = scal + 2*16*4;
  static constexpr int bytes = end > 2*4*32*W*8 ? end : 2*4*32*W*8;
};

// four 128-byte rows of a 2-D tensor (rows r.x..r.w, from column 0) into
// consecutive rows of shared memory (address dst), completing on the
// mbarrier at shared address b
__device__ __forceinline__ void tma_gather4(unsigned dst, const CUtensorMap *m, int4 r, unsigned b)
{
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
               :: "r"(dst), "l"(m), "r"(0), "r"(r.x), "r"(r.y), "r"(r.z), "r"(r.w), "r"(b) : "memory");
}
// the box of a 3-D tensor at (0, y, 0) into shared memory, completing on b
__device__ __forceinline__ void tma_tile3d_y(unsigned dst, const CUtensorMap *m, int y, unsigned b)
{
  asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4}], [%5];"
               :: "r"(dst), "l"(m), "r"(0), "r"(y), "r"(0), "r"(b) : "memory");
}
// the box of a 2-D tensor at (x, y) into shared memory, completing on b
__device__ __forceinline__ void tma_tile2d(unsigned dst, const CUtensorMap *m, int x, int y, unsigned b)
{
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3}], [%4];"
               :: "r"(dst), "l"(m), "r"(x), "r"(y), "r"(b) : "memory");
}
// mbar_wait with the wait suspended in hardware between polls (up to a
// microsecond a poll, woken by the phase's completion) instead of spinning
// on issue slots; false when the phase has not completed within `limit`
// clock64 cycles
__device__ __forceinline__ bool mbar_wait_sleep(unsigned a, unsigned ph, long long limit)
{
  const long long t0 = clock64();
  while(true) {
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(a), "r"(ph), "r"(1000u) : "memory");
    if(ok) return true;
    if(clock64() - t0 > limit) return false;
  }
}

// FP32 spinors and links (double-stored), 16 slots, 16 rhs; modes 0-3 and the
// norms as stag_dslash_mr.  tm_in: the input spinors as rows of 32 floats,
// [colour*Vh + site], box one row; tm_in3: the same as [colour][site][32
// floats], box 3 x 8 x 32; tm_lk: the links as [slot*9 + entry][2V floats],
// box 16 floats x 9 rows.  Needs Vh a multiple of 8 (the launcher checks).
template <int NR_, int ST, int MINB, int W>
__global__ void __launch_bounds__(32*W, MINB)
stag_dslash_tma(qllg_stag_args a, const __grid_constant__ CUtensorMap tm_in,
                const __grid_constant__ CUtensorMap tm_in3, const __grid_constant__ CUtensorMap tm_lk)
{
  extern __shared__ __align__(128) unsigned char tsm[];
  typedef float T;
  typedef TmaLayout<ST,W> Lo;
  constexpr int TB = 32*W;
  constexpr int NR = 16, R = 4, Q = 4, PS = QLLG_F32, PX = QLLG_F32;
  T *s_ca = (T *)(tsm + Lo::scal), *s_alpha = s_ca + NR;
  const Geo G = make_geo(a.g);
  const size_t total = (size_t)G.Vh*NR;
  const int p = a.out_parity;
  const int loff = p ? G.Vh : 0;
  const int tid = threadIdx.x, w = W == 1 ? 0 : tid >> 5, lane = tid & 31;
  const int e = lane >> 2, q = lane & 3, sw = e & 1;
  const bool skip = a.done && *(volatile const int *)a.done;     // uniform
  uint64_t *bars = (uint64_t *)(tsm + Lo::bar) + w*ST;
  int *nbt = (int *)(tsm + Lo::nbt) + w*16*3*8;
  const unsigned char *spw = tsm + Lo::sp + w*ST*kTmSp;
  const unsigned char *lkw = tsm + Lo::lk + w*ST*kTmLkPad;
  // the same as shared-window addresses, for the copies and the waits
  const unsigned bars_s = smem_addr(bars), spw_s = smem_addr(spw), lkw_s = smem_addr(lkw);
  // the copies need 128-byte aligned destinations (block-uniform)
  bool ok = (smem_addr(tsm) & 127u) == 0;
  if(lane == 0) {
    for(int s=0; s<ST; s++) mbar_init(&bars[s], 1);
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
  unsigned actm = 0;                     // bit jp: rhs q*R + jp active
#pragma unroll
  for(int jp=0; jp<R; jp++) if(!a.active || a.active[q*R + jp]) actm |= 1u << jp;
  const bool allact = actm == (1u << R) - 1;
  const int ngroups = G.Vh/8;
  const int gstride = gridDim.x*W;
  // the issue pointer: group, slot and stage of the next slot to copy
  int ig = blockIdx.x*W + w, isl = 0, ibuf = 0, cbuf = 0;
  unsigned ph = 0;                       // bit s: parity of stage s's next phase
  unsigned issued = 0, consumed = 0;
  unsigned cmask = 0;                    // W == 1: bit s: slot s's 8 neighbours consecutive
  int xf[4];                             // W == 1: coordinates of the group's first site
  auto issue = [&]() {
    if(ig < ngroups && ok) {
      if(isl == 0) {
        // the neighbours' spinor rows of the group's sites: lane 4e + q
        // takes the four slots of direction q of site e
        int xs[4];
        site_coords(G, p, ig*8 + e, xs);
        unsigned ball[4];
#pragma unroll
        for(int k=0; k<4; k++) {
          const int n = nbr_index(G, xs, q, (k & 1 ? 3 : 1)*(k & 2 ? -1 : 1));
#pragma unroll
          for(int c=0; c<3; c++) nbt[((4*q + k)*3 + c)*8 + e] = c*G.Vh + n;
          if constexpr (W == 1) {
            // site e's neighbour follows site e - 1's (lane 4(e - 1) + q)
            const int prev = __shfl_up_sync(0xffffffffu, n, 4);
            ball[k] = __ballot_sync(0xffffffffu, e == 0 || n == prev + 1);
          }
        }
        if constexpr (W == 1) {
          cmask = 0;
#pragma unroll
          for(int qq=0; qq<4; qq++)
#pragma unroll
            for(int k=0; k<4; k++)
              if(((ball[k] >> qq) & 0x11111111u) == 0x11111111u) cmask |= 1u << (4*qq + k);
          site_coords(G, p, ig*8, xf);
        }
        __syncwarp();
      }
      // W == 1: the first site's neighbour in this slot, from block-uniform
      // values only
      int nf = 0;
      if constexpr (W == 1)
        nf = nbr_index(G, xf, isl >> 2, (isl & 1 ? 3 : 1)*(isl & 2 ? -1 : 1));
      if(lane == 0 && !a.wait_test) {
        const unsigned bar = bars_s + ibuf*8, sp = spw_s + ibuf*kTmSp;
        // the lanes' reads of this stage (ordered by the warp barrier after
        // them) come before the copies' writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bars[ibuf], kTmSp + kTmLk);
        if(W == 1 && ((cmask >> isl) & 1)) {
          tma_tile3d_y(sp, &tm_in3, nf, bar);
        } else {
          const int4 *rows = (const int4 *)(nbt + isl*24);
#pragma unroll
          for(int c=0; c<3; c++) {
            tma_gather4(sp + c*1024, &tm_in, rows[2*c], bar);
            tma_gather4(sp + c*1024 + 512, &tm_in, rows[2*c + 1], bar);
          }
        }
        tma_tile2d(lkw_s + ibuf*kTmLkPad, &tm_lk, 2*(loff + ig*8), isl*9, bar);
      }
      issued++;
      if(++isl == 16) { isl = 0; ig += gstride; }
      ibuf = ibuf + 1 == ST ? 0 : ibuf + 1;
    }
  };
  if(!skip) {
#pragma unroll
    for(int i=0; i<ST-1; i++) issue();
    for(int g = blockIdx.x*W + w; g < ngroups && ok; g += gstride) {
      const int site = g*8 + e;
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
      for(int sl=0; sl<16; sl++) {
        issue();
        if(!__all_sync(0xffffffffu, mbar_wait_sleep(bars_s + cbuf*8, (ph >> cbuf) & 1, a.wait_cycles))) {
          ok = false;
          break;
        }
        ph ^= 1u << cbuf;
        consumed++;
        const unsigned char *sp = spw + cbuf*kTmSp;
        const unsigned char *lk = lkw + cbuf*kTmLkPad;
        Cx<T> U[9];
#pragma unroll
        for(int k=0; k<9; k++) {
          const float2 u = *(const float2 *)(lk + k*64 + e*8);
          U[k].r = u.x; U[k].i = u.y;
        }
#pragma unroll
        for(int L=0; L<2; L++) {
          const int h = L ^ sw;
          Cx<T> v[2][3];
#pragma unroll
          for(int c=0; c<3; c++) {
            const float4 u = *(const float4 *)(sp + c*1024 + e*128 + q*32 + h*16);
            v[0][c].r = u.x; v[0][c].i = u.y; v[1][c].r = u.z; v[1][c].i = u.w;
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
        cbuf = cbuf + 1 == ST ? 0 : cbuf + 1;
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
    if(!ok) {
      atomicExch(&g_bulk_err, 1);
      // let the copies issued and not consumed land before the ring is
      // reused by the reduction or the block leaves
      if(!a.wait_test) {
        for(unsigned c = consumed; c < issued; c++) {
          mbar_wait_sleep(bars_s + cbuf*8, (ph >> cbuf) & 1, kBkWait);
          ph ^= 1u << cbuf;
          cbuf = cbuf + 1 == ST ? 0 : cbuf + 1;
        }
      }
    }
  }
  // the norm sums per rhs of the thread (accumulator j holds rhs j ^ 2sw)
  double red[2][R];
#pragma unroll
  for(int jp=0; jp<R; jp++) {
    red[0][jp] = sw ? acc0[jp ^ 2].get() : acc0[jp].get();
    red[1][jp] = sw ? acc1[jp ^ 2].get() : acc1[jp].get();
  }
  __syncthreads();                  // the ring is idle: the reduction reuses it
  double *shm = (double *)tsm;
  if(a.mode == 3) {
    if(skip) return;
    double *res[2] = {a.sc->tmp, NULL};
    if(grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, TB)) {
      __syncthreads();
      if(threadIdx.x == 0) {
        if(a.mixed) cg_finish_mixed(a.sc, NR);
        else cg_finish_plain(a.sc, NR);
      }
    }
  } else if(a.norm_out || a.norm_self) {
    double *res[2] = {a.norm_out, a.norm_self};
    grid_reduce_mr<2,R>(red, NR, Q, a.partial, a.counter, shm, res, TB);
  }
}

// ------------------------------------------------------------ the launcher
typedef CUresult (*TmaEncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, through the runtime (no link to the driver
// library); NULL where the driver does not have it
TmaEncodeFn tma_encoder()
{
  static TmaEncodeFn fn = NULL;
  static int tried = 0;
  if(!tried) {
    tried = 1;
    void *f = NULL;
    cudaDriverEntryPointQueryResult qr;
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &qr)
         == cudaSuccess && qr == cudaDriverEntryPointSuccess)
      fn = (TmaEncodeFn)f;
    else
      cudaGetLastError();
  }
  return fn;
}

// an FP32 tensor map of rank 2 or 3 (extents n[] from the innermost, byte
// pitches pitch[] of the outer dimensions, box[]), cached by address and
// shape: the solvers reuse a handful of vectors and one link buffer per
// operator
int tma_map(CUtensorMap *out, const void *base, int rank, const uint64_t *n, const uint64_t *pitch,
            const uint32_t *box)
{
  struct Ent { const void *base; int rank; uint64_t n[3]; uint32_t box[3]; CUtensorMap m; };
  static Ent cache[24];
  static int used = 0, next = 0;
  for(int i=0; i<used; i++) {
    const Ent &E = cache[i];
    bool same = E.base == base && E.rank == rank;
    for(int d=0; d<rank && same; d++) same = E.n[d] == n[d] && E.box[d] == box[d];
    if(same) { *out = E.m; return 0; }
  }
  TmaEncodeFn enc = tma_encoder();
  if(!enc) { qllg_set_error("tensor-map encoder not available"); return -1; }
  cuuint64_t dims[3], strides[2];
  cuuint32_t bx[3], estr[3] = {1, 1, 1};
  for(int d=0; d<rank; d++) { dims[d] = n[d]; bx[d] = box[d]; }
  for(int d=0; d<rank-1; d++) strides[d] = pitch[d];
  Ent &E = cache[next];
  if(enc(&E.m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, (void *)base, dims, strides, bx, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    qllg_set_error("cuTensorMapEncodeTiled failed");
    return -1;
  }
  E.base = base; E.rank = rank;
  for(int d=0; d<rank; d++) { E.n[d] = n[d]; E.box[d] = box[d]; }
  *out = E.m;
  next = (next + 1) % 24;
  if(used < 24) used++;
  return 0;
}

bool tma_ok(const qllg_stag_args *a)
{
  return !a->fb && a->g.Vh % 8 == 0 && ((uintptr_t)a->links & 15u) == 0 &&
         ((uintptr_t)a->in & 15u) == 0 && tma_encoder() != NULL;
}

template <int NR_, int ST, int MINB, int W>
int launch_tma(const qllg_stag_args *a)
{
  constexpr int smem = TmaLayout<ST,W>::bytes;
  static int blocks_per_sm = 0;
  if(!blocks_per_sm) {
    if(qllg_check_cuda(cudaFuncSetAttribute(stag_dslash_tma<NR_,ST,MINB,W>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "tma smem") ||
       qllg_check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &blocks_per_sm, stag_dslash_tma<NR_,ST,MINB,W>, 32*W, smem), "occupancy")) return -1;
    if(blocks_per_sm < 1) blocks_per_sm = 1;
  }
  if(a->preload) return 0;
  const uint64_t Vh = (uint64_t)a->g.Vh, V = (uint64_t)a->g.V;
  CUtensorMap tin, tin3, tlk;
  // spinors: rows of 16 rhs x 2 floats, [colour*Vh + site] (one row a box)
  // and [colour][site][32 floats] (3 x 8 rows a box); links: rows of the
  // full lattice's V sites x 2 floats, [slot*9 + entry] (16 floats x 9 rows)
  const uint64_t n_in[2] = {32, 3*Vh}, p_in[1] = {128};
  const uint32_t b_in[2] = {32, 1};
  const uint64_t n_in3[3] = {32, Vh, 3}, p_in3[2] = {128, 128*Vh};
  const uint32_t b_in3[3] = {32, 8, 3};
  const uint64_t n_lk[2] = {2*V, 16*9}, p_lk[1] = {8*V};
  const uint32_t b_lk[2] = {16, 9};
  if(tma_map(&tin, a->in, 2, n_in, p_in, b_in) || tma_map(&tin3, a->in, 3, n_in3, p_in3, b_in3) ||
     tma_map(&tlk, a->links, 2, n_lk, p_lk, b_lk)) return -1;
  const size_t ngroups = Vh/8;
  const size_t need = (ngroups + W - 1)/W;
  size_t maxg = (size_t)qllg_num_sms()*blocks_per_sm;
  if(a->rb && maxg > (size_t)a->rb->maxblocks) maxg = a->rb->maxblocks;
  int grid = (int)(need < maxg ? need : maxg);
  if(grid < 1) grid = 1;
  qllg_stag_args A = *a;
  A.partial = a->rb ? a->rb->partial : NULL;
  A.counter = a->rb ? a->rb->counter : NULL;
  A.wait_cycles = (long long)(qllg_get_param("wait_polls")*100.0);
  A.wait_test = qllg_get_param("bulk_wait_test") != 0;
  stag_dslash_tma<NR_,ST,MINB,W><<<grid, 32*W, smem, qllg_stream()>>>(A, tin, tin3, tlk);
  return qllg_launched("stag_dslash_tma launch");
}
