// k_mixed.cu -- kernels of the mixed-precision (reliable-update) CG:
// the sloppy recurrence runs in 16-bit or FP32 storage with FP32
// arithmetic, and the flagged right-hand sides periodically replace the
// sloppy residual by the FP64 true residual b - A x (Clark et al., "Solving
// Lattice QCD systems of equations using mixed precision solvers on GPUs",
// Comput. Phys. Commun. 181 (2010) 1517, the reliable-update scheme of
// Sleijpen and van der Vorst).  The recurrence itself is cgSolveT's scaled
// form (lib/cg.c:77-115): p += r/|r|^2, a = 1/<p,Ap>.
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kT = 256;

#define GRID_LOOP(t, total) \
  for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < (total); \
      t += (size_t)gridDim.x*blockDim.x)

int grid_for(size_t total, qllg_redbuf *rb)
{
  size_t g = (total + kT - 1)/kT, m = (size_t)qllg_num_sms()*8;
  if(g > m) g = m;
  if(rb && g > (size_t)rb->maxblocks) g = rb->maxblocks;
  return g < 1 ? 1 : (int)g;
}

// start from an initial guess: x64 holds it and t64 = A x64 (computed by
// the caller in FP64); r64 = b - t64, rs = r64 rounded, xs = p = 0, and
// the scalars of a fresh solve with |r|^2 = |b - A x0|^2 (rsq_stop holds
// the relative target on entry and becomes absolute, as in mcg_init)
template <int PS, int NR>
__global__ void __launch_bounds__(kT)
mcg_init_guess_k(void *r64, void *xs, void *rs, void *p, const void *b, const void *t64,
                 int nsites, qllg_cg_scalars *s, double *partial, unsigned *counter)
{
  __shared__ double shm[2*kT];
  size_t total = (size_t)nsites*NR;
  double red[2] = {0, 0};
  GRID_LOOP(t, total) {
    Cx<double> bv[3], tv[3];
    SpinorIO<QLLG_F64,3>::load(b, total, t, bv);
    SpinorIO<QLLG_F64,3>::load(t64, total, t, tv);
    Cx<float> rf[3], zf[3];
#pragma unroll
    for(int c=0; c<3; c++) {
      red[1] += bv[c].r*bv[c].r + bv[c].i*bv[c].i;
      tv[c].r = bv[c].r - tv[c].r; tv[c].i = bv[c].i - tv[c].i;
      red[0] += tv[c].r*tv[c].r + tv[c].i*tv[c].i;
      rf[c].r = (float)tv[c].r; rf[c].i = (float)tv[c].i; zf[c].r = 0; zf[c].i = 0;
    }
    SpinorIO<QLLG_F64,3>::store(r64, total, t, tv);
    SpinorIO<VecPrec<PS>::value,3>::store(rs, total, t, rf);
    SpinorIO<QLLG_F32,3>::store(xs, total, t, zf);
    SpinorIO<PS,3>::store(p, total, t, zf);
  }
  double *res[2] = {s->tmp, s->prev};
  if(grid_reduce<2>(red, NR, threadIdx.x % NR, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        const double r2 = s->tmp[q], bs = s->prev[q];
        s->bsq[q] = bs; s->rsq[q] = r2; s->maxr2[q] = r2;
        s->rsq_stop[q] *= bs;
        s->iters[q] = 0; s->ru[q] = 0; s->nru[q] = 0;
        s->active[q] = (bs > 0 && s->maxits > 0 && r2 >= s->rsq_stop[q]) ? 1 : 0;
        any |= s->active[q];
      }
      s->done = !any;
      s->no_ru = 1;
      s->count = 0;
    }
  }
}

template <int PX, int PS, int NR>
__global__ void __launch_bounds__(kT)
mcg_init_k(void *x64, void *r64, void *xs, void *rs, void *p, const void *b, int nsites,
           qllg_cg_scalars *s, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  double red[1] = {0};
  GRID_LOOP(t, total) {
    Cx<double> v[3], z[3];
    SpinorIO<QLLG_F64,3>::load(b, total, t, v);
#pragma unroll
    for(int c=0; c<3; c++) { z[c].r = 0; z[c].i = 0; red[0] += v[c].r*v[c].r + v[c].i*v[c].i; }
    SpinorIO<QLLG_F64,3>::store(r64, total, t, v);
    SpinorIO<QLLG_F64,3>::store(x64, total, t, z);
    Cx<float> vf[3], zf[3];
#pragma unroll
    for(int c=0; c<3; c++) { vf[c].r = (float)v[c].r; vf[c].i = (float)v[c].i; zf[c].r = 0; zf[c].i = 0; }
    SpinorIO<VecPrec<PS>::value,3>::store(rs, total, t, vf);
    SpinorIO<PX,3>::store(xs, total, t, zf);
    SpinorIO<PS,3>::store(p, total, t, zf);
  }
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, threadIdx.x % NR, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        double bs = s->tmp[q];
        s->bsq[q] = bs; s->rsq[q] = bs; s->maxr2[q] = bs;
        s->rsq_stop[q] *= bs;
        s->iters[q] = 0; s->ru[q] = 0; s->nru[q] = 0;
        s->active[q] = (bs > 0 && s->maxits > 0) ? 1 : 0;
        any |= s->active[q];
      }
      s->done = !any;
      s->no_ru = 1;
      s->count = 0;
    }
  }
}

// admit right-hand sides into columns of a running batch (continuous
// batching): the admitted columns get x64 = xs = p = 0, r64 = rs = b and
// fresh scalars; every other column, and its scalars, is left as it is.
// A column's arithmetic never involves another column, so a request gives
// the same result whichever columns run beside it.
template <int PS, int NR>
__global__ void __launch_bounds__(kT)
mcg_admit_k(void *x64, void *r64, void *xs, void *rs, void *p, const void *b, int nsites,
            qllg_cg_scalars *s, qllg_admit_args ad, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  double red[1] = {0};
  if(ad.mask[rhs]) {
    GRID_LOOP(t, total) {
      Cx<double> v[3], z[3];
      SpinorIO<QLLG_F64,3>::load(b, total, t, v);
#pragma unroll
      for(int c=0; c<3; c++) { z[c].r = 0; z[c].i = 0; red[0] += v[c].r*v[c].r + v[c].i*v[c].i; }
      SpinorIO<QLLG_F64,3>::store(r64, total, t, v);
      SpinorIO<QLLG_F64,3>::store(x64, total, t, z);
      Cx<float> vf[3], zf[3];
#pragma unroll
      for(int c=0; c<3; c++) { vf[c].r = (float)v[c].r; vf[c].i = (float)v[c].i; zf[c].r = 0; zf[c].i = 0; }
      SpinorIO<VecPrec<PS>::value,3>::store(rs, total, t, vf);
      SpinorIO<QLLG_F32,3>::store(xs, total, t, zf);
      SpinorIO<PS,3>::store(p, total, t, zf);
    }
  }
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        if(ad.mask[q]) {
          double bs = s->tmp[q];
          s->bsq[q] = bs; s->rsq[q] = bs; s->maxr2[q] = bs; s->prev[q] = bs;
          s->rsq_stop[q] = ad.tol2[q]*bs;
          s->mass2[q] = ad.mass2[q];
          s->iters[q] = 0; s->ru[q] = 0; s->nru[q] = 0;
          s->active[q] = (bs > 0 && s->maxits > 0) ? 1 : 0;
        }
        any |= s->active[q];
      }
      s->done = !any;
    }
  }
}

template <int PS, int NR>
__global__ void mcg_p_k(void *p, const void *rs, int nsites, qllg_cg_scalars *s)
{
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->done || !s->active[rhs]) return;
  const float beta = (float)(1.0/s->rsq[rhs]);
  GRID_LOOP(t, total) {
    Cx<float> pv[3], rv[3];
    SpinorIO<PS,3>::load(p, total, t, pv);
    SpinorIO<PS,3>::load(rs, total, t, rv);
#pragma unroll
    for(int c=0; c<3; c++) { pv[c].r = fmaf(beta, rv[c].r, pv[c].r); pv[c].i = fmaf(beta, rv[c].i, pv[c].i); }
    SpinorIO<PS,3>::store(p, total, t, pv);
  }
}

template <int PX, int PS, int NR>
__global__ void __launch_bounds__(kT)
mcg_update_k(void *xs, void *rs, const void *p, const void *Ap, int nsites,
             qllg_cg_scalars *s, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  const bool skip = *(volatile int *)&s->done;
  if(skip) return;
  Acc<float> acc;
  if(s->active[rhs]) {
    const float alpha = (float)(1.0/(s->mass2[rhs]*s->pnorm[rhs] + s->vnorm[rhs]));
    GRID_LOOP(t, total) {
      Cx<float> xv[3], rv[3], pv[3], av[3];
      SpinorIO<PX,3>::load(xs, total, t, xv);
      SpinorIO<PS,3>::load(rs, total, t, rv);
      SpinorIO<PS,3>::load(p, total, t, pv);
      SpinorIO<PS,3>::load(Ap, total, t, av);
#pragma unroll
      for(int c=0; c<3; c++) {
        xv[c].r = fmaf(alpha, pv[c].r, xv[c].r); xv[c].i = fmaf(alpha, pv[c].i, xv[c].i);
        rv[c].r = fmaf(-alpha, av[c].r, rv[c].r); rv[c].i = fmaf(-alpha, av[c].i, rv[c].i);
      }
      acc.norm(rv);
      SpinorIO<PX,3>::store(xs, total, t, xv);
      SpinorIO<PS,3>::store(rs, total, t, rv);
    }
  }
  double red[1] = {acc.get()};
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int anyru = 0;
      for(int q=0; q<NR; q++) {
        s->ru[q] = 0;
        if(!s->active[q]) continue;
        double r2 = s->tmp[q];
        s->iters[q]++;
        s->rsq[q] = r2;
        s->ru[q] = ru_kind(s, q, r2);
        anyru |= s->ru[q] != 0;
      }
      s->no_ru = !anyru;
      s->count++;
    }
  }
}

template <int PX, int NC, int NR>
__global__ void mcg_accum_k(void *x64, void *xs, int nsites, qllg_cg_scalars *s)
{
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->no_ru || !s->ru[rhs]) return;
  GRID_LOOP(t, total) {
    Cx<double> xv[NC];
    Cx<float> sv[NC], z[NC];
    SpinorIO<QLLG_F64,NC>::load(x64, total, t, xv);
    SpinorIO<PX,NC>::load(xs, total, t, sv);
#pragma unroll
    for(int c=0; c<NC; c++) { xv[c].r += sv[c].r; xv[c].i += sv[c].i; z[c].r = 0; z[c].i = 0; }
    SpinorIO<QLLG_F64,NC>::store(x64, total, t, xv);
    SpinorIO<PX,NC>::store(xs, total, t, z);
  }
}

template <int PS, int NC, int NR>
__global__ void __launch_bounds__(kT)
mcg_residual_k(void *r64, void *rs, const void *b, const void *t64, int nsites, int stdform,
               qllg_cg_scalars *s, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->no_ru) return;   // uniform: written by the previous kernel
  double red[1] = {0};
  if(s->ru[rhs]) {
    GRID_LOOP(t, total) {
      Cx<double> bv[NC], tv[NC];
      SpinorIO<QLLG_F64,NC>::load(b, total, t, bv);
      SpinorIO<QLLG_F64,NC>::load(t64, total, t, tv);
      Cx<float> f[NC];
#pragma unroll
      for(int c=0; c<NC; c++) {
        tv[c].r = bv[c].r - tv[c].r; tv[c].i = bv[c].i - tv[c].i;
        red[0] += tv[c].r*tv[c].r + tv[c].i*tv[c].i;
        f[c].r = (float)tv[c].r; f[c].i = (float)tv[c].i;
      }
      SpinorIO<QLLG_F64,NC>::store(r64, total, t, tv);
      SpinorIO<PS,NC>::store(rs, total, t, f);
    }
  }
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        if(s->ru[q]) {
          double r2 = s->tmp[q];
          if(stdform) s->alpha[q] = r2/s->prev[q];
          s->rsq[q] = r2;
          s->maxr2[q] = r2;
          s->nru[q]++;
          if(!(r2 >= s->rsq_stop[q] && s->iters[q] < s->maxits)) s->active[q] = 0;
        }
        any |= s->active[q];
      }
      /* ru[] and no_ru stay set for the re-orthogonalisation that follows;
       * the next sloppy update clears them (or, once every rhs is done,
       * nothing else runs) */
      s->done = !any;
      if(!any) s->no_ru = 1;
    }
  }
}

template <int PS, int NR>
__global__ void __launch_bounds__(kT)
mcg_orth_dot_k(const void *p, const void *rs, int nsites, qllg_cg_scalars *s,
               double *partial, unsigned *counter)
{
  __shared__ double shm[2*kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->no_ru) return;
  Acc<float> acc0, acc1;
  if(s->ru[rhs]) {
    GRID_LOOP(t, total) {
      Cx<float> pv[3], rv[3];
      SpinorIO<PS,3>::load(p, total, t, pv);
      SpinorIO<VecPrec<PS>::value,3>::load(rs, total, t, rv);
      float re = 0, im = 0;
#pragma unroll
      for(int c=0; c<3; c++) {
        re = fmaf(rv[c].r, pv[c].r, re); re = fmaf(rv[c].i, pv[c].i, re);
        im = fmaf(rv[c].r, pv[c].i, im); im = fmaf(-rv[c].i, pv[c].r, im);
      }
      acc0.add(re);
      acc1.add(im);
    }
  }
  double red[2] = {acc0.get(), acc1.get()};
  double *res[2] = {s->orth_re, s->orth_im};
  if(grid_reduce<2>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      for(int q=0; q<NR; q++) {
        double r2 = s->rsq[q];
        s->orth_re[q] = (s->ru[q] && r2 > 0) ? s->orth_re[q]/r2 : 0;
        s->orth_im[q] = (s->ru[q] && r2 > 0) ? s->orth_im[q]/r2 : 0;
      }
    }
  }
}

template <int PS, int NR>
__global__ void mcg_orth_axpy_k(void *p, const void *rs, int nsites, qllg_cg_scalars *s)
{
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->no_ru || !s->ru[rhs]) return;
  const float cr = (float)s->orth_re[rhs], ci = (float)s->orth_im[rhs];
  GRID_LOOP(t, total) {
    Cx<float> pv[3], rv[3];
    SpinorIO<PS,3>::load(p, total, t, pv);
    SpinorIO<VecPrec<PS>::value,3>::load(rs, total, t, rv);
#pragma unroll
    for(int c=0; c<3; c++) {
      pv[c].r -= cr*rv[c].r - ci*rv[c].i;
      pv[c].i -= cr*rv[c].i + ci*rv[c].r;
    }
    SpinorIO<PS,3>::store(p, total, t, pv);
  }
}

#define NR_SWITCH(nrhs, ...) \
  switch(nrhs) { \
  case 1: { constexpr int NR = 1; __VA_ARGS__; } break; \
  case 2: { constexpr int NR = 2; __VA_ARGS__; } break; \
  case 4: { constexpr int NR = 4; __VA_ARGS__; } break; \
  case 8: { constexpr int NR = 8; __VA_ARGS__; } break; \
  case 16: { constexpr int NR = 16; __VA_ARGS__; } break; \
  default: qllg_set_error("nrhs %d not in {1,2,4,8,16}", nrhs); return -1; }

#define PXS_SWITCH(px, ps, ...) \
  if(px == QLLG_F32 && ps == QLLG_I16) { constexpr int PX = QLLG_F32, PS = QLLG_I16; __VA_ARGS__; } \
  else if(px == QLLG_F32 && ps == QLLG_F32) { constexpr int PX = QLLG_F32, PS = QLLG_F32; __VA_ARGS__; } \
  else if(px == QLLG_I16 && ps == QLLG_I16) { constexpr int PX = QLLG_I16, PS = QLLG_I16; __VA_ARGS__; } \
  else { qllg_set_error("mixed CG: precisions %d/%d", px, ps); return -1; }

int done(const char *w) { return qllg_launched(w); }

} // namespace

extern "C" int
qllg_k_mcg_reortho(int ps, void *p, const void *rs, int nsites, int nrhs, qllg_cg_scalars *s,
                   qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  if(ps == QLLG_I16) {
    NR_SWITCH(nrhs, (mcg_orth_dot_k<QLLG_I16,NR><<<g,kT,0,st>>>(p, rs, nsites, s, rb->partial, rb->counter)));
    if(done("mcg_orth_dot")) return -1;
    NR_SWITCH(nrhs, (mcg_orth_axpy_k<QLLG_I16,NR><<<g,kT,0,st>>>(p, rs, nsites, s)));
  } else if(ps == QLLG_F32) {
    NR_SWITCH(nrhs, (mcg_orth_dot_k<QLLG_F32,NR><<<g,kT,0,st>>>(p, rs, nsites, s, rb->partial, rb->counter)));
    if(done("mcg_orth_dot")) return -1;
    NR_SWITCH(nrhs, (mcg_orth_axpy_k<QLLG_F32,NR><<<g,kT,0,st>>>(p, rs, nsites, s)));
  } else { qllg_set_error("mcg_reortho: precision %d", ps); return -1; }
  return done("mcg_orth_axpy");
}

extern "C" int
qllg_k_mcg_init(int px, int ps, void *x64, void *r64, void *xs, void *rs, void *p,
                const void *b, int nsites, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  PXS_SWITCH(px, ps, NR_SWITCH(nrhs, (mcg_init_k<PX,PS,NR><<<g,kT,0,st>>>(x64, r64, xs, rs, p, b,
                                      nsites, s, rb->partial, rb->counter))));
  return done("mcg_init");
}

extern "C" int
qllg_k_mcg_init_guess(int ps, void *r64, void *xs, void *rs, void *p, const void *b,
                      const void *t64, int nsites, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  if(ps == QLLG_F32) {
    NR_SWITCH(nrhs, (mcg_init_guess_k<QLLG_F32,NR><<<g,kT,0,st>>>(r64, xs, rs, p, b, t64, nsites, s,
                                                                 rb->partial, rb->counter)));
  } else if(ps == QLLG_I16) {
    NR_SWITCH(nrhs, (mcg_init_guess_k<QLLG_I16,NR><<<g,kT,0,st>>>(r64, xs, rs, p, b, t64, nsites, s,
                                                                 rb->partial, rb->counter)));
  } else { qllg_set_error("mcg_init_guess: precision %d", ps); return -1; }
  return done("mcg_init_guess");
}

extern "C" int
qllg_k_mcg_admit(int ps, void *x64, void *r64, void *xs, void *rs, void *p, const void *b,
                 int nsites, int nrhs, qllg_cg_scalars *s, const qllg_admit_args *ad,
                 qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  if(ps == QLLG_F32) {
    NR_SWITCH(nrhs, (mcg_admit_k<QLLG_F32,NR><<<g,kT,0,st>>>(x64, r64, xs, rs, p, b, nsites, s, *ad,
                                                           rb->partial, rb->counter)));
  } else if(ps == QLLG_I16) {
    NR_SWITCH(nrhs, (mcg_admit_k<QLLG_I16,NR><<<g,kT,0,st>>>(x64, r64, xs, rs, p, b, nsites, s, *ad,
                                                           rb->partial, rb->counter)));
  } else { qllg_set_error("mcg_admit: precision %d", ps); return -1; }
  return done("mcg_admit");
}

extern "C" int
qllg_k_mcg_update_p(int ps, void *p, const void *rs, int nsites, int nrhs, qllg_cg_scalars *s)
{
  int g = grid_for((size_t)nsites*nrhs, 0);
  cudaStream_t st = qllg_stream();
  if(ps == QLLG_I16) { NR_SWITCH(nrhs, (mcg_p_k<QLLG_I16,NR><<<g,kT,0,st>>>(p, rs, nsites, s))); }
  else if(ps == QLLG_F32) { NR_SWITCH(nrhs, (mcg_p_k<QLLG_F32,NR><<<g,kT,0,st>>>(p, rs, nsites, s))); }
  else { qllg_set_error("mcg_update_p: precision %d", ps); return -1; }
  return done("mcg_update_p");
}

extern "C" int
qllg_k_mcg_update(int px, int ps, void *xs, void *rs, const void *p, const void *Ap,
                  int nsites, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  PXS_SWITCH(px, ps, NR_SWITCH(nrhs, (mcg_update_k<PX,PS,NR><<<g,kT,0,st>>>(xs, rs, p, Ap, nsites,
                                      s, rb->partial, rb->counter))));
  return done("mcg_update");
}

extern "C" int
qllg_k_mcg_accum(int px, void *x64, void *xs, int nsites, int ncomp, int nrhs, qllg_cg_scalars *s)
{
  int g = grid_for((size_t)nsites*nrhs, 0);
  cudaStream_t st = qllg_stream();
  if(px == QLLG_F32 && ncomp == 3) { NR_SWITCH(nrhs, (mcg_accum_k<QLLG_F32,3,NR><<<g,kT,0,st>>>(x64, xs, nsites, s))); }
  else if(px == QLLG_I16 && ncomp == 3) { NR_SWITCH(nrhs, (mcg_accum_k<QLLG_I16,3,NR><<<g,kT,0,st>>>(x64, xs, nsites, s))); }
  else if(px == QLLG_F32 && ncomp == 12) { NR_SWITCH(nrhs, (mcg_accum_k<QLLG_F32,12,NR><<<g,kT,0,st>>>(x64, xs, nsites, s))); }
  else { qllg_set_error("mcg_accum: precision %d components %d", px, ncomp); return -1; }
  return done("mcg_accum");
}

extern "C" int
qllg_k_mcg_residual(int ps, void *r64, void *rs, const void *b, const void *t64, int nsites,
                    int ncomp, int nrhs, int stdform, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  if(ps == QLLG_I16 && ncomp == 3) { NR_SWITCH(nrhs, (mcg_residual_k<QLLG_I16,3,NR><<<g,kT,0,st>>>(r64, rs, b, t64, nsites, stdform, s, rb->partial, rb->counter))); }
  else if(ps == QLLG_F32 && ncomp == 3) { NR_SWITCH(nrhs, (mcg_residual_k<QLLG_F32,3,NR><<<g,kT,0,st>>>(r64, rs, b, t64, nsites, stdform, s, rb->partial, rb->counter))); }
  else if(ps == QLLG_F32 && ncomp == 12) { NR_SWITCH(nrhs, (mcg_residual_k<QLLG_F32,12,NR><<<g,kT,0,st>>>(r64, rs, b, t64, nsites, stdform, s, rb->partial, rb->counter))); }
  else { qllg_set_error("mcg_residual: precision %d components %d", ps, ncomp); return -1; }
  return done("mcg_residual");
}

// ----------------------------------------------------- standard-form CG
namespace {

template <int PX, int PS, int NC, int NR>
__global__ void __launch_bounds__(kT)
scg_init_k(void *x, void *r, void *p, const void *b64, void *x64, void *r64, int nsites,
           qllg_cg_scalars *s, double *partial, unsigned *counter)
{
  typedef typename Calc<PX, PS>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  double red[1] = {0};
  GRID_LOOP(t, total) {
    Cx<double> bv[NC], z[NC];
    SpinorIO<QLLG_F64,NC>::load(b64, total, t, bv);
    Cx<T> bt[NC], zt[NC];
#pragma unroll
    for(int c=0; c<NC; c++) {
      red[0] += bv[c].r*bv[c].r + bv[c].i*bv[c].i;
      z[c].r = 0; z[c].i = 0; zt[c].r = 0; zt[c].i = 0;
      bt[c].r = (T)bv[c].r; bt[c].i = (T)bv[c].i;
    }
    SpinorIO<PX,NC>::store(x, total, t, zt);
    SpinorIO<PS,NC>::store(r, total, t, bt);
    SpinorIO<PS,NC>::store(p, total, t, bt);
    if(x64) SpinorIO<QLLG_F64,NC>::store(x64, total, t, z);
    if(r64) SpinorIO<QLLG_F64,NC>::store(r64, total, t, bv);
  }
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, threadIdx.x % NR, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        double bs = s->tmp[q];
        s->bsq[q] = bs; s->rsq[q] = bs; s->maxr2[q] = bs; s->prev[q] = bs;
        s->rsq_stop[q] *= bs;
        s->iters[q] = 0; s->ru[q] = 0; s->nru[q] = 0;
        s->active[q] = (bs > 0 && s->maxits > 0) ? 1 : 0;
        any |= s->active[q];
      }
      s->done = !any;
      s->no_ru = 1;
      s->count = 0;
    }
  }
}

template <int PX, int PS, int NC, int NR>
__global__ void __launch_bounds__(kT)
scg_xr_k(void *x, void *r, const void *p, const void *Ap, int nsites, qllg_cg_scalars *s,
         double *partial, unsigned *counter)
{
  typedef typename Calc<PX, PS>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->done) return;
  Acc<T> acc;
  if(s->active[rhs]) {
    const T alpha = (T)(s->rsq[rhs]/s->pnorm[rhs]);
    GRID_LOOP(t, total) {
      Cx<T> xv[NC], rv[NC], pv[NC], av[NC];
      SpinorIO<PX,NC>::load(x, total, t, xv);
      SpinorIO<PS,NC>::load(r, total, t, rv);
      SpinorIO<PS,NC>::load(p, total, t, pv);
      SpinorIO<PS,NC>::load(Ap, total, t, av);
#pragma unroll
      for(int c=0; c<NC; c++) {
        xv[c].r = fma(alpha, pv[c].r, xv[c].r); xv[c].i = fma(alpha, pv[c].i, xv[c].i);
        rv[c].r = fma(-alpha, av[c].r, rv[c].r); rv[c].i = fma(-alpha, av[c].i, rv[c].i);
      }
      acc.norm(rv);
      SpinorIO<PX,NC>::store(x, total, t, xv);
      SpinorIO<PS,NC>::store(r, total, t, rv);
    }
  }
  double red[1] = {acc.get()};
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) cg_finish_std(s, NR);
  }
}

template <int PS, int NC, int NR>
__global__ void scg_p_k(void *p, const void *r, int nsites, qllg_cg_scalars *s)
{
  typedef typename Calc<PS, PS>::T T;
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->done || !s->active[rhs]) return;
  const T beta = (T)s->alpha[rhs];
  GRID_LOOP(t, total) {
    Cx<T> pv[NC], rv[NC];
    SpinorIO<PS,NC>::load(p, total, t, pv);
    SpinorIO<PS,NC>::load(r, total, t, rv);
#pragma unroll
    for(int c=0; c<NC; c++) { pv[c].r = fma(beta, pv[c].r, rv[c].r); pv[c].i = fma(beta, pv[c].i, rv[c].i); }
    SpinorIO<PS,NC>::store(p, total, t, pv);
  }
}

} // namespace

#define SCG_SWITCH(px, ps, ncomp, ...) \
  if(px == QLLG_F64 && ps == QLLG_F64 && ncomp == 3) { constexpr int PX = QLLG_F64, PS = QLLG_F64, NC = 3; __VA_ARGS__; } \
  else if(px == QLLG_F64 && ps == QLLG_F64 && ncomp == 12) { constexpr int PX = QLLG_F64, PS = QLLG_F64, NC = 12; __VA_ARGS__; } \
  else if(px == QLLG_F32 && ps == QLLG_F32 && ncomp == 3) { constexpr int PX = QLLG_F32, PS = QLLG_F32, NC = 3; __VA_ARGS__; } \
  else if(px == QLLG_F32 && ps == QLLG_F32 && ncomp == 12) { constexpr int PX = QLLG_F32, PS = QLLG_F32, NC = 12; __VA_ARGS__; } \
  else if(px == QLLG_F32 && ps == QLLG_I16 && ncomp == 3) { constexpr int PX = QLLG_F32, PS = QLLG_I16, NC = 3; __VA_ARGS__; } \
  else { qllg_set_error("standard CG: precisions %d/%d components %d", px, ps, ncomp); return -1; }

extern "C" int
qllg_k_scg_init(int px, int ps, void *x, void *r, void *p, const void *b64, void *x64,
                void *r64, int nsites, int ncomp, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  SCG_SWITCH(px, ps, ncomp, NR_SWITCH(nrhs, (scg_init_k<PX,PS,NC,NR><<<g,kT,0,st>>>(x, r, p, b64, x64, r64, nsites, s, rb->partial, rb->counter))));
  return done("scg_init");
}

extern "C" int
qllg_k_scg_update_xr(int px, int ps, void *x, void *r, const void *p, const void *Ap, int nsites,
                     int ncomp, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nrhs, rb);
  cudaStream_t st = qllg_stream();
  SCG_SWITCH(px, ps, ncomp, NR_SWITCH(nrhs, (scg_xr_k<PX,PS,NC,NR><<<g,kT,0,st>>>(x, r, p, Ap, nsites, s, rb->partial, rb->counter))));
  return done("scg_update_xr");
}

extern "C" int
qllg_k_scg_update_p(int prec, void *p, const void *r, int nsites, int ncomp, int nrhs,
                    qllg_cg_scalars *s)
{
  int g = grid_for((size_t)nsites*nrhs, 0);
  cudaStream_t st = qllg_stream();
  SCG_SWITCH(prec, prec, ncomp, NR_SWITCH(nrhs, (scg_p_k<PS,NC,NR><<<g,kT,0,st>>>(p, r, nsites, s))));
  return done("scg_update_p");
}
