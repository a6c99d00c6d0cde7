// k_cgms.cu -- multishift CG kernels (cgmsSolveT, lib/cgms.c:6-179).
// The scalar recurrences (zeta, alpha, beta per shift) run in FP64 on the
// GPU in single-thread kernels; the vector updates of all shifts are fused
// into one pass over the lattice (2N+3 vector streams per iteration).
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kT = 256;

#define GRID_LOOP(t, total) \
  for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < (total); \
      t += (size_t)gridDim.x*blockDim.x)

__global__ void cgms_pre_k(qllg_cgms_scalars *s)
{
  if(threadIdx.x != 0 || s->done) return;
  if(s->iteration > 0) {
    for(int i=0; i<s->n; i++) {     // lib/cgms.c:163-167
      s->bo[i] = s->b[i];
      s->zo[i] = s->z[i];
      s->z[i] = s->zn[i];
    }
  }
  s->oldrsq = s->rsq;
}

__global__ void cgms_coef_k(qllg_cgms_scalars *s)
{
  if(threadIdx.x != 0 || s->done) return;
  s->iteration++;
  double pkp = s->mass2*s->pnorm + s->vnorm;   // li.Anorm2 of dslashp2
  pkp *= s->s[0]*s->s[0];
  s->pkp = pkp;
  if(pkp <= 0) { s->done = 1; return; }
  s->b[0] = s->rsq/pkp;
  s->zn[0] = 1;
  for(int i=1; i<s->n; i++) {
    double c1;
    s->zn[i] = s->z[i]*s->zo[i]*s->bo[0];
    c1 = s->b[0]*s->a[0]*(s->zo[i] - s->z[i]);
    c1 += s->zo[i]*s->bo[0]*(1 + s->shifts[i]*s->b[0]);
    if(c1 != 0.0) s->zn[i] /= c1;
    else s->zn[i] = 0;
    if(s->z[i] != 0.0) s->b[i] = s->b[0]*s->zn[i]/s->z[i];
    else s->zn[i] = s->b[i] = 0;
  }
}

template <int P>
__global__ void __launch_bounds__(kT)
cgms_xr_k(void *out, void *r, const void *ps, const void *Ap, int nsites, size_t fs,
          qllg_cgms_scalars *s, double *partial, unsigned *counter)
{
  typedef typename Calc<P,P>::T T;
  __shared__ double shm[kT];
  __shared__ T coef[QLLG_MAXSHIFT];
  if(*(volatile int *)&s->done) return;        // uniform: set by the previous kernel
  const int n = s->n;
  for(int i=threadIdx.x; i<n; i+=blockDim.x) coef[i] = (T)(s->b[i]*s->s[i]);
  __syncthreads();
  const T t0 = -(T)(s->b[0]*s->s[0]);
  const size_t total = (size_t)nsites;
  Acc<T> acc;
  GRID_LOOP(t, total) {
    Cx<T> pv[3], ov[3];
    for(int i=0; i<n; i++) {
      const void *pi = (const char *)ps + fs*i;
      void *oi = (char *)out + fs*i;
      SpinorIO<P,3>::load(pi, total, t, pv);
      SpinorIO<P,3>::load(oi, total, t, ov);
#pragma unroll
      for(int c=0; c<3; c++) { ov[c].r = fma(coef[i], pv[c].r, ov[c].r); ov[c].i = fma(coef[i], pv[c].i, ov[c].i); }
      SpinorIO<P,3>::store(oi, total, t, ov);
    }
    Cx<T> rv[3], av[3];
    SpinorIO<P,3>::load(r, total, t, rv);
    SpinorIO<P,3>::load(Ap, total, t, av);
#pragma unroll
    for(int c=0; c<3; c++) {
      rv[c].r = fma(t0, av[c].r, rv[c].r); rv[c].i = fma(t0, av[c].i, rv[c].i);
    }
    acc.norm(rv);
    SpinorIO<P,3>::store(r, total, t, rv);
  }
  double red[1] = {acc.get()};
  double rsq = 0;
  double *res[1] = {&s->pkp};   // scratch slot for the sum
  if(grid_reduce<1>(red, 1, 0, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      rsq = s->pkp;
      s->rsq = rsq;
      if((s->iteration >= s->itnlim) || (s->rsqstop <= 0 || rsq < s->rsqstop)) {
        s->done = 1;
      } else {
        s->a[0] = rsq/s->oldrsq;                   // lib/cgms.c:130-135
        for(int i=1; i<n; i++) {
          double c2 = s->z[i]*s->b[0];
          if(c2 != 0.0) s->a[i] = s->a[0]*s->zn[i]*s->b[i]/c2;
          else s->a[i] = 0;
        }
      }
    }
  }
}

template <int P>
__global__ void cgms_p_k(void *ps, const void *r, int nsites, size_t fs, qllg_cgms_scalars *s)
{
  typedef typename Calc<P,P>::T T;
  __shared__ T ca[QLLG_MAXSHIFT], cz[QLLG_MAXSHIFT];
  __shared__ int live[QLLG_MAXSHIFT];
  if(*(volatile int *)&s->done) return;
  const int n = s->n;
  for(int i=threadIdx.x; i<n; i+=blockDim.x) {
    ca[i] = (T)s->a[i]; cz[i] = (T)s->zn[i]; live[i] = (i == 0) || (s->s[i] != 0);
  }
  __syncthreads();
  const size_t total = (size_t)nsites;
  GRID_LOOP(t, total) {
    Cx<T> rv[3], pv[3];
    SpinorIO<P,3>::load(r, total, t, rv);
    for(int i=0; i<n; i++) {
      if(!live[i]) continue;
      void *pi = (char *)ps + fs*i;
      SpinorIO<P,3>::load(pi, total, t, pv);
      if(i == 0) {
#pragma unroll
        for(int c=0; c<3; c++) { pv[c].r = fma(ca[0], pv[c].r, rv[c].r); pv[c].i = fma(ca[0], pv[c].i, rv[c].i); }
      } else {
#pragma unroll
        for(int c=0; c<3; c++) {
          T tr = cz[i]*rv[c].r, ti = cz[i]*rv[c].i;
          pv[c].r = fma(ca[i], pv[c].r, tr); pv[c].i = fma(ca[i], pv[c].i, ti);
        }
      }
      SpinorIO<P,3>::store(pi, total, t, pv);
    }
  }
}

// ------------------------------------------------ many rhs at once (FP32)
// The vectors are FP32 fields [3][nsites][NR] (one per shift for p and the
// solutions); every rhs column keeps its own recurrence, in FP64, exactly
// as the single-rhs kernels above do for one.
__global__ void mcgms_pre_k(qllg_mcgms_scalars *s)
{
  const int r = threadIdx.x;
  if(r >= s->nr || s->done || !s->active[r]) return;
  if(s->iteration[r] > 0) {
    for(int i=0; i<s->n; i++) {
      s->bo[r][i] = s->b[r][i];
      s->zo[r][i] = s->z[r][i];
      s->z[r][i] = s->zn[r][i];
    }
  }
  s->oldrsq[r] = s->rsq[r];
}

__global__ void mcgms_coef_k(qllg_mcgms_scalars *s)
{
  const int r = threadIdx.x;
  if(r >= s->nr || s->done || !s->active[r]) return;
  s->iteration[r]++;
  const double pkp = s->mass2[r]*s->pnorm[r] + s->vnorm[r];
  if(pkp <= 0) { s->active[r] = 0; return; }
  const double b0 = s->rsq[r]/pkp;
  s->b[r][0] = b0;
  s->zn[r][0] = 1;
  for(int i=1; i<s->n; i++) {
    double zn = s->z[r][i]*s->zo[r][i]*s->bo[r][0];
    double c1 = b0*s->a[r][0]*(s->zo[r][i] - s->z[r][i]);
    c1 += s->zo[r][i]*s->bo[r][0]*(1 + s->shifts[i]*b0);
    zn = c1 != 0.0 ? zn/c1 : 0;
    s->zn[r][i] = zn;
    s->b[r][i] = s->z[r][i] != 0.0 ? b0*zn/s->z[r][i] : 0;
    if(s->z[r][i] == 0.0) s->zn[r][i] = 0;
  }
}

template <int NR>
__global__ void __launch_bounds__(kT)
mcgms_xr_k(void *out, void *r, const void *ps, const void *Ap, int nsites, size_t fs,
           qllg_mcgms_scalars *s, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  if(*(volatile int *)&s->done) return;
  const int rhs = threadIdx.x % NR, n = s->n;
  const size_t total = (size_t)nsites*NR;
  Acc<float> acc;
  if(s->active[rhs]) {
    const float t0 = -(float)s->b[rhs][0];
    GRID_LOOP(t, total) {
      Cx<float> pv[3], ov[3];
      for(int i=0; i<n; i++) {
        const float ci = (float)s->b[rhs][i];
        const void *pi = (const char *)ps + fs*i;
        void *oi = (char *)out + fs*i;
        SpinorIO<QLLG_F32,3>::load(pi, total, t, pv);
        SpinorIO<QLLG_F32,3>::load(oi, total, t, ov);
#pragma unroll
        for(int c=0; c<3; c++) { ov[c].r = fmaf(ci, pv[c].r, ov[c].r); ov[c].i = fmaf(ci, pv[c].i, ov[c].i); }
        SpinorIO<QLLG_F32,3>::store(oi, total, t, ov);
      }
      Cx<float> rv[3], av[3];
      SpinorIO<QLLG_F32,3>::load(r, total, t, rv);
      SpinorIO<QLLG_F32,3>::load(Ap, total, t, av);
#pragma unroll
      for(int c=0; c<3; c++) { rv[c].r = fmaf(t0, av[c].r, rv[c].r); rv[c].i = fmaf(t0, av[c].i, rv[c].i); }
      acc.norm(rv);
      SpinorIO<QLLG_F32,3>::store(r, total, t, rv);
    }
  }
  double red[1] = {acc.get()};
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<s->nr; q++) {
        if(!s->active[q]) continue;
        const double rsq = s->tmp[q];
        s->rsq[q] = rsq;
        if(s->iteration[q] >= s->itnlim || rsq < s->rsqstop[q]) {
          s->active[q] = 0;
        } else {
          s->a[q][0] = rsq/s->oldrsq[q];                   // lib/cgms.c:130-135
          for(int i=1; i<n; i++) {
            const double c2 = s->z[q][i]*s->b[q][0];
            s->a[q][i] = c2 != 0.0 ? s->a[q][0]*s->zn[q][i]*s->b[q][i]/c2 : 0;
          }
          any = 1;
        }
      }
      s->done = !any;
    }
  }
}

template <int NR>
__global__ void mcgms_p_k(void *ps, const void *r, int nsites, size_t fs, qllg_mcgms_scalars *s)
{
  if(*(volatile int *)&s->done) return;
  const int rhs = threadIdx.x % NR, n = s->n;
  if(!s->active[rhs]) return;
  const size_t total = (size_t)nsites*NR;
  GRID_LOOP(t, total) {
    Cx<float> rv[3], pv[3];
    SpinorIO<QLLG_F32,3>::load(r, total, t, rv);
    for(int i=0; i<n; i++) {
      void *pi = (char *)ps + fs*i;
      const float ca = (float)s->a[rhs][i], cz = (float)s->zn[rhs][i];
      SpinorIO<QLLG_F32,3>::load(pi, total, t, pv);
      if(i == 0) {
#pragma unroll
        for(int c=0; c<3; c++) { pv[c].r = fmaf(ca, pv[c].r, rv[c].r); pv[c].i = fmaf(ca, pv[c].i, rv[c].i); }
      } else {
#pragma unroll
        for(int c=0; c<3; c++) {
          const float tr = cz*rv[c].r, ti = cz*rv[c].i;
          pv[c].r = fmaf(ca, pv[c].r, tr); pv[c].i = fmaf(ca, pv[c].i, ti);
        }
      }
      SpinorIO<QLLG_F32,3>::store(pi, total, t, pv);
    }
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

int grid_for(size_t total, qllg_redbuf *rb)
{
  size_t g = (total + kT - 1)/kT, m = (size_t)qllg_num_sms()*8;
  if(g > m) g = m;
  if(rb && g > (size_t)rb->maxblocks) g = rb->maxblocks;
  return g < 1 ? 1 : (int)g;
}

int done(const char *w) { return qllg_launched(w); }

} // namespace

extern "C" int
qllg_k_cgms_pre(qllg_cgms_scalars *s)
{
  cgms_pre_k<<<1, 32, 0, qllg_stream()>>>(s);
  return done("cgms_pre");
}

extern "C" int
qllg_k_cgms_coef(qllg_cgms_scalars *s)
{
  cgms_coef_k<<<1, 32, 0, qllg_stream()>>>(s);
  return done("cgms_coef");
}

extern "C" int
qllg_k_cgms_update_xr(int prec, void *out, void *r, const void *ps, const void *Ap, int nsites,
                      qllg_cgms_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites, rb);
  if(prec == QLLG_F64)
    cgms_xr_k<QLLG_F64><<<g, kT, 0, qllg_stream()>>>(out, r, ps, Ap, nsites, qllg_spinor_bytes(prec, 3)*(size_t)nsites, s, rb->partial, rb->counter);
  else if(prec == QLLG_F32)
    cgms_xr_k<QLLG_F32><<<g, kT, 0, qllg_stream()>>>(out, r, ps, Ap, nsites, qllg_spinor_bytes(prec, 3)*(size_t)nsites, s, rb->partial, rb->counter);
  else { qllg_set_error("cgms: precision %d", prec); return -1; }
  return done("cgms_update_xr");
}

extern "C" int
qllg_k_cgms_update_p(int prec, void *ps, const void *r, int nsites, qllg_cgms_scalars *s)
{
  int g = grid_for((size_t)nsites, 0);
  if(prec == QLLG_F64) cgms_p_k<QLLG_F64><<<g, kT, 0, qllg_stream()>>>(ps, r, nsites, qllg_spinor_bytes(prec, 3)*(size_t)nsites, s);
  else if(prec == QLLG_F32) cgms_p_k<QLLG_F32><<<g, kT, 0, qllg_stream()>>>(ps, r, nsites, qllg_spinor_bytes(prec, 3)*(size_t)nsites, s);
  else { qllg_set_error("cgms: precision %d", prec); return -1; }
  return done("cgms_update_p");
}

extern "C" int
qllg_k_mcgms_pre(qllg_mcgms_scalars *s)
{
  mcgms_pre_k<<<1, QLLG_MAXRHS, 0, qllg_stream()>>>(s);
  return done("mcgms_pre");
}

extern "C" int
qllg_k_mcgms_coef(qllg_mcgms_scalars *s)
{
  mcgms_coef_k<<<1, QLLG_MAXRHS, 0, qllg_stream()>>>(s);
  return done("mcgms_coef");
}

extern "C" int
qllg_k_mcgms_update_xr(void *out, void *r, const void *ps, const void *Ap, int nsites, int nr,
                       size_t fs, qllg_mcgms_scalars *s, qllg_redbuf *rb)
{
  int g = grid_for((size_t)nsites*nr, rb);
  NR_SWITCH(nr, (mcgms_xr_k<NR><<<g, kT, 0, qllg_stream()>>>(out, r, ps, Ap, nsites, fs, s,
                                                             rb->partial, rb->counter)));
  return done("mcgms_update_xr");
}

extern "C" int
qllg_k_mcgms_update_p(void *ps, const void *r, int nsites, int nr, size_t fs, qllg_mcgms_scalars *s)
{
  int g = grid_for((size_t)nsites*nr, 0);
  NR_SWITCH(nr, (mcgms_p_k<NR><<<g, kT, 0, qllg_stream()>>>(ps, r, nsites, fs, s)));
  return done("mcgms_update_p");
}
