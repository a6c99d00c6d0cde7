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
