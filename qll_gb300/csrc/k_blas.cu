// k_blas.cu -- streaming vector kernels of the solvers (sm_103a):
// layout transposes between the reference's host layout and the device
// layout, precision conversion, axpby, norms with the deterministic grid
// reduction, and the fused CG update steps of cgSolveT (lib/cg.c:77-115).
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kT = 256;

size_t g_max_grid = 0;

int grid_for(size_t total, const void *fn, qllg_redbuf *rb)
{
  (void)fn;
  if(!g_max_grid) g_max_grid = (size_t)qllg_num_sms()*8;
  size_t need = (total + kT - 1)/kT;
  size_t g = need < g_max_grid ? need : g_max_grid;
  if(rb && g > (size_t)rb->maxblocks) g = rb->maxblocks;
  return g < 1 ? 1 : (int)g;
}

#define GRID_LOOP(t, total) \
  for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < (total); \
      t += (size_t)gridDim.x*blockDim.x)

// ------------------------------------------------------------ transposes
template <int P, int NC, typename S>
__global__ void from_aos(void *dev, const S *stage, int nsites, int nrhs, size_t rstride)
{
  typedef typename Real<P>::T T;
  size_t total = (size_t)nsites*nrhs;
  GRID_LOOP(t, total) {
    int site = (int)(t / nrhs), rhs = (int)(t % nrhs);
    const S *src = stage + rhs*rstride + (size_t)site*2*NC;
    Cx<T> v[NC];
#pragma unroll
    for(int c=0; c<NC; c++) { v[c].r = (T)src[2*c]; v[c].i = (T)src[2*c+1]; }
    SpinorIO<P,NC>::store(dev, total, t, v);
  }
}

// The same for three colours and several rhs, through shared memory: a
// block takes 32 sites, reads each rhs's 32 sites as one contiguous run and
// writes each colour's 32 x NR complex values as one contiguous run.  (The
// plain kernel's warps read from NR host blocks at once, which measured 25
// GB/s for 16 rhs at 32^3x64.)
template <int P, typename S, int NR>
__global__ void __launch_bounds__(kT)
from_aos3_tiled(void *dev, const S *stage, int nsites, size_t rstride)
{
  typedef typename Real<P>::T T;
  constexpr int TS = 32, W = 6*TS + 1;          // reals per rhs in the tile, padded
  __shared__ S tile[NR*W];
  const size_t total = (size_t)nsites*NR;
  for(int s0 = blockIdx.x*TS; s0 < nsites; s0 += gridDim.x*TS) {
    const int ns = nsites - s0 < TS ? nsites - s0 : TS;
    for(int e = threadIdx.x; e < NR*6*TS; e += blockDim.x) {
      const int r = e/(6*TS), k = e % (6*TS);
      if(k < 6*ns) tile[r*W + k] = stage[r*rstride + (size_t)s0*6 + k];
    }
    __syncthreads();
    for(int e = threadIdx.x; e < 3*TS*NR; e += blockDim.x) {
      const int c = e/(TS*NR), rem = e % (TS*NR), si = rem/NR, r = rem % NR;
      if(si < ns) {
        Cx<T> v;
        v.r = (T)tile[r*W + 6*si + 2*c];
        v.i = (T)tile[r*W + 6*si + 2*c + 1];
        SpinorIO<P,1>::store(dev, 0, c*total + (size_t)(s0 + si)*NR + r, &v);
      }
    }
    __syncthreads();
  }
}

template <int P, int NC, typename S>
__global__ void to_aos(const void *dev, S *stage, int nsites, int nrhs, size_t rstride)
{
  typedef typename Calc<P,P>::T T;
  size_t total = (size_t)nsites*nrhs;
  GRID_LOOP(t, total) {
    int site = (int)(t / nrhs), rhs = (int)(t % nrhs);
    S *dst = stage + rhs*rstride + (size_t)site*2*NC;
    Cx<T> v[NC];
    SpinorIO<P,NC>::load(dev, total, t, v);
#pragma unroll
    for(int c=0; c<NC; c++) { dst[2*c] = (S)v[c].r; dst[2*c+1] = (S)v[c].i; }
  }
}

// site order and matrix convention of an embedding code (QDP/QLA or MILC)
// <-> the reference's one-lane order: foreign site s is QLL site perm[s]
// (identity when perm is NULL); with transpose, n = 18 reals are a 3x3
// complex matrix stored row-major (entry 3*row + col), the reference's
// being column-major (packM/unpackM's transpose, qopstag.c:123-196)
__global__ void aos_from_foreign_k(double *out, const double *in, const int *perm, int V, int n,
                                   int transpose)
{
  for(size_t s = (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < (size_t)V;
      s += (size_t)gridDim.x*blockDim.x) {
    const size_t q = perm ? (size_t)perm[s] : s;
    const double *src = in + s*n;
    double *dst = out + q*n;
    if(transpose) {
#pragma unroll
      for(int r=0; r<3; r++)
#pragma unroll
        for(int c=0; c<3; c++) {
          dst[2*(3*c + r)] = src[2*(3*r + c)];
          dst[2*(3*c + r) + 1] = src[2*(3*r + c) + 1];
        }
    } else {
      for(int e=0; e<n; e++) dst[e] = src[e];
    }
  }
}

__global__ void aos_to_foreign_k(double *out, const double *in, const int *perm, int V, int n)
{
  for(size_t s = (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < (size_t)V;
      s += (size_t)gridDim.x*blockDim.x) {
    const size_t q = perm ? (size_t)perm[s] : s;
    for(int e=0; e<n; e++) out[s*n + e] = in[q*n + e];
  }
}

// one column (rhs col of nrhs) of an FP64 device vector <-> a contiguous
// [nsites][6] double array (the continuous-batching solver moves requests
// in and out of single columns while the others keep running)
__global__ void column_from_aos_k(void *dev, const double *stage, int nsites, int nrhs, int col)
{
  const size_t total = (size_t)nsites*nrhs;
  for(size_t s = (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < (size_t)nsites;
      s += (size_t)gridDim.x*blockDim.x) {
    Cx<double> v[3];
#pragma unroll
    for(int c=0; c<3; c++) { v[c].r = stage[6*s + 2*c]; v[c].i = stage[6*s + 2*c + 1]; }
    SpinorIO<QLLG_F64,3>::store(dev, total, s*nrhs + col, v);
  }
}

__global__ void column_to_aos_k(const void *dev, double *stage, int nsites, int nrhs, int col)
{
  const size_t total = (size_t)nsites*nrhs;
  for(size_t s = (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < (size_t)nsites;
      s += (size_t)gridDim.x*blockDim.x) {
    Cx<double> v[3];
    SpinorIO<QLLG_F64,3>::load(dev, total, s*nrhs + col, v);
#pragma unroll
    for(int c=0; c<3; c++) { stage[6*s + 2*c] = v[c].r; stage[6*s + 2*c + 1] = v[c].i; }
  }
}

// column jd of an [3][nsites][nd] field (precision PD) = column js of an
// [3][nsites][ns] field (precision PS)
template <int PD, int PSRC>
__global__ void column_copy_k(void *dst, int nd, int jd, const void *src, int ns, int js, int nsites)
{
  typedef typename Calc<PD,PSRC>::T T;
  for(size_t s = (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < (size_t)nsites;
      s += (size_t)gridDim.x*blockDim.x) {
    Cx<T> v[3];
    SpinorIO<PSRC,3>::load(src, (size_t)nsites*ns, s*ns + js, v);
    SpinorIO<PD,3>::store(dst, (size_t)nsites*nd, s*nd + jd, v);
  }
}

// a chunk of a graph-captured solver loop: at most n more trips
__global__ void chunk_limit_k(int *loops, int *limit, int n)
{
  if(threadIdx.x == 0 && blockIdx.x == 0) *limit = *loops + n;
}

template <int PO, int PI, int NC>
__global__ void convert_k(void *out, const void *in, int nsites, int nrhs, const int *active)
{
  typedef typename Calc<PO,PI>::T T;
  size_t total = (size_t)nsites*nrhs;
  GRID_LOOP(t, total) {
    if(active && !active[t % nrhs]) continue;
    Cx<T> v[NC];
    SpinorIO<PI,NC>::load(in, total, t, v);
    SpinorIO<PO,NC>::store(out, total, t, v);
  }
}

// --------------------------------------------------------------- links
template <typename S>
__global__ void link_maxabs(const S *stage, int V, unsigned *mx)
{
  float m = 0.f;
  size_t total = (size_t)V*18;
  GRID_LOOP(t, total) m = fmaxf(m, fabsf((float)stage[t]));
  for(int o=16; o>0; o>>=1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

template <int P, typename S>
__global__ void link_from_aos(void *dev, const float *scale, const S *stage, int V)
{
  GRID_LOOP(i, (size_t)V) {
    const S *m = stage + i*18;
    if(P == QLLG_F64) {
      double2 *d = (double2 *)dev;
#pragma unroll
      for(int k=0; k<9; k++) d[k*(size_t)V + i] = make_double2((double)m[2*k], (double)m[2*k+1]);
    } else if(P == QLLG_F32) {
      float2 *d = (float2 *)dev;
#pragma unroll
      for(int k=0; k<9; k++) d[k*(size_t)V + i] = make_float2((float)m[2*k], (float)m[2*k+1]);
    } else {
      float s = *scale;
      float inv = s > 0.f ? 32767.0f/s : 0.f;
      uint32_t w[9];
#pragma unroll
      for(int k=0; k<9; k++) w[k] = pack_s16((float)m[2*k]*inv, (float)m[2*k+1]*inv);
      char *b = (char *)dev;
      ((int4 *)b)[i] = make_int4((int)w[0], (int)w[1], (int)w[2], (int)w[3]);
      ((int4 *)(b + 16*(size_t)V))[i] = make_int4((int)w[4], (int)w[5], (int)w[6], (int)w[7]);
      ((int *)(b + 32*(size_t)V))[i] = (int)w[8];
    }
  }
}

template <typename D2, typename S>
__global__ void link_to_aos(const void *dev, S *stage, int V)
{
  const D2 *d = (const D2 *)dev;
  GRID_LOOP(i, (size_t)V) {
    S *m = stage + i*18;
#pragma unroll
    for(int k=0; k<9; k++) { D2 t = d[k*(size_t)V + i]; m[2*k] = (S)t.x; m[2*k+1] = (S)t.y; }
  }
}

__global__ void link_f64_maxabs(const double *dev, int V, unsigned *mx)
{
  float m = 0.f;
  GRID_LOOP(t, (size_t)V*18) m = fmaxf(m, (float)fabs(dev[t]));
  for(int o=16; o>0; o>>=1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

template <int P>
__global__ void link_from_f64(void *dev, const float *scale, const double *in, int V)
{
  const double2 *d = (const double2 *)in;
  GRID_LOOP(i, (size_t)V) {
    double2 e[9];
#pragma unroll
    for(int k=0; k<9; k++) e[k] = d[k*(size_t)V + i];
    if(P == QLLG_F32) {
      float2 *o = (float2 *)dev;
#pragma unroll
      for(int k=0; k<9; k++) o[k*(size_t)V + i] = make_float2((float)e[k].x, (float)e[k].y);
    } else {
      float s = *scale;
      float inv = s > 0.f ? 32767.0f/s : 0.f;
      uint32_t w[9];
#pragma unroll
      for(int k=0; k<9; k++) w[k] = pack_s16((float)e[k].x*inv, (float)e[k].y*inv);
      char *b = (char *)dev;
      ((int4 *)b)[i] = make_int4((int)w[0], (int)w[1], (int)w[2], (int)w[3]);
      ((int4 *)(b + 16*(size_t)V))[i] = make_int4((int)w[4], (int)w[5], (int)w[6], (int)w[7]);
      ((int *)(b + 32*(size_t)V))[i] = (int)w[8];
    }
  }
}

// FP64 values -> double-float (hi, lo) pairs, value by value (links: a slot
// is 9 V complex entries, laid out as in FP64)
__global__ void to_df_k(float2 *out, const double *in, size_t n)
{
  GRID_LOOP(i, n) {
    const dfl d(in[i]);
    out[i] = make_float2(d.h, d.l);
  }
}

// FP64 spinor columns <-> double-float, for the rhs whose active[] entry is
// eq (any nonzero one when eq is 0, every rhs when active is NULL);
// nothing when *skip is set.  The conversion back may run in place.
template <int NR, bool TO>
__global__ void __launch_bounds__(kT)
spinor_df_k(void *out, const void *in, int nsites, int ncomp, const int *active, int eq,
            const int *skip)
{
  // threads over (component, site, k-th flagged rhs) only
  __shared__ int list[NR];
  __shared__ int nact_s;
  if(skip && *(volatile const int *)skip) return;          // uniform
  if(threadIdx.x == 0) {
    int n = 0;
    for(int r=0; r<NR; r++)
      if(!active || (active[r] && (!eq || active[r] == eq))) list[n++] = r;
    nact_s = n;
  }
  __syncthreads();
  const int nact = nact_s;
  if(!nact) return;
  const size_t work = (size_t)nsites*ncomp*nact;
  GRID_LOOP(w, work) {
    const size_t t = (w/nact)*NR + list[w % nact];
    if(TO) {
      const double2 d = ((const double2 *)in)[t];
      const dfl re(d.x), im(d.y);
      ((float4 *)out)[t] = make_float4(re.h, re.l, im.h, im.l);
    } else {
      const float4 q = ((const float4 *)in)[t];
      ((double2 *)out)[t] = make_double2((double)q.x + (double)q.y, (double)q.z + (double)q.w);
    }
  }
}

// FP64 slot -> reconstruct-12 FP32 (see LinkR): the Naik rows are rounded
// to FP32 first and row 2 rebuilt from the rounded rows exactly as the
// Dslash rebuilds it; the sign is the one that matches the stored row 2,
// and a link whose row 2 does not follow from rows 0, 1 (not c W with W in
// SU(3)) raises *bad
__global__ void link_to_f32r_k(char *out, const double *in, int V, int naik, unsigned char *signs,
                               int bit, int *bad)
{
  const double2 *d = (const double2 *)in;
  GRID_LOOP(i, (size_t)V) {
    Cx<float> m[9];
    double2 e[9];
#pragma unroll
    for(int k=0; k<9; k++) { e[k] = d[k*(size_t)V + i]; m[k].r = (float)e[k].x; m[k].i = (float)e[k].y; }
    if(!naik) {
      float4 *q = (float4 *)out;
#pragma unroll
      for(int k=0; k<4; k++)
        q[k*(size_t)V + i] = make_float4(m[2*k].r, m[2*k].i, m[2*k + 1].r, m[2*k + 1].i);
      ((float2 *)(out + 64*(size_t)V))[i] = make_float2(m[8].r, m[8].i);
      continue;
    }
    float4 *q = (float4 *)out;
    q[i] = make_float4(m[0].r, m[0].i, m[3].r, m[3].i);
    q[(size_t)V + i] = make_float4(m[6].r, m[6].i, m[1].r, m[1].i);
    q[2*(size_t)V + i] = make_float4(m[4].r, m[4].i, m[7].r, m[7].i);
    Cx<float> r[9];
#pragma unroll
    for(int k=0; k<9; k++) r[k] = m[k];
    LinkR::rebuild_row2(r, false);
    double dot = 0, n2 = 0, err = 0;
#pragma unroll
    for(int c=0; c<3; c++) {
      dot += e[3*c + 2].x*r[3*c + 2].r + e[3*c + 2].y*r[3*c + 2].i;
      n2 += e[3*c + 2].x*e[3*c + 2].x + e[3*c + 2].y*e[3*c + 2].y;
    }
    const bool neg = dot < 0;
#pragma unroll
    for(int c=0; c<3; c++) {
      const double xr = (neg ? -r[3*c + 2].r : r[3*c + 2].r) - e[3*c + 2].x;
      const double xi = (neg ? -r[3*c + 2].i : r[3*c + 2].i) - e[3*c + 2].y;
      err += xr*xr + xi*xi;
    }
    if(!(err <= 1e-10*n2)) atomicOr(bad, 1);       // relative 1e-5
    unsigned char sgn = bit ? signs[i] : 0;
    signs[i] = (unsigned char)(sgn | ((neg ? 1 : 0) << bit));
  }
}

// ------------------------------------------------------------ axpby/norm
template <int PY, int PX, int NC, int NR>
__global__ void axpby_k(void *y, const void *x, const double *a, double a0,
                        const double *b, double b0, int nsites, const int *active)
{
  typedef typename Calc<PY,PX>::T T;
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(active && !active[rhs]) return;
  const T ca = (T)(a ? a[rhs] : a0), cb = (T)(b ? b[rhs] : b0);
  GRID_LOOP(t, total) {
    Cx<T> yv[NC], xv[NC];
    SpinorIO<PX,NC>::load(x, total, t, xv);
    if(ca != (T)0) {
      SpinorIO<PY,NC>::load(y, total, t, yv);
#pragma unroll
      for(int c=0; c<NC; c++) { yv[c].r = fma(cb, xv[c].r, ca*yv[c].r); yv[c].i = fma(cb, xv[c].i, ca*yv[c].i); }
    } else {
#pragma unroll
      for(int c=0; c<NC; c++) { yv[c].r = cb*xv[c].r; yv[c].i = cb*xv[c].i; }
    }
    SpinorIO<PY,NC>::store(y, total, t, yv);
  }
}

// y = y + b x, the exact form of X_veq_X_plus_r_times_X (lib/vla.c:767-786)
template <int P, int NC, int NR>
__global__ void xpay_k(void *y, const void *x, const double *b, double b0, double bsign,
                       int nsites, const int *active)
{
  typedef typename Calc<P,P>::T T;
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(active && !active[rhs]) return;
  const T cb = (T)(bsign*(b ? b[rhs] : b0));
  GRID_LOOP(t, total) {
    Cx<T> yv[NC], xv[NC];
    SpinorIO<P,NC>::load(x, total, t, xv);
    SpinorIO<P,NC>::load(y, total, t, yv);
#pragma unroll
    for(int c=0; c<NC; c++) { yv[c].r = fma(cb, xv[c].r, yv[c].r); yv[c].i = fma(cb, xv[c].i, yv[c].i); }
    SpinorIO<P,NC>::store(y, total, t, yv);
  }
}

template <int P, int NC, int NR>
__global__ void __launch_bounds__(kT) norm2_k(const void *x, int nsites, double *out,
                                               double *partial, unsigned *counter)
{
  typedef typename Calc<P,P>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  double red[1] = {0};
  GRID_LOOP(t, total) {
    Cx<T> v[NC];
    SpinorIO<P,NC>::load(x, total, t, v);
#pragma unroll
    for(int c=0; c<NC; c++) red[0] += (double)v[c].r*v[c].r + (double)v[c].i*v[c].i;
  }
  double *res[1] = {out};
  grid_reduce<1>(red, NR, threadIdx.x % NR, partial, counter, shm, res);
}

// --------------------------------------------------------------- CG steps
template <int P, int NC, int NR>
__global__ void __launch_bounds__(kT) cg_init_k(void *x, void *r, void *p, const void *b,
                                                 int nsites, qllg_cg_scalars *s,
                                                 double *partial, unsigned *counter)
{
  typedef typename Calc<P,P>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  double red[1] = {0};
  GRID_LOOP(t, total) {
    Cx<T> v[NC], z[NC];
    SpinorIO<P,NC>::load(b, total, t, v);
#pragma unroll
    for(int c=0; c<NC; c++) { z[c].r = 0; z[c].i = 0; red[0] += (double)v[c].r*v[c].r + (double)v[c].i*v[c].i; }
    SpinorIO<P,NC>::store(r, total, t, v);
    SpinorIO<P,NC>::store(x, total, t, z);
    SpinorIO<P,NC>::store(p, total, t, z);
  }
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, threadIdx.x % NR, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        double bs = s->tmp[q];
        s->bsq[q] = bs;
        s->rsq[q] = bs;
        s->rsq_stop[q] *= bs;
        s->iters[q] = 0;
        s->active[q] = (bs > 0 && s->maxits > 0) ? 1 : 0;
        any |= s->active[q];
      }
      s->done = !any;
      s->count = 0;
    }
  }
}

template <int P, int NC, int NR>
__global__ void __launch_bounds__(kT) cg_xr_k(void *x, void *r, const void *p, const void *Ap,
                                               int nsites, qllg_cg_scalars *s,
                                               double *partial, unsigned *counter)
{
  typedef typename Calc<P,P>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  const bool skip = *(volatile int *)&s->done;
  Acc<T> acc;
  if(!skip && s->active[rhs]) {
    const T alpha = (T)(1.0/(s->mass2[rhs]*s->pnorm[rhs] + s->vnorm[rhs]));
    GRID_LOOP(t, total) {
      Cx<T> xv[NC], rv[NC], pv[NC], av[NC];
      SpinorIO<P,NC>::load(x, total, t, xv);
      SpinorIO<P,NC>::load(r, total, t, rv);
      SpinorIO<P,NC>::load(p, total, t, pv);
      SpinorIO<P,NC>::load(Ap, total, t, av);
#pragma unroll
      for(int c=0; c<NC; c++) {
        xv[c].r = fma(alpha, pv[c].r, xv[c].r); xv[c].i = fma(alpha, pv[c].i, xv[c].i);
        rv[c].r = fma(-alpha, av[c].r, rv[c].r); rv[c].i = fma(-alpha, av[c].i, rv[c].i);
      }
      acc.norm(rv);
      SpinorIO<P,NC>::store(x, total, t, xv);
      SpinorIO<P,NC>::store(r, total, t, rv);
    }
  }
  if(skip) return;   // uniform over the grid
  double red[1] = {acc.get()};
  double *res[1] = {s->tmp};
  if(grid_reduce<1>(red, NR, rhs, partial, counter, shm, res)) {
    __syncthreads();
    if(threadIdx.x == 0) {
      int any = 0;
      for(int q=0; q<NR; q++) {
        if(s->active[q]) {
          s->rsq[q] = s->tmp[q];
          s->iters[q]++;
          if(!(s->rsq[q] >= s->rsq_stop[q] && s->iters[q] < s->maxits)) s->active[q] = 0;
        }
        any |= s->active[q];
      }
      s->done = !any;
      s->count++;
    }
  }
}

template <int P, int NC, int NR>
__global__ void cg_p_k(void *p, const void *r, int nsites, qllg_cg_scalars *s)
{
  typedef typename Calc<P,P>::T T;
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->done || !s->active[rhs]) return;
  const T beta = (T)(1.0/s->rsq[rhs]);
  GRID_LOOP(t, total) {
    Cx<T> pv[NC], rv[NC];
    SpinorIO<P,NC>::load(p, total, t, pv);
    SpinorIO<P,NC>::load(r, total, t, rv);
#pragma unroll
    for(int c=0; c<NC; c++) { pv[c].r = fma(beta, rv[c].r, pv[c].r); pv[c].i = fma(beta, rv[c].i, pv[c].i); }
    SpinorIO<P,NC>::store(p, total, t, pv);
  }
}

template <int P, int NR>
__global__ void __launch_bounds__(kT)
cg_p_norm_k(void *p, const void *r, int nsites, qllg_cg_scalars *s, double *partial,
            unsigned *counter)
{
  typedef typename Calc<P,P>::T T;
  __shared__ double shm[kT];
  size_t total = (size_t)nsites*NR;
  const int rhs = threadIdx.x % NR;
  if(*(volatile int *)&s->done) return;        // uniform
  Acc<T> acc;
  if(s->active[rhs]) {
    const T beta = (T)(1.0/s->rsq[rhs]);
    GRID_LOOP(t, total) {
      Cx<T> pv[3], rv[3];
      SpinorIO<P,3>::load(p, total, t, pv);
      SpinorIO<VecPrec<P>::value,3>::load(r, total, t, rv);
#pragma unroll
      for(int c=0; c<3; c++) {
        pv[c].r = fma(beta, rv[c].r, pv[c].r); pv[c].i = fma(beta, rv[c].i, pv[c].i);
      }
      SpinorIO<P,3>::store(p, total, t, pv);
      acc.norm(pv);
    }
  }
  double red[1] = {acc.get()};
  double *res[1] = {s->pnorm};
  grid_reduce<1>(red, NR, rhs, partial, counter, shm, res);
}

// ---------------------------------------------------------- dispatch
#define NR_SWITCH(nrhs, ...) \
  switch(nrhs) { \
  case 1: { constexpr int NR = 1; __VA_ARGS__; } break; \
  case 2: { constexpr int NR = 2; __VA_ARGS__; } break; \
  case 4: { constexpr int NR = 4; __VA_ARGS__; } break; \
  case 8: { constexpr int NR = 8; __VA_ARGS__; } break; \
  case 16: { constexpr int NR = 16; __VA_ARGS__; } break; \
  default: qllg_set_error("nrhs %d not in {1,2,4,8,16}", nrhs); return -1; }

// precision x colour count for kernels on one field type
#define PN_SWITCH(prec, ncomp, ...) \
  if(prec == QLLG_F64 && ncomp == 3) { constexpr int P = QLLG_F64, NC = 3; __VA_ARGS__; } \
  else if(prec == QLLG_F32 && ncomp == 3) { constexpr int P = QLLG_F32, NC = 3; __VA_ARGS__; } \
  else if(prec == QLLG_I16 && ncomp == 3) { constexpr int P = QLLG_I16, NC = 3; __VA_ARGS__; } \
  else if(prec == QLLG_F64 && ncomp == 12) { constexpr int P = QLLG_F64, NC = 12; __VA_ARGS__; } \
  else if(prec == QLLG_F32 && ncomp == 12) { constexpr int P = QLLG_F32, NC = 12; __VA_ARGS__; } \
  else { qllg_set_error("unsupported precision %d / components %d", prec, ncomp); return -1; }

int done(const char *what) { return qllg_launched(what); }
} // namespace
static int done_check(const char *w) { return qllg_launched(w); }
namespace {

} // namespace

extern "C" int
qllg_k_spinor_from_aos(int prec, void *dev, const void *stage, int dbl, int nsites, int ncomp,
                       int nrhs, size_t rs)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
  if(ncomp == 3 && nrhs > 1 && (prec == QLLG_F64 || prec == QLLG_F32)) {
    const int gt = grid_for((size_t)nsites*(kT/32), 0, 0);    // 32 sites per block
#define FT(P_) \
    if(dbl) { NR_SWITCH(nrhs, (from_aos3_tiled<P_,double,NR><<<gt,kT,0,st>>>(dev, (const double *)stage, nsites, rs))); } \
    else { NR_SWITCH(nrhs, (from_aos3_tiled<P_,float,NR><<<gt,kT,0,st>>>(dev, (const float *)stage, nsites, rs))); }
    if(prec == QLLG_F64) { FT(QLLG_F64) } else { FT(QLLG_F32) }
#undef FT
    return done("from_aos");
  }
  PN_SWITCH(prec, ncomp, {
    if(dbl) from_aos<P,NC,double><<<g,kT,0,st>>>(dev, (const double *)stage, nsites, nrhs, rs);
    else from_aos<P,NC,float><<<g,kT,0,st>>>(dev, (const float *)stage, nsites, nrhs, rs);
  });
  return done("from_aos");
}

extern "C" int
qllg_k_spinor_to_aos(int prec, const void *dev, void *stage, int dbl, int nsites, int ncomp,
                     int nrhs, size_t rs)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    if(dbl) to_aos<P,NC,double><<<g,kT,0,st>>>(dev, (double *)stage, nsites, nrhs, rs);
    else to_aos<P,NC,float><<<g,kT,0,st>>>(dev, (float *)stage, nsites, nrhs, rs);
  });
  return done("to_aos");
}

extern "C" int
qllg_k_aos_from_foreign(double *out, const double *in, const int *perm, int V, int n, int transpose)
{
  if(transpose && n != 18) { qllg_set_error("aos_from_foreign: transpose needs 18 reals"); return -1; }
  aos_from_foreign_k<<<grid_for((size_t)V, 0, 0), kT, 0, qllg_stream()>>>(out, in, perm, V, n,
                                                                          transpose);
  return done("aos_from_foreign");
}

extern "C" int
qllg_k_aos_to_foreign(double *out, const double *in, const int *perm, int V, int n)
{
  aos_to_foreign_k<<<grid_for((size_t)V, 0, 0), kT, 0, qllg_stream()>>>(out, in, perm, V, n);
  return done("aos_to_foreign");
}

extern "C" int
qllg_k_column_from_aos(void *dev, const double *stage, int nsites, int nrhs, int col)
{
  column_from_aos_k<<<grid_for((size_t)nsites, 0, 0), kT, 0, qllg_stream()>>>(dev, stage, nsites,
                                                                              nrhs, col);
  return done("column_from_aos");
}

extern "C" int
qllg_k_column_to_aos(const void *dev, double *stage, int nsites, int nrhs, int col)
{
  column_to_aos_k<<<grid_for((size_t)nsites, 0, 0), kT, 0, qllg_stream()>>>(dev, stage, nsites,
                                                                            nrhs, col);
  return done("column_to_aos");
}

extern "C" int
qllg_k_column_copy(int pd, void *dst, int nd, int jd, int psrc, const void *src, int ns, int js,
                   int nsites)
{
  const int g = grid_for((size_t)nsites, 0, 0);
  cudaStream_t st = qllg_stream();
#define CC(A,B) if(pd == A && psrc == B) { \
    column_copy_k<A,B><<<g,kT,0,st>>>(dst, nd, jd, src, ns, js, nsites); \
    return done("column_copy"); }
  CC(QLLG_F64, QLLG_F64) CC(QLLG_F64, QLLG_F32) CC(QLLG_F32, QLLG_F64) CC(QLLG_F32, QLLG_F32)
#undef CC
  qllg_set_error("column_copy: precisions %d/%d", pd, psrc);
  return -1;
}

extern "C" int
qllg_k_chunk_limit(int *loops, int *limit, int n)
{
  chunk_limit_k<<<1, 32, 0, qllg_stream()>>>(loops, limit, n);
  return done("chunk_limit");
}

extern "C" int
qllg_k_spinor_convert(int po, void *out, int pi, const void *in, int nsites, int ncomp,
                      int nrhs, const int *active)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
#define CONV(A,B) if(po == A && pi == B) { \
    if(ncomp == 3) convert_k<A,B,3><<<g,kT,0,st>>>(out, in, nsites, nrhs, active); \
    else if(ncomp == 12 && A != QLLG_I16 && B != QLLG_I16) \
      convert_k<(A==QLLG_I16?QLLG_F32:A),(B==QLLG_I16?QLLG_F32:B),12><<<g,kT,0,st>>>(out, in, nsites, nrhs, active); \
    else { qllg_set_error("convert: components %d", ncomp); return -1; } \
    return done("convert"); }
  CONV(QLLG_F64, QLLG_F64) CONV(QLLG_F64, QLLG_F32) CONV(QLLG_F64, QLLG_I16)
  CONV(QLLG_F32, QLLG_F64) CONV(QLLG_F32, QLLG_F32) CONV(QLLG_F32, QLLG_I16)
  CONV(QLLG_I16, QLLG_F64) CONV(QLLG_I16, QLLG_F32) CONV(QLLG_I16, QLLG_I16)
#undef CONV
  qllg_set_error("convert: precisions %d <- %d", po, pi);
  return -1;
}

extern "C" int
qllg_k_link_from_aos(int prec, void *dev, float *scale, const void *stage, int dbl, int V)
{
  cudaStream_t st = qllg_stream();
  int g = grid_for((size_t)V, 0, 0);
  if(prec == QLLG_I16) {
    if(qllg_check_cuda(cudaMemsetAsync(scale, 0, sizeof(float), st), "memset")) return -1;
    int g2 = grid_for((size_t)V*18, 0, 0);
    if(dbl) link_maxabs<double><<<g2,kT,0,st>>>((const double *)stage, V, (unsigned *)scale);
    else link_maxabs<float><<<g2,kT,0,st>>>((const float *)stage, V, (unsigned *)scale);
  }
#define LF(P) if(prec == P) { \
    if(dbl) link_from_aos<P,double><<<g,kT,0,st>>>(dev, scale, (const double *)stage, V); \
    else link_from_aos<P,float><<<g,kT,0,st>>>(dev, scale, (const float *)stage, V); \
    return done("link_from_aos"); }
  LF(QLLG_F64) LF(QLLG_F32) LF(QLLG_I16)
#undef LF
  qllg_set_error("link_from_aos: precision %d", prec);
  return -1;
}

extern "C" int
qllg_k_link_to_aos(int prec, const void *dev, void *stage, int dbl, int V)
{
  int g = grid_for((size_t)V, 0, 0);
  cudaStream_t st = qllg_stream();
  if(prec == QLLG_F64) {
    if(dbl) link_to_aos<double2,double><<<g,kT,0,st>>>(dev, (double *)stage, V);
    else link_to_aos<double2,float><<<g,kT,0,st>>>(dev, (float *)stage, V);
  } else if(prec == QLLG_F32) {
    if(dbl) link_to_aos<float2,double><<<g,kT,0,st>>>(dev, (double *)stage, V);
    else link_to_aos<float2,float><<<g,kT,0,st>>>(dev, (float *)stage, V);
  } else { qllg_set_error("link_to_aos: precision %d", prec); return -1; }
  return done("link_to_aos");
}

extern "C" int
qllg_k_link_convert(int prec, void *out, float *scale, const double *in, int V)
{
  cudaStream_t st = qllg_stream();
  int g = grid_for((size_t)V, 0, 0);
  if(prec == QLLG_F32) {
    link_from_f64<QLLG_F32><<<g,kT,0,st>>>(out, scale, in, V);
  } else if(prec == QLLG_I16) {
    if(qllg_check_cuda(cudaMemsetAsync(scale, 0, sizeof(float), st), "memset")) return -1;
    link_f64_maxabs<<<grid_for((size_t)V*18, 0, 0),kT,0,st>>>(in, V, (unsigned *)scale);
    link_from_f64<QLLG_I16><<<g,kT,0,st>>>(out, scale, in, V);
  } else if(prec == QLLG_DF) {
    to_df_k<<<grid_for((size_t)V*18, 0, 0),kT,0,st>>>((float2 *)out, in, (size_t)V*18);
  } else {
    qllg_set_error("link_convert: precision %d", prec);
    return -1;
  }
  return done("link_convert");
}

extern "C" int
qllg_k_spinor_df(int to_df, void *out, const void *in, int nsites, int ncomp, int nrhs,
                 const int *active, int eq, const int *skip)
{
  // sized for one flagged rhs: with more, the grid-stride loop takes them
  const int g = grid_for((size_t)nsites*ncomp, 0, 0);
  cudaStream_t st = qllg_stream();
  if(to_df) { NR_SWITCH(nrhs, (spinor_df_k<NR,true><<<g,kT,0,st>>>(out, in, nsites, ncomp, active, eq, skip))); }
  else { NR_SWITCH(nrhs, (spinor_df_k<NR,false><<<g,kT,0,st>>>(out, in, nsites, ncomp, active, eq, skip))); }
  return done("spinor_df");
}

extern "C" int
qllg_k_link_to_f32r(void *out, const double *in, int V, int naik, unsigned char *signs, int bit,
                    int *bad)
{
  link_to_f32r_k<<<grid_for((size_t)V, 0, 0), kT, 0, qllg_stream()>>>((char *)out, in, V, naik,
                                                                      signs, bit, bad);
  return done("link_to_f32r");
}

extern "C" int
qllg_k_axpby(int py, void *y, int px, const void *x, const double *a, double a0,
             const double *b, double b0, int nsites, int ncomp, int nrhs, const int *active)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
#define AX(A,B) if(py == A && px == B) { \
    if(ncomp == 3) { NR_SWITCH(nrhs, (axpby_k<A,B,3,NR><<<g,kT,0,st>>>(y, x, a, a0, b, b0, nsites, active))); } \
    else if(ncomp == 12 && A != QLLG_I16 && B != QLLG_I16) { \
      NR_SWITCH(nrhs, (axpby_k<(A==QLLG_I16?QLLG_F32:A),(B==QLLG_I16?QLLG_F32:B),12,NR><<<g,kT,0,st>>>(y, x, a, a0, b, b0, nsites, active))); } \
    else { qllg_set_error("axpby: components %d", ncomp); return -1; } \
    return done("axpby"); }
  AX(QLLG_F64, QLLG_F64) AX(QLLG_F64, QLLG_F32) AX(QLLG_F32, QLLG_F32)
  AX(QLLG_F32, QLLG_F64) AX(QLLG_I16, QLLG_I16) AX(QLLG_F32, QLLG_I16) AX(QLLG_I16, QLLG_F32)
#undef AX
  qllg_set_error("axpby: precisions %d <- %d", py, px);
  return -1;
}

extern "C" int
qllg_k_xpay(int prec, void *y, const void *x, const double *b, double b0, double bsign,
            int nsites, int ncomp, int nrhs, const int *active)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    NR_SWITCH(nrhs, (xpay_k<P,NC,NR><<<g,kT,0,st>>>(y, x, b, b0, bsign, nsites, active)));
  });
  return done("xpay");
}

extern "C" int
qllg_k_norm2(int prec, const void *x, int nsites, int ncomp, int nrhs, double *out,
             qllg_redbuf *rb)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, rb);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    NR_SWITCH(nrhs, (norm2_k<P,NC,NR><<<g,kT,0,st>>>(x, nsites, out, rb->partial, rb->counter)));
  });
  return done("norm2");
}

extern "C" int
qllg_k_zero(int prec, void *x, int nsites, int ncomp, int nrhs)
{
  /* all-zero bits are 0.0 in every storage format (the 16-bit one has a
   * zero scale); never read x, which may hold stale NaN patterns */
  size_t bytes = (prec == QLLG_I16 ? 16u : (prec == QLLG_F64 ? 16u : 8u)*ncomp)*(size_t)nsites*nrhs;
  return qllg_check_cuda(cudaMemsetAsync(x, 0, bytes, qllg_stream()), "zero");
}

extern "C" int
qllg_k_copy(int prec, void *y, const void *x, int nsites, int ncomp, int nrhs)
{
  return qllg_k_axpby(prec, y, prec, x, NULL, 0.0, NULL, 1.0, nsites, ncomp, nrhs, NULL);
}

extern "C" int
qllg_k_cg_init(int prec, void *x, void *r, void *p, const void *b, int nsites, int ncomp,
               int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, rb);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    NR_SWITCH(nrhs, (cg_init_k<P,NC,NR><<<g,kT,0,st>>>(x, r, p, b, nsites, s, rb->partial, rb->counter)));
  });
  return done("cg_init");
}

extern "C" int
qllg_k_cg_update_xr(int prec, void *x, void *r, const void *p, const void *Ap, int nsites,
                    int ncomp, int nrhs, qllg_cg_scalars *s, qllg_redbuf *rb)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, rb);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    NR_SWITCH(nrhs, (cg_xr_k<P,NC,NR><<<g,kT,0,st>>>(x, r, p, Ap, nsites, s, rb->partial, rb->counter)));
  });
  return done("cg_update_xr");
}

extern "C" int
qllg_k_cg_update_p(int prec, void *p, const void *r, int nsites, int ncomp, int nrhs,
                   qllg_cg_scalars *s)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, 0);
  cudaStream_t st = qllg_stream();
  PN_SWITCH(prec, ncomp, {
    NR_SWITCH(nrhs, (cg_p_k<P,NC,NR><<<g,kT,0,st>>>(p, r, nsites, s)));
  });
  return done("cg_update_p");
}

extern "C" int
qllg_k_cg_update_p_norm(int prec, void *p, const void *r, int nsites, int nrhs,
                        qllg_cg_scalars *s, qllg_redbuf *rb)
{
  size_t total = (size_t)nsites*nrhs;
  int g = grid_for(total, 0, rb);
  cudaStream_t st = qllg_stream();
  if(prec == QLLG_F64) { NR_SWITCH(nrhs, (cg_p_norm_k<QLLG_F64,NR><<<g,kT,0,st>>>(p, r, nsites, s, rb->partial, rb->counter))); }
  else if(prec == QLLG_F32) { NR_SWITCH(nrhs, (cg_p_norm_k<QLLG_F32,NR><<<g,kT,0,st>>>(p, r, nsites, s, rb->partial, rb->counter))); }
  else if(prec == QLLG_I16) { NR_SWITCH(nrhs, (cg_p_norm_k<QLLG_I16,NR><<<g,kT,0,st>>>(p, r, nsites, s, rb->partial, rb->counter))); }
  else { qllg_set_error("cg_update_p_norm: precision %d", prec); return -1; }
  return done("cg_update_p_norm");
}

// the WHILE condition of a graph-captured solver loop: continue while the
// done flag is clear and the iteration cap is not reached (the cap makes the
// loop end even if a flag were never set)
__global__ void loop_cond_k(cudaGraphConditionalHandle h, int *done, int *loops, const int *limit)
{
  if(threadIdx.x == 0) {
    int n = ++*loops;
    cudaGraphSetConditional(h, (!*(volatile int *)done && n < *limit) ? 1u : 0u);
  }
}

extern "C" int
qllg_k_loop_cond(unsigned long long handle, int *done, int *loops, const int *limit)
{
  loop_cond_k<<<1, 32, 0, qllg_stream()>>>((cudaGraphConditionalHandle)handle, done, loops, limit);
  return done_check("loop_cond");
}

// the IF condition of a graph's reliable-update block: taken when some rhs
// is flagged for an update (*no_ru clear); *trips counts the times taken
__global__ void ru_cond_k(cudaGraphConditionalHandle h, const int *no_ru, int *trips)
{
  if(threadIdx.x == 0) {
    const int take = !*(volatile const int *)no_ru;
    if(take) ++*trips;
    cudaGraphSetConditional(h, take ? 1u : 0u);
  }
}

extern "C" int
qllg_k_ru_cond(unsigned long long handle, const int *no_ru, int *trips)
{
  ru_cond_k<<<1, 32, 0, qllg_stream()>>>((cudaGraphConditionalHandle)handle, no_ru, trips);
  return done_check("ru_cond");
}

// ------------------------------------------------ host <-> device copies
// A copy between device memory and page-locked host memory done by the SMs,
// which reach the host buffer through its mapped device address over the
// CPU-GPU link, instead of by a copy engine.  On GB300 (805 MB, 64 KB host
// pages) a copy-engine transfer of a host buffer that the GPU has not
// touched for a while (after a one-second solve, or after 0.5 s idle) took
// 35-90 ms against 3.9 ms when repeated at once; the SM copy takes 3.9-4.0
// ms in both cases.  16-byte accesses: the caller checks that both ends are
// 16-byte aligned and the size a multiple of 16.
__global__ void copy16_k(const int4 *__restrict__ src, int4 *__restrict__ dst, size_t n)
{
  GRID_LOOP(t, n) dst[t] = src[t];
}

extern "C" int
qllg_k_copy16(void *dst, const void *src, size_t bytes)
{
  const size_t n = bytes/16;
  size_t g = (n + kT - 1)/kT, m = (size_t)qllg_num_sms()*32;
  if(g > m) g = m;
  if(g < 1) g = 1;
  copy16_k<<<(int)g, kT, 0, qllg_stream()>>>((const int4 *)src, (int4 *)dst, n);
  return done_check("copy16");
}
