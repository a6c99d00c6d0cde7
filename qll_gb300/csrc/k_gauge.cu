// k_gauge.cu -- 3x3 matrix-field kernels (sm_103a) behind fat7/asqtad
// smearing, the plaquette, double-stored links and the generic
// transporter: shifted gathers, products M N, M N^dagger, M^dagger N with an
// optional neighbour shift of the right factor, axpy, and adjoints.  The
// per-element arithmetic follows PeqMtimesX / PeqMtimesXa / PeqMatimesX
// (lib/vla.c:929-1078).  Fields are full-lattice [9][V] double2/float2
// (entry 3*column + row) in QLL site order.
#include "kcommon.cuh"

using namespace qk;

namespace {

constexpr int kT = 256;

#define GRID_LOOP(t, total) \
  for(size_t t = (size_t)blockIdx.x*blockDim.x + threadIdx.x; t < (total); \
      t += (size_t)gridDim.x*blockDim.x)

// full-lattice index of the neighbour x + len*mu of full-lattice site s
__device__ __forceinline__ size_t full_nbr(const Geo &G, int s, int mu, int len) {
  int p = s >= G.Vh;
  int i = s - p*G.Vh;
  int x[4];
  site_coords(G, p, i, x);
  int q = p ^ (len & 1);
  return (size_t)q*G.Vh + nbr_index(G, x, mu, len);
}

template <typename T> struct MIO;
template <> struct MIO<double> {
  static __device__ __forceinline__ void load(const void *b, size_t V, size_t s, Cx<double> m[9]) {
    const double2 *p = (const double2 *)b;
#pragma unroll
    for(int k=0; k<9; k++) { double2 t = p[k*V + s]; m[k].r = t.x; m[k].i = t.y; }
  }
  static __device__ __forceinline__ void store(void *b, size_t V, size_t s, const Cx<double> m[9]) {
    double2 *p = (double2 *)b;
#pragma unroll
    for(int k=0; k<9; k++) p[k*V + s] = make_double2(m[k].r, m[k].i);
  }
};
template <> struct MIO<float> {
  static __device__ __forceinline__ void load(const void *b, size_t V, size_t s, Cx<float> m[9]) {
    const float2 *p = (const float2 *)b;
#pragma unroll
    for(int k=0; k<9; k++) { float2 t = p[k*V + s]; m[k].r = t.x; m[k].i = t.y; }
  }
  static __device__ __forceinline__ void store(void *b, size_t V, size_t s, const Cx<float> m[9]) {
    float2 *p = (float2 *)b;
#pragma unroll
    for(int k=0; k<9; k++) p[k*V + s] = make_float2(m[k].r, m[k].i);
  }
};

// out = c * op(A)(x) op(B)(nbr(x)), or out += ... when acc
// kind 0: A B, 1: A B^dagger, 2: A^dagger B
template <typename T>
__global__ void mat_mul_k(void *out, const void *A, const void *B, qllg_geom g, int kind,
                          int mu, int len, int acc)
{
  const Geo G = make_geo(g);
  const size_t V = g.V;
  GRID_LOOP(s, V) {
    Cx<T> a[9], b[9], r[9];
    MIO<T>::load(A, V, s, a);
    size_t sb = len ? full_nbr(G, (int)s, mu, len) : s;
    MIO<T>::load(B, V, sb, b);
    if(acc) MIO<T>::load(out, V, s, r);
    else {
#pragma unroll
      for(int k=0; k<9; k++) { r[k].r = 0; r[k].i = 0; }
    }
#pragma unroll
    for(int i=0; i<3; i++) {          // column of the result
#pragma unroll
      for(int l=0; l<3; l++) {
        Cx<T> v = (kind == 1) ? b[3*l + i] : b[3*i + l];
        if(kind == 1) v.i = -v.i;
#pragma unroll
        for(int j=0; j<3; j++) {
          Cx<T> m = (kind == 2) ? a[3*j + l] : a[3*l + j];
          if(kind == 2) m.i = -m.i;
          r[3*i+j].r = fma(m.r, v.r, r[3*i+j].r);
          r[3*i+j].i = fma(m.r, v.i, r[3*i+j].i);
        }
#pragma unroll
        for(int j=0; j<3; j++) {
          Cx<T> m = (kind == 2) ? a[3*j + l] : a[3*l + j];
          if(kind == 2) m.i = -m.i;
          r[3*i+j].r = fma(-m.i, v.i, r[3*i+j].r);
          r[3*i+j].i = fma(m.i, v.r, r[3*i+j].i);
        }
      }
    }
    MIO<T>::store(out, V, s, r);
  }
}

// out(x) = sgn * in(nbr(x)) (adj: its adjoint); len 0 = no shift
template <typename T>
__global__ void mat_shift_k(void *out, const void *in, qllg_geom g, int mu, int len, int adj,
                            double sgn)
{
  const Geo G = make_geo(g);
  const size_t V = g.V;
  GRID_LOOP(s, V) {
    Cx<T> m[9], r[9];
    size_t sb = len ? full_nbr(G, (int)s, mu, len) : s;
    MIO<T>::load(in, V, sb, m);
#pragma unroll
    for(int row=0; row<3; row++)
#pragma unroll
      for(int col=0; col<3; col++) {
        Cx<T> e = adj ? m[3*row + col] : m[3*col + row];
        if(adj) e.i = -e.i;
        r[3*col + row].r = (T)sgn*e.r;
        r[3*col + row].i = (T)sgn*e.i;
      }
    MIO<T>::store(out, V, s, r);
  }
}

// out = a*out + c*in (a = 0 does not read out)
template <typename T>
__global__ void mat_axpy_k(T *out, const T *in, double a, double c, size_t n)
{
  const T ta = (T)a, tc = (T)c;
  GRID_LOOP(i, n) out[i] = (ta == (T)0) ? tc*in[i] : fma(tc, in[i], ta*out[i]);
}

// out[i] = out[i] + c*in[i] exactly as X_vpeq_r_times_X (lib/vla.c:749-765)
template <typename T>
__global__ void mat_peq_k(T *out, const T *in, double c, size_t n)
{
  const T tc = (T)c;
  GRID_LOOP(i, n) out[i] = fma(tc, in[i], out[i]);
}

// plaquette sum over sites of Re tr[(U_i(x) U_j(x+i))^dagger U_j(x) U_i(x+j)]
template <typename T>
__global__ void __launch_bounds__(kT)
plaq_k(const void *ui, const void *uj, qllg_geom g, int i, int j, double *out,
       double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  const Geo G = make_geo(g);
  const size_t V = g.V;
  double red[1] = {0};
  GRID_LOOP(s, V) {
    Cx<T> a[9], b[9], c[9], d[9];
    MIO<T>::load(ui, V, s, a);
    MIO<T>::load(uj, V, full_nbr(G, (int)s, i, 1), b);
    MIO<T>::load(uj, V, s, c);
    MIO<T>::load(ui, V, full_nbr(G, (int)s, j, 1), d);
    // A = a b, B = c d; sum_k Re(conj(A_k) B_k)
    double acc = 0;
#pragma unroll
    for(int col=0; col<3; col++)
#pragma unroll
      for(int row=0; row<3; row++) {
        double Ar = 0, Ai = 0, Br = 0, Bi = 0;
#pragma unroll
        for(int l=0; l<3; l++) {
          Cx<T> x1 = a[3*l + row], y1 = b[3*col + l];
          Ar += (double)x1.r*y1.r - (double)x1.i*y1.i;
          Ai += (double)x1.r*y1.i + (double)x1.i*y1.r;
          Cx<T> x2 = c[3*l + row], y2 = d[3*col + l];
          Br += (double)x2.r*y2.r - (double)x2.i*y2.i;
          Bi += (double)x2.r*y2.i + (double)x2.i*y2.r;
        }
        acc += Ar*Br + Ai*Bi;
      }
    red[0] += acc;
  }
  double *res[1] = {out};
  grid_reduce<1>(red, 1, 0, partial, counter, shm, res);
}

int grid_for(size_t total)
{
  size_t g = (total + kT - 1)/kT, m = (size_t)qllg_num_sms()*8;
  if(g > m) g = m;
  return g < 1 ? 1 : (int)g;
}

int done(const char *w) { return qllg_launched(w); }

} // namespace

extern "C" int
qllg_k_mat_mul(int prec, void *out, const void *A, const void *B, const qllg_geom *g,
               int kind, int mu, int len, int acc)
{
  int gr = grid_for((size_t)g->V);
  if(prec == QLLG_F64) mat_mul_k<double><<<gr, kT, 0, qllg_stream()>>>(out, A, B, *g, kind, mu, len, acc);
  else mat_mul_k<float><<<gr, kT, 0, qllg_stream()>>>(out, A, B, *g, kind, mu, len, acc);
  return done("mat_mul");
}

extern "C" int
qllg_k_mat_shift(int prec, void *out, const void *in, const qllg_geom *g, int mu, int len,
                 int adj, double sgn)
{
  int gr = grid_for((size_t)g->V);
  if(prec == QLLG_F64) mat_shift_k<double><<<gr, kT, 0, qllg_stream()>>>(out, in, *g, mu, len, adj, sgn);
  else mat_shift_k<float><<<gr, kT, 0, qllg_stream()>>>(out, in, *g, mu, len, adj, sgn);
  return done("mat_shift");
}

extern "C" int
qllg_k_mat_axpy(int prec, void *out, const void *in, double a, double c, size_t nreal)
{
  int gr = grid_for(nreal);
  if(prec == QLLG_F64) mat_axpy_k<double><<<gr, kT, 0, qllg_stream()>>>((double *)out, (const double *)in, a, c, nreal);
  else mat_axpy_k<float><<<gr, kT, 0, qllg_stream()>>>((float *)out, (const float *)in, a, c, nreal);
  return done("mat_axpy");
}

extern "C" int
qllg_k_mat_peq(int prec, void *out, const void *in, double c, size_t nreal)
{
  int gr = grid_for(nreal);
  if(prec == QLLG_F64) mat_peq_k<double><<<gr, kT, 0, qllg_stream()>>>((double *)out, (const double *)in, c, nreal);
  else mat_peq_k<float><<<gr, kT, 0, qllg_stream()>>>((float *)out, (const float *)in, c, nreal);
  return done("mat_peq");
}

extern "C" int
qllg_k_plaq(int prec, const void *ui, const void *uj, const qllg_geom *g, int i, int j,
            double *out, qllg_redbuf *rb)
{
  int gr = grid_for((size_t)g->V);
  if(gr > rb->maxblocks) gr = rb->maxblocks;
  if(prec == QLLG_F64) plaq_k<double><<<gr, kT, 0, qllg_stream()>>>(ui, uj, *g, i, j, out, rb->partial, rb->counter);
  else plaq_k<float><<<gr, kT, 0, qllg_stream()>>>(ui, uj, *g, i, j, out, rb->partial, rb->counter);
  return done("plaq");
}

// ---------------------------------------------------- host-layout fields
namespace {

template <typename T>
__global__ void aos_shift_k(T *out, const T *in, int nelem, qllg_geom g, int mu, int len)
{
  const Geo G = make_geo(g);
  GRID_LOOP(s, (size_t)g.V) {
    size_t k = full_nbr(G, (int)s, mu, len);
    for(int e=0; e<nelem; e++) out[s*nelem + e] = in[k*nelem + e];
  }
}

// PeqMtimesX with ldv columns (lib/vla.c:929-964) on host-layout fields
template <typename T>
__global__ void aos_transport_k(T *out, const T *u, const T *in, int nelem, qllg_geom g,
                                int mu, int len)
{
  const Geo G = make_geo(g);
  const int ldv = nelem/6;
  GRID_LOOP(s, (size_t)g.V) {
    size_t k = full_nbr(G, (int)s, mu, len);
    const T *m = u + s*18;
    T *r = out + s*nelem;
    const T *v = in + k*nelem;
    for(int i=0; i<ldv; i++) {
      for(int l=0; l<3; l++) {
        T vr = v[(3*i+l)*2], vi = v[(3*i+l)*2+1];
        for(int j=0; j<3; j++) {
          const T *mj = m + (j + 3*l)*2;
          T *rj = r + (3*i+j)*2;
          rj[0] = fma(mj[0], vr, rj[0]);
          rj[1] = fma(mj[0], vi, rj[1]);
        }
        for(int j=0; j<3; j++) {
          const T *mj = m + (j + 3*l)*2;
          T *rj = r + (3*i+j)*2;
          rj[0] = fma(-mj[1], vi, rj[0]);
          rj[1] = fma(mj[1], vr, rj[1]);
        }
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kT)
aos_sum_k(const T *x, size_t a, size_t b, int sq, double *out, double *partial, unsigned *counter)
{
  __shared__ double shm[kT];
  double red[1] = {0};
  for(size_t i = a + (size_t)blockIdx.x*blockDim.x + threadIdx.x; i < b;
      i += (size_t)gridDim.x*blockDim.x) {
    double v = x[i];
    red[0] += sq ? v*v : v;
  }
  double *res[1] = {out};
  grid_reduce<1>(red, 1, 0, partial, counter, shm, res);
}

} // namespace

extern "C" int
qllg_k_aos_shift(int prec, void *out, const void *in, int nelem, const qllg_geom *g, int mu, int len)
{
  int gr = grid_for((size_t)g->V);
  if(prec == QLLG_F64) aos_shift_k<double><<<gr, kT, 0, qllg_stream()>>>((double *)out, (const double *)in, nelem, *g, mu, len);
  else aos_shift_k<float><<<gr, kT, 0, qllg_stream()>>>((float *)out, (const float *)in, nelem, *g, mu, len);
  return done("aos_shift");
}

extern "C" int
qllg_k_aos_transport(int prec, void *out, const void *u, const void *in, int nelem,
                     const qllg_geom *g, int mu, int len)
{
  int gr = grid_for((size_t)g->V);
  if(prec == QLLG_F64) aos_transport_k<double><<<gr, kT, 0, qllg_stream()>>>((double *)out, (const double *)u, (const double *)in, nelem, *g, mu, len);
  else aos_transport_k<float><<<gr, kT, 0, qllg_stream()>>>((float *)out, (const float *)u, (const float *)in, nelem, *g, mu, len);
  return done("aos_transport");
}

extern "C" int
qllg_k_aos_sum(int prec, const void *x, int nelem, int s0, int s1, int sq, double *out,
               qllg_redbuf *rb)
{
  size_t a = (size_t)nelem*s0, b = (size_t)nelem*s1;
  int gr = grid_for(b - a);
  if(gr > rb->maxblocks) gr = rb->maxblocks;
  if(prec == QLLG_F64) aos_sum_k<double><<<gr, kT, 0, qllg_stream()>>>((const double *)x, a, b, sq, out, rb->partial, rb->counter);
  else aos_sum_k<float><<<gr, kT, 0, qllg_stream()>>>((const float *)x, a, b, sq, out, rb->partial, rb->counter);
  return done("aos_sum");
}

// ------------------------------------------------------ re-unitarisation
// makeU (lib/vla.c:1635-1665, makeUsite) on host-layout sites [s0, s1) of
// nc x nc complex matrices, 2 nc^2 reals a site: vector i (2 nc reals from
// 2 nc i) is normalised, then for each earlier vector j its projection
// <v_j, v_i> v_j is removed and v_i normalised again -- the reference's
// order, including the normalisation after every projection.  nc <= 3.
namespace {
template <typename T>
__global__ void make_u_k(T *m, int nc, size_t s0, size_t s1)
{
  for(size_t s = s0 + (size_t)blockIdx.x*blockDim.x + threadIdx.x; s < s1; s += (size_t)gridDim.x*blockDim.x) {
    T *ms = m + (size_t)2*nc*nc*s;
    T v[18];
    for(int k=0; k<2*nc*nc; k++) v[k] = ms[k];
    for(int i=0; i<nc; i++) {
      T *vi = v + 2*nc*i;
      T n = vi[0]*vi[0];
      for(int k=1; k<2*nc; k++) n = fma(vi[k], vi[k], n);
      T ni = (T)1/sqrt(n);
      for(int k=0; k<2*nc; k++) vi[k] = ni*vi[k];
      for(int j=0; j<i; j++) {
        const T *vj = v + 2*nc*j;
        // d = <v_j, v_i> (conjugate on v_j)
        T dr = vj[0]*vi[0], di = vj[0]*vi[1];
        dr = fma(vj[1], vi[1], dr);
        di = fma(-vj[1], vi[0], di);
        for(int k=2; k<2*nc; k+=2) {
          dr = fma(vj[k], vi[k], dr);
          di = fma(vj[k], vi[k+1], di);
          dr = fma(vj[k+1], vi[k+1], dr);
          di = fma(-vj[k+1], vi[k], di);
        }
        // v_i -= d v_j
        for(int k=0; k<2*nc; k+=2) {
          T x0 = vi[k], x1 = vi[k+1];
          x0 = fma(-dr, vj[k], x0);
          x1 = fma(-dr, vj[k+1], x1);
          x0 = fma(di, vj[k+1], x0);
          x1 = fma(-di, vj[k], x1);
          vi[k] = x0; vi[k+1] = x1;
        }
        n = vi[0]*vi[0];
        for(int k=1; k<2*nc; k++) n = fma(vi[k], vi[k], n);
        ni = (T)1/sqrt(n);
        for(int k=0; k<2*nc; k++) vi[k] = ni*vi[k];
      }
    }
    for(int k=0; k<2*nc*nc; k++) ms[k] = v[k];
  }
}
} // namespace

extern "C" int
qllg_k_make_u(int prec, void *m, int nc, size_t s0, size_t s1)
{
  if(nc < 1 || nc > 3) { qllg_set_error("makeU: nc %d (1 to 3)", nc); return -1; }
  if(s1 <= s0) return 0;
  int gr = grid_for(s1 - s0);
  if(prec == QLLG_F64) make_u_k<double><<<gr, kT, 0, qllg_stream()>>>((double *)m, nc, s0, s1);
  else make_u_k<float><<<gr, kT, 0, qllg_stream()>>>((float *)m, nc, s0, s1);
  return done("make_u");
}
