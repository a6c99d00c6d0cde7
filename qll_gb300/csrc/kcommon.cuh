// kcommon.cuh -- device helpers shared by the libqll_gb300 kernels:
// lattice geometry of the even-odd site order, field loads/stores in the
// three storage precisions, and the deterministic grid reduction.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "qllg_internal.h"

namespace qk {

// ------------------------------------------------------------- precisions
template <int P> struct Real;
template <> struct Real<QLLG_F64> { typedef double T; typedef double2 V2; };
template <> struct Real<QLLG_F32> { typedef float T; typedef float2 V2; };
template <> struct Real<QLLG_I16> { typedef float T; typedef float2 V2; };
template <> struct Real<QLLG_F32R> { typedef float T; typedef float2 V2; };
template <> struct Real<QLLG_DF> { typedef float T; typedef float4 V2; };

// storage of the residual/solution vectors that go with Dslash operands of
// precision P: 16-bit Dslash operands keep FP32 recurrence vectors
template <int P> struct VecPrec { static constexpr int value = (P == QLLG_F64) ? QLLG_F64 : QLLG_F32; };

// ----------------------------------------------------------- double-float
// A real as the unevaluated sum h + l of two floats with |l| <= ulp(h)/2,
// about 48 significant bits, computed with FP32 instructions only: this
// part runs FP32 at many times its FP64 rate.  Products use Dekker's exact
// product through fma (a.h*b.h = p + e exactly), sums Knuth's TwoSum; the
// cross terms a.h*b.l + a.l*b.h are rounded once more and a.l*b.l is
// dropped, so a product or a fused multiply-add is good to about 2^-47
// relative.  __fmul_rn/__fadd_rn/__fsub_rn keep the compiler from
// contracting the error terms into fmas.
// a*b + c with one rounding, for every arithmetic type of the Dslash
// kernels (double-float below)
__device__ __forceinline__ float kfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double kfma(double a, double b, double c) { return ::fma(a, b, c); }

struct dfl {
  float h, l;
  __device__ __forceinline__ dfl() {}
  __device__ __forceinline__ dfl(float hh, float ll) : h(hh), l(ll) {}
  __device__ __forceinline__ dfl(double d) {
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
  }
  __device__ __forceinline__ explicit operator double() const { return (double)h + (double)l; }
};
__device__ __forceinline__ dfl df_fast2sum(float s, float e) {   // needs |s| >= |e| or s = 0
  const float h = __fadd_rn(s, e);
  return dfl(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ dfl operator-(const dfl &a) { return dfl(-a.h, -a.l); }
__device__ __forceinline__ dfl operator+(const dfl &a, const dfl &b) {
  const float s = __fadd_rn(a.h, b.h);                  // TwoSum(a.h, b.h) = s + err
  const float bb = __fsub_rn(s, a.h);
  const float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  return df_fast2sum(s, __fadd_rn(err, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dfl operator-(const dfl &a, const dfl &b) { return a + (-b); }
__device__ __forceinline__ dfl &operator+=(dfl &a, const dfl &b) { a = a + b; return a; }
__device__ __forceinline__ dfl &operator-=(dfl &a, const dfl &b) { a = a - b; return a; }
__device__ __forceinline__ dfl operator*(const dfl &a, const dfl &b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast2sum(p, e);
}
__device__ __forceinline__ dfl kfma(const dfl &a, const dfl &b, const dfl &c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = __fadd_rn(c.h, p);                    // TwoSum(c.h, p) = s + err
  const float bb = __fsub_rn(s, c.h);
  const float err = __fadd_rn(__fsub_rn(c.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  return df_fast2sum(s, __fadd_rn(err, __fadd_rn(c.l, e)));
}

// arithmetic type of a kernel that reads precision A and writes B
template <int A, int B> struct Calc { typedef float T; };
template <int B> struct Calc<QLLG_F64, B> { typedef double T; };
template <int A> struct Calc<A, QLLG_F64> { typedef double T; };
template <> struct Calc<QLLG_F64, QLLG_F64> { typedef double T; };
template <> struct Calc<QLLG_DF, QLLG_DF> { typedef dfl T; };

// ---------------------------------------------------------------- geometry
struct Geo {
  int L0, L1, L2, L3, X0h, Vh;
};
__host__ __device__ inline Geo make_geo(const qllg_geom &g) {
  Geo r; r.L0 = g.L[0]; r.L1 = g.L[1]; r.L2 = g.L[2]; r.L3 = g.L[3];
  r.X0h = g.L[0]/2; r.Vh = g.Vh; return r;
}

// coordinates of site i of parity p (x0 fastest; lexicographic index / 2)
__device__ __forceinline__ void site_coords(const Geo &G, int p, int i, int x[4]) {
  int x0h = i % G.X0h; int r = i / G.X0h;
  x[1] = r % G.L1; r /= G.L1;
  x[2] = r % G.L2; x[3] = r / G.L2;
  x[0] = 2*x0h + ((p + x[1] + x[2] + x[3]) & 1);
}

// index within its parity block of the site x shifted by d along mu
__device__ __forceinline__ int nbr_index(const Geo &G, const int x[4], int mu, int d) {
  int y0 = x[0], y1 = x[1], y2 = x[2], y3 = x[3];
  if(mu == 0)      { y0 += d; y0 += (y0 < 0) ? G.L0 : 0; y0 -= (y0 >= G.L0) ? G.L0 : 0; }
  else if(mu == 1) { y1 += d; y1 += (y1 < 0) ? G.L1 : 0; y1 -= (y1 >= G.L1) ? G.L1 : 0; }
  else if(mu == 2) { y2 += d; y2 += (y2 < 0) ? G.L2 : 0; y2 -= (y2 >= G.L2) ? G.L2 : 0; }
  else             { y3 += d; y3 += (y3 < 0) ? G.L3 : 0; y3 -= (y3 >= G.L3) ? G.L3 : 0; }
  return (y0 + G.L0*(y1 + G.L1*(y2 + G.L2*y3))) >> 1;
}

// -------------------------------------------------------------- complex
template <typename T> struct Cx { T r, i; };

template <typename T>
__device__ __forceinline__ void cmac(Cx<T> &acc, const Cx<T> &m, const Cx<T> &v) {
  acc.r = kfma(m.r, v.r, acc.r); acc.i = kfma(m.i, v.r, acc.i);
  acc.r = kfma(-m.i, v.i, acc.r); acc.i = kfma(m.r, v.i, acc.i);
}

// cmac for FP32 on packed pairs (fma.rn.f32x2, sm_100 and later): the same
// two fused multiply-adds per component in the same order, so the result is
// bitwise that of cmac, in two instructions instead of four
__device__ __forceinline__ void cmac_f2(Cx<float> &acc, const Cx<float> &m, const Cx<float> &v) {
  asm("{\n\t.reg .b64 a, m, n, p, q;\n\t"
      "mov.b64 a, {%0, %1};\n\t"
      "mov.b64 m, {%2, %3};\n\t"
      "mov.b64 n, {%4, %2};\n\t"
      "mov.b64 p, {%5, %5};\n\t"
      "mov.b64 q, {%6, %6};\n\t"
      "fma.rn.f32x2 a, m, p, a;\n\t"
      "fma.rn.f32x2 a, n, q, a;\n\t"
      "mov.b64 {%0, %1}, a;\n\t}"
      : "+f"(acc.r), "+f"(acc.i) : "f"(m.r), "f"(m.i), "f"(-m.i), "f"(v.r), "f"(v.i));
}

// ------------------------------------------------------------ spinor I/O
// nc colour(-spin) complex components per site; idx = site*nrhs + rhs;
// stride = nsites*nrhs (component-major for FP64/FP32)
template <int P, int NC> struct SpinorIO;

template <int NC> struct SpinorIO<QLLG_F64, NC> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, size_t stride, size_t idx, Cx<T> v[NC]) {
    const double2 *p = (const double2 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) { double2 t = __ldg(p + c*stride + idx); v[c].r = (T)t.x; v[c].i = (T)t.y; }
  }
  template <typename T>
  static __device__ __forceinline__ void store(void *b, size_t stride, size_t idx, const Cx<T> v[NC]) {
    double2 *p = (double2 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) p[c*stride + idx] = make_double2((double)v[c].r, (double)v[c].i);
  }
};

template <int NC> struct SpinorIO<QLLG_F32, NC> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, size_t stride, size_t idx, Cx<T> v[NC]) {
    const float2 *p = (const float2 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) { float2 t = __ldg(p + c*stride + idx); v[c].r = (T)t.x; v[c].i = (T)t.y; }
  }
  template <typename T>
  static __device__ __forceinline__ void store(void *b, size_t stride, size_t idx, const Cx<T> v[NC]) {
    float2 *p = (float2 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) p[c*stride + idx] = make_float2((float)v[c].r, (float)v[c].i);
  }
};

// double-float spinor: one float4 (re.h, re.l, im.h, im.l) per complex
// component, laid out as FP64
template <int NC> struct SpinorIO<QLLG_DF, NC> {
  static __device__ __forceinline__ void load(const void *b, size_t stride, size_t idx, Cx<dfl> v[NC]) {
    const float4 *p = (const float4 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) {
      float4 t = __ldg(p + c*stride + idx);
      v[c].r = dfl(t.x, t.y); v[c].i = dfl(t.z, t.w);
    }
  }
  static __device__ __forceinline__ void store(void *b, size_t stride, size_t idx, const Cx<dfl> v[NC]) {
    float4 *p = (float4 *)b;
#pragma unroll
    for(int c=0; c<NC; c++) p[c*stride + idx] = make_float4(v[c].r.h, v[c].r.l, v[c].i.h, v[c].i.l);
  }
};

// exact int16 -> float: bias the value into the low mantissa bits of 2^23
__device__ __forceinline__ float s16lo(uint32_t w) {
  return __uint_as_float(0x4B000000u | ((w ^ 0x8000u) & 0xFFFFu)) - 8421376.0f;
}
__device__ __forceinline__ float s16hi(uint32_t w) {
  return __uint_as_float(0x4B000000u | ((w >> 16) ^ 0x8000u)) - 8421376.0f;
}
__device__ __forceinline__ uint32_t pack_s16(float a, float b) {
  int ia = __float2int_rn(a), ib = __float2int_rn(b);
  return (uint32_t)(ia & 0xFFFF) | ((uint32_t)ib << 16);
}

// 16-bit spinor: three colour components in one int4 per (site,rhs)
template <> struct SpinorIO<QLLG_I16, 3> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, size_t, size_t idx, Cx<T> v[3]) {
    int4 w = __ldg((const int4 *)b + idx);
    float s = __int_as_float(w.w) * (1.0f/32767.0f);
    v[0].r = s16lo(w.x)*s; v[0].i = s16hi(w.x)*s;
    v[1].r = s16lo(w.y)*s; v[1].i = s16hi(w.y)*s;
    v[2].r = s16lo(w.z)*s; v[2].i = s16hi(w.z)*s;
  }
  template <typename T>
  static __device__ __forceinline__ void store(void *b, size_t, size_t idx, const Cx<T> v[3]) {
    float m = 0.f;
#pragma unroll
    for(int c=0; c<3; c++) { m = fmaxf(m, fabsf((float)v[c].r)); m = fmaxf(m, fabsf((float)v[c].i)); }
    float inv = (m > 0.f) ? 32767.0f/m : 0.f;
    int4 w;
    w.x = (int)pack_s16((float)v[0].r*inv, (float)v[0].i*inv);
    w.y = (int)pack_s16((float)v[1].r*inv, (float)v[1].i*inv);
    w.z = (int)pack_s16((float)v[2].r*inv, (float)v[2].i*inv);
    w.w = __float_as_int(m);
    ((int4 *)b)[idx] = w;
  }
};

// four consecutive rhs (idx0, a multiple of 4) of one site, all three
// colours: FP32 as two 16-byte loads per colour (the buffer and stride must
// keep idx0 16-byte aligned: the launchers check the base pointers); other
// precisions one load per rhs
template <int P> struct Spinor4 {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, size_t stride, size_t idx0, Cx<T> v[4][3]) {
#pragma unroll
    for(int j=0; j<4; j++) SpinorIO<P,3>::load(b, stride, idx0 + j, v[j]);
  }
  template <typename T>
  static __device__ __forceinline__ void store(void *b, size_t stride, size_t idx0, const Cx<T> v[4][3]) {
#pragma unroll
    for(int j=0; j<4; j++) SpinorIO<P,3>::store(b, stride, idx0 + j, v[j]);
  }
};
template <> struct Spinor4<QLLG_F32> {
  // the two consecutive rhs at idx (even): one 16-byte load per colour
  template <typename T>
  static __device__ __forceinline__ void load_pair(const void *b, size_t stride, size_t idx,
                                                   Cx<T> v[2][3]) {
#pragma unroll
    for(int c=0; c<3; c++) {
      float4 q = __ldg((const float4 *)((const float2 *)b + c*stride + idx));
      v[0][c].r = q.x; v[0][c].i = q.y; v[1][c].r = q.z; v[1][c].i = q.w;
    }
  }
  template <typename T>
  static __device__ __forceinline__ void store_pair(void *b, size_t stride, size_t idx,
                                                    const Cx<T> v[2][3]) {
#pragma unroll
    for(int c=0; c<3; c++)
      *(float4 *)((float2 *)b + c*stride + idx) =
        make_float4((float)v[0][c].r, (float)v[0][c].i, (float)v[1][c].r, (float)v[1][c].i);
  }
  // rhs 2h and 2h+1 only: one 16-byte load per colour
  template <typename T>
  static __device__ __forceinline__ void load_half(const void *b, size_t stride, size_t idx0, int h,
                                                   Cx<T> v[2][3]) {
#pragma unroll
    for(int c=0; c<3; c++) {
      float4 q = __ldg((const float4 *)((const float2 *)b + c*stride + idx0) + h);
      v[0][c].r = q.x; v[0][c].i = q.y; v[1][c].r = q.z; v[1][c].i = q.w;
    }
  }
  template <typename T>
  static __device__ __forceinline__ void store_half(void *b, size_t stride, size_t idx0, int h,
                                                    const Cx<T> v[2][3]) {
#pragma unroll
    for(int c=0; c<3; c++)
      ((float4 *)((float2 *)b + c*stride + idx0))[h] =
        make_float4((float)v[0][c].r, (float)v[0][c].i, (float)v[1][c].r, (float)v[1][c].i);
  }
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, size_t stride, size_t idx0, Cx<T> v[4][3]) {
#pragma unroll
    for(int c=0; c<3; c++) {
      const float4 *p = (const float4 *)((const float2 *)b + c*stride + idx0);
      float4 lo = __ldg(p), hi = __ldg(p + 1);
      v[0][c].r = lo.x; v[0][c].i = lo.y; v[1][c].r = lo.z; v[1][c].i = lo.w;
      v[2][c].r = hi.x; v[2][c].i = hi.y; v[3][c].r = hi.z; v[3][c].i = hi.w;
    }
  }
  template <typename T>
  static __device__ __forceinline__ void store(void *b, size_t stride, size_t idx0, const Cx<T> v[4][3]) {
#pragma unroll
    for(int c=0; c<3; c++) {
      float4 *p = (float4 *)((float2 *)b + c*stride + idx0);
      p[0] = make_float4((float)v[0][c].r, (float)v[0][c].i, (float)v[1][c].r, (float)v[1][c].i);
      p[1] = make_float4((float)v[2][c].r, (float)v[2][c].i, (float)v[3][c].r, (float)v[3][c].i);
    }
  }
};

// --------------------------------------------------------------- link I/O
// slot-major stores; V = sites of the full lattice
template <int P> struct LinkIO;

template <> struct LinkIO<QLLG_F64> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, int slot, size_t V, size_t site, const float *, Cx<T> m[9]) {
    const double2 *p = (const double2 *)b + (size_t)slot*9*V + site;
#pragma unroll
    for(int k=0; k<9; k++) { double2 t = __ldg(p + k*V); m[k].r = (T)t.x; m[k].i = (T)t.y; }
  }
};
template <> struct LinkIO<QLLG_F32> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, int slot, size_t V, size_t site, const float *, Cx<T> m[9]) {
    const float2 *p = (const float2 *)b + (size_t)slot*9*V + site;
#pragma unroll
    for(int k=0; k<9; k++) { float2 t = __ldg(p + k*V); m[k].r = (T)t.x; m[k].i = (T)t.y; }
  }
};
// double-float links: one float4 per complex entry, laid out as FP64
template <> struct LinkIO<QLLG_DF> {
  static __device__ __forceinline__ void load(const void *b, int slot, size_t V, size_t site, const float *, Cx<dfl> m[9]) {
    const float4 *p = (const float4 *)b + (size_t)slot*9*V + site;
#pragma unroll
    for(int k=0; k<9; k++) { float4 t = __ldg(p + k*V); m[k].r = dfl(t.x, t.y); m[k].i = dfl(t.z, t.w); }
  }
};
// reconstruct-12 FP32 links.  A fat slot is [4][V] float4 (entries 2k,
// 2k+1) + [V] float2 (entry 8).  A Naik slot is rows 0 and 1 as [3][V]
// float4: (e0, e3), (e6, e1), (e4, e7) (entry 3*col + row); row 2 is
// s conj(r0 x r1)/|r0|, the third row of c W for W in SU(3), c real, |c| =
// |r0|, s = sign(c) from the per-site sign bit.
struct LinkR {
  static __device__ __forceinline__ void fat(const char *p, size_t V, size_t site, Cx<float> m[9]) {
    const float4 *q = (const float4 *)p;
#pragma unroll
    for(int k=0; k<4; k++) {
      float4 w = __ldg(q + k*V + site);
      m[2*k].r = w.x; m[2*k].i = w.y; m[2*k + 1].r = w.z; m[2*k + 1].i = w.w;
    }
    float2 e = __ldg((const float2 *)(p + 64*V) + site);
    m[8].r = e.x; m[8].i = e.y;
  }
  static __device__ __forceinline__ void naik(const char *p, size_t V, size_t site, bool neg,
                                              Cx<float> m[9]) {
    const float4 *q = (const float4 *)p;
    float4 a = __ldg(q + site), b = __ldg(q + V + site), c = __ldg(q + 2*V + site);
    m[0].r = a.x; m[0].i = a.y; m[3].r = a.z; m[3].i = a.w;
    m[6].r = b.x; m[6].i = b.y; m[1].r = b.z; m[1].i = b.w;
    m[4].r = c.x; m[4].i = c.y; m[7].r = c.z; m[7].i = c.w;
    rebuild_row2(m, neg);
  }
  // entries 2, 5, 8 (row 2) from rows 0 and 1
  static __device__ __forceinline__ void rebuild_row2(Cx<float> m[9], bool neg) {
    const float n2 = m[0].r*m[0].r + m[0].i*m[0].i + m[3].r*m[3].r + m[3].i*m[3].i +
                     m[6].r*m[6].r + m[6].i*m[6].i;
    const float f = (neg ? -1.f : 1.f)*rsqrtf(n2);
#pragma unroll
    for(int c=0; c<3; c++) {
      const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
      // (r0 x r1)_c = r0[c1] r1[c2] - r0[c2] r1[c1]; r_k[col] is entry 3*col + k
      const Cx<float> a = m[3*c1], b = m[3*c2 + 1], d = m[3*c2], e = m[3*c1 + 1];
      const float xr = (a.r*b.r - a.i*b.i) - (d.r*e.r - d.i*e.i);
      const float xi = (a.r*b.i + a.i*b.r) - (d.r*e.i + d.i*e.r);
      m[3*c + 2].r = f*xr;
      m[3*c + 2].i = -f*xi;
    }
  }
};

// 16-bit link: per slot [V] int4 (entries 0..3), [V] int4 (4..7), [V] int (8)
template <> struct LinkIO<QLLG_I16> {
  template <typename T>
  static __device__ __forceinline__ void load(const void *b, int slot, size_t V, size_t site, const float *scale, Cx<T> m[9]) {
    const char *base = (const char *)b + (size_t)slot*36*V;
    int4 a = __ldg((const int4 *)base + site);
    int4 c = __ldg((const int4 *)(base + 16*V) + site);
    int e = __ldg((const int *)(base + 32*V) + site);
    float s = __ldg(scale + slot) * (1.0f/32767.0f);
    m[0].r = s16lo(a.x)*s; m[0].i = s16hi(a.x)*s;
    m[1].r = s16lo(a.y)*s; m[1].i = s16hi(a.y)*s;
    m[2].r = s16lo(a.z)*s; m[2].i = s16hi(a.z)*s;
    m[3].r = s16lo(a.w)*s; m[3].i = s16hi(a.w)*s;
    m[4].r = s16lo(c.x)*s; m[4].i = s16hi(c.x)*s;
    m[5].r = s16lo(c.y)*s; m[5].i = s16hi(c.y)*s;
    m[6].r = s16lo(c.z)*s; m[6].i = s16hi(c.z)*s;
    m[7].r = s16lo(c.w)*s; m[7].i = s16hi(c.w)*s;
    m[8].r = s16lo(e)*s;   m[8].i = s16hi(e)*s;
  }
};

// ------------------------------------------------- per-thread accumulators
// Sums of squares and dot products that a thread accumulates before the
// block/grid tree (which is FP64).  FP64 data accumulate in FP64.  FP32
// data accumulate in FP32 with Kahan compensation, one compensated add per
// (site, rhs): the FP64 pipe of this part runs at a small fraction of the
// FP32 rate, and converting every product to double made the norms of the
// FP32 kernels FP64-bound.  The compensated sum keeps the thread's partial
// to about one FP32 rounding of the total.
template <typename T> struct Acc;
template <> struct Acc<double> {
  double s = 0;
  __device__ __forceinline__ void add(double x) { s += x; }
  template <int N> __device__ __forceinline__ void norm(const Cx<double> (&v)[N]) {
#pragma unroll
    for(int c=0; c<N; c++) s += v[c].r*v[c].r + v[c].i*v[c].i;
  }
  __device__ __forceinline__ double get() const { return s; }
};
// double-float data: the norm in FP64 (only diagnostics use it)
template <> struct Acc<dfl> {
  double s = 0;
  template <int N> __device__ __forceinline__ void norm(const Cx<dfl> (&v)[N]) {
#pragma unroll
    for(int c=0; c<N; c++) {
      const double r = (double)v[c].r, i = (double)v[c].i;
      s += r*r + i*i;
    }
  }
  __device__ __forceinline__ double get() const { return s; }
};
template <> struct Acc<float> {
  float s = 0, e = 0;
  __device__ __forceinline__ void add(float x) {
    float y = x - e;
    float t = s + y;
    e = (t - s) - y;
    s = t;
  }
  template <int N> __device__ __forceinline__ void norm(const Cx<float> (&v)[N]) {
    float q = 0;
#pragma unroll
    for(int c=0; c<N; c++) { q = fmaf(v[c].r, v[c].r, q); q = fmaf(v[c].i, v[c].i, q); }
    add(q);
  }
  __device__ __forceinline__ double get() const { return (double)s - (double)e; }
};

// ------------------------------------------------------------ reductions
// Block partial sums per rhs, then the last block to finish folds the
// partials of all blocks in a fixed order, so results are bitwise
// repeatable for a fixed grid.  nr reductions of nrhs values each.
template <int NR>
__device__ __forceinline__ bool grid_reduce(double (&val)[NR], int nrhs, int rhs,
                                            double *partial, unsigned *counter,
                                            double *shm /* blockDim*NR */,
                                            double *result[NR]) {
  const int tid = threadIdx.x, nt = blockDim.x;
#pragma unroll
  for(int q=0; q<NR; q++) shm[q*nt + tid] = val[q];
  __syncthreads();
  // fold threads of equal rhs: thread t holds rhs t % nrhs
  if(tid < nrhs) {
#pragma unroll
    for(int q=0; q<NR; q++) {
      double s = 0;
      for(int t=tid; t<nt; t+=nrhs) s += shm[q*nt + t];
      partial[(size_t)blockIdx.x*(2*QLLG_MAXRHS) + q*QLLG_MAXRHS + tid] = s;
    }
  }
  __threadfence();
  __shared__ bool last;
  __syncthreads();
  if(tid == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if(!last) return false;
  __threadfence();
  // all partials visible: K = NR*nrhs sums (a power of two dividing the
  // block size); thread t adds blocks j, j+J, ... of sum c = t % K with
  // j = t / K, then a fixed tree over j.
  const int nb = gridDim.x;
  const int K = NR*nrhs, J = nt / K;
  const int c = tid % K, j = tid / K;
  const int q = c / nrhs, r = c % nrhs;
  double s = 0;
  for(int b=j; b<nb; b+=J)
    s += ((volatile double *)partial)[(size_t)b*(2*QLLG_MAXRHS) + q*QLLG_MAXRHS + r];
  shm[tid] = s;
  __syncthreads();
  for(int w=J/2; w>0; w>>=1) {
    if(j < w) shm[c + K*j] += shm[c + K*(j + w)];
    __syncthreads();
  }
  if(j == 0) {
#pragma unroll
    for(int qq=0; qq<NR; qq++) if(qq == q && result[qq]) result[qq][r] = shm[c];
  }
  if(tid == 0) *counter = 0u;
  return true;
}

// Same reduction when each thread holds R right-hand sides: thread t works
// on rhs q*R + j (j < R) with q = t % Q and Q = nrhs/R threads per site.
// ntr: the first ntr threads of the block hold values (0: all); the others
// (a producer warp) only take part in the barriers
template <int NRED, int R>
__device__ __forceinline__ bool grid_reduce_mr(double (&val)[NRED][R], int nrhs, int Q,
                                               double *partial, unsigned *counter,
                                               double *shm /* NRED*R*blockDim */,
                                               double *result[NRED], int ntr = 0,
                                               bool pairs = false) {
  const int tid = threadIdx.x, nt = ntr ? ntr : blockDim.x;
  const bool in = tid < nt;
  if(in) {
#pragma unroll
    for(int n=0; n<NRED; n++)
#pragma unroll
      for(int j=0; j<R; j++) shm[(n*R + j)*nt + tid] = val[n][j];
  }
  __syncthreads();
  {
    const int K = NRED*nrhs, J = nt/K, c = tid % K, l = tid / K;
    const int n = c / nrhs, r = c % nrhs;
    // thread q of a site holds rhs q*R + j, or with pairs the rhs pairs
    // h*2Q + 2q (+1), j = 2h (+1)
    const int j = pairs ? 2*(r/(2*Q)) + (r & 1) : r % R;
    const int qq = pairs ? (r % (2*Q))/2 : r / R;
    double s = 0;
    if(in) for(int i=l; i<nt/Q; i+=J) s += shm[(n*R + j)*nt + qq + Q*i];
    __syncthreads();
    if(in) shm[tid] = s;
    __syncthreads();
    for(int w=J/2; w>0; w>>=1) {
      if(in && l < w) shm[c + K*l] += shm[c + K*(l + w)];
      __syncthreads();
    }
    if(in && l == 0) partial[(size_t)blockIdx.x*(2*QLLG_MAXRHS) + n*QLLG_MAXRHS + r] = shm[c];
  }
  __threadfence();
  __shared__ bool last;
  __syncthreads();
  if(tid == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if(!last) return false;
  __threadfence();
  const int nb = gridDim.x;
  const int K = NRED*nrhs, J = nt / K;
  const int c = tid % K, l = tid / K;
  const int q = c / nrhs, r = c % nrhs;
  double s = 0;
  if(in)
    for(int b=l; b<nb; b+=J)
      s += ((volatile double *)partial)[(size_t)b*(2*QLLG_MAXRHS) + q*QLLG_MAXRHS + r];
  if(in) shm[tid] = s;
  __syncthreads();
  for(int w=J/2; w>0; w>>=1) {
    if(in && l < w) shm[c + K*l] += shm[c + K*(l + w)];
    __syncthreads();
  }
  if(in && l == 0) {
#pragma unroll
    for(int qq=0; qq<NRED; qq++) if(qq == q && result[qq]) result[qq][r] = shm[c];
  }
  if(tid == 0) *counter = 0u;
  return true;
}

// ------------------------------------------------ CG bookkeeping (last block)
// plain CG (cgSolveT's loop test, lib/cg.c:115): keep iterating while
// |r|^2 >= rsq_stop and iters < maxits; the new |r|^2 of each rhs is in tmp
__device__ inline void cg_finish_plain(qllg_cg_scalars *s, int nr) {
  int any = 0;
  for(int q=0; q<nr; q++) {
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

// mixed CG: flag a reliable update when the sloppy residual fell by delta
// since the last one, passed the target, hit maxits or is not a number
// the reliable update rhs q takes after an iteration with |r|^2 = r2: 0
// none; 1 an intermediate one (r2 fell by delta^2 since the last); 2 a final
// candidate (converged, iteration limit, or not a number), on which the
// solve of that rhs may stop, so its residual b - A x must be FP64
__device__ __forceinline__ int ru_kind(const qllg_cg_scalars *s, int q, double r2) {
  if(r2 < s->rsq_stop[q] || s->iters[q] >= s->maxits || !(r2 == r2)) return 2;
  return r2 < s->delta2*s->maxr2[q] ? 1 : 0;
}

__device__ inline void cg_finish_mixed(qllg_cg_scalars *s, int nr) {
  int anyru = 0;
  for(int q=0; q<nr; q++) {
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

// standard-form CG (r -= alpha Ap, then p = r + beta p with beta in
// alpha[]): the bookkeeping after |r|^2 of the update is reduced into
// tmp[]; mixed (delta2 > 0): reliable-update flags instead of stopping
__device__ inline void cg_finish_std(qllg_cg_scalars *s, int nr) {
  int anyru = 0, any = 0;
  const bool mixed = s->delta2 > 0;
  for(int q=0; q<nr; q++) {
    s->ru[q] = 0;
    if(s->active[q]) {
      double r2 = s->tmp[q];
      s->iters[q]++;
      s->prev[q] = s->rsq[q];
      s->rsq[q] = r2;
      s->alpha[q] = r2/s->prev[q];
      if(mixed) {
        s->ru[q] = ru_kind(s, q, r2);
        anyru |= s->ru[q] != 0;
      } else if(!(r2 >= s->rsq_stop[q] && s->iters[q] < s->maxits)) {
        s->active[q] = 0;
      }
    }
    any |= s->active[q];
  }
  s->no_ru = !anyru;
  s->done = !any;
  s->count++;
}

} // namespace qk
