// gb_spin.cuh -- site-pair (f32x2) spin algebra of the FP32 / FP16 Wilson hopping term:
// the half-spinor projections and reconstructions of Grid's TwoSpinor.h:75-330
// (spProj / accumRecon), the SU(3) x two-spinor product, and the shared-memory stride of
// a staged 4D site's links.  Used by the per-site gather kernel (gb_dhop.cu) and the
// t-stream kernel (gb_dhop_stream.cu).
#pragma once

#include "gb_device.cuh"

namespace gb {

// =======================================================================================
// FP32 / FP16 storage: two 5D sites (s5, s5+1) per thread in packed f32x2 arithmetic.
// Every operation acts identically on both lanes, so the site-pair layout needs no lane
// shuffles; each link element is read once from shared memory and broadcast to both
// lanes.
// =======================================================================================
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }
// a + S*b
template <int S> __device__ __forceinline__ float2 adds2(float2 a, float2 b) { return S > 0 ? add2(a, b) : sub2(a, b); }

template <int MU, int S>
__device__ __forceinline__ void project2(const Pair12& f, float2 (&hr)[6], float2 (&hi)[6]) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float2 f0r = f.re[c], f0i = f.im[c], f1r = f.re[3 + c], f1i = f.im[3 + c];
    const float2 f2r = f.re[6 + c], f2i = f.im[6 + c], f3r = f.re[9 + c], f3i = f.im[9 + c];
    if (MU == 0) {  // h0 = f0 + S i f3, h1 = f1 + S i f2
      hr[c] = adds2<-S>(f0r, f3i); hi[c] = adds2<S>(f0i, f3r);
      hr[3 + c] = adds2<-S>(f1r, f2i); hi[3 + c] = adds2<S>(f1i, f2r);
    } else if (MU == 1) {  // h0 = f0 - S f3, h1 = f1 + S f2
      hr[c] = adds2<-S>(f0r, f3r); hi[c] = adds2<-S>(f0i, f3i);
      hr[3 + c] = adds2<S>(f1r, f2r); hi[3 + c] = adds2<S>(f1i, f2i);
    } else if (MU == 2) {  // h0 = f0 + S i f2, h1 = f1 - S i f3
      hr[c] = adds2<-S>(f0r, f2i); hi[c] = adds2<S>(f0i, f2r);
      hr[3 + c] = adds2<S>(f1r, f3i); hi[3 + c] = adds2<-S>(f1i, f3r);
    } else {  // h0 = f0 + S f2, h1 = f1 + S f3
      hr[c] = adds2<S>(f0r, f2r); hi[c] = adds2<S>(f0i, f2i);
      hr[3 + c] = adds2<S>(f1r, f3r); hi[3 + c] = adds2<S>(f1i, f3i);
    }
  }
}

// acc (+)= n * reconstruction of u, n the per-lane factor of the neighbour's storage
// (1 for FP32, whose adds are then exactly a + u and a - u); FIRST assigns
template <int MU, int S, bool FIRST>
__device__ __forceinline__ void reconstruct2(Pair12& r, const float2 (&ur)[6], const float2 (&ui)[6], float2 n) {
  const float2 np = n, nn = make_float2(-n.x, -n.y);
  // a + T n b, T = +-1
  auto acc = [&](int T, float2 a, float2 b) { return __ffma2_rn(b, T > 0 ? np : nn, a); };
  const int SP = S, SM = -S;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float2 u0r = ur[c], u0i = ui[c], u1r = ur[3 + c], u1i = ui[3 + c];
    if (FIRST) {
      const float2 zero = f2(0.f);
      r.re[c] = acc(1, zero, u0r); r.im[c] = acc(1, zero, u0i);
      r.re[3 + c] = acc(1, zero, u1r); r.im[3 + c] = acc(1, zero, u1i);
      if (MU == 0) {  // r2 = -S i u1, r3 = -S i u0
        r.re[6 + c] = acc(SP, zero, u1i); r.im[6 + c] = acc(SM, zero, u1r);
        r.re[9 + c] = acc(SP, zero, u0i); r.im[9 + c] = acc(SM, zero, u0r);
      } else if (MU == 1) {  // r2 = S u1, r3 = -S u0
        r.re[6 + c] = acc(SP, zero, u1r); r.im[6 + c] = acc(SP, zero, u1i);
        r.re[9 + c] = acc(SM, zero, u0r); r.im[9 + c] = acc(SM, zero, u0i);
      } else if (MU == 2) {  // r2 = -S i u0, r3 = S i u1
        r.re[6 + c] = acc(SP, zero, u0i); r.im[6 + c] = acc(SM, zero, u0r);
        r.re[9 + c] = acc(SM, zero, u1i); r.im[9 + c] = acc(SP, zero, u1r);
      } else {  // r2 = S u0, r3 = S u1
        r.re[6 + c] = acc(SP, zero, u0r); r.im[6 + c] = acc(SP, zero, u0i);
        r.re[9 + c] = acc(SP, zero, u1r); r.im[9 + c] = acc(SP, zero, u1i);
      }
    } else {
      r.re[c] = acc(1, r.re[c], u0r); r.im[c] = acc(1, r.im[c], u0i);
      r.re[3 + c] = acc(1, r.re[3 + c], u1r); r.im[3 + c] = acc(1, r.im[3 + c], u1i);
      if (MU == 0) {
        r.re[6 + c] = acc(SP, r.re[6 + c], u1i); r.im[6 + c] = acc(SM, r.im[6 + c], u1r);
        r.re[9 + c] = acc(SP, r.re[9 + c], u0i); r.im[9 + c] = acc(SM, r.im[9 + c], u0r);
      } else if (MU == 1) {
        r.re[6 + c] = acc(SP, r.re[6 + c], u1r); r.im[6 + c] = acc(SP, r.im[6 + c], u1i);
        r.re[9 + c] = acc(SM, r.re[9 + c], u0r); r.im[9 + c] = acc(SM, r.im[9 + c], u0i);
      } else if (MU == 2) {
        r.re[6 + c] = acc(SP, r.re[6 + c], u0i); r.im[6 + c] = acc(SM, r.im[6 + c], u0r);
        r.re[9 + c] = acc(SM, r.re[9 + c], u1i); r.im[9 + c] = acc(SP, r.im[9 + c], u1r);
      } else {
        r.re[6 + c] = acc(SP, r.re[6 + c], u0r); r.im[6 + c] = acc(SP, r.im[6 + c], u0i);
        r.re[9 + c] = acc(SP, r.re[9 + c], u1r); r.im[9 + c] = acc(SP, r.im[9 + c], u1i);
      }
    }
  }
}

// Links in shared memory: per 4D site 8 legs x 9 complex as (re, im) float pairs, one
// 4D site every kLinkStride floats.  The stride (592 B) keeps each site's TMA destination
// 16-byte aligned and puts the (up to 8) sites one warp touches on distinct bank pairs,
// so a warp's 64-bit link load is one conflict-free broadcast wavefront.
constexpr int kLinkStride = 148;

// u = U h on both spins; U: 9 (re, im) in shared memory, broadcast to both lanes
__device__ __forceinline__ void su3_mul2(const float2* __restrict__ U, const float2 (&hr)[6], const float2 (&hi)[6],
                                         float2 (&ur)[6], float2 (&ui)[6]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float2 w0 = U[a * 3 + 0], w1 = U[a * 3 + 1], w2 = U[a * 3 + 2];
    const float2 r0 = f2(w0.x), i0 = f2(w0.y);
    const float2 r1 = f2(w1.x), i1 = f2(w1.y);
    const float2 r2 = f2(w2.x), i2 = f2(w2.y);
#pragma unroll
    for (int sp = 0; sp < 2; sp++) {
      const int o = sp * 3;
      float2 p = __fmul2_rn(r0, hr[o]);
      float2 q = __fmul2_rn(i0, hi[o]);
      float2 xi = __fmul2_rn(r0, hi[o]);
      xi = __ffma2_rn(i0, hr[o], xi);
      p = __ffma2_rn(r1, hr[o + 1], p);
      q = __ffma2_rn(i1, hi[o + 1], q);
      xi = __ffma2_rn(r1, hi[o + 1], xi);
      xi = __ffma2_rn(i1, hr[o + 1], xi);
      p = __ffma2_rn(r2, hr[o + 2], p);
      q = __ffma2_rn(i2, hi[o + 2], q);
      xi = __ffma2_rn(r2, hi[o + 2], xi);
      xi = __ffma2_rn(i2, hr[o + 2], xi);
      ur[o + a] = sub2(p, q);
      ui[o + a] = xi;
    }
  }
}

// The two x legs of a t-stream thread: which of +x / -x reaches the input site with the
// thread's own checkerboard index depends on the parity of the site's row, so the x legs
// take their projector sign at run time (s2 = (S, S), S = +-1).  Same roundings as
// project2<0, S> / reconstruct2<0, S, false> with n = 1: a +- b exactly rounded.
__device__ __forceinline__ void project2_x(const Pair12& f, float2 s2, float2 (&hr)[6], float2 (&hi)[6]) {
  const float2 m2 = make_float2(-s2.x, -s2.y);
#pragma unroll
  for (int c = 0; c < 3; c++) {  // h0 = f0 + S i f3, h1 = f1 + S i f2
    hr[c] = __ffma2_rn(f.im[9 + c], m2, f.re[c]);
    hi[c] = __ffma2_rn(f.re[9 + c], s2, f.im[c]);
    hr[3 + c] = __ffma2_rn(f.im[6 + c], m2, f.re[3 + c]);
    hi[3 + c] = __ffma2_rn(f.re[6 + c], s2, f.im[3 + c]);
  }
}
__device__ __forceinline__ void reconstruct2_x(Pair12& r, const float2 (&ur)[6], const float2 (&ui)[6], float2 s2) {
  const float2 one = f2(1.f), m2 = make_float2(-s2.x, -s2.y);
#pragma unroll
  for (int c = 0; c < 3; c++) {  // r0 += u0, r1 += u1, r2 += -S i u1, r3 += -S i u0
    r.re[c] = __ffma2_rn(ur[c], one, r.re[c]);
    r.im[c] = __ffma2_rn(ui[c], one, r.im[c]);
    r.re[3 + c] = __ffma2_rn(ur[3 + c], one, r.re[3 + c]);
    r.im[3 + c] = __ffma2_rn(ui[3 + c], one, r.im[3 + c]);
    r.re[6 + c] = __ffma2_rn(ui[3 + c], s2, r.re[6 + c]);
    r.im[6 + c] = __ffma2_rn(ur[3 + c], m2, r.im[6 + c]);
    r.re[9 + c] = __ffma2_rn(ui[c], s2, r.re[9 + c]);
    r.im[9 + c] = __ffma2_rn(ur[c], m2, r.im[9 + c]);
  }
}

}  // namespace gb
