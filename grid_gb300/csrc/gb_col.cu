// gb_col.cu -- fused s-column kernels of the Cayley 5D operators (FP32 / FP16 site-pair layout).
//
// Every Cayley 5D operator acts on each spin-colour component of each (4D site, rhs)
// column of Ls values on its own, because the chiral projectors P+- are diagonal in spin:
// M5D (CayleyFermion5Dcache.h:41-115) couples s to s-1 (P+ components, non-dagger) or
// s+1 (P- components), and MooeeInv (CayleyFermion5Dcache.h:117-230) is an LDU solve
// along s.  A CTA stages Q columns x 12 components of its input(s) in shared memory with
// coalesced 16-byte loads, one thread per (component, column) runs a short program of
// these operators on its column in registers, and the CTA stores the result coalesced.
// FP16 fields are decoded with their per-site norms on the way in and get new norms (the
// largest |re|, |im| of each 5D site) on the way out.
//
// Programs: out = A(x) + zc * B(y) with
//   A in {M5D, INV, M5D(INV(x)), INV(M5D(x))},  B in {none, y, M5D(y)},
// one dagger flag for the whole program.  They fuse the steps of
// SchurDiagMooeeOperator::Mpc / MpcDag (LinearOperator.h:330-349) that touch no
// neighbour in 4D: Mpc = Mooee - DhopOE M5D MooeeInv DhopEO M5D, and
// MpcDag = MooeeDag - M5Ddag DhopOE^dag MooeeInvDag M5Ddag DhopEO^dag.
#include <atomic>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {

// columns per CTA and the shared-memory slot of one column (an odd number of float4, so
// the column reads of a quarter warp fall on distinct banks)
// (with two input tiles 16 columns, so that several CTAs fit an SM's shared memory)
template <int LS, int NIN = 1> __host__ __device__ constexpr int col_q() { return (LS >= 16 || NIN > 1) ? 16 : 32; }
template <int LS> __host__ __device__ constexpr int col_stride() { return (LS / 2) % 2 == 0 ? LS / 2 + 1 : LS / 2; }

template <int LS> struct ColCoef {
  float d1[LS], u1[LS], l1[LS];  // M5D of A
  float d2[LS], u2[LS], l2[LS];  // M5D of B
  float lee[LS], leem[LS], uee[LS], ueem[LS], dinv[LS];  // LDU factors (dagger-swapped)
};

struct ColParams {
  const void* x;
  const void* y;
  void* out;
  const float* xn;  // FP16: per-5D-site norms
  const float* yn;
  float* outn;
  size_t np;  // 16-byte vectors per plane (site pairs per half field)
  size_t nq;  // columns: 4D sites x right-hand sides
  float zc;
  // RUPD (the last program of MpcDag in the CG): instead of storing out, r -= a out with
  // each right-hand side's CG scalar a, and per-CTA sums of |r|^2 per right-hand side into
  // rpart[CTA][nrhs] (the layout of the norm partials); nrhs divides the tile's columns
  void* r;
  float* rn;  // FP16: the per-5D-site norms of r
  double* rpart;
  const CGScalars* cg;
  int nrhs;
};

// stage one input into the [12][Q][ST] float4 tile: FP32 copies the vectors, FP16 decodes
// the two components of each vector with the norms of the pair's sites
template <class T, int LS, int Q> struct ColIO;
template <int LS, int Q> struct ColIO<float, LS, Q> {
  static __device__ __forceinline__ void load(const void* src, const float*, float*, float4* tile, size_t np, size_t q0,
                                              int nv) {
    constexpr int H = LS / 2, ST = col_stride<LS>();
    const float4* x = static_cast<const float4*>(src);
#pragma unroll 4
    for (int e = threadIdx.x; e < 12 * Q * H; e += 12 * Q) {
      const int k = e / (Q * H), r = e - k * (Q * H);
      if (r < nv) {
        const int qq = r / H, m = r - qq * H;
        tile[(k * Q + qq) * ST + m] = __ldg(x + size_t(k) * np + q0 * H + r);
      }
    }
  }
  static __device__ __forceinline__ void store(void* dst, float*, float*, float4* tile, size_t np, size_t q0, int nv) {
    constexpr int H = LS / 2, ST = col_stride<LS>();
    float4* o = static_cast<float4*>(dst);
#pragma unroll 4
    for (int e = threadIdx.x; e < 12 * Q * H; e += 12 * Q) {
      const int k = e / (Q * H), r = e - k * (Q * H);
      if (r < nv) {
        const int qq = r / H, m = r - qq * H;
        o[size_t(k) * np + q0 * H + r] = tile[(k * Q + qq) * ST + m];
      }
    }
  }
};
template <int LS, int Q> struct ColIO<__half, LS, Q> {
  // snorm: Q * LS floats of shared memory for the CTA's site norms
  static __device__ __forceinline__ void load(const void* src, const float* norms, float* snorm, float4* tile,
                                              size_t np, size_t q0, int nv) {
    constexpr int H = LS / 2, ST = col_stride<LS>();
    for (int e = threadIdx.x; e < 2 * nv; e += 12 * Q) snorm[e] = __ldg(norms + q0 * LS + e);
    __syncthreads();
    const uint4* x = static_cast<const uint4*>(src);
    for (int e = threadIdx.x; e < 6 * Q * H; e += 12 * Q) {
      const int g = e / (Q * H), r = e - g * (Q * H);
      if (r < nv) {
        const int qq = r / H, m = r - qq * H;
        const uint4 v = __ldg(x + size_t(g) * np + q0 * H + r);
        const __half2* h = reinterpret_cast<const __half2*>(&v);
        const float n0 = snorm[qq * LS + 2 * m], n1 = snorm[qq * LS + 2 * m + 1];
        const float2 a = __half22float2(h[0]), b = __half22float2(h[1]), c = __half22float2(h[2]),
                     d = __half22float2(h[3]);
        tile[((2 * g) * Q + qq) * ST + m] = make_float4(a.x * n0, a.y * n1, b.x * n0, b.y * n1);
        tile[((2 * g + 1) * Q + qq) * ST + m] = make_float4(c.x * n0, c.y * n1, d.x * n0, d.y * n1);
      }
    }
    __syncthreads();  // snorm is reused by the next input
  }
  static __device__ __forceinline__ void store(void* dst, float* norms, float* snorm, float4* tile, size_t np,
                                               size_t q0, int nv) {
    constexpr int H = LS / 2, ST = col_stride<LS>();
    // the norm of each 5D site: the largest |re|, |im| over its 12 components
    for (int e = threadIdx.x; e < 2 * nv; e += 12 * Q) {
      const int qq = e / LS, sl = e - qq * LS, m = sl >> 1, l = sl & 1;
      float mx = 0.f;
#pragma unroll
      for (int k = 0; k < 12; k++) {
        const float4 v = tile[(k * Q + qq) * ST + m];
        mx = fmaxf(mx, fmaxf(fabsf(l ? v.y : v.x), fabsf(l ? v.w : v.z)));
      }
      snorm[e] = mx;
      norms[q0 * LS + e] = mx;
    }
    __syncthreads();
    uint4* o = static_cast<uint4*>(dst);
    for (int e = threadIdx.x; e < 6 * Q * H; e += 12 * Q) {
      const int g = e / (Q * H), r = e - g * (Q * H);
      if (r < nv) {
        const int qq = r / H, m = r - qq * H;
        const float m0 = snorm[qq * LS + 2 * m], m1 = snorm[qq * LS + 2 * m + 1];
        const float2 inv = make_float2(m0 > 0.f ? 1.0f / m0 : 0.f, m1 > 0.f ? 1.0f / m1 : 0.f);
        const float4 a = tile[((2 * g) * Q + qq) * ST + m], b = tile[((2 * g + 1) * Q + qq) * ST + m];
        uint4 v;
        __half2* h = reinterpret_cast<__half2*>(&v);
        h[0] = __float22half2_rn(__fmul2_rn(make_float2(a.x, a.y), inv));
        h[1] = __float22half2_rn(__fmul2_rn(make_float2(a.z, a.w), inv));
        h[2] = __float22half2_rn(__fmul2_rn(make_float2(b.x, b.y), inv));
        h[3] = __float22half2_rn(__fmul2_rn(make_float2(b.z, b.w), inv));
        o[size_t(g) * np + q0 * H + r] = v;
      }
    }
  }
};

// chi_s = d_s x_s + (l_s x_{s-1} | u_s x_{s+1}) with the wrap inside the column
template <int LS, bool DAG>
__device__ __forceinline__ void col_m5d(const float (&xr)[LS], const float (&xi)[LS], float (&yr)[LS], float (&yi)[LS],
                                        const float* d, const float* u, const float* l, bool upper) {
  const bool from_minus = DAG ? !upper : upper;
#pragma unroll
  for (int s = 0; s < LS; s++) {
    const float c = from_minus ? l[s] : u[s];
    const float nr = from_minus ? xr[(s + LS - 1) % LS] : xr[(s + 1) % LS];
    const float ni = from_minus ? xi[(s + LS - 1) % LS] : xi[(s + 1) % LS];
    yr[s] = fmaf(c, nr, d[s] * xr[s]);
    yi[s] = fmaf(c, ni, d[s] * xi[s]);
  }
}

// in place LDU solve along s: forward sweep with lee (first chirality) or the leem
// column (second), backward sweep with uee (second) or the ueem column (first)
template <int LS>
__device__ __forceinline__ void col_inv(float (&r)[LS], float (&i)[LS], const ColCoef<LS>& c, bool first) {
  float pr = 0.f, pi = 0.f, ar = 0.f, ai = 0.f;
#pragma unroll
  for (int s = 0; s < LS; s++) {
    float xr = r[s], xi = i[s];
    if (s < LS - 1) {
      if (first) {
        if (s > 0) { xr = fmaf(-c.lee[s - 1], pr, xr); xi = fmaf(-c.lee[s - 1], pi, xi); }
      } else {
        ar = fmaf(c.leem[s], xr, ar); ai = fmaf(c.leem[s], xi, ai);
      }
      pr = xr; pi = xi;
    } else {
      if (first) { xr = fmaf(-c.lee[LS - 2], pr, xr); xi = fmaf(-c.lee[LS - 2], pi, xi); }
      else { xr -= ar; xi -= ai; }
      xr *= c.dinv[LS - 1]; xi *= c.dinv[LS - 1];
    }
    r[s] = xr; i[s] = xi;
  }
  const float lr = r[LS - 1], li = i[LS - 1];
  float nr = lr, ni = li;
#pragma unroll
  for (int s = LS - 2; s >= 0; s--) {
    float xr = r[s] * c.dinv[s], xi = i[s] * c.dinv[s];
    if (!first) { xr = fmaf(-c.uee[s], nr, xr); xi = fmaf(-c.uee[s], ni, xi); }
    else { xr = fmaf(-c.ueem[s], lr, xr); xi = fmaf(-c.ueem[s], li, xi); }
    r[s] = xr; i[s] = xi;
    nr = xr; ni = xi;
  }
}

template <int LS>
__device__ __forceinline__ void col_read(const float4* slot, float (&r)[LS], float (&i)[LS]) {
#pragma unroll
  for (int m = 0; m < LS / 2; m++) {
    const float4 v = slot[m];
    r[2 * m] = v.x; r[2 * m + 1] = v.y;
    i[2 * m] = v.z; i[2 * m + 1] = v.w;
  }
}

// the program on one (component, column): slot (and yslot) hold its LS values as LS/2
// float4 (re_s, re_s+1, im_s, im_s+1); the result replaces slot
template <int LS, bool DAG, int OPA, int OPB>
__device__ __forceinline__ void col_run(float4* slot, const float4* yslot, float zc, const ColCoef<LS>& c,
                                        bool upper) {
  constexpr int H = LS / 2;
  const bool first = DAG ? !upper : upper;
  float xr[LS], xi[LS], orr[LS], oi[LS];
  col_read<LS>(slot, xr, xi);
  if (OPA == COL_M5D) {
    col_m5d<LS, DAG>(xr, xi, orr, oi, c.d1, c.u1, c.l1, upper);
  } else if (OPA == COL_INV) {
    col_inv<LS>(xr, xi, c, first);
#pragma unroll
    for (int s = 0; s < LS; s++) { orr[s] = xr[s]; oi[s] = xi[s]; }
  } else if (OPA == COL_INV_M5D) {
    col_inv<LS>(xr, xi, c, first);
    col_m5d<LS, DAG>(xr, xi, orr, oi, c.d1, c.u1, c.l1, upper);
  } else {  // COL_M5D_INV
    col_m5d<LS, DAG>(xr, xi, orr, oi, c.d1, c.u1, c.l1, upper);
    col_inv<LS>(orr, oi, c, first);
  }
  if (OPB != COLB_NONE) {
    float yr[LS], yi[LS];
    col_read<LS>(yslot, yr, yi);
    if (OPB == COLB_M5D) {
      col_m5d<LS, DAG>(yr, yi, xr, xi, c.d2, c.u2, c.l2, upper);
#pragma unroll
      for (int s = 0; s < LS; s++) { yr[s] = xr[s]; yi[s] = xi[s]; }
    }
#pragma unroll
    for (int s = 0; s < LS; s++) { orr[s] = fmaf(zc, yr[s], orr[s]); oi[s] = fmaf(zc, yi[s], oi[s]); }
  }
#pragma unroll
  for (int m = 0; m < H; m++) slot[m] = make_float4(orr[2 * m], orr[2 * m + 1], oi[2 * m], oi[2 * m + 1]);
}

template <class T, int LS, bool DAG, int OPA, int OPB>
__global__ void __launch_bounds__(12 * col_q<LS, OPB != COLB_NONE ? 2 : 1>()) col_kernel(const ColParams p,
                                                                                        const ColCoef<LS> c) {
  constexpr int Q = col_q<LS, OPB != COLB_NONE ? 2 : 1>(), H = LS / 2, ST = col_stride<LS>();
  extern __shared__ float4 col_tile[];  // [inputs][12][Q][ST], then Q * LS norms (FP16)
  float4* tx = col_tile;
  float4* ty = col_tile + 12 * Q * ST;
  float* snorm = reinterpret_cast<float*>(col_tile + (OPB != COLB_NONE ? 2 : 1) * 12 * Q * ST);
  const int t = threadIdx.x;
  const size_t q0 = size_t(blockIdx.x) * Q;
  const int qn = p.nq - q0 < size_t(Q) ? int(p.nq - q0) : Q;
  const int nv = qn * H;  // vectors of one plane in this CTA
  ColIO<T, LS, Q>::load(p.x, p.xn, snorm, tx, p.np, q0, nv);
  if (OPB != COLB_NONE) ColIO<T, LS, Q>::load(p.y, p.yn, snorm, ty, p.np, q0, nv);
  __syncthreads();
  const int k = t / Q, qq = t - k * Q;
  if (qq < qn) col_run<LS, DAG, OPA, OPB>(tx + (k * Q + qq) * ST, ty + (k * Q + qq) * ST, p.zc, c, k < 6);
  __syncthreads();
  ColIO<T, LS, Q>::store(p.out, p.outn, snorm, tx, p.np, q0, nv);
}

// FP32 programs as a persistent kernel: each CTA walks its tiles of 16 columns with the
// next tile's inputs arriving by cp.async (16-byte copies straight into the padded,
// bank-conflict-free shared layout) in a second stage while the current one computes
// and stores.  No wait spins: cp.async.wait_group waits on the thread's own copies.
#ifndef GB_COL_PIPE_Q
#define GB_COL_PIPE_Q 16
#endif
#ifndef GB_COL_STAGES
#define GB_COL_STAGES 2
#endif
constexpr int kColPipeQ = GB_COL_PIPE_Q;     // columns per tile
constexpr int kColStages = GB_COL_STAGES;    // tiles in flight per CTA

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// columns [q0, q0 + nv / H) of all 12 planes into a [12][Q][ST] tile
template <int LS>
__device__ __forceinline__ void col_issue(const float4* x, float4* tile, size_t np, size_t q0, int nv) {
  constexpr int Q = kColPipeQ, H = LS / 2, ST = col_stride<LS>();
#pragma unroll 4
  for (int e = threadIdx.x; e < 12 * Q * H; e += 12 * Q) {
    const int k = e / (Q * H), r = e - k * (Q * H);
    if (r < nv) {
      const int qq = r / H, m = r - qq * H;
      cp_async16(tile + (k * Q + qq) * ST + m, x + size_t(k) * np + q0 * H + r);
    }
  }
}

template <int LS, bool DAG, int OPA, int OPB, bool RUPD>
__global__ void __launch_bounds__(12 * kColPipeQ) col_pipe_kernel(const ColParams p, const ColCoef<LS> c) {
  constexpr int Q = kColPipeQ, H = LS / 2, ST = col_stride<LS>(), NIN = OPB != COLB_NONE ? 2 : 1;
  constexpr int TILE = 12 * Q * ST;   // float4 of one input tile
  extern __shared__ float4 col_ring[];  // [kColStages][NIN][12][Q][ST]
  const size_t ntiles = (p.nq + Q - 1) / Q;
  const float4* xs = static_cast<const float4*>(p.x);
  const float4* ys = static_cast<const float4*>(p.y);
  float4* o = static_cast<float4*>(p.out);
  const int t = threadIdx.x, k = t / Q, qq = t - k * Q;
  auto vectors = [&](size_t tile) { return int(min(p.nq - tile * Q, size_t(Q))) * H; };
  auto issue = [&](size_t tile, int st) {  // one commit group per stage fill, empty past the end
    if (tile < ntiles) {
      float4* base = col_ring + size_t(st) * NIN * TILE;
      col_issue<LS>(xs, base, p.np, tile * Q, vectors(tile));
      if (NIN == 2) col_issue<LS>(ys, base + TILE, p.np, tile * Q, vectors(tile));
    }
    cp_async_commit();
  };
  size_t tile = blockIdx.x;
  // RUPD: -a per right-hand side; |r|^2 of each element of the tile, then per column (one
  // (4D site, rhs) each; tiles start at a multiple of nrhs columns, so column q2 of every
  // tile belongs to right-hand side q2 % nrhs), FP32 per tile and FP64 across tiles
  __shared__ float sma[kColPipeQ];
  __shared__ float cn[RUPD ? 12 * Q * H : 1];
  double colacc = 0.0;  // thread t < Q: |r|^2 of column t of this CTA's tiles
  if (RUPD && t < p.nrhs) sma[t] = -float(p.cg[t].a);  // read after the loop's first barrier
  for (int k0 = 0; k0 < kColStages - 1; k0++) issue(tile + size_t(k0) * gridDim.x, k0);
  for (int st = 0; tile < ntiles; tile += gridDim.x, st = st + 1 == kColStages ? 0 : st + 1) {
    // refill the stage computed last (stored out before the last barrier), then wait for
    // this stage's group: all but the newest kColStages - 1 groups have landed
    issue(tile + size_t(kColStages - 1) * gridDim.x, st == 0 ? kColStages - 1 : st - 1);
    const int nv = vectors(tile);
    // RUPD: this thread's H vectors of r (the ones its store loop updates) are loaded
    // before the wait, so they arrive while the tile lands and its columns compute
    float4 rv[RUPD ? H : 1];
    if (RUPD) {
#pragma unroll
      for (int j = 0; j < H; j++) {
        const int e = t + j * 12 * Q, kk = e / (Q * H), r = e - kk * (Q * H);
        if (r < nv) rv[j] = static_cast<const float4*>(p.r)[size_t(kk) * p.np + tile * Q * H + r];
      }
    }
    cp_async_wait<kColStages - 1>();
    __syncthreads();
    float4* base = col_ring + size_t(st) * NIN * TILE;
    if (qq < nv / H) col_run<LS, DAG, OPA, OPB>(base + (k * Q + qq) * ST, base + TILE + (k * Q + qq) * ST, p.zc, c, k < 6);
    __syncthreads();
    if (RUPD) {
#pragma unroll
      for (int j = 0; j < H; j++) {
        const int e = t + j * 12 * Q, kk = e / (Q * H), r = e - kk * (Q * H);
        if (r < nv) {
          const int q2 = r / H, m = r - q2 * H;
          const float4 v = base[(kk * Q + q2) * ST + m];
          const float ma = sma[q2 % p.nrhs];
          float4 w = rv[j];
          w.x = fmaf(ma, v.x, w.x); w.y = fmaf(ma, v.y, w.y);
          w.z = fmaf(ma, v.z, w.z); w.w = fmaf(ma, v.w, w.w);
          static_cast<float4*>(p.r)[size_t(kk) * p.np + tile * Q * H + r] = w;
          cn[(kk * Q + q2) * H + m] = fmaf(w.x, w.x, fmaf(w.y, w.y, fmaf(w.z, w.z, w.w * w.w)));
        }
      }
      __syncthreads();
      if (t < nv / H) {
        float s = 0.f;
        for (int kk = 0; kk < 12; kk++)
#pragma unroll
          for (int m = 0; m < H; m++) s += cn[(kk * Q + t) * H + m];
        colacc += double(s);
      }
    } else {
#pragma unroll 4
      for (int e = t; e < 12 * Q * H; e += 12 * Q) {
        const int kk = e / (Q * H), r = e - kk * (Q * H);
        if (r < nv) {
          const int q2 = r / H, m = r - q2 * H;
          o[size_t(kk) * p.np + tile * Q * H + r] = base[(kk * Q + q2) * ST + m];
        }
      }
    }
    __syncthreads();  // the stage is read out before it is refilled
  }
  cp_async_wait<0>();
  if (RUPD) {  // per right-hand side: its columns' sums in column order
    __shared__ double csum[kColPipeQ];
    if (t < Q) csum[t] = colacc;
    __syncthreads();
    if (t < p.nrhs) {
      double s = 0.0;
      for (int q2 = t; q2 < Q; q2 += p.nrhs) s += csum[q2];
      p.rpart[size_t(blockIdx.x) * p.nrhs + t] = s;
    }
  }
}

// FP16 programs on the same ring: each stage holds a tile's raw vectors (6 planes of
// 16-byte vectors, two components of a site pair each, in their global order) and its
// per-site norms, fetched by cp.async; after they land the CTA decodes them into the
// float tile, runs the program and stores through the FP16 encoder (fresh norms).
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

template <int LS>
__device__ __forceinline__ void col_issue_half(const uint4* x, const float* xn, uint4* raw, float* rnorm, size_t np,
                                               size_t q0, int nv) {
  constexpr int Q = kColPipeQ, H = LS / 2;
  for (int e = threadIdx.x; e < 6 * Q * H; e += 12 * Q) {
    const int g = e / (Q * H), r = e - g * (Q * H);
    if (r < nv) cp_async16(raw + g * (Q * H) + r, x + size_t(g) * np + q0 * H + r);
  }
  for (int e = threadIdx.x; e < 2 * nv; e += 12 * Q) cp_async4(rnorm + e, xn + q0 * LS + e);
}

template <int LS>
__device__ __forceinline__ void col_decode_half(const uint4* raw, const float* rnorm, float4* tile, int nv) {
  constexpr int Q = kColPipeQ, H = LS / 2, ST = col_stride<LS>();
  for (int e = threadIdx.x; e < 6 * Q * H; e += 12 * Q) {
    const int g = e / (Q * H), r = e - g * (Q * H);
    if (r < nv) {
      const int qq = r / H, m = r - qq * H;
      const uint4 v = raw[g * (Q * H) + r];
      const __half2* h = reinterpret_cast<const __half2*>(&v);
      const float n0 = rnorm[qq * LS + 2 * m], n1 = rnorm[qq * LS + 2 * m + 1];
      const float2 a = __half22float2(h[0]), b = __half22float2(h[1]), c = __half22float2(h[2]),
                   d = __half22float2(h[3]);
      tile[((2 * g) * Q + qq) * ST + m] = make_float4(a.x * n0, a.y * n1, b.x * n0, b.y * n1);
      tile[((2 * g + 1) * Q + qq) * ST + m] = make_float4(c.x * n0, c.y * n1, d.x * n0, d.y * n1);
    }
  }
}

// RUPD (the last program of MpcDag in the CG, two inputs): r is a third raw input of the
// ring; after the program it is decoded into the y tile (free by then), r -= a[rhs] out is
// formed there and stored through the FP16 encoder, and |r|^2 (before encoding, as the
// separate update pass sums it) is summed per column and right-hand side as in
// col_pipe_kernel.
template <int LS, bool DAG, int OPA, int OPB, bool RUPD>
__global__ void __launch_bounds__(12 * kColPipeQ) col_pipe_half_kernel(const ColParams p, const ColCoef<LS> c) {
  constexpr int Q = kColPipeQ, H = LS / 2, ST = col_stride<LS>(), NIN = OPB != COLB_NONE ? 2 : 1;
  constexpr int NRING = NIN + (RUPD ? 1 : 0);  // raw inputs staged per tile
  constexpr int RAW = 6 * Q * H;      // uint4 of one input's raw tile
  constexpr int TILE = 12 * Q * ST;   // float4 of one input's decoded tile
  // [NIN float tiles][kColStages][NRING][raw tile][Q * LS norms], then Q * LS floats of scratch
  extern __shared__ float4 col_half_smem[];
  float4* ftile = col_half_smem;
  uint4* ring = reinterpret_cast<uint4*>(col_half_smem + NIN * TILE);
  constexpr int SLOT = RAW + Q * LS / 4;  // uint4 per input per stage (norms packed 4 per uint4)
  float* snorm = reinterpret_cast<float*>(ring + size_t(kColStages) * NRING * SLOT);
  const size_t ntiles = (p.nq + Q - 1) / Q;
  const uint4* xs = static_cast<const uint4*>(p.x);
  const uint4* ys = static_cast<const uint4*>(p.y);
  const int t = threadIdx.x, k = t / Q, qq = t - k * Q;
  auto vectors = [&](size_t tile) { return int(min(p.nq - tile * Q, size_t(Q))) * H; };
  auto slot = [&](int st, int j) { return ring + (size_t(st) * NRING + j) * SLOT; };
  auto issue = [&](size_t tile, int st) {
    if (tile < ntiles) {
      col_issue_half<LS>(xs, p.xn, slot(st, 0), reinterpret_cast<float*>(slot(st, 0) + RAW), p.np, tile * Q,
                         vectors(tile));
      if (NIN == 2)
        col_issue_half<LS>(ys, p.yn, slot(st, 1), reinterpret_cast<float*>(slot(st, 1) + RAW), p.np, tile * Q,
                           vectors(tile));
      if (RUPD)
        col_issue_half<LS>(static_cast<const uint4*>(p.r), p.rn, slot(st, NIN),
                           reinterpret_cast<float*>(slot(st, NIN) + RAW), p.np, tile * Q, vectors(tile));
    }
    cp_async_commit();
  };
  __shared__ float sma[kColPipeQ];
  __shared__ float cn[RUPD ? 12 * Q * H : 1];
  double colacc = 0.0;  // thread t < Q: |r|^2 of column t of this CTA's tiles
  if (RUPD && t < p.nrhs) sma[t] = -float(p.cg[t].a);  // read after the loop's first barrier
  size_t tile = blockIdx.x;
  for (int k0 = 0; k0 < kColStages - 1; k0++) issue(tile + size_t(k0) * gridDim.x, k0);
  for (int st = 0; tile < ntiles; tile += gridDim.x, st = st + 1 == kColStages ? 0 : st + 1) {
    issue(tile + size_t(kColStages - 1) * gridDim.x, st == 0 ? kColStages - 1 : st - 1);
    cp_async_wait<kColStages - 1>();
    __syncthreads();
    const int nv = vectors(tile);
    for (int j = 0; j < NIN; j++)
      col_decode_half<LS>(slot(st, j), reinterpret_cast<const float*>(slot(st, j) + RAW), ftile + j * TILE, nv);
    __syncthreads();
    if (qq < nv / H) col_run<LS, DAG, OPA, OPB>(ftile + (k * Q + qq) * ST, ftile + TILE + (k * Q + qq) * ST, p.zc, c, k < 6);
    __syncthreads();
    if (RUPD) {
      float4* rt = ftile + TILE;  // the y tile, read by the program only
      col_decode_half<LS>(slot(st, NIN), reinterpret_cast<const float*>(slot(st, NIN) + RAW), rt, nv);
      __syncthreads();
      for (int e = t; e < 12 * Q * H; e += 12 * Q) {
        const int kk = e / (Q * H), r = e - kk * (Q * H);
        if (r < nv) {
          const int q2 = r / H, m = r - q2 * H, i = (kk * Q + q2) * ST + m;
          const float ma = sma[q2 % p.nrhs];
          const float4 v = ftile[i];
          float4 w = rt[i];
          w.x = fmaf(ma, v.x, w.x); w.y = fmaf(ma, v.y, w.y);
          w.z = fmaf(ma, v.z, w.z); w.w = fmaf(ma, v.w, w.w);
          rt[i] = w;
          cn[(kk * Q + q2) * H + m] = fmaf(w.x, w.x, fmaf(w.y, w.y, fmaf(w.z, w.z, w.w * w.w)));
        }
      }
      __syncthreads();
      if (t < nv / H) {
        float s = 0.f;
        for (int kk = 0; kk < 12; kk++)
#pragma unroll
          for (int m = 0; m < H; m++) s += cn[(kk * Q + t) * H + m];
        colacc += double(s);
      }
      ColIO<__half, LS, Q>::store(p.r, p.rn, snorm, rt, p.np, tile * Q, nv);
    } else {
      ColIO<__half, LS, Q>::store(p.out, p.outn, snorm, ftile, p.np, tile * Q, nv);
    }
    __syncthreads();  // the float tile and this stage are read out before they are reused
  }
  cp_async_wait<0>();
  if (RUPD) {  // per right-hand side: its columns' sums in column order
    __shared__ double csum[kColPipeQ];
    if (t < Q) csum[t] = colacc;
    __syncthreads();
    if (t < p.nrhs) {
      double s = 0.0;
      for (int q2 = t; q2 < Q; q2 += p.nrhs) s += csum[q2];
      p.rpart[size_t(blockIdx.x) * p.nrhs + t] = s;
    }
  }
}

template <int LS> static void fill_col(const Op* op, int dag, const ColCoefsHost& h, ColCoef<LS>& c) {
  const std::vector<double>& lee = dag ? op->uee : op->lee;
  const std::vector<double>& leem = dag ? op->ueem : op->leem;
  const std::vector<double>& uee = dag ? op->lee : op->uee;
  const std::vector<double>& ueem = dag ? op->leem : op->ueem;
  for (int s = 0; s < LS; s++) {
    c.d1[s] = h.d1.empty() ? 0.f : float(h.d1[s]);
    c.u1[s] = h.u1.empty() ? 0.f : float(h.u1[s]);
    c.l1[s] = h.l1.empty() ? 0.f : float(h.l1[s]);
    c.d2[s] = h.d2.empty() ? 0.f : float(h.d2[s]);
    c.u2[s] = h.u2.empty() ? 0.f : float(h.u2[s]);
    c.l2[s] = h.l2.empty() ? 0.f : float(h.l2[s]);
    c.lee[s] = float(lee[s]); c.leem[s] = float(leem[s]);
    c.uee[s] = float(uee[s]); c.ueem[s] = float(ueem[s]);
    c.dinv[s] = float(1.0 / op->dee[s]);
  }
}

#ifndef GB_COL_PIPE
#define GB_COL_PIPE 1
#endif

template <int LS, bool DAG, int OPA, int OPB, bool RUPD = false>
static int col_pipe_go(Op* op, const ColParams& p, const ColCoef<LS>& c, int* r_parts = nullptr) {
  constexpr int NIN = OPB != COLB_NONE ? 2 : 1;
  const size_t smem = size_t(kColStages) * NIN * 12 * kColPipeQ * col_stride<LS>() * sizeof(float4);
  static std::atomic<int> per_sm{0};
  static std::atomic<int> sms{0};
  if (per_sm.load() == 0) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(col_pipe_kernel<LS, DAG, OPA, OPB, RUPD>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int n = 0, dev = 0, count = 0;
    GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, col_pipe_kernel<LS, DAG, OPA, OPB, RUPD>,
                                                                12 * kColPipeQ, smem));
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev));
    sms.store(count);
    per_sm.store(n > 0 ? n : 1);
  }
  const size_t ntiles = (p.nq + kColPipeQ - 1) / kColPipeQ;
  size_t slots = size_t(per_sm.load()) * size_t(sms.load());
  if (RUPD && slots > size_t(2) * kRedBlocks) slots = size_t(2) * kRedBlocks;  // the partial buffer's [CTA][nrhs]
  const unsigned blocks = unsigned(ntiles < slots ? ntiles : slots);
  col_pipe_kernel<LS, DAG, OPA, OPB, RUPD><<<blocks, 12 * kColPipeQ, smem, op->stream>>>(p, c);
  GB_CHECK_CUDA(cudaGetLastError());
  if (r_parts) *r_parts = RUPD ? int(blocks) : 0;
  return GB_OK;
}

template <int LS, bool DAG, int OPA, int OPB, bool RUPD = false>
static int col_pipe_half_go(Op* op, const ColParams& p, const ColCoef<LS>& c, int* r_parts = nullptr) {
  constexpr int Q = kColPipeQ, NIN = OPB != COLB_NONE ? 2 : 1, NRING = NIN + (RUPD ? 1 : 0);
  constexpr size_t RAW = size_t(6) * Q * (LS / 2), SLOT = RAW + Q * LS / 4;
  const size_t smem = size_t(NIN) * 12 * Q * col_stride<LS>() * sizeof(float4) +
                      size_t(kColStages) * NRING * SLOT * sizeof(uint4) + size_t(Q) * LS * sizeof(float);
  static std::atomic<int> per_sm{0};
  static std::atomic<int> sms{0};
  if (per_sm.load() == 0) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(col_pipe_half_kernel<LS, DAG, OPA, OPB, RUPD>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int n = 0, dev = 0, count = 0;
    GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, col_pipe_half_kernel<LS, DAG, OPA, OPB, RUPD>,
                                                                12 * Q, smem));
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev));
    sms.store(count);
    per_sm.store(n > 0 ? n : 1);
  }
  const size_t ntiles = (p.nq + Q - 1) / Q;
  size_t slots = size_t(per_sm.load()) * size_t(sms.load());
  if (RUPD && slots > size_t(2) * kRedBlocks) slots = size_t(2) * kRedBlocks;  // the partial buffer's [CTA][nrhs]
  const unsigned blocks = unsigned(ntiles < slots ? ntiles : slots);
  col_pipe_half_kernel<LS, DAG, OPA, OPB, RUPD><<<blocks, 12 * Q, smem, op->stream>>>(p, c);
  GB_CHECK_CUDA(cudaGetLastError());
  if (r_parts) *r_parts = RUPD ? int(blocks) : 0;
  return GB_OK;
}

template <class T, int LS, bool DAG, int OPA, int OPB>
static int col_go(Op* op, const ColParams& p, const ColCoef<LS>& c) {
  if (GB_COL_PIPE && sizeof(T) == 4) return col_pipe_go<LS, DAG, OPA, OPB>(op, p, c);
  if (GB_COL_PIPE && sizeof(T) == 2) return col_pipe_half_go<LS, DAG, OPA, OPB>(op, p, c);
  constexpr int Q = col_q<LS, OPB != COLB_NONE ? 2 : 1>();
  const size_t smem = size_t(OPB != COLB_NONE ? 2 : 1) * 12 * Q * col_stride<LS>() * sizeof(float4) +
                      (sizeof(T) == 2 ? size_t(Q) * LS * sizeof(float) : 0);
  static std::atomic<bool> configured{false};
  if (!configured.load()) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(col_kernel<T, LS, DAG, OPA, OPB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(smem)));
    configured.store(true);
  }
  const unsigned blocks = unsigned((p.nq + Q - 1) / Q);
  col_kernel<T, LS, DAG, OPA, OPB><<<blocks, 12 * Q, smem, op->stream>>>(p, c);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// the programs the operators use; the others are not instantiated
template <class T, int LS>
static int col_ls(Op* op, int opa, int opb, int dag, const ColParams& p, const ColCoefsHost& h, int* r_parts) {
  ColCoef<LS> c;
  fill_col<LS>(op, dag, h, c);
  if (GB_COL_PIPE && p.r && dag && opa == COL_M5D && opb == COLB_M5D) {
    if (sizeof(T) == 4) return col_pipe_go<LS, true, COL_M5D, COLB_M5D, true>(op, p, c, r_parts);
    return col_pipe_half_go<LS, true, COL_M5D, COLB_M5D, true>(op, p, c, r_parts);
  }
  const int key = (dag ? 100 : 0) + opa * 10 + opb;
  switch (key) {
    case 0 + COL_M5D * 10 + COLB_NONE: return col_go<T, LS, false, COL_M5D, COLB_NONE>(op, p, c);
    case 100 + COL_M5D * 10 + COLB_NONE: return col_go<T, LS, true, COL_M5D, COLB_NONE>(op, p, c);
    case 0 + COL_M5D * 10 + COLB_IDENT: return col_go<T, LS, false, COL_M5D, COLB_IDENT>(op, p, c);
    case 100 + COL_M5D * 10 + COLB_IDENT: return col_go<T, LS, true, COL_M5D, COLB_IDENT>(op, p, c);
    case 0 + COL_INV * 10 + COLB_NONE: return col_go<T, LS, false, COL_INV, COLB_NONE>(op, p, c);
    case 100 + COL_INV * 10 + COLB_NONE: return col_go<T, LS, true, COL_INV, COLB_NONE>(op, p, c);
    case 0 + COL_INV_M5D * 10 + COLB_NONE: return col_go<T, LS, false, COL_INV_M5D, COLB_NONE>(op, p, c);
    case 100 + COL_M5D_INV * 10 + COLB_NONE: return col_go<T, LS, true, COL_M5D_INV, COLB_NONE>(op, p, c);
    case 100 + COL_M5D * 10 + COLB_M5D: return col_go<T, LS, true, COL_M5D, COLB_M5D>(op, p, c);
  }
  set_error("column program (%d, %d, dag %d) is not instantiated", opa, opb, dag);
  return GB_ERR_UNSUPPORTED;
}

bool col_available(const Op* op, int prec) {
  if (op->kind != 1 || op->zmobius || (prec != GB_F32 && prec != GB_F16)) return false;
  switch (op->Ls) {
    case 4: case 6: case 8: case 10: case 12: case 16: case 20: case 24: return true;
  }
  return false;
}

int launch_col(Op* op, int opa, int opb, int dag, HalfView x, HalfView y, HalfView out, double zc,
               const ColCoefsHost& h, HalfView* r_upd, int* r_parts) {
  if (r_parts) *r_parts = 0;
  if (!col_available(op, x.prec) || out.prec != x.prec || (opb != COLB_NONE && y.prec != x.prec)) {
    set_error("column kernel: FP32 or FP16 Moebius fields with an instantiated Ls expected");
    return GB_ERR_UNSUPPORTED;
  }
  ColParams p;
  p.x = x.data; p.y = y.data; p.out = out.data;
  p.xn = x.norms; p.yn = y.norms; p.outn = out.norms;
  p.np = op->n5() >> 1;
  p.nq = size_t(op->half4) * op->nrhs;
  p.zc = float(zc);
  const bool rupd = r_upd && r_parts && r_upd->prec == x.prec && kColPipeQ % op->nrhs == 0 && dag &&
                    opa == COL_M5D && opb == COLB_M5D;
  p.r = rupd ? r_upd->data : nullptr;
  p.rn = rupd ? r_upd->norms : nullptr;
  p.rpart = rupd ? op->d_partial : nullptr;
  p.cg = op->d_cg;
  p.nrhs = op->nrhs;
  int* parts = rupd ? r_parts : nullptr;
  const bool half = x.prec == GB_F16;
  switch (op->Ls) {
#define GB_COL_LS(L) \
  case L: return half ? col_ls<__half, L>(op, opa, opb, dag, p, h, parts) : col_ls<float, L>(op, opa, opb, dag, p, h, parts);
    GB_COL_LS(4) GB_COL_LS(6) GB_COL_LS(8) GB_COL_LS(10) GB_COL_LS(12) GB_COL_LS(16) GB_COL_LS(20) GB_COL_LS(24)
#undef GB_COL_LS
  }
  set_error("column kernel: Ls = %d not instantiated", op->Ls);
  return GB_ERR_UNSUPPORTED;
}

}  // namespace gb
