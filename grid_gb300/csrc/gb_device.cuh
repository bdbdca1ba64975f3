// gb_device.cuh -- device helpers: spinor plane I/O, TMA bulk copies with bounded
// mbarrier waits, reductions.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "gb_df64.cuh"
#include "gb_internal.h"

namespace gb {

// ---------------------------------------------------------------------------------------
// Spinor register form: 12 complex components, index spin*3 + colour.
// ---------------------------------------------------------------------------------------
template <class R> struct Spinor {
  R re[12], im[12];
};

// Loads one 5D site's spinor from the plane layout.  T selects the storage:
//   double -> 12 double2 planes, one site per vector; float / __half -> the site-pair
//   layout described below.
template <class R> struct SpinorIO;

template <> struct SpinorIO<double> {
  static __device__ __forceinline__ void load(const void* base, const float*, size_t n5, size_t i, Spinor<double>& f) {
    const double2* p = static_cast<const double2*>(base);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      double2 v = __ldg(p + size_t(k) * n5 + i);
      f.re[k] = v.x; f.im[k] = v.y;
    }
  }
  // only the components of spins {0,1} (upper = true) or {2,3}
  static __device__ __forceinline__ void load_half(const void* base, const float*, size_t n5, size_t i, bool upper,
                                                   Spinor<double>& f) {
    const double2* p = static_cast<const double2*>(base);
    const int k0 = upper ? 0 : 6;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      double2 v = __ldg(p + size_t(k0 + k) * n5 + i);
      f.re[k0 + k] = v.x; f.im[k0 + k] = v.y;
    }
  }
  static __device__ __forceinline__ void store(void* base, float*, size_t n5, size_t i, const Spinor<double>& f) {
    double2* p = static_cast<double2*>(base);
#pragma unroll
    for (int k = 0; k < 12; k++) p[size_t(k) * n5 + i] = make_double2(f.re[k], f.im[k]);
  }
};

// FP64 storage with double-float arithmetic (the hopping term of operators created with
// GB_FLAG_DF64): the FP64 planes, each double split into (hi, lo) floats on load and
// hi + lo rounded back to a double on store.
struct DF64 {};
template <> struct SpinorIO<DF64> {
  static __device__ __forceinline__ void load(const void* base, const float*, size_t n5, size_t i, Spinor<dfloat>& f) {
    const double2* p = static_cast<const double2*>(base);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const double2 v = __ldg(p + size_t(k) * n5 + i);
      f.re[k] = df::split(v.x);
      f.im[k] = df::split(v.y);
    }
  }
  static __device__ __forceinline__ void store(void* base, float*, size_t n5, size_t i, const Spinor<dfloat>& f) {
    double2* p = static_cast<double2*>(base);
#pragma unroll
    for (int k = 0; k < 12; k++) p[size_t(k) * n5 + i] = make_double2(df::to_double(f.re[k]), df::to_double(f.im[k]));
  }
};

// FP32 and FP16 use the site-pair layout: a 16-byte vector holds data of the two 5D
// sites (i, i+1), i even, so a thread can compute both with packed f32x2 arithmetic.
//   FP32: 12 planes (complex component k) of n5/2 float4 = (re_i, re_i+1, im_i, im_i+1)
//   FP16: 6 planes (components 2q, 2q+1) of n5/2 16-byte vectors of 8 halves
//         (re_2q@i, re_2q@i+1, im_2q@i, im_2q@i+1, re_2q+1@i, re_2q+1@i+1, im_2q+1@i, im_2q+1@i+1),
//         each site's values divided by its norm (max |re|,|im| of the site), one float per site.
// SpinorIO<float/__half> read or write ONE site of that layout (scalar accesses; used by
// the kernels that are not on the hot path); PairIO below moves whole vectors.
template <> struct SpinorIO<float> {
  static __device__ __forceinline__ void load(const void* base, const float*, size_t n5, size_t i, Spinor<float>& f) {
    const float* p = static_cast<const float*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const float* v = p + (size_t(k) * np + q) * 4;
      f.re[k] = __ldg(v + l);
      f.im[k] = __ldg(v + 2 + l);
    }
  }
  static __device__ __forceinline__ void load_half(const void* base, const float*, size_t n5, size_t i, bool upper,
                                                   Spinor<float>& f) {
    const float* p = static_cast<const float*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1), k0 = upper ? 0 : 6;
#pragma unroll
    for (int k = k0; k < k0 + 6; k++) {
      const float* v = p + (size_t(k) * np + q) * 4;
      f.re[k] = __ldg(v + l);
      f.im[k] = __ldg(v + 2 + l);
    }
  }
  static __device__ __forceinline__ void store(void* base, float*, size_t n5, size_t i, const Spinor<float>& f) {
    float* p = static_cast<float*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      float* v = p + (size_t(k) * np + q) * 4;
      v[l] = f.re[k];
      v[2 + l] = f.im[k];
    }
  }
};

template <> struct SpinorIO<__half> {
  static __device__ __forceinline__ void load(const void* base, const float* norms, size_t n5, size_t i,
                                              Spinor<float>& f) {
    const __half* p = static_cast<const __half*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1);
    const float nrm = __ldg(norms + i);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const __half* v = p + (size_t(k >> 1) * np + q) * 8 + (k & 1) * 4;
      f.re[k] = __half2float(v[l]) * nrm;
      f.im[k] = __half2float(v[2 + l]) * nrm;
    }
  }
  static __device__ __forceinline__ void load_half(const void* base, const float* norms, size_t n5, size_t i,
                                                   bool upper, Spinor<float>& f) {
    const __half* p = static_cast<const __half*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1), k0 = upper ? 0 : 6;
    const float nrm = __ldg(norms + i);
#pragma unroll
    for (int k = k0; k < k0 + 6; k++) {
      const __half* v = p + (size_t(k >> 1) * np + q) * 8 + (k & 1) * 4;
      f.re[k] = __half2float(v[l]) * nrm;
      f.im[k] = __half2float(v[2 + l]) * nrm;
    }
  }
  static __device__ __forceinline__ void store(void* base, float* norms, size_t n5, size_t i, const Spinor<float>& f) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) m = fmaxf(m, fmaxf(fabsf(f.re[k]), fabsf(f.im[k])));
    const float inv = m > 0.f ? 1.0f / m : 0.f;
    __half* p = static_cast<__half*>(base);
    const size_t np = n5 >> 1, q = i >> 1;
    const int l = int(i & 1);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      __half* v = p + (size_t(k >> 1) * np + q) * 8 + (k & 1) * 4;
      v[l] = __float2half_rn(f.re[k] * inv);
      v[2 + l] = __float2half_rn(f.im[k] * inv);
    }
    norms[i] = m;
  }
};

// ---------------------------------------------------------------------------------------
// Site pairs: component k of sites (i, i+1) as packed float2 (lane 0 = site i).
// ---------------------------------------------------------------------------------------
struct Pair12 {
  float2 re[12], im[12];
};

template <class T> struct PairIO;
template <> struct PairIO<float> {
  // the loaded vectors of one site pair, before conversion (a prefetch buffer)
  struct Raw {
    float4 v[12];
  };
  static __device__ __forceinline__ void load_raw(const void* base, const float2*, size_t np, size_t q, Raw& r) {
    const float4* p = static_cast<const float4*>(base) + q;
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = __ldg(p + size_t(k) * np);
  }
  static __device__ __forceinline__ void decode(const Raw& r, Pair12& f) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      f.re[k] = make_float2(r.v[k].x, r.v[k].y);
      f.im[k] = make_float2(r.v[k].z, r.v[k].w);
    }
  }
  // the stored values and the per-lane factor that scales them to the field's values
  // (a linear consumer may apply the factor late); FP32 stores the values themselves
  static __device__ __forceinline__ void decode_unscaled(const Raw& r, Pair12& f) { decode(r, f); }
  static __device__ __forceinline__ float2 scale(const Raw&) { return make_float2(1.f, 1.f); }
  // q = pair index (= i/2), np = pairs per plane
  static __device__ __forceinline__ void load(const void* base, const float2*, size_t np, size_t q, Pair12& f) {
    const float4* p = static_cast<const float4*>(base) + q;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const float4 v = __ldg(p + size_t(k) * np);
      f.re[k] = make_float2(v.x, v.y);
      f.im[k] = make_float2(v.z, v.w);
    }
  }
  // components [k0, k0+6): one chirality
  static __device__ __forceinline__ void load6(const void* base, const float2*, size_t np, size_t q, int k0, Pair12& f) {
    const float4* p = static_cast<const float4*>(base) + q;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const float4 v = __ldg(p + size_t(k0 + k) * np);
      f.re[k0 + k] = make_float2(v.x, v.y);
      f.im[k0 + k] = make_float2(v.z, v.w);
    }
  }
  static __device__ __forceinline__ void store(void* base, float2*, size_t np, size_t q, const Pair12& f) {
    float4* p = static_cast<float4*>(base) + q;
#pragma unroll
    for (int k = 0; k < 12; k++) p[size_t(k) * np] = make_float4(f.re[k].x, f.re[k].y, f.im[k].x, f.im[k].y);
  }
  // store, and return |stored site|^2 per lane
  static __device__ __forceinline__ float2 store_n2(void* base, float2* n, size_t np, size_t q, const Pair12& f) {
    store(base, n, np, q, f);
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 12; k++) s = __ffma2_rn(f.re[k], f.re[k], __ffma2_rn(f.im[k], f.im[k], s));
    return s;
  }
};

template <> struct PairIO<__half> {
  struct Raw {
    uint4 v[6];
    float2 n;
  };
  static __device__ __forceinline__ void load_raw(const void* base, const float2* norms, size_t np, size_t q, Raw& r) {
    const uint4* p = static_cast<const uint4*>(base) + q;
    r.n = __ldg(norms + q);
#pragma unroll
    for (int g = 0; g < 6; g++) r.v[g] = __ldg(p + size_t(g) * np);
  }
  static __device__ __forceinline__ void decode(const Raw& r, Pair12& f) {
#pragma unroll
    for (int g = 0; g < 6; g++) {
      const __half2* h = reinterpret_cast<const __half2*>(&r.v[g]);
      f.re[2 * g] = __fmul2_rn(__half22float2(h[0]), r.n);
      f.im[2 * g] = __fmul2_rn(__half22float2(h[1]), r.n);
      f.re[2 * g + 1] = __fmul2_rn(__half22float2(h[2]), r.n);
      f.im[2 * g + 1] = __fmul2_rn(__half22float2(h[3]), r.n);
    }
  }
  // the halves as floats, without the per-site norms (scale() returns them)
  static __device__ __forceinline__ void decode_unscaled(const Raw& r, Pair12& f) {
#pragma unroll
    for (int g = 0; g < 6; g++) {
      const __half2* h = reinterpret_cast<const __half2*>(&r.v[g]);
      f.re[2 * g] = __half22float2(h[0]);
      f.im[2 * g] = __half22float2(h[1]);
      f.re[2 * g + 1] = __half22float2(h[2]);
      f.im[2 * g + 1] = __half22float2(h[3]);
    }
  }
  static __device__ __forceinline__ float2 scale(const Raw& r) { return r.n; }
  static __device__ __forceinline__ void load(const void* base, const float2* norms, size_t np, size_t q, Pair12& f) {
    const uint4* p = static_cast<const uint4*>(base) + q;
    const float2 n = __ldg(norms + q);
#pragma unroll
    for (int g = 0; g < 6; g++) {
      const uint4 v = __ldg(p + size_t(g) * np);
      const __half2* h = reinterpret_cast<const __half2*>(&v);
      f.re[2 * g] = __fmul2_rn(__half22float2(h[0]), n);
      f.im[2 * g] = __fmul2_rn(__half22float2(h[1]), n);
      f.re[2 * g + 1] = __fmul2_rn(__half22float2(h[2]), n);
      f.im[2 * g + 1] = __fmul2_rn(__half22float2(h[3]), n);
    }
  }
  static __device__ __forceinline__ void load6(const void* base, const float2* norms, size_t np, size_t q, int k0,
                                               Pair12& f) {
    const uint4* p = static_cast<const uint4*>(base) + q;
    const float2 n = __ldg(norms + q);
#pragma unroll
    for (int g = k0 / 2; g < k0 / 2 + 3; g++) {
      const uint4 v = __ldg(p + size_t(g) * np);
      const __half2* h = reinterpret_cast<const __half2*>(&v);
      f.re[2 * g] = __fmul2_rn(__half22float2(h[0]), n);
      f.im[2 * g] = __fmul2_rn(__half22float2(h[1]), n);
      f.re[2 * g + 1] = __fmul2_rn(__half22float2(h[2]), n);
      f.im[2 * g + 1] = __fmul2_rn(__half22float2(h[3]), n);
    }
  }
  static __device__ __forceinline__ void store(void* base, float2* norms, size_t np, size_t q, const Pair12& f) {
    float m0 = 0.f, m1 = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      m0 = fmaxf(m0, fmaxf(fabsf(f.re[k].x), fabsf(f.im[k].x)));
      m1 = fmaxf(m1, fmaxf(fabsf(f.re[k].y), fabsf(f.im[k].y)));
    }
    const float2 inv = make_float2(m0 > 0.f ? 1.0f / m0 : 0.f, m1 > 0.f ? 1.0f / m1 : 0.f);
    uint4* p = static_cast<uint4*>(base) + q;
#pragma unroll
    for (int g = 0; g < 6; g++) {
      uint4 v;
      __half2* h = reinterpret_cast<__half2*>(&v);
      h[0] = __float22half2_rn(__fmul2_rn(f.re[2 * g], inv));
      h[1] = __float22half2_rn(__fmul2_rn(f.im[2 * g], inv));
      h[2] = __float22half2_rn(__fmul2_rn(f.re[2 * g + 1], inv));
      h[3] = __float22half2_rn(__fmul2_rn(f.im[2 * g + 1], inv));
      p[size_t(g) * np] = v;
    }
    norms[q] = make_float2(m0, m1);
  }
  // store, and return |stored site|^2 per lane: the squares of the halves as a later load
  // decodes them, times the site norm squared
  static __device__ __forceinline__ float2 store_n2(void* base, float2* norms, size_t np, size_t q, const Pair12& f) {
    float m0 = 0.f, m1 = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      m0 = fmaxf(m0, fmaxf(fabsf(f.re[k].x), fabsf(f.im[k].x)));
      m1 = fmaxf(m1, fmaxf(fabsf(f.re[k].y), fabsf(f.im[k].y)));
    }
    const float2 inv = make_float2(m0 > 0.f ? 1.0f / m0 : 0.f, m1 > 0.f ? 1.0f / m1 : 0.f);
    uint4* p = static_cast<uint4*>(base) + q;
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int g = 0; g < 6; g++) {
      uint4 v;
      __half2* h = reinterpret_cast<__half2*>(&v);
      h[0] = __float22half2_rn(__fmul2_rn(f.re[2 * g], inv));
      h[1] = __float22half2_rn(__fmul2_rn(f.im[2 * g], inv));
      h[2] = __float22half2_rn(__fmul2_rn(f.re[2 * g + 1], inv));
      h[3] = __float22half2_rn(__fmul2_rn(f.im[2 * g + 1], inv));
      p[size_t(g) * np] = v;
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const float2 d = __half22float2(h[e]);
        s = __ffma2_rn(d, d, s);
      }
    }
    norms[q] = make_float2(m0, m1);
    return make_float2(s.x * m0 * m0, s.y * m1 * m1);
  }
};

// arithmetic type for a storage type
template <class T> struct Arith { using type = T; };
template <> struct Arith<__half> { using type = float; };
template <> struct Arith<DF64> { using type = dfloat; };

// ---------------------------------------------------------------------------------------
// TMA bulk copy global -> shared with an mbarrier and a bounded wait.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// bytes must be a multiple of 16; both addresses 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Returns true when phase `parity` of the barrier completed within the poll budget.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls = (1u << 24)) {
  uint32_t ok = 0;
  for (uint32_t it = 0; it < max_polls; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// ---------------------------------------------------------------------------------------
// Block reductions over per-thread FP64 values, one result per right-hand side.
// blockDim = L5 * m with m a power of two; a thread's rhs is (tid % L5) / Ls.
// ---------------------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void block_reduce_rhs(const double (&v)[NV], int L5, int Ls, int nrhs, double* out) {
  extern __shared__ double red_smem[];
  const int t = threadIdx.x, B = blockDim.x;
  if (nrhs == 1) {
    // warp shuffle then one value per warp
    double w[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double x = v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      w[k] = x;
    }
    const int nw = (B + 31) >> 5;
    if ((t & 31) == 0)
      for (int k = 0; k < NV; k++) red_smem[k * 32 + (t >> 5)] = w[k];
    __syncthreads();
    if (t < 32) {
#pragma unroll
      for (int k = 0; k < NV; k++) {
        double x = t < nw ? red_smem[k * 32 + t] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (t == 0) out[size_t(blockIdx.x) * NV + k] = x;
      }
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < NV; k++) red_smem[k * B + t] = v[k];
  __syncthreads();
  for (int stride = (B / L5) >> 1; stride >= 1; stride >>= 1) {
    if (t < L5 * stride)
      for (int k = 0; k < NV; k++) red_smem[k * B + t] += red_smem[k * B + t + L5 * stride];
    __syncthreads();
  }
  if (t < nrhs) {
    for (int k = 0; k < NV; k++) {
      double sum = 0;
      for (int s = 0; s < Ls; s++) sum += red_smem[k * B + t * Ls + s];
      out[(size_t(blockIdx.x) * nrhs + t) * NV + k] = sum;
    }
  }
}

}  // namespace gb
