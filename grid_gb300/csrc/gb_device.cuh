// gb_device.cuh -- device helpers: spinor plane I/O, TMA bulk copies with bounded
// mbarrier waits, reductions.
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "gb_internal.h"

namespace gb {

// ---------------------------------------------------------------------------------------
// Spinor register form: 12 complex components, index spin*3 + colour.
// ---------------------------------------------------------------------------------------
template <class R> struct Spinor {
  R re[12], im[12];
};

// Loads one 5D site's spinor from the plane layout.  T selects the storage:
//   double -> 12 double2 planes; float -> 6 float4 planes;
//   __half -> 3 planes of 8 halves scaled by the per-site norm.
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

template <> struct SpinorIO<float> {
  static __device__ __forceinline__ void load(const void* base, const float*, size_t n5, size_t i, Spinor<float>& f) {
    const float4* p = static_cast<const float4*>(base);
#pragma unroll
    for (int g = 0; g < 6; g++) {
      float4 v = __ldg(p + size_t(g) * n5 + i);
      f.re[2 * g] = v.x; f.im[2 * g] = v.y; f.re[2 * g + 1] = v.z; f.im[2 * g + 1] = v.w;
    }
  }
  static __device__ __forceinline__ void load_half(const void* base, const float*, size_t n5, size_t i, bool upper,
                                                   Spinor<float>& f) {
    const float4* p = static_cast<const float4*>(base);
    const int g0 = upper ? 0 : 3;
#pragma unroll
    for (int g = 0; g < 3; g++) {
      float4 v = __ldg(p + size_t(g0 + g) * n5 + i);
      const int k = 2 * (g0 + g);
      f.re[k] = v.x; f.im[k] = v.y; f.re[k + 1] = v.z; f.im[k + 1] = v.w;
    }
  }
  static __device__ __forceinline__ void store(void* base, float*, size_t n5, size_t i, const Spinor<float>& f) {
    float4* p = static_cast<float4*>(base);
#pragma unroll
    for (int g = 0; g < 6; g++)
      p[size_t(g) * n5 + i] = make_float4(f.re[2 * g], f.im[2 * g], f.re[2 * g + 1], f.im[2 * g + 1]);
  }
};

// FP16 storage, FP32 arithmetic: plane q (0..2) holds complex components 4q..4q+3 as
// 8 halves; every component is stored divided by the site's max |re|,|im| (the norm).
struct Half8 { __half2 h[4]; };

template <> struct SpinorIO<__half> {
  static __device__ __forceinline__ void load(const void* base, const float* norms, size_t n5, size_t i,
                                              Spinor<float>& f) {
    const uint4* p = static_cast<const uint4*>(base);
    const float nrm = __ldg(norms + i);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      uint4 v = __ldg(p + size_t(q) * n5 + i);
      const __half2* h = reinterpret_cast<const __half2*>(&v);
#pragma unroll
      for (int c = 0; c < 4; c++) {
        float2 z = __half22float2(h[c]);
        f.re[4 * q + c] = z.x * nrm; f.im[4 * q + c] = z.y * nrm;
      }
    }
  }
  // planes straddle the chiralities: read the site and keep the requested six components
  static __device__ __forceinline__ void load_half(const void* base, const float* norms, size_t n5, size_t i,
                                                   bool upper, Spinor<float>& f) {
    Spinor<float> t;
    load(base, norms, n5, i, t);
    const int k0 = upper ? 0 : 6;
#pragma unroll
    for (int k = 0; k < 6; k++) { f.re[k0 + k] = t.re[k0 + k]; f.im[k0 + k] = t.im[k0 + k]; }
  }
  static __device__ __forceinline__ void store(void* base, float* norms, size_t n5, size_t i, const Spinor<float>& f) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) m = fmaxf(m, fmaxf(fabsf(f.re[k]), fabsf(f.im[k])));
    const float inv = m > 0.f ? 1.0f / m : 0.f;
    uint4* p = static_cast<uint4*>(base);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      uint4 v;
      __half2* h = reinterpret_cast<__half2*>(&v);
#pragma unroll
      for (int c = 0; c < 4; c++) h[c] = __floats2half2_rn(f.re[4 * q + c] * inv, f.im[4 * q + c] * inv);
      p[size_t(q) * n5 + i] = v;
    }
    norms[i] = m;
  }
};

// arithmetic type for a storage type
template <class T> struct Arith { using type = T; };
template <> struct Arith<__half> { using type = float; };

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
