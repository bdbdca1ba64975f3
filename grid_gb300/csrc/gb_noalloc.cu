// gb_noalloc.cu -- norm2 of a field without any device allocation.
//
// Who needs it: code that owns a field but may not call cudaMalloc/cudaFree when it
// measures it -- a request loop that runs inside a fixed HBM budget handed out by an
// admission controller (every byte of device memory is accounted for before work is
// admitted, so a solver step must not grow the footprint), or a host thread that drives
// the GPU from a context where allocator calls are forbidden or too slow (allocation
// synchronises the device and can stall other streams).  gb_field_norm2 reduces through
// a scratch buffer that belongs to the operator; this variant reduces through one fixed
// array in the library's static device memory instead, so nothing is allocated per call
// or per operator.
//
// The scratch array lives in every GPU that loads this library until the process exits
// (kScratchDoubles doubles = 64.1 KB).  Every call shares it: calls whose kernels overlap
// on the GPU (different streams, or different host threads) race on it and must be
// serialised by the caller.  Each call overwrites every partial sum it later reads, so
// nothing has to be cleared between calls.
#include <cuda_fp16.h>

#include <mutex>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {
namespace {

constexpr int kNaMaxRhs = 16;     // right-hand sides per field
constexpr int kNaMaxBlocks = 256; // CTAs per checkerboard half
constexpr int kScratchDoubles = 2 * kNaMaxBlocks * kNaMaxRhs + kNaMaxRhs;

// partial sums [half][block][rhs], then the per-rhs results
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// host-side device addresses of g_noalloc_scratch, one per device, found once
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_device(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) {
    set_error("norm2 (no allocation): device %d out of range", device);
    return GB_ERR_BAD_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[device]) {
    int cur = 0;
    GB_CHECK_CUDA(cudaGetDevice(&cur));
    if (cur != device) GB_CHECK_CUDA(cudaSetDevice(device));
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != device) cudaSetDevice(cur);
    if (e != cudaSuccess || !p) {
      set_error("norm2 (no allocation): cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return GB_ERR_CUDA;
    }
    g_scratch_ptr[device] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[device];
  return GB_OK;
}

// per-thread FP64 sums of |x|^2 over a grid-stride loop whose stride is a multiple of
// L5, so every thread stays on one right-hand side
template <class T>
__global__ void __launch_bounds__(256) norm2_static_kernel(const void* x, const float* xn, size_t n5, int L5, int Ls,
                                                           int nrhs, double* partial) {
  using R = typename Arith<T>::type;
  double v[1] = {0.0};
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n5; i += stride) {
    Spinor<R> f;
    SpinorIO<T>::load(x, xn, n5, i, f);
    R s = 0;
#pragma unroll
    for (int k = 0; k < 12; k++) s = fma(f.re[k], f.re[k], fma(f.im[k], f.im[k], s));
    v[0] += double(s);
  }
  block_reduce_rhs<1>(v, L5, Ls, nrhs, partial);
}

// out[rhs] = sum over parts of partial[part][rhs], fixed order
__global__ void norm2_static_final(const double* partial, int nparts, int nrhs, double* out) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double s = 0;
  for (int b = 0; b < nparts; b++) s += partial[size_t(b) * nrhs + r];
  out[r] = s;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_field_norm2_noalloc(gb_field_t f, double* out) {
  if (!f || !out) { set_error("norm2 (no allocation): null argument"); return GB_ERR_BAD_ARG; }
  Op* op = f->op;
  if (op->nrhs > kNaMaxRhs) {
    set_error("norm2 (no allocation): %d right-hand sides exceed the static scratch limit of %d", op->nrhs_user, kNaMaxRhs);
    return GB_ERR_UNSUPPORTED;
  }
  double* scratch = nullptr;
  GB_TRY(scratch_for_device(op->device, &scratch));
  // CTA shape as the operator's reductions use, grid capped to the static partial space
  int m = 1;
  while (op->L5 * m * 2 <= 256) m *= 2;
  const int B = op->nrhs == 1 ? 256 : op->L5 * m;
  if (B > 256) {  // the kernel's launch bound: blockDim is a multiple of L5
    set_error("norm2 (no allocation): L5 = %d above 256 is not supported", op->L5);
    return GB_ERR_UNSUPPORTED;
  }
  size_t need = (f->n5 + B - 1) / B;
  const int g = int(need < size_t(kNaMaxBlocks) ? (need < 1 ? 1 : need) : size_t(kNaMaxBlocks));
  const size_t smem = size_t(op->nrhs == 1 ? 32 : B) * sizeof(double);
  const int halves = f->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) {
    HalfView v = half_view(f, h);
    double* part = scratch + size_t(h) * g * op->nrhs;
    switch (v.prec) {
      case GB_F64: norm2_static_kernel<double><<<g, B, smem, op->stream>>>(v.data, v.norms, f->n5, op->L5, op->Ls, op->nrhs, part); break;
      case GB_F32: norm2_static_kernel<float><<<g, B, smem, op->stream>>>(v.data, v.norms, f->n5, op->L5, op->Ls, op->nrhs, part); break;
      case GB_F16: norm2_static_kernel<__half><<<g, B, smem, op->stream>>>(v.data, v.norms, f->n5, op->L5, op->Ls, op->nrhs, part); break;
      default: set_error("norm2 (no allocation): bad precision"); return GB_ERR_BAD_ARG;
    }
    GB_CHECK_CUDA(cudaGetLastError());
  }
  double* result = scratch + size_t(2) * kNaMaxBlocks * kNaMaxRhs;
  norm2_static_final<<<1, 32 * ((op->nrhs + 31) / 32), 0, op->stream>>>(scratch, g * halves, op->nrhs, result);
  GB_CHECK_CUDA(cudaGetLastError());
  GB_CHECK_CUDA(cudaMemcpyAsync(out, result, size_t(op->nrhs_user) * sizeof(double), cudaMemcpyDefault, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}
