// gb_blas.cu -- field linear algebra, FP64 reductions, layout conversion, gauge import.
//
// Reductions follow Grid's rankInnerProduct / sumD / axpy_norm
// (Grid/lattice/Lattice_reduction.h:202-372): per-site products in the field's
// precision, accumulation over sites in FP64, one result per right-hand side.  The
// partial sums of a fixed grid of CTAs are combined in a fixed order by a second kernel,
// so a reduction is bit-reproducible from run to run.
#include <cuda_fp16.h>

#include "gb_device.cuh"

namespace gb {

// ---------------------------------------------------------------------------------------
// Elementwise: z = a x + b y ; copy with precision change ; zero
// ---------------------------------------------------------------------------------------
template <class TZ, class TX, class TY>
__global__ void __launch_bounds__(256) axpby_kernel(void* z, float* zn, double a, const void* x, const float* xn, double b,
                                                    const void* y, const float* yn, size_t n5, int use_y) {
  using R = typename Arith<TZ>::type;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  Spinor<typename Arith<TX>::type> fx;
  SpinorIO<TX>::load(x, xn, n5, i, fx);
  Spinor<R> o;
  if (use_y) {
    Spinor<typename Arith<TY>::type> fy;
    SpinorIO<TY>::load(y, yn, n5, i, fy);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      o.re[k] = R(a) * R(fx.re[k]) + R(b) * R(fy.re[k]);
      o.im[k] = R(a) * R(fx.im[k]) + R(b) * R(fy.im[k]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 12; k++) { o.re[k] = R(a) * R(fx.re[k]); o.im[k] = R(a) * R(fx.im[k]); }
  }
  SpinorIO<TZ>::store(z, zn, n5, i, o);
}

template <class TZ, class TX>
__global__ void __launch_bounds__(256) convert_kernel(void* z, float* zn, const void* x, const float* xn, size_t n5) {
  using R = typename Arith<TZ>::type;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  Spinor<typename Arith<TX>::type> fx;
  SpinorIO<TX>::load(x, xn, n5, i, fx);
  Spinor<R> o;
#pragma unroll
  for (int k = 0; k < 12; k++) { o.re[k] = R(fx.re[k]); o.im[k] = R(fx.im[k]); }
  SpinorIO<TZ>::store(z, zn, n5, i, o);
}

static inline unsigned nblk(size_t n) { return unsigned((n + 255) / 256); }

template <class TZ, class TX, class TY>
static int axpby_t(Op* op, HalfView z, double a, HalfView x, double b, HalfView y, size_t n5, int use_y) {
  axpby_kernel<TZ, TX, TY><<<nblk(n5), 256, 0, op->stream>>>(z.data, z.norms, a, x.data, x.norms, b, y.data, y.norms,
                                                            n5, use_y);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_axpby(Op* op, HalfView z, double a, HalfView x, double b, HalfView y, size_t n5) {
  if (x.prec != z.prec || y.prec != z.prec) {
    set_error("axpby: mixed precisions");
    return GB_ERR_BAD_ARG;
  }
  if (z.prec != GB_F64) return launch_axpby_pair(op, z, a, x, b, y, n5, 1);
  return axpby_t<double, double, double>(op, z, a, x, b, y, n5, 1);
}

int launch_scale(Op* op, HalfView z, double a, HalfView x, size_t n5) {
  if (x.prec != z.prec) {
    set_error("scale: mixed precisions");
    return GB_ERR_BAD_ARG;
  }
  if (z.prec != GB_F64) return launch_axpby_pair(op, z, a, x, 0.0, x, n5, 0);
  return axpby_t<double, double, double>(op, z, a, x, 0, x, n5, 0);
}

template <class TZ, class TX> static int convert_t(Op* op, HalfView z, HalfView x, size_t n5) {
  convert_kernel<TZ, TX><<<nblk(n5), 256, 0, op->stream>>>(z.data, z.norms, x.data, x.norms, n5);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_copy(Op* op, HalfView dst, HalfView src, size_t n5) {
  if (dst.prec == src.prec) {
    GB_CHECK_CUDA(cudaMemcpyAsync(dst.data, src.data, n5 * spinor_bytes(dst.prec), cudaMemcpyDeviceToDevice, op->stream));
    if (dst.prec == GB_F16)
      GB_CHECK_CUDA(cudaMemcpyAsync(dst.norms, src.norms, n5 * sizeof(float), cudaMemcpyDeviceToDevice, op->stream));
    return GB_OK;
  }
#define GB_CONV(PD, TD, PS, TS) \
  if (dst.prec == PD && src.prec == PS) return convert_t<TD, TS>(op, dst, src, n5);
  GB_CONV(GB_F64, double, GB_F32, float)
  GB_CONV(GB_F64, double, GB_F16, __half)
  GB_CONV(GB_F32, float, GB_F64, double)
  GB_CONV(GB_F32, float, GB_F16, __half)
  GB_CONV(GB_F16, __half, GB_F64, double)
  GB_CONV(GB_F16, __half, GB_F32, float)
#undef GB_CONV
  return GB_ERR_BAD_ARG;
}

int launch_zero(Op* op, HalfView z, size_t n5) {
  GB_CHECK_CUDA(cudaMemsetAsync(z.data, 0, n5 * spinor_bytes(z.prec), op->stream));
  if (z.prec == GB_F16) GB_CHECK_CUDA(cudaMemsetAsync(z.norms, 0, n5 * sizeof(float), op->stream));
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Reductions
// ---------------------------------------------------------------------------------------
struct RedShape {
  int L5, Ls, nrhs;
};

// kind 0: |x|^2 ; kind 1: <x|y> ; kind 2: z = a x + y (a from host), |z|^2 ;
// kind 3: r = r - a[rhs] mmp (a from the device CG scalars), |r|^2
template <class T, int KIND>
__global__ void __launch_bounds__(256) reduce_kernel(const RedShape sh, const void* x, const float* xn, const void* y,
                                                     const float* yn, void* z, float* zn, double a,
                                                     const CGScalars* cg, size_t n5, double* partial) {
  using R = typename Arith<T>::type;
  constexpr int NV = KIND == 1 ? 2 : 1;
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = 0.0;
  const size_t stride = size_t(gridDim.x) * blockDim.x;  // a multiple of L5
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  R ar = R(a);
  if (KIND == 3) {
    const int rhs = int(i % sh.L5) / sh.Ls;
    ar = -R(cg[rhs].a);
  }
  for (; i < n5; i += stride) {
    Spinor<R> fx;
    SpinorIO<T>::load(x, xn, n5, i, fx);
    if (KIND == 0) {
      R s = 0;
#pragma unroll
      for (int k = 0; k < 12; k++) s = fma(fx.re[k], fx.re[k], fma(fx.im[k], fx.im[k], s));
      v[0] += double(s);
    } else if (KIND == 1) {
      Spinor<R> fy;
      SpinorIO<T>::load(y, yn, n5, i, fy);
      R sr = 0, si = 0;
#pragma unroll
      for (int k = 0; k < 12; k++) {
        sr = fma(fx.re[k], fy.re[k], fma(fx.im[k], fy.im[k], sr));
        si = fma(fx.re[k], fy.im[k], fma(-fx.im[k], fy.re[k], si));
      }
      v[0] += double(sr);
      v[1] += double(si);
    } else {
      // KIND 2: z = a*x + y ; KIND 3: z(=y) = y - a*x
      Spinor<R> fy;
      SpinorIO<T>::load(y, yn, n5, i, fy);
      R s = 0;
#pragma unroll
      for (int k = 0; k < 12; k++) {
        fy.re[k] = fma(ar, fx.re[k], fy.re[k]);
        fy.im[k] = fma(ar, fx.im[k], fy.im[k]);
        s = fma(fy.re[k], fy.re[k], fma(fy.im[k], fy.im[k], s));
      }
      SpinorIO<T>::store(z, zn, n5, i, fy);
      v[0] += double(s);
    }
  }
  block_reduce_rhs<NV>(v, sh.L5, sh.Ls, sh.nrhs, partial);
}

int red_grid(Op* op, size_t n5, int* blocks, int* threads) {
  int L5 = op->L5;
  int m = 1;
  while (L5 * m * 2 <= 256) m *= 2;
  int B = op->nrhs == 1 ? 256 : L5 * m;
  if (B > 256) {  // the kernel's launch bound: blockDim is a multiple of L5
    set_error("reduction: FP64 fields with L5 = %d above 256 are not supported", L5);
    return GB_ERR_UNSUPPORTED;
  }
  size_t need = (n5 + B - 1) / B;
  int g = int(need < size_t(kRedBlocks) ? need : size_t(kRedBlocks));
  if (g < 1) g = 1;
  *blocks = g;
  *threads = B;
  return GB_OK;
}

template <class T, int KIND>
static int reduce_t(Op* op, HalfView x, HalfView y, HalfView z, double a, size_t n5, double* partial) {
  int g, B;
  GB_TRY(red_grid(op, n5, &g, &B));
  RedShape sh{op->L5, op->Ls, op->nrhs};
  const int NV = KIND == 1 ? 2 : 1;
  size_t smem = size_t(NV) * (op->nrhs == 1 ? 32 : B) * sizeof(double);
  reduce_kernel<T, KIND><<<g, B, smem, op->stream>>>(sh, x.data, x.norms, y.data, y.norms, z.data, z.norms, a, op->d_cg,
                                                     n5, partial);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// FP32 / FP16 fields reduce through the pair kernels (gb_pair.cu), whose partial count
// red_parts() reports; FP64 through reduce_kernel
int launch_norm2_partial(Op* op, HalfView x, size_t n5, double* partial) {
  if (x.prec != GB_F64) return launch_reduce_pair(op, 0, x, x, x, 0.0, n5, partial);
  return reduce_t<double, 0>(op, x, x, x, 0.0, n5, partial);
}
int launch_inner_partial(Op* op, HalfView a, HalfView b, size_t n5, double* partial) {
  if (a.prec != b.prec) { set_error("innerProduct: mixed precisions"); return GB_ERR_BAD_ARG; }
  if (a.prec != GB_F64) return launch_reduce_pair(op, 1, a, b, a, 0.0, n5, partial);
  return reduce_t<double, 1>(op, a, b, a, 0.0, n5, partial);
}
// z = a x + y, |z|^2
int launch_axpy_norm_partial(Op* op, HalfView z, double a, HalfView x, HalfView y, size_t n5, double* partial) {
  if (x.prec != y.prec || z.prec != x.prec) { set_error("axpy_norm: mixed precisions"); return GB_ERR_BAD_ARG; }
  if (x.prec != GB_F64) return launch_reduce_pair(op, 2, x, y, z, a, n5, partial);
  return reduce_t<double, 2>(op, x, y, z, a, n5, partial);
}
// r -= a[rhs] mmp, |r|^2: Grid's axpy_norm(r, -a, mmp, r) with the device CG scalars
int launch_cg_r_update(Op* op, HalfView r, HalfView mmp, size_t n5, double* partial) {
  if (r.prec != mmp.prec) { set_error("CG update: mixed precisions"); return GB_ERR_BAD_ARG; }
  if (r.prec != GB_F64) return launch_reduce_pair(op, 3, mmp, r, r, 0.0, n5, partial);
  return reduce_t<double, 3>(op, mmp, r, r, 0.0, n5, partial);
}

// partial: [nparts][nrhs][nv] -> out[nrhs][nv]; one CTA per rhs, fixed summation order
__global__ void reduce_final_kernel(const double* partial, int nparts, int nrhs, int nv, double* out) {
  __shared__ double sm[256][2];
  const int rhs = blockIdx.x, t = threadIdx.x;
  double s0 = 0, s1 = 0;
  for (int b = t; b < nparts; b += blockDim.x) {
    s0 += partial[(size_t(b) * nrhs + rhs) * nv];
    if (nv > 1) s1 += partial[(size_t(b) * nrhs + rhs) * nv + 1];
  }
  sm[t][0] = s0;
  sm[t][1] = s1;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (t < st) { sm[t][0] += sm[t + st][0]; sm[t][1] += sm[t + st][1]; }
    __syncthreads();
  }
  if (t == 0) {
    out[rhs * nv] = sm[0][0];
    if (nv > 1) out[rhs * nv + 1] = sm[0][1];
  }
}

int launch_reduce_final(Op* op, const double* partial, int nparts, int nv, double* out) {
  reduce_final_kernel<<<op->nrhs, 256, 0, op->stream>>>(partial, nparts, op->nrhs, nv, out);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// CG scalars (ConjugateGradient.h:151-200, ConjugateGradientReliableUpdate.h:163-251),
// one set per right-hand side.  A right-hand side that has converged keeps a = b = 0,
// so its solution stays fixed while the others iterate.
// ---------------------------------------------------------------------------------------
__global__ void cg_init_kernel(CGScalars* cg, const double* ssq, const double* cp, int nrhs, double tol, double delta,
                               int* flags) {
  const int r = threadIdx.x;
  __shared__ int nd;
  if (r == 0) nd = 0;
  __syncthreads();
  if (r < nrhs) {
    CGScalars s;
    s.ssq = ssq[r];
    s.rsq = tol * tol * ssq[r];
    s.cp = cp[r];
    s.c = cp[r];
    s.cprev = cp[r];
    s.maxres = cp[r];
    s.delta = delta;
    s.a = 0; s.b = 0; s.d = 0;
    s.done = (cp[r] <= s.rsq) ? 1 : 0;
    s.iter = 0;
    s.relup = 0;
    s.pad = 0;
    cg[r] = s;
    if (s.done) atomicAdd(&nd, 1);
  }
  __syncthreads();
  if (r == 0) { flags[0] = (nd == nrhs); flags[1] = 0; }
}

// sum over b of partial[b * stride + offset] by one CTA (a power of two, at most 1024
// threads) in a fixed order (strided per-thread sums, then a tree); every thread gets the
// result
__device__ double cta_sum_fixed(const double* partial, int nparts, int stride, int offset) {
  __shared__ double sm[1024];
  double s = 0;
  // unrolled so that several loads are in flight before the (ordered) adds
#pragma unroll 8
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += partial[size_t(b) * stride + offset];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sm[threadIdx.x] += sm[threadIdx.x + st];
    __syncthreads();
  }
  const double r = sm[0];
  __syncthreads();
  return r;
}

// launched with 256 threads, 1024 above 2048 partial sums (one per CTA of an FP32 Dhop):
// the partial sums of every right-hand side are reduced by the whole CTA (a single thread
// walking thousands of partials would take ~100 us)
__global__ void __launch_bounds__(1024) cg_alpha_kernel(CGScalars* cg, const double* partial, int nparts, int nrhs,
                                                       int nv) {
  for (int r = 0; r < nrhs; r++) {
    const double d = cta_sum_fixed(partial, nparts, nrhs * nv, r * nv);
    if (threadIdx.x == 0) {
      cg[r].d = d;
      cg[r].a = cg[r].done ? 0.0 : cg[r].c / d;
    }
  }
}

__global__ void __launch_bounds__(1024) cg_beta_kernel(CGScalars* cg, const double* partial, int nparts, int nrhs,
                                                      int* flags) {
  int nd = 0, nr = 0;
  for (int r = 0; r < nrhs; r++) {
    const double cp = cta_sum_fixed(partial, nparts, nrhs, r);
    if (threadIdx.x == 0) {
      CGScalars s = cg[r];
      if (!s.done) {
        s.cp = cp;
        s.b = cp / s.c;
        s.cprev = s.c;
        s.c = cp;
        s.iter += 1;
        if (cp > s.maxres) s.maxres = cp;
        if (cp <= s.rsq) s.done = 1;
        else if (cp < s.delta * s.maxres) s.relup = 1;
      } else {
        s.b = 0.0;
      }
      cg[r] = s;
      nd += s.done;
      nr += (s.relup && !s.done);
    }
  }
  if (threadIdx.x == 0) { flags[0] = (nd == nrhs); flags[1] = nr; }
}

__global__ void cg_relup_reset_kernel(CGScalars* cg, const double* cp_true, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  CGScalars s = cg[r];
  if (!s.done) {
    s.cp = cp_true[r];
    s.b = cp_true[r] / s.cprev;
    s.c = cp_true[r];
    s.maxres = cp_true[r];
  }
  s.relup = 0;
  cg[r] = s;
}

static inline int rhs_threads(const Op* op) { return 32 * ((op->nrhs + 31) / 32); }

int launch_cg_init(Op* op, const double* d_ssq, const double* d_cp, double tol, double delta) {
  cg_init_kernel<<<1, rhs_threads(op), 0, op->stream>>>(op->d_cg, d_ssq, d_cp, op->nrhs, tol, delta, op->d_all_done);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}
// the scalar kernels reduce the per-block partial sums themselves, in a fixed order
static inline int sum_threads(int nparts) { return nparts > 2048 ? 1024 : 256; }
int launch_cg_alpha(Op* op, const double* partial, int nparts, int nv) {
  cg_alpha_kernel<<<1, sum_threads(nparts), 0, op->stream>>>(op->d_cg, partial, nparts, op->nrhs, nv);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}
// The device-resident CG loop (a CUDA graph whose conditional WHILE node repeats a
// captured chunk of iterations).  flags = op->d_all_done: [0] every right-hand side has
// converged, [1] right-hand sides that want a reliable update (both written by
// cg_beta_kernel each iteration), [2] chunks run in this launch, [3] the most chunks one
// launch may run.  arm sets [2], [3] before a launch; check decides after every chunk.
__global__ void cg_loop_arm_kernel(int* flags, int max_chunks) {
  flags[2] = 0;
  flags[3] = max_chunks;
}
__global__ void cg_loop_check_kernel(cudaGraphConditionalHandle h, int* flags) {
  const int n = ++flags[2];
  cudaGraphSetConditional(h, (!flags[0] && !flags[1] && n < flags[3]) ? 1u : 0u);
}
int launch_cg_loop_arm(Op* op, int max_chunks) {
  cg_loop_arm_kernel<<<1, 1, 0, op->stream>>>(op->d_all_done, max_chunks);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}
int launch_cg_loop_check(Op* op, cudaGraphConditionalHandle h) {
  cg_loop_check_kernel<<<1, 1, 0, op->stream>>>(h, op->d_all_done);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_cg_beta(Op* op, const double* partial_norm, int nparts) {
  cg_beta_kernel<<<1, sum_threads(nparts), 0, op->stream>>>(op->d_cg, partial_norm, nparts, op->nrhs, op->d_all_done);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}
int launch_cg_relup_reset(Op* op, const double* d_cp_true) {
  cg_relup_reset_kernel<<<1, rhs_threads(op), 0, op->stream>>>(op->d_cg, d_cp_true, op->nrhs);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// p = b p + r   (the second line of ConjugateGradient.h:175-183)
template <class T>
__global__ void __launch_bounds__(256) cg_p_kernel(const RedShape sh, void* p, float* pn, const void* r, const float* rn,
                                                   const CGScalars* cg, size_t n5) {
  using R = typename Arith<T>::type;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  const int rhs = int(i % sh.L5) / sh.Ls;
  const R b = R(cg[rhs].b);
  Spinor<R> fp, fr;
  SpinorIO<T>::load(p, pn, n5, i, fp);
  SpinorIO<T>::load(r, rn, n5, i, fr);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    fp.re[k] = fma(b, fp.re[k], fr.re[k]);
    fp.im[k] = fma(b, fp.im[k], fr.im[k]);
  }
  SpinorIO<T>::store(p, pn, n5, i, fp);
}

int launch_cg_p_update(Op* op, HalfView p, HalfView r, size_t n5) {
  if (p.prec != GB_F64) return launch_cg_p_pair(op, p, r, n5);
  RedShape sh{op->L5, op->Ls, op->nrhs};
  cg_p_kernel<double><<<nblk(n5), 256, 0, op->stream>>>(sh, p.data, p.norms, r.data, r.norms, op->d_cg, n5);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// psi += a p, then (PUPD) p = b p + r: the CG's linear combination after the residual
// update (ConjugateGradient.h:174-183), FP64 fields
template <bool PUPD>
__global__ void __launch_bounds__(256) cg_xp_kernel(const RedShape sh, double2* psi, double2* p, const double2* r,
                                                    const CGScalars* cg, size_t n5) {
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  const CGScalars& c = cg[int(i % sh.L5) / sh.Ls];
  const double a = c.a, b = c.b;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const double2 pk = p[size_t(k) * n5 + i];
    double2 x = psi[size_t(k) * n5 + i];
    x.x = fma(a, pk.x, x.x);
    x.y = fma(a, pk.y, x.y);
    psi[size_t(k) * n5 + i] = x;
    if (PUPD) {
      const double2 rk = r[size_t(k) * n5 + i];
      p[size_t(k) * n5 + i] = make_double2(fma(b, pk.x, rk.x), fma(b, pk.y, rk.y));
    }
  }
}

int launch_cg_xp_update(Op* op, HalfView psi, HalfView p, HalfView r, size_t n5, int update_p) {
  if (p.prec != r.prec) { set_error("CG update: mixed precisions"); return GB_ERR_BAD_ARG; }
  if (p.prec != GB_F64) return launch_cg_xp_pair(op, psi, p, r, n5, update_p);
  if (psi.prec != GB_F64) { set_error("CG update: FP64 fields expected"); return GB_ERR_BAD_ARG; }
  RedShape sh{op->L5, op->Ls, op->nrhs};
  auto* x = static_cast<double2*>(psi.data);
  auto* pp = static_cast<double2*>(p.data);
  auto* rr = static_cast<const double2*>(r.data);
  if (update_p) cg_xp_kernel<true><<<nblk(n5), 256, 0, op->stream>>>(sh, x, pp, rr, op->d_cg, n5);
  else cg_xp_kernel<false><<<nblk(n5), 256, 0, op->stream>>>(sh, x, pp, rr, op->d_cg, n5);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Layout conversion between canonical FP64 and the device planes
// ---------------------------------------------------------------------------------------
struct GeoParams {
  int L[4];
  int64_t half4, vol4;
  int L5, Ls, nrhs, nrhs_user;
};

__device__ __forceinline__ int64_t cb_to_site(int64_t xcb, int parity, const GeoParams& g) {
  const int Lxh = g.L[0] >> 1;
  const int64_t row = xcb / Lxh;
  const int xh = int(xcb - row * Lxh);
  const int y = int(row % g.L[1]);
  const int64_t zt = row / g.L[1];
  const int z = int(zt % g.L[2]);
  const int t = int(zt / g.L[2]);
  const int x = 2 * xh + ((parity + y + z + t) & 1);
  return row * g.L[0] + x;
}

// canonical host layout <-> device layout; CR is the canonical real type (double or float:
// Grid's LatticeFermionD / LatticeFermionF host data)
template <class CR> struct Canon2;
template <> struct Canon2<double> { using type = double2; };
template <> struct Canon2<float> { using type = float2; };

template <class T, class CR, bool IMPORT>
__global__ void __launch_bounds__(256) layout_kernel(const GeoParams g, CR* canon, void* dev, float* devn, int parity,
                                                     int canon_full) {
  using R = typename Arith<T>::type;
  using C2 = typename Canon2<CR>::type;
  const size_t n5 = size_t(g.half4) * g.L5;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  const int64_t xcb = int64_t(i / g.L5);
  const int s5 = int(i - size_t(xcb) * g.L5);
  const int rhs = s5 / g.Ls, s = s5 - rhs * g.Ls;
  Spinor<R> f;
  if (rhs >= g.nrhs_user) {  // the padding right-hand side: zeros, absent from the host array
    if (IMPORT) {
#pragma unroll
      for (int k = 0; k < 12; k++) { f.re[k] = R(0); f.im[k] = R(0); }
      SpinorIO<T>::store(dev, devn, n5, i, f);
    }
    return;
  }
  const int64_t c4 = canon_full ? cb_to_site(xcb, parity, g) : xcb;
  const int64_t n4c = canon_full ? g.vol4 : g.half4;
  C2* c = reinterpret_cast<C2*>(canon) + ((size_t(rhs) * n4c + c4) * g.Ls + s) * 12;
  if (IMPORT) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const C2 v = c[k];
      f.re[k] = R(v.x); f.im[k] = R(v.y);
    }
    SpinorIO<T>::store(dev, devn, n5, i, f);
  } else {
    SpinorIO<T>::load(dev, devn, n5, i, f);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      C2 v;
      v.x = CR(f.re[k]);
      v.y = CR(f.im[k]);
      c[k] = v;
    }
  }
}

static GeoParams geo(const Op* op) {
  GeoParams g;
  for (int k = 0; k < 4; k++) g.L[k] = op->dims[k];
  g.half4 = op->half4;
  g.vol4 = op->vol4;
  g.L5 = op->L5;
  g.Ls = op->Ls;
  g.nrhs = op->nrhs;
  g.nrhs_user = op->nrhs_user;
  return g;
}

template <class CR, bool IMPORT>
static int layout_p(Op* op, CR* canon, HalfView v, int parity, int canon_full) {
  GeoParams g = geo(op);
  const size_t n5 = op->n5();
  switch (v.prec) {
    case GB_F64: layout_kernel<double, CR, IMPORT><<<nblk(n5), 256, 0, op->stream>>>(g, canon, v.data, v.norms, parity, canon_full); break;
    case GB_F32: layout_kernel<float, CR, IMPORT><<<nblk(n5), 256, 0, op->stream>>>(g, canon, v.data, v.norms, parity, canon_full); break;
    case GB_F16: layout_kernel<__half, CR, IMPORT><<<nblk(n5), 256, 0, op->stream>>>(g, canon, v.data, v.norms, parity, canon_full); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_import_half(Op* op, const void* canon, int canon_prec, HalfView out, int parity, int canon_is_full) {
  if (canon_prec == GB_F32)
    return layout_p<float, true>(op, static_cast<float*>(const_cast<void*>(canon)), out, parity, canon_is_full);
  return layout_p<double, true>(op, static_cast<double*>(const_cast<void*>(canon)), out, parity, canon_is_full);
}
int launch_export_half(Op* op, HalfView in, void* canon, int canon_prec, int parity, int canon_is_full) {
  if (canon_prec == GB_F32) return layout_p<float, false>(op, static_cast<float*>(canon), in, parity, canon_is_full);
  return layout_p<double, false>(op, static_cast<double*>(canon), in, parity, canon_is_full);
}

// ---------------------------------------------------------------------------------------
// 4D <-> 5D surface fields of a Moebius operator (CayleyFermion5DImplementation.h:57-129)
// and 4D slices of a 5D field (InsertSlice / ExtractSlice along the fifth dimension,
// Grid/lattice/Lattice_transfer.h:999-1070).  One thread per (rhs, 4D site) of a canonical
// 4D field c4[rhs][site][12].
//   SURF_INSERT   spins 0,1 (P+) of the 4D spinor at s = 0 and spins 2,3 (P-) at s = Ls-1,
//                 zeros in the other halves of those two sites; every other s untouched
//                 (the caller zeroes the field first)
//   SURF_EXTRACT  the 4D spinor back: with arg != 0 spins 0,1 come from s = Ls-1 and spins
//                 2,3 from s = 0 (ExportPhysicalFermionSolution), otherwise the reverse
//                 (ExportPhysicalFermionSource)
//   SLICE_INSERT / SLICE_EXTRACT  the whole spinor at s = arg
// ---------------------------------------------------------------------------------------
enum { SURF_INSERT = 0, SURF_EXTRACT = 1, SLICE_INSERT = 2, SLICE_EXTRACT = 3 };

template <class T, int MODE>
__global__ void __launch_bounds__(256) surface_kernel(const GeoParams g, double* c4, void* even, float* even_n,
                                                      void* odd, float* odd_n, int arg) {
  using R = typename Arith<T>::type;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(g.vol4) * g.nrhs_user) return;
  const int rhs = int(t / size_t(g.vol4));
  const int64_t site = int64_t(t - size_t(rhs) * g.vol4);
  int sum = 0;
  {
    int64_t r = site;
    for (int k = 0; k < 4; k++) { sum += int(r % g.L[k]); r /= g.L[k]; }
  }
  const int parity = sum & 1;
  void* base = parity ? odd : even;
  float* nrm = parity ? odd_n : even_n;
  const size_t n5 = size_t(g.half4) * g.L5;
  const size_t i0 = size_t(site >> 1) * g.L5 + size_t(rhs) * g.Ls;  // s = 0
  const size_t i1 = i0 + g.Ls - 1;                                   // s = Ls-1
  double2* c = reinterpret_cast<double2*>(c4) + (size_t(rhs) * g.vol4 + site) * 12;
  Spinor<R> a, b;
  if (MODE == SURF_INSERT) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const double2 v = c[k];
      const bool up = k < 6;
      a.re[k] = up ? R(v.x) : R(0); a.im[k] = up ? R(v.y) : R(0);
      b.re[k] = up ? R(0) : R(v.x); b.im[k] = up ? R(0) : R(v.y);
    }
    SpinorIO<T>::store(base, nrm, n5, i0, a);
    SpinorIO<T>::store(base, nrm, n5, i1, b);
  } else if (MODE == SURF_EXTRACT) {
    SpinorIO<T>::load(base, nrm, n5, i0, a);
    SpinorIO<T>::load(base, nrm, n5, i1, b);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const bool from_last = (k < 6) == (arg != 0);
      c[k] = from_last ? make_double2(double(b.re[k]), double(b.im[k])) : make_double2(double(a.re[k]), double(a.im[k]));
    }
  } else if (MODE == SLICE_INSERT) {
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const double2 v = c[k];
      a.re[k] = R(v.x); a.im[k] = R(v.y);
    }
    SpinorIO<T>::store(base, nrm, n5, i0 + arg, a);
  } else {
    SpinorIO<T>::load(base, nrm, n5, i0 + arg, a);
#pragma unroll
    for (int k = 0; k < 12; k++) c[k] = make_double2(double(a.re[k]), double(a.im[k]));
  }
}

template <int MODE>
static int surface_p(Op* op, double* c4, HalfView even, HalfView odd, int arg) {
  const GeoParams g = geo(op);
  const size_t n = size_t(op->vol4) * op->nrhs_user;
  switch (even.prec) {
    case GB_F64: surface_kernel<double, MODE><<<nblk(n), 256, 0, op->stream>>>(g, c4, even.data, even.norms, odd.data, odd.norms, arg); break;
    case GB_F32: surface_kernel<float, MODE><<<nblk(n), 256, 0, op->stream>>>(g, c4, even.data, even.norms, odd.data, odd.norms, arg); break;
    case GB_F16: surface_kernel<__half, MODE><<<nblk(n), 256, 0, op->stream>>>(g, c4, even.data, even.norms, odd.data, odd.norms, arg); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}
int launch_surface_insert(Op* op, const double* c4, HalfView even, HalfView odd) {
  return surface_p<SURF_INSERT>(op, const_cast<double*>(c4), even, odd, 0);
}
int launch_surface_extract(Op* op, HalfView even, HalfView odd, double* c4, int solution) {
  return surface_p<SURF_EXTRACT>(op, c4, even, odd, solution);
}
int launch_slice(Op* op, double* c4, HalfView even, HalfView odd, int s, int insert) {
  if (s < 0 || s >= op->Ls) { set_error("slice %d outside [0, %d)", s, op->Ls); return GB_ERR_BAD_ARG; }
  return insert ? surface_p<SLICE_INSERT>(op, c4, even, odd, s) : surface_p<SLICE_EXTRACT>(op, c4, even, odd, s);
}

// ---------------------------------------------------------------------------------------
// CayleyFermion5D::P / Pdag (CayleyFermion5DImplementation.h:70-88): chi_s = P- psi_s +
// P+ psi_{s+1} (P) or P+ psi_{s-1} (Pdag), s cyclic within each right-hand side's block of
// Ls.  One thread per output 5D site of one checkerboard half; in and out are distinct.
// ---------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) chiral_shift_kernel(const GeoParams g, const void* in, const float* in_n,
                                                           void* out, float* out_n, int dag) {
  using R = typename Arith<T>::type;
  const size_t n5 = size_t(g.half4) * g.L5;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  const int s5 = int(i % g.L5);
  const int s = s5 % g.Ls;
  const int sp = dag ? (s + g.Ls - 1) % g.Ls : (s + 1) % g.Ls;
  const size_t j = i - s + sp;
  Spinor<R> a, b;
  SpinorIO<T>::load(in, in_n, n5, i, a);
  SpinorIO<T>::load(in, in_n, n5, j, b);
#pragma unroll
  for (int k = 0; k < 6; k++) { a.re[k] = b.re[k]; a.im[k] = b.im[k]; }
  SpinorIO<T>::store(out, out_n, n5, i, a);
}

int launch_chiral_shift(Op* op, HalfView in, HalfView out, int dag) {
  if (in.prec != out.prec) { set_error("P: mixed field precisions"); return GB_ERR_BAD_ARG; }
  const GeoParams g = geo(op);
  const size_t n = op->n5();
  switch (in.prec) {
    case GB_F64: chiral_shift_kernel<double><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dag); break;
    case GB_F32: chiral_shift_kernel<float><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dag); break;
    case GB_F16: chiral_shift_kernel<__half><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dag); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// DoubleStore (Grid/qcd/action/fermion/WilsonImpl.h:127-171) with ImportGauge's -1/2
// (WilsonFermion5DImplementation.h:149-180), for the links of output parity p.
// ---------------------------------------------------------------------------------------
struct PhaseParams {
  double re[4], im[4];
};

template <class L>
__global__ void __launch_bounds__(256) double_store_kernel(const GeoParams g, const PhaseParams ph, const double2* U,
                                                           L* out, int parity, int recon12) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(g.half4) * 8) return;
  const int64_t xcb = int64_t(t >> 3);
  const int leg = int(t & 7);
  const int mu = leg & 3;
  const int64_t site = cb_to_site(xcb, parity, g);
  int x[4];
  {
    int64_t r = site;
    for (int k = 0; k < 4; k++) { x[k] = int(r % g.L[k]); r /= g.L[k]; }
  }
  double pr = 1, pi = 0;
  int64_t src = site;
  if (leg < 4) {
    if (x[mu] == g.L[mu] - 1) { pr = ph.re[mu]; pi = ph.im[mu]; }
  } else {
    if (x[mu] == 0) { pr = ph.re[mu]; pi = -ph.im[mu]; }
    int xs[4] = {x[0], x[1], x[2], x[3]};
    xs[mu] = (xs[mu] - 1 + g.L[mu]) % g.L[mu];
    src = xs[0] + int64_t(g.L[0]) * (xs[1] + int64_t(g.L[1]) * (xs[2] + int64_t(g.L[2]) * xs[3]));
  }
  const double2* u = U + (size_t(src) * 4 + mu) * 9;
  const int rows = recon12 ? 2 : 3;  // 12-real links keep rows 0 and 1
  L* o = out + (size_t(xcb) * 8 + leg) * (rows * 6);
  for (int a = 0; a < rows; a++)
    for (int b = 0; b < 3; b++) {
      // forward: U[a][b]; backward: conj(U[b][a])
      const double2 v = leg < 4 ? u[a * 3 + b] : make_double2(u[b * 3 + a].x, -u[b * 3 + a].y);
      const double re = -0.5 * (pr * v.x - pi * v.y);
      const double im = -0.5 * (pr * v.y + pi * v.x);
      o[(a * 3 + b) * 2] = L(re);
      o[(a * 3 + b) * 2 + 1] = L(im);
    }
}

int launch_double_store(Op* op, const double* U_canon, int parity) {
  GeoParams g = geo(op);
  PhaseParams ph;
  for (int k = 0; k < 4; k++) { ph.re[k] = op->phases[k].real(); ph.im[k] = op->phases[k].imag(); }
  const size_t n = size_t(op->half4) * 8;
  const double2* U = reinterpret_cast<const double2*>(U_canon);
  if (op->prec == GB_F64)
    double_store_kernel<double><<<nblk(n), 256, 0, op->stream>>>(g, ph, U, static_cast<double*>(op->links[parity]), parity,
                                                                 op->recon12 ? 1 : 0);
  else
    double_store_kernel<float><<<nblk(n), 256, 0, op->stream>>>(g, ph, U, static_cast<float*>(op->links[parity]), parity,
                                                                op->recon12 ? 1 : 0);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb

// ---------------------------------------------------------------------------------------
// The bounded-wait contract of every device wait, exercised on its own: one thread polls
// a device flag with a poll budget and, when the budget runs out, records the failure in
// a status word the host reads and returns -- no trap, the context stays usable.
// ---------------------------------------------------------------------------------------
namespace gb {
namespace {
__global__ void bounded_flag_wait_kernel(const volatile int* flag, int expect, long long max_polls, int* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long long i = 0;
  while (*flag != expect && i < max_polls) {
    __nanosleep(1000);
    i++;
  }
  *status = (*flag == expect) ? 0 : 1;
}
}  // namespace
}  // namespace gb

extern "C" int gb_bounded_wait_test(gb_op_t op, int set_flag, long long max_polls) {
  using namespace gb;
  if (!op || max_polls < 1 || max_polls > (1ll << 22)) { set_error("bounded wait test: 1 <= max_polls <= 2^22"); return GB_ERR_BAD_ARG; }
  int* d = nullptr;  // d[0]: the flag, d[1]: the status
  GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), 2 * sizeof(int), op->stream));
  struct Free { int* p; cudaStream_t s; ~Free() { cudaFreeAsync(p, s); } } guard{d, op->stream};
  const int init[2] = {set_flag ? 1 : 0, -1};
  GB_CHECK_CUDA(cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, op->stream));
  bounded_flag_wait_kernel<<<1, 32, 0, op->stream>>>(d, 1, max_polls, d + 1);
  GB_CHECK_CUDA(cudaGetLastError());
  int status = -1;
  GB_CHECK_CUDA(cudaMemcpyAsync(&status, d + 1, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  if (status != 0) {
    set_error("device wait gave up after %lld polls (flag never set)", max_polls);
    return GB_ERR_TIMEOUT;
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Per-slot chiral complex scaling and the fifth-dimension transforms of the
// Fourier-accelerated Pauli-Villars solve (FourierAcceleratedPV.h:56-237) and of the
// twisted-mass 5D Wilson operator (WilsonTMFermion5D.h:82-135).
// ---------------------------------------------------------------------------------------
namespace gb {
namespace {

// out_i = d(slot, chirality) x_i + zc z_i, d = dr + i di per slot for spins 0,1 (P+) and
// spins 2,3 (P-); slots are the L5 positions s5 of a 5D site index
struct ChiralCoef {
  double up_re[kMaxSlots], up_im[kMaxSlots], dn_re[kMaxSlots], dn_im[kMaxSlots];
};

template <class T>
__global__ void __launch_bounds__(256) chiral_scale_kernel(const GeoParams g, const void* x, const float* xn, const void* z,
                                                           const float* zn, double zc, void* out, float* outn,
                                                           const ChiralCoef c) {
  using R = typename Arith<T>::type;
  const size_t n5 = size_t(g.half4) * g.L5;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n5) return;
  const int s5 = int(i % g.L5);
  Spinor<R> a;
  SpinorIO<T>::load(x, xn, n5, i, a);
  Spinor<R> b;
  if (z) SpinorIO<T>::load(z, zn, n5, i, b);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const R dr = R(k < 6 ? c.up_re[s5] : c.dn_re[s5]);
    const R di = R(k < 6 ? c.up_im[s5] : c.dn_im[s5]);
    R re = dr * a.re[k] - di * a.im[k];
    R im = dr * a.im[k] + di * a.re[k];
    if (z) { re += R(zc) * b.re[k]; im += R(zc) * b.im[k]; }
    a.re[k] = re;
    a.im[k] = im;
  }
  SpinorIO<T>::store(out, outn, n5, i, a);
}

// out_{r,k} = sum_s mat[k][s] in_{r,s} along each rhs block of Ls slots; one thread per
// (half-site, rhs, output slot k)
template <class T>
__global__ void __launch_bounds__(256) dft_s_kernel(const GeoParams g, const void* in, const float* inn, void* out,
                                                    float* outn, const double2* mat) {
  using R = typename Arith<T>::type;
  const size_t n5 = size_t(g.half4) * g.L5;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n5) return;
  const size_t xcb = t / g.L5;
  const int s5 = int(t - xcb * g.L5);
  const int r = s5 / g.Ls, k = s5 - r * g.Ls;
  const size_t base = xcb * g.L5 + size_t(r) * g.Ls;
  R accr[12], acci[12];
#pragma unroll
  for (int q = 0; q < 12; q++) { accr[q] = R(0); acci[q] = R(0); }
  for (int s = 0; s < g.Ls; s++) {
    Spinor<R> a;
    SpinorIO<T>::load(in, inn, n5, base + s, a);
    const double2 m = mat[size_t(k) * g.Ls + s];
    const R mr = R(m.x), mi = R(m.y);
#pragma unroll
    for (int q = 0; q < 12; q++) {
      accr[q] += mr * a.re[q] - mi * a.im[q];
      acci[q] += mr * a.im[q] + mi * a.re[q];
    }
  }
  Spinor<R> o;
#pragma unroll
  for (int q = 0; q < 12; q++) { o.re[q] = accr[q]; o.im[q] = acci[q]; }
  SpinorIO<T>::store(out, outn, n5, t, o);
}

// slot t of dst (L5 = L5d) = slot s of src (L5 = L5s), same 4D checkerboard half
template <class T>
__global__ void __launch_bounds__(256) copy_slot_kernel(int64_t half4, const void* src, const float* srcn, int L5s, int s,
                                                        void* dst, float* dstn, int L5d, int tslot) {
  using R = typename Arith<T>::type;
  const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (x >= half4) return;
  Spinor<R> a;
  SpinorIO<T>::load(src, srcn, size_t(half4) * L5s, size_t(x) * L5s + s, a);
  SpinorIO<T>::store(dst, dstn, size_t(half4) * L5d, size_t(x) * L5d + tslot, a);
}

}  // namespace

int launch_chiral_scale(Op* op, HalfView x, const HalfView* z, double zc, HalfView out, const double* up_re,
                        const double* up_im, const double* dn_re, const double* dn_im) {
  if (op->L5 > kMaxSlots) { set_error("chiral scaling: L5 = %d above %d", op->L5, kMaxSlots); return GB_ERR_UNSUPPORTED; }
  if (x.prec != out.prec || (z && z->prec != x.prec)) { set_error("chiral scaling: mixed precisions"); return GB_ERR_BAD_ARG; }
  ChiralCoef c;
  for (int s = 0; s < kMaxSlots; s++) {
    const bool in = s < op->L5;
    c.up_re[s] = in ? up_re[s] : 0; c.up_im[s] = in ? up_im[s] : 0;
    c.dn_re[s] = in ? dn_re[s] : 0; c.dn_im[s] = in ? dn_im[s] : 0;
  }
  const GeoParams g = geo(op);
  const size_t n = op->n5();
  const void* zd = z ? z->data : nullptr;
  const float* zn = z ? z->norms : nullptr;
  switch (x.prec) {
    case GB_F64: chiral_scale_kernel<double><<<nblk(n), 256, 0, op->stream>>>(g, x.data, x.norms, zd, zn, zc, out.data, out.norms, c); break;
    case GB_F32: chiral_scale_kernel<float><<<nblk(n), 256, 0, op->stream>>>(g, x.data, x.norms, zd, zn, zc, out.data, out.norms, c); break;
    case GB_F16: chiral_scale_kernel<__half><<<nblk(n), 256, 0, op->stream>>>(g, x.data, x.norms, zd, zn, zc, out.data, out.norms, c); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_dft_s(Op* op, HalfView in, HalfView out, const double* mat_host) {
  if (in.prec != out.prec) { set_error("DFT along s: mixed precisions"); return GB_ERR_BAD_ARG; }
  const int Ls = op->Ls;
  double2* dmat = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dmat), size_t(Ls) * Ls * sizeof(double2), op->stream));
  struct Free { double2* p; cudaStream_t s; ~Free() { cudaFreeAsync(p, s); } } guard{dmat, op->stream};
  GB_CHECK_CUDA(cudaMemcpyAsync(dmat, mat_host, size_t(Ls) * Ls * sizeof(double2), cudaMemcpyHostToDevice, op->stream));
  const GeoParams g = geo(op);
  const size_t n = op->n5();
  switch (in.prec) {
    case GB_F64: dft_s_kernel<double><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dmat); break;
    case GB_F32: dft_s_kernel<float><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dmat); break;
    case GB_F16: dft_s_kernel<__half><<<nblk(n), 256, 0, op->stream>>>(g, in.data, in.norms, out.data, out.norms, dmat); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  // the host matrix must outlive the copy: wait before returning
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}

int launch_copy_slot(Op* op, HalfView src, int L5s, int s, HalfView dst, int L5d, int t) {
  if (src.prec != dst.prec) { set_error("slot copy: mixed precisions"); return GB_ERR_BAD_ARG; }
  const size_t n = size_t(op->half4);
  switch (src.prec) {
    case GB_F64: copy_slot_kernel<double><<<nblk(n), 256, 0, op->stream>>>(op->half4, src.data, src.norms, L5s, s, dst.data, dst.norms, L5d, t); break;
    case GB_F32: copy_slot_kernel<float><<<nblk(n), 256, 0, op->stream>>>(op->half4, src.data, src.norms, L5s, s, dst.data, dst.norms, L5d, t); break;
    case GB_F16: copy_slot_kernel<__half><<<nblk(n), 256, 0, op->stream>>>(op->half4, src.data, src.norms, L5s, s, dst.data, dst.norms, L5d, t); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
