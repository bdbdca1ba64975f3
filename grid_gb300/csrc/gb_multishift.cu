// gb_multishift.cu -- ConjugateGradientMultiShift on device-resident fields.
//
// Solves (A + m_s) psi_s = src for every shift m_s at once from the Krylov space of the
// lightest shift m_0 (Grid/algorithms/iterative/ConjugateGradientMultiShift.h:76-330),
// A = MdagM (full fields) or MpcDagMpc (odd fields).  The shifted search directions and
// solutions follow Grid's recurrences:
//   a = c/cp;  p = a p + r;  ps_0 = a ps_0 + r;  ps_s = z_s r + a z_s bs_s/(z'_s b) ps_s
//   d = <p, (A + m_0) p>;  b = -cp/d;  r += b (A + m_0) p;  c = |r|^2
//   z_s <- z_s z'_s bp / (b a (z'_s - z_s) + z'_s bp (1 - (m_s - m_0) b));  bs_s = b z_s / z'_s
//   psi_s -= bs_s ps_s;  shift s stops when c z_s^2 < tol_s^2 |src|^2
// All scalars live on the device and one fused pass per iteration updates every psi_s,
// ps_s and p while reading r once (Grid does this in 2 + 2 nshift passes).  The host polls
// the "all converged" flag every check_every iterations.  Fields are treated as flat
// arrays of 16-byte words (the update is elementwise, so the layout does not matter);
// FP64 and FP32 fields are supported.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {

namespace {

constexpr int kMaxShift = 32;
constexpr int kMsBlocks = 1216;  // reduction CTAs (8 per SM)

struct MSState {
  double a, b, bp, c, cp, d, m0;
  int all_done, iter, frozen, pad1;  // frozen: every update done after all shifts converged
  double mass[kMaxShift], rsq[kMaxShift], z[kMaxShift][2], bs[kMaxShift], as[kMaxShift], zr[kMaxShift];
  int iz, nshift;
  int psi_upd[kMaxShift], ps_upd[kMaxShift], conv[kMaxShift], iters[kMaxShift];
};

template <class V> struct Word;
template <> struct Word<double2> {
  using R = double;
  static __device__ __forceinline__ double2 axpby(R a, const double2& x, R b, const double2& y) {
    return make_double2(fma(a, x.x, b * y.x), fma(a, x.y, b * y.y));
  }
  static __device__ __forceinline__ double dot(const double2& x, const double2& y) { return x.x * y.x + x.y * y.y; }
};
template <> struct Word<float4> {
  using R = float;
  static __device__ __forceinline__ float4 axpby(R a, const float4& x, R b, const float4& y) {
    return make_float4(fmaf(a, x.x, b * y.x), fmaf(a, x.y, b * y.y), fmaf(a, x.z, b * y.z), fmaf(a, x.w, b * y.w));
  }
  static __device__ __forceinline__ double dot(const float4& x, const float4& y) {
    return double(x.x) * y.x + double(x.y) * y.y + double(x.z) * y.z + double(x.w) * y.w;
  }
};

struct MSFields {
  void* ps[kMaxShift];
  void* psi[kMaxShift];
};

// block sum of two doubles into partial[2*blockIdx.x + {0,1}]
__device__ __forceinline__ void block_sum2(double a, double b, double* partial) {
  __shared__ double sa[32], sb[32];
  for (int o = 16; o; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sa[w] = a; sb[w] = b; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    a = l < nw ? sa[l] : 0.0;
    b = l < nw ? sb[l] : 0.0;
    for (int o = 16; o; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (l == 0) { partial[2 * blockIdx.x] = a; partial[2 * blockIdx.x + 1] = b; }
  }
}

// partial: <x, y> and <x, x> (real parts)
template <class V> __global__ void __launch_bounds__(256) ms_dot_kernel(const V* x, const V* y, size_t nw, double* partial) {
  double s1 = 0, s2 = 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nw; i += size_t(gridDim.x) * blockDim.x) {
    const V a = x[i], b = y[i];
    s1 += Word<V>::dot(a, b);
    s2 += Word<V>::dot(a, a);
  }
  block_sum2(s1, s2, partial);
}

// r += b (mmp + m0 p); partial |r|^2
template <class V>
__global__ void __launch_bounds__(256) ms_r_kernel(V* r, const V* mmp, const V* p, size_t nw, const MSState* st,
                                                   double* partial) {
  using R = typename Word<V>::R;
  if (st->frozen) return;
  const R b = R(st->b), bm = R(st->b * st->m0);
  double s1 = 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nw; i += size_t(gridDim.x) * blockDim.x) {
    V v = Word<V>::axpby(b, mmp[i], R(1), r[i]);
    v = Word<V>::axpby(bm, p[i], R(1), v);
    r[i] = v;
    s1 += Word<V>::dot(v, v);
  }
  block_sum2(s1, 0.0, partial);
}

// the fused vector pass: psi_s -= bs_s ps_s (previous iteration), ps_s = zr_s r + as_s ps_s,
// p = a p + r (this iteration)
template <class V>
__global__ void __launch_bounds__(256) ms_update_kernel(V* p, const V* r, const MSFields f, size_t nw,
                                                        const MSState* st, int do_p) {
  using R = typename Word<V>::R;
  if (st->frozen) return;
  const int ns = st->nshift;
  const R a = R(st->a);
  do_p = do_p && !st->all_done;  // after convergence only the pending psi update is left
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nw; i += size_t(gridDim.x) * blockDim.x) {
    const V rv = r[i];
    for (int s = 0; s < ns; s++) {
      V* ps = static_cast<V*>(f.ps[s]);
      if (!st->psi_upd[s] && !st->ps_upd[s]) continue;
      V pv = ps[i];
      if (st->psi_upd[s]) {
        V* psi = static_cast<V*>(f.psi[s]);
        psi[i] = Word<V>::axpby(R(-st->bs[s]), pv, R(1), psi[i]);
      }
      if (do_p && st->ps_upd[s]) ps[i] = Word<V>::axpby(R(st->zr[s]), rv, R(st->as[s]), pv);
    }
    if (do_p) p[i] = Word<V>::axpby(a, p[i], R(1), rv);
  }
}

// psi_s = -bs_s src ; ps_s = src (set-up)
template <class V>
__global__ void __launch_bounds__(256) ms_setup_kernel(const V* src, const MSFields f, size_t nw, const MSState* st) {
  using R = typename Word<V>::R;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nw; i += size_t(gridDim.x) * blockDim.x) {
    const V v = src[i];
    for (int s = 0; s < st->nshift; s++) {
      static_cast<V*>(f.ps[s])[i] = v;
      static_cast<V*>(f.psi[s])[i] = Word<V>::axpby(R(-st->bs[s]), v, R(0), v);
    }
  }
}

// sum of partial[2 i + which] by the whole CTA (256 threads) in a fixed order
__device__ double sum_partials(const double* partial, int n, int which) {
  __shared__ double sm[256];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[2 * i + which];
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

// after the first A p: d, b, z, bs (ConjugateGradientMultiShift.h:152-176)
__global__ void ms_init_kernel(MSState* st, const double* partial, int nparts) {
  const double s0 = sum_partials(partial, nparts, 0), s1 = sum_partials(partial, nparts, 1);
  if (threadIdx.x) return;
  const double d = s0 + st->m0 * s1;
  st->d = d;
  st->b = -st->cp / d;
  st->iz = 0;
  st->z[0][0] = st->z[0][1] = 1.0;
  st->bs[0] = st->b;
  for (int s = 1; s < st->nshift; s++) {
    st->z[s][1] = 1.0;
    st->z[s][0] = 1.0 / (1.0 - st->b * (st->mass[s] - st->mass[0]));
    st->bs[s] = st->b * st->z[s][0];
  }
  for (int s = 0; s < st->nshift; s++) { st->psi_upd[s] = 0; st->ps_upd[s] = 1; st->conv[s] = 0; st->iters[s] = 0; }
}

// after r = src + b A p: c, then this iteration's p/ps coefficients (loop top of Grid's)
__global__ void ms_coef_kernel(MSState* st, const double* partial, int nparts) {
  const double s0 = sum_partials(partial, nparts, 0);
  if (threadIdx.x) return;
  st->c = s0;
  const double a = st->c / st->cp;
  st->a = a;
  const int iz = st->iz;
  st->as[0] = a;
  st->zr[0] = 1.0;
  for (int s = 1; s < st->nshift; s++) {
    st->zr[s] = st->z[s][iz];
    st->as[s] = a * st->z[s][iz] * st->bs[s] / (st->z[s][1 - iz] * st->b);
  }
  st->cp = st->c;
}

// after d = <p, A p>: d, b
__global__ void ms_mid_kernel(MSState* st, const double* partial, int nparts) {
  if (st->frozen) return;  // uniform: read by every thread before any write
  const double s0 = sum_partials(partial, nparts, 0), s1 = sum_partials(partial, nparts, 1);
  if (threadIdx.x) return;
  if (st->all_done) {  // the update pass before this kernel applied the last psi update
    st->frozen = 1;
    return;
  }
  st->d = s0 + st->m0 * s1;
  st->bp = st->b;
  st->b = -st->cp / st->d;
}

// after r += b A p: c, z, bs, convergence, then the next iteration's coefficients
__global__ void ms_post_kernel(MSState* st, const double* partial, int nparts) {
  if (st->frozen) return;
  const double c = sum_partials(partial, nparts, 0);
  if (threadIdx.x) return;
  st->c = c;
  const double b = st->b, bp = st->bp, a = st->a;
  st->bs[0] = b;
  const int iz = 1 - st->iz;
  st->iz = iz;
  st->iter++;
  for (int s = 1; s < st->nshift; s++) {
    if (st->conv[s]) continue;
    const double z0 = st->z[s][1 - iz], z1 = st->z[s][iz];
    st->z[s][iz] = z0 * z1 * bp / (b * a * (z1 - z0) + z1 * bp * (1.0 - (st->mass[s] - st->mass[0]) * b));
    st->bs[s] = b * st->z[s][iz] / z0;
  }
  int all = 1;
  for (int s = 0; s < st->nshift; s++) {
    st->psi_upd[s] = !st->conv[s];  // psi_s -= bs_s ps_s in the next pass
    if (!st->conv[s]) {
      st->iters[s] = st->iter;
      const double css = c * st->z[s][iz] * st->z[s][iz];
      if (css < st->rsq[s]) st->conv[s] = 1;
      else all = 0;
    }
    st->ps_upd[s] = !st->conv[s];
  }
  st->all_done = all;
  // next iteration's a, as, zr (ConjugateGradientMultiShift.h:196-217)
  const double an = c / st->cp;
  st->a = an;
  st->as[0] = an;
  st->zr[0] = 1.0;
  for (int s = 1; s < st->nshift; s++) {
    st->zr[s] = st->z[s][iz];
    st->as[s] = an * st->z[s][iz] * st->bs[s] / (st->z[s][1 - iz] * b);
  }
  st->cp = c;
}

struct Timer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double seconds() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

size_t field_words(const Field* f) { return (f->full() ? 2 : 1) * f->half_bytes() / 16; }

template <class V> struct MS {
  Op* op;
  size_t nw;
  double* partial;
  MSState* st;
  unsigned blocks() const {
    const size_t b = (nw + 255) / 256;
    return unsigned(b < size_t(kMsBlocks) ? b : size_t(kMsBlocks));
  }
  int dot(const Field* x, const Field* y) {
    ms_dot_kernel<V><<<blocks(), 256, 0, op->stream>>>(static_cast<const V*>(x->data), static_cast<const V*>(y->data), nw,
                                                      partial);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
  }
  int r_update(Field* r, const Field* mmp, const Field* p) {
    ms_r_kernel<V><<<blocks(), 256, 0, op->stream>>>(static_cast<V*>(r->data), static_cast<const V*>(mmp->data),
                                                    static_cast<const V*>(p->data), nw, st, partial);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
  }
  int update(Field* p, const Field* r, const MSFields& f, int do_p) {
    ms_update_kernel<V><<<blocks(), 256, 0, op->stream>>>(static_cast<V*>(p->data), static_cast<const V*>(r->data), f,
                                                         nw, st, do_p);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
  }
  int setup(const Field* src, const MSFields& f) {
    ms_setup_kernel<V><<<blocks(), 256, 0, op->stream>>>(static_cast<const V*>(src->data), f, nw, st);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
  }
  int scalar(void (*k)(MSState*, const double*, int)) {
    k<<<1, 256, 0, op->stream>>>(st, partial, int(blocks()));
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
  }
};

template <class V>
int multishift(Op* op, int kind, Field* src, int ns, const double* shifts, const double* tols, Field** psi,
               int maxit, int check_every, gb_multishift_result* R) {
  Timer tm;
  Field *p, *mmp, *r, *t;
  GB_TRY(ws_get(op, kind == 0 ? GB_FULL : GB_ODD, src->prec, kind == 0 ? WS_MS_P_FULL : WS_MS_P, &p));
  GB_TRY(ws_get(op, kind == 0 ? GB_FULL : GB_ODD, src->prec, kind == 0 ? WS_MS_MMP_FULL : WS_MS_MMP, &mmp));
  GB_TRY(ws_get(op, kind == 0 ? GB_FULL : GB_ODD, src->prec, kind == 0 ? WS_MS_R_FULL : WS_MS_R, &r));
  GB_TRY(ws_get(op, kind == 0 ? GB_FULL : GB_ODD, src->prec, kind == 0 ? WS_MS_T_FULL : WS_MS_T, &t));
  MSFields f;
  std::memset(&f, 0, sizeof(f));
  std::vector<Field*> ps(ns);
  for (int s = 0; s < ns; s++) {
    GB_TRY(ws_get(op, kind == 0 ? GB_FULL : GB_ODD, src->prec, (kind == 0 ? WS_MS_PS_FULL : WS_MS_PS) + s, &ps[s]));
    f.ps[s] = ps[s]->data;
    f.psi[s] = psi[s]->data;
    psi[s]->subset = src->subset;
  }
  if (!src->full()) p->subset = mmp->subset = r->subset = t->subset = src->subset;
  MS<V> ms{op, field_words(src), op->d_partial, nullptr};  // kMsBlocks <= kRedBlocks partial pairs
  MSState* st = nullptr;
  MSState* hst = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&st), sizeof(MSState), op->stream));
  struct Free { MSState* d; MSState* h; cudaStream_t s; ~Free() { if (d) cudaFreeAsync(d, s); if (h) cudaFreeHost(h); } }
      guard{st, nullptr, op->stream};
  GB_CHECK_CUDA(cudaMallocHost(reinterpret_cast<void**>(&hst), sizeof(MSState)));
  guard.h = hst;
  ms.st = st;

  // |src|^2 and the per-shift targets (ConjugateGradientMultiShift.h:130-150)
  GB_TRY(ms.dot(src, src));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  std::vector<double> part(2 * ms.blocks());
  GB_CHECK_CUDA(cudaMemcpy(part.data(), op->d_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost));
  double ssq = 0;
  for (unsigned i = 0; i < ms.blocks(); i++) ssq += part[2 * i];
  std::memset(hst, 0, sizeof(MSState));
  hst->nshift = ns;
  hst->m0 = shifts[0];
  hst->cp = ssq;
  for (int s = 0; s < ns; s++) {
    hst->mass[s] = shifts[s];
    hst->rsq[s] = ssq * tols[s] * tols[s];
  }
  std::memset(R, 0, sizeof(*R));
  R->nshift = ns;
  if (ssq == 0.0) {  // trivial source
    for (int s = 0; s < ns; s++) { GB_TRY(field_zero(psi[s])); R->iterations_shift[s] = 1; }
    R->converged = 1;
    R->seconds = tm.seconds();
    return GB_OK;
  }
  GB_CHECK_CUDA(cudaMemcpyAsync(st, hst, sizeof(MSState), cudaMemcpyHostToDevice, op->stream));
  // r = p = src ; mmp = A p ; d = <p, (A + m0) p> ; b ; z ; bs ; r += b (A + m0) p ; c
  GB_TRY(field_copy(r, src));
  GB_TRY(field_copy(p, src));
  GB_TRY(op_hermop(op, kind, p, mmp));
  GB_TRY(ms.dot(p, mmp));
  GB_TRY(ms.scalar(ms_init_kernel));
  GB_TRY(ms.r_update(r, mmp, p));
  GB_TRY(ms.setup(src, f));  // psi_s = -bs_s src, ps_s = src
  GB_TRY(ms.scalar(ms_coef_kernel));
  const int chunk = check_every > 0 ? check_every : 10;
  int k = 0;
  bool done = false;
  while (!done && k < maxit) {
    const int m = std::min(chunk, maxit - k);
    for (int j = 0; j < m; j++) {
      GB_TRY(ms.update(p, r, f, 1));  // psi (previous), ps, p
      GB_TRY(op_hermop(op, kind, p, mmp));
      GB_TRY(ms.dot(p, mmp));
      GB_TRY(ms.scalar(ms_mid_kernel));
      GB_TRY(ms.r_update(r, mmp, p));
      GB_TRY(ms.scalar(ms_post_kernel));
    }
    k += m;
    GB_CHECK_CUDA(cudaMemcpyAsync(hst, st, sizeof(MSState), cudaMemcpyDeviceToHost, op->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
    done = hst->all_done != 0;
  }
  // the last psi update (psi_s -= bs_s ps_s for the shifts still running at the last step)
  GB_TRY(ms.update(p, r, f, 0));
  GB_CHECK_CUDA(cudaMemcpyAsync(hst, st, sizeof(MSState), cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  // true residuals |(A + m_s) psi_s - src| / |src|  (ConjugateGradientMultiShift.h:296-305)
  for (int s = 0; s < ns; s++) {
    GB_TRY(op_hermop(op, kind, psi[s], mmp));
    GB_TRY(field_axpby(t, 1.0, shifts[s], mmp, psi[s]));
    GB_TRY(field_axpby(t, 1.0, -1.0, t, src));
    GB_TRY(ms.dot(t, t));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
    GB_CHECK_CUDA(cudaMemcpy(part.data(), op->d_partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost));
    double rn = 0;
    for (unsigned i = 0; i < ms.blocks(); i++) rn += part[2 * i];
    R->true_residual_shift[s] = std::sqrt(rn / ssq);
    R->iterations_shift[s] = hst->iters[s];
  }
  R->iterations = hst->iter;
  R->converged = hst->all_done;
  R->seconds = tm.seconds();
  R->flops = hermop_flops(op, kind) * R->iterations;
  GB_TRY(check_device_error(op));
  if (!R->converged) {
    set_error("multishift CG did not converge in %d iterations", maxit);
    return GB_ERR_NOT_CONVERGED;
  }
  return GB_OK;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_cg_multishift(gb_op_t op, int kind, gb_field_t src, int nshift, const double* shifts,
                                const double* tolerances, gb_field_t* psi, int max_iterations, int check_every,
                                gb_multishift_result* res) {
  if (!op || !src || !shifts || !tolerances || !psi || !res) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (!op->gauge_loaded) { set_error("operator has no gauge field"); return GB_ERR_BAD_ARG; }
  if (nshift < 1 || nshift > kMaxShift) { set_error("nshift = %d outside [1, %d]", nshift, kMaxShift); return GB_ERR_BAD_ARG; }
  if (kind != 0 && kind != 1) { set_error("kind must be 0 (MdagM) or 1 (MpcDagMpc)"); return GB_ERR_BAD_ARG; }
  if (max_iterations < 1) { set_error("max_iterations < 1"); return GB_ERR_BAD_ARG; }
  if (op->nrhs_user != 1) { set_error("multishift CG: one right-hand side"); return GB_ERR_UNSUPPORTED; }
  if (src->prec != op->prec || (op->prec != GB_F64 && op->prec != GB_F32)) {
    set_error("multishift CG: FP64 or FP32 fields of the operator's precision");
    return GB_ERR_UNSUPPORTED;
  }
  if (!ops_conformable(src->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; }
  if (kind == 0 && !src->full()) { set_error("MdagM multishift: full fields expected"); return GB_ERR_BAD_PARITY; }
  if (kind == 1 && src->subset != GB_ODD) { set_error("Schur multishift: odd source expected"); return GB_ERR_BAD_PARITY; }
  for (int s = 0; s < nshift; s++) {
    if (!psi[s] || !ops_conformable(psi[s]->op, op) || psi[s]->prec != src->prec || psi[s]->full() != src->full()) {
      set_error("psi[%d] is not conformable to the source", s);
      return GB_ERR_BAD_ARG;
    }
    if (shifts[s] < shifts[0]) { set_error("shift %d is lighter than shift 0 (the primary must be the lightest)", s); return GB_ERR_BAD_ARG; }
    if (!(tolerances[s] > 0)) { set_error("tolerance %d must be positive", s); return GB_ERR_BAD_ARG; }
    for (int u = 0; u < s; u++)
      if (psi[u] == psi[s] || psi[s] == src) { set_error("psi fields must be distinct from each other and src"); return GB_ERR_BAD_ARG; }
  }
  std::vector<Field*> ps(nshift);
  for (int s = 0; s < nshift; s++) ps[s] = psi[s];
  if (op->prec == GB_F64)
    return multishift<double2>(op, kind, src, nshift, shifts, tolerances, ps.data(), max_iterations, check_every, res);
  return multishift<float4>(op, kind, src, nshift, shifts, tolerances, ps.data(), max_iterations, check_every, res);
}
