// gb_5d.cu -- fifth-dimension kernels of the Cayley / Moebius operator.
//
// m5d_kernel: Grid's CayleyFermion5D::M5D / M5Ddag
//   (Grid/qcd/action/fermion/implementation/CayleyFermion5Dcache.h:41-115)
//     non-dag: chi[s] = d[s] phi[s] + u[s] P- psi[s+1] + l[s] P+ psi[s-1]
//     dag    : chi[s] = d[s] phi[s] + u[s] P+ psi[s+1] + l[s] P- psi[s-1]
//   periodic in s within each right-hand side's block of Ls slots, plus an optional
//   fused "+ zc * z" term (the axpy of SchurDiagMooeeOperator::Mpc).
// mooee_inv_kernel: Grid's CayleyFermion5D::MooeeInv / MooeeInvDag, the LDU forward and
//   backward sweeps along s (CayleyFermion5Dcache.h:117-230).  The sweeps act on each
//   spin-colour component separately, so one thread owns one 16-byte plane vector of
//   one (4D site, rhs) and keeps the whole s column in registers.
#include <cuda_fp16.h>

#include "gb_device.cuh"

namespace gb {

template <class R> struct Coef5 {
  R d[kMaxLs], u[kMaxLs], l[kMaxLs];
};

struct M5Params {
  const void* psi; const float* psi_n;
  const void* phi; const float* phi_n;
  void* chi; float* chi_n;
  const void* z; const float* z_n;
  double zc;
  size_t n5;
  int L5, Ls;
};

template <class T, bool DAG, bool ZTERM>
__global__ void __launch_bounds__(256) m5d_kernel(const M5Params p, const Coef5<typename Arith<T>::type> c) {
  using R = typename Arith<T>::type;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.n5) return;
  const int s5 = int(i % p.L5);
  const int s = s5 % p.Ls;
  const size_t base = i - s;
  const size_t ip = base + (s + 1 == p.Ls ? 0 : s + 1);
  const size_t im = base + (s == 0 ? p.Ls - 1 : s - 1);
  Spinor<R> f, a;
  SpinorIO<T>::load(p.phi, p.phi_n, p.n5, i, f);
  // upper spins (P+) come from s-1 (non-dag) or s+1 (dag); lower spins (P-) the other one
  SpinorIO<T>::load_half(p.psi, p.psi_n, p.n5, DAG ? ip : im, true, a);
  SpinorIO<T>::load_half(p.psi, p.psi_n, p.n5, DAG ? im : ip, false, a);
  const R d = c.d[s];
  const R cu = DAG ? c.u[s] : c.l[s];  // coefficient of the upper-spin neighbour
  const R cl = DAG ? c.l[s] : c.u[s];  // coefficient of the lower-spin neighbour
  Spinor<R> o;
#pragma unroll
  for (int k = 0; k < 6; k++) {
    o.re[k] = fma(cu, a.re[k], d * f.re[k]);
    o.im[k] = fma(cu, a.im[k], d * f.im[k]);
  }
#pragma unroll
  for (int k = 6; k < 12; k++) {
    o.re[k] = fma(cl, a.re[k], d * f.re[k]);
    o.im[k] = fma(cl, a.im[k], d * f.im[k]);
  }
  if (ZTERM) {
    Spinor<R> z;
    SpinorIO<T>::load(p.z, p.z_n, p.n5, i, z);
    const R zc = R(p.zc);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      o.re[k] = fma(zc, z.re[k], o.re[k]);
      o.im[k] = fma(zc, z.im[k], o.im[k]);
    }
  }
  SpinorIO<T>::store(p.chi, p.chi_n, p.n5, i, o);
}

template <class T, bool DAG, bool ZTERM>
static int launch_m5d_t(Op* op, const M5Params& p, const double* lower, const double* diag, const double* upper) {
  using R = typename Arith<T>::type;
  Coef5<R> c;
  for (int s = 0; s < op->Ls; s++) { c.d[s] = R(diag[s]); c.u[s] = R(upper[s]); c.l[s] = R(lower[s]); }
  const unsigned blocks = unsigned((p.n5 + 255) / 256);
  m5d_kernel<T, DAG, ZTERM><<<blocks, 256, 0, op->stream>>>(p, c);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

template <class T>
static int launch_m5d_p(Op* op, const M5Params& p, const double* l, const double* d, const double* u, int dag) {
  const bool z = p.z != nullptr;
  if (dag) return z ? launch_m5d_t<T, true, true>(op, p, l, d, u) : launch_m5d_t<T, true, false>(op, p, l, d, u);
  return z ? launch_m5d_t<T, false, true>(op, p, l, d, u) : launch_m5d_t<T, false, false>(op, p, l, d, u);
}

int launch_m5d_z(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
                 const double* upper, int dag, size_t n5, const HalfView* z, double zc, int* norm_parts) {
  if (norm_parts) *norm_parts = 0;
  if (op->Ls > kMaxLs) {
    set_error("M5D: Ls = %d exceeds %d", op->Ls, kMaxLs);
    return GB_ERR_UNSUPPORTED;
  }
  if (psi.prec != phi.prec || psi.prec != chi.prec || (z && z->prec != psi.prec)) {
    set_error("M5D: mixed field precisions");
    return GB_ERR_BAD_ARG;
  }
  M5Params p;
  p.psi = psi.data; p.psi_n = psi.norms;
  p.phi = phi.data; p.phi_n = phi.norms;
  p.chi = chi.data; p.chi_n = chi.norms;
  p.z = z ? z->data : nullptr; p.z_n = z ? z->norms : nullptr;
  p.zc = zc;
  p.n5 = n5;
  p.L5 = op->L5;
  p.Ls = op->Ls;
  // FP32 / FP16 (site-pair layout, Ls even): one thread per pair of s slots
  if (psi.prec != GB_F64) return launch_m5d_pair(op, psi, phi, chi, lower, diag, upper, dag, n5, z, zc, norm_parts);
  return launch_m5d_p<double>(op, p, lower, diag, upper, dag);
}

int launch_m5d(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
               const double* upper, int dag, size_t n5) {
  return launch_m5d_z(op, psi, phi, chi, lower, diag, upper, dag, n5, nullptr, 0.0, nullptr);
}

// ---------------------------------------------------------------------------------------
// MooeeInv
// ---------------------------------------------------------------------------------------
template <class R> struct LduCoef {
  R lee[kMaxLs], leem[kMaxLs], uee[kMaxLs], ueem[kMaxLs], dinv[kMaxLs];
};

struct InvParams {
  const void* in; const float* in_n;
  void* out; float* out_n;
  size_t n5;
  size_t nq;  // (4D site, rhs) pairs
  int L5, Ls, nplanes;
};

template <class V> struct VecOps;
template <> struct VecOps<double2> {
  using R = double;
  static __device__ __forceinline__ double2 zero() { return make_double2(0, 0); }
  static __device__ __forceinline__ double2 axpy(R a, double2 x, double2 y) { return make_double2(fma(a, x.x, y.x), fma(a, x.y, y.y)); }
  static __device__ __forceinline__ double2 scale(R a, double2 x) { return make_double2(a * x.x, a * x.y); }
};
template <> struct VecOps<float4> {
  using R = float;
  static __device__ __forceinline__ float4 zero() { return make_float4(0, 0, 0, 0); }
  static __device__ __forceinline__ float4 axpy(R a, float4 x, float4 y) {
    return make_float4(fmaf(a, x.x, y.x), fmaf(a, x.y, y.y), fmaf(a, x.z, y.z), fmaf(a, x.w, y.w));
  }
  static __device__ __forceinline__ float4 scale(R a, float4 x) { return make_float4(a * x.x, a * x.y, a * x.z, a * x.w); }
};

// one thread per (plane, 4D site, rhs); plane-major thread order.  LS > 0: compile-time
// Ls with the column in registers; LS == 0: runtime Ls, the forward sweep's values are
// re-read from the output.
template <class V, bool DAG, int LS>
__global__ void __launch_bounds__(256) mooee_inv_kernel(const InvParams p, const LduCoef<typename VecOps<V>::R> c) {
  using Ops = VecOps<V>;
  using R = typename Ops::R;
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= p.nq * p.nplanes) return;
  const int g = int(t / p.nq);
  const size_t q = t - size_t(g) * p.nq;
  const int Ls = LS > 0 ? LS : p.Ls;
  const int nrhs = p.L5 / p.Ls;
  const size_t x = q / nrhs;
  const int rhs = int(q - x * nrhs);
  const size_t i0 = x * p.L5 + size_t(rhs) * Ls;
  const V* in = static_cast<const V*>(p.in) + size_t(g) * p.n5 + i0;
  V* out = static_cast<V*>(p.out) + size_t(g) * p.n5 + i0;
  const bool upper = g < p.nplanes / 2;
  // the chirality propagated by the forward sweep: P+ (non-dag) or P- (dag)
  const bool first = DAG ? !upper : upper;
  constexpr int NB = LS > 0 ? LS : 1;
  V col[NB];
  V prev = Ops::zero(), acc = Ops::zero(), r;
#pragma unroll
  for (int s = 0; s < Ls - 1; s++) {
    r = __ldg(in + s);
    if (first) { if (s > 0) r = Ops::axpy(-c.lee[s - 1], prev, r); }
    else acc = Ops::axpy(c.leem[s], r, acc);
    if (LS > 0) col[s < NB ? s : 0] = r; else out[s] = r;
    prev = r;
  }
  r = __ldg(in + Ls - 1);
  if (first) r = Ops::axpy(-c.lee[Ls - 2], prev, r);
  else r = Ops::axpy(R(-1), acc, r);
  r = Ops::scale(c.dinv[Ls - 1], r);
  out[Ls - 1] = r;
  const V last = r;
  V nxt = r;
#pragma unroll
  for (int s = Ls - 2; s >= 0; s--) {
    V v = LS > 0 ? col[s < NB ? s : 0] : out[s];
    v = Ops::scale(c.dinv[s], v);
    if (!first) v = Ops::axpy(-c.uee[s], nxt, v);
    else v = Ops::axpy(-c.ueem[s], last, v);
    out[s] = v;
    nxt = v;
  }
}

// FP16 storage: one thread per (4D site, rhs) on whole spinors, arithmetic in FP32.
template <bool DAG>
__global__ void __launch_bounds__(128) mooee_inv_half_kernel(const InvParams p, const LduCoef<float> c) {
  const size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= p.nq) return;
  const int Ls = p.Ls;
  const int nrhs = p.L5 / Ls;
  const size_t x = q / nrhs;
  const int rhs = int(q - x * nrhs);
  const size_t i0 = x * p.L5 + size_t(rhs) * Ls;
  Spinor<float> prev, acc, r, last, nxt;
  for (int k = 0; k < 12; k++) { prev.re[k] = prev.im[k] = acc.re[k] = acc.im[k] = 0.f; }
  // chirality of component k: k < 6 upper
  for (int s = 0; s < Ls - 1; s++) {
    SpinorIO<__half>::load(p.in, p.in_n, p.n5, i0 + s, r);
    for (int k = 0; k < 12; k++) {
      const bool first = DAG ? (k >= 6) : (k < 6);
      if (first) { if (s > 0) { r.re[k] -= c.lee[s - 1] * prev.re[k]; r.im[k] -= c.lee[s - 1] * prev.im[k]; } }
      else { acc.re[k] += c.leem[s] * r.re[k]; acc.im[k] += c.leem[s] * r.im[k]; }
    }
    // the forward column passes through the FP16 output between the two sweeps, like
    // every FP16 intermediate; continue with the rounded value so both sweeps agree
    SpinorIO<__half>::store(p.out, p.out_n, p.n5, i0 + s, r);
    SpinorIO<__half>::load(p.out, p.out_n, p.n5, i0 + s, r);
    prev = r;
  }
  SpinorIO<__half>::load(p.in, p.in_n, p.n5, i0 + Ls - 1, r);
  for (int k = 0; k < 12; k++) {
    const bool first = DAG ? (k >= 6) : (k < 6);
    if (first) { r.re[k] -= c.lee[Ls - 2] * prev.re[k]; r.im[k] -= c.lee[Ls - 2] * prev.im[k]; }
    else { r.re[k] -= acc.re[k]; r.im[k] -= acc.im[k]; }
    r.re[k] *= c.dinv[Ls - 1]; r.im[k] *= c.dinv[Ls - 1];
  }
  SpinorIO<__half>::store(p.out, p.out_n, p.n5, i0 + Ls - 1, r);
  last = r;
  nxt = r;
  for (int s = Ls - 2; s >= 0; s--) {
    Spinor<float> v;
    SpinorIO<__half>::load(p.out, p.out_n, p.n5, i0 + s, v);
    for (int k = 0; k < 12; k++) {
      const bool first = DAG ? (k >= 6) : (k < 6);
      v.re[k] *= c.dinv[s]; v.im[k] *= c.dinv[s];
      if (!first) { v.re[k] -= c.uee[s] * nxt.re[k]; v.im[k] -= c.uee[s] * nxt.im[k]; }
      else { v.re[k] -= c.ueem[s] * last.re[k]; v.im[k] -= c.ueem[s] * last.im[k]; }
    }
    SpinorIO<__half>::store(p.out, p.out_n, p.n5, i0 + s, v);
    nxt = v;
  }
}

// FP32 site-pair layout: one thread per (complex component k, 4D site, rhs); the s column
// of that component is Ls/2 float4 vectors (re_s, re_s+1, im_s, im_s+1), kept in
// registers for compile-time LS (LS == 0: runtime Ls, column re-read from the output).
template <bool DAG, int LS>
__global__ void __launch_bounds__(256) mooee_inv_pair_kernel(const InvParams p, const LduCoef<float> c) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= p.nq * 12) return;
  const int k = int(t / p.nq);
  const size_t q = t - size_t(k) * p.nq;
  const int Ls = LS > 0 ? LS : p.Ls;
  const int nrhs = p.L5 / p.Ls;
  const size_t x = q / nrhs;
  const int rhs = int(q - x * nrhs);
  const size_t np = p.n5 >> 1;
  const size_t q0 = (x * p.L5 + size_t(rhs) * Ls) >> 1;  // first pair of the column
  const float4* in = static_cast<const float4*>(p.in) + size_t(k) * np + q0;
  float4* out = static_cast<float4*>(p.out) + size_t(k) * np + q0;
  const bool first = DAG ? (k >= 6) : (k < 6);
  constexpr int NB = LS > 0 ? LS : 2;
  float cr[NB], ci[NB];
  float pr = 0.f, pi = 0.f, ar = 0.f, ai = 0.f;
  // forward sweep, pairs of s
#pragma unroll
  for (int m = 0; m < (LS > 0 ? LS / 2 : 1); m++) {
    if (LS == 0) break;
    const float4 v = __ldg(in + m);
    float re[2] = {v.x, v.y}, im[2] = {v.z, v.w};
#pragma unroll
    for (int l = 0; l < 2; l++) {
      const int s = 2 * m + l;
      float r = re[l], i = im[l];
      if (s < Ls - 1) {
        if (first) { if (s > 0) { r = fmaf(-c.lee[s - 1], pr, r); i = fmaf(-c.lee[s - 1], pi, i); } }
        else { ar = fmaf(c.leem[s], r, ar); ai = fmaf(c.leem[s], i, ai); }
        pr = r; pi = i;
      } else {
        if (first) { r = fmaf(-c.lee[Ls - 2], pr, r); i = fmaf(-c.lee[Ls - 2], pi, i); }
        else { r -= ar; i -= ai; }
        r *= c.dinv[Ls - 1]; i *= c.dinv[Ls - 1];
      }
      cr[s < NB ? s : 0] = r; ci[s < NB ? s : 0] = i;
    }
  }
  if (LS == 0) {  // runtime Ls: same sweep through the output
    for (int m = 0; m < Ls / 2; m++) {
      const float4 v = __ldg(in + m);
      float re[2] = {v.x, v.y}, im[2] = {v.z, v.w};
      float o[4];
      for (int l = 0; l < 2; l++) {
        const int s = 2 * m + l;
        float r = re[l], i = im[l];
        if (s < Ls - 1) {
          if (first) { if (s > 0) { r = fmaf(-c.lee[s - 1], pr, r); i = fmaf(-c.lee[s - 1], pi, i); } }
          else { ar = fmaf(c.leem[s], r, ar); ai = fmaf(c.leem[s], i, ai); }
          pr = r; pi = i;
        } else {
          if (first) { r = fmaf(-c.lee[Ls - 2], pr, r); i = fmaf(-c.lee[Ls - 2], pi, i); }
          else { r -= ar; i -= ai; }
          r *= c.dinv[Ls - 1]; i *= c.dinv[Ls - 1];
        }
        o[l] = r; o[2 + l] = i;
      }
      out[m] = make_float4(o[0], o[1], o[2], o[3]);
    }
  }
  // backward sweep: chi_s = chi_s / d_s - (uee[s] P_second chi_{s+1} | ueem[s] P_first chi_{Ls-1})
  float lr, li;
  if (LS > 0) { lr = cr[NB - 1]; li = ci[NB - 1]; }
  else { const float4 v = out[Ls / 2 - 1]; lr = v.y; li = v.w; }
  float nr = lr, ni = li;
  if (LS > 0) {
#pragma unroll
    for (int s = (LS > 0 ? LS : 2) - 2; s >= 0; s--) {
      float r = cr[s] * c.dinv[s], i = ci[s] * c.dinv[s];
      if (!first) { r = fmaf(-c.uee[s], nr, r); i = fmaf(-c.uee[s], ni, i); }
      else { r = fmaf(-c.ueem[s], lr, r); i = fmaf(-c.ueem[s], li, i); }
      cr[s] = r; ci[s] = i;
      nr = r; ni = i;
    }
#pragma unroll
    for (int m = 0; m < (LS > 0 ? LS / 2 : 1); m++) out[m] = make_float4(cr[2 * m], cr[2 * m + 1], ci[2 * m], ci[2 * m + 1]);
  } else {
    for (int m = Ls / 2 - 1; m >= 0; m--) {
      float4 v = out[m];
      float re[2] = {v.x, v.y}, im[2] = {v.z, v.w};
      for (int l = 1; l >= 0; l--) {
        const int s = 2 * m + l;
        if (s == Ls - 1) continue;
        float r = re[l] * c.dinv[s], i = im[l] * c.dinv[s];
        if (!first) { r = fmaf(-c.uee[s], nr, r); i = fmaf(-c.uee[s], ni, i); }
        else { r = fmaf(-c.ueem[s], lr, r); i = fmaf(-c.ueem[s], li, i); }
        re[l] = r; im[l] = i;
        nr = r; ni = i;
      }
      out[m] = make_float4(re[0], re[1], im[0], im[1]);
    }
  }
}

template <bool DAG> static int launch_inv_pair(Op* op, const InvParams& p, const LduCoef<float>& c) {
  const size_t n = p.nq * 12;
  const unsigned blocks = unsigned((n + 255) / 256);
  switch (op->Ls) {
#define GB_INVP_CASE(L) \
  case L: mooee_inv_pair_kernel<DAG, L><<<blocks, 256, 0, op->stream>>>(p, c); break;
    GB_INVP_CASE(2) GB_INVP_CASE(4) GB_INVP_CASE(6) GB_INVP_CASE(8) GB_INVP_CASE(10) GB_INVP_CASE(12)
    GB_INVP_CASE(14) GB_INVP_CASE(16) GB_INVP_CASE(20) GB_INVP_CASE(24) GB_INVP_CASE(32)
#undef GB_INVP_CASE
    default: mooee_inv_pair_kernel<DAG, 0><<<blocks, 256, 0, op->stream>>>(p, c); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

template <class V, bool DAG>
static int launch_inv_v(Op* op, const InvParams& p, const LduCoef<typename VecOps<V>::R>& c) {
  const size_t n = p.nq * p.nplanes;
  const unsigned blocks = unsigned((n + 255) / 256);
  switch (op->Ls) {
#define GB_INV_CASE(L) \
  case L: mooee_inv_kernel<V, DAG, L><<<blocks, 256, 0, op->stream>>>(p, c); break;
    GB_INV_CASE(4) GB_INV_CASE(6) GB_INV_CASE(8) GB_INV_CASE(10) GB_INV_CASE(12) GB_INV_CASE(16)
    GB_INV_CASE(20) GB_INV_CASE(24) GB_INV_CASE(32)
#undef GB_INV_CASE
    default: mooee_inv_kernel<V, DAG, 0><<<blocks, 256, 0, op->stream>>>(p, c); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

template <class R> static void fill_ldu(const Op* op, int dag, LduCoef<R>& c) {
  // MooeeInvDag uses the transposed factors: (lee,leem) <-> (uee,ueem)
  const std::vector<double>& lee = dag ? op->uee : op->lee;
  const std::vector<double>& leem = dag ? op->ueem : op->leem;
  const std::vector<double>& uee = dag ? op->lee : op->uee;
  const std::vector<double>& ueem = dag ? op->leem : op->ueem;
  for (int s = 0; s < op->Ls; s++) {
    c.lee[s] = R(lee[s]); c.leem[s] = R(leem[s]); c.uee[s] = R(uee[s]); c.ueem[s] = R(ueem[s]);
    c.dinv[s] = R(1.0 / op->dee[s]);
  }
}

int launch_mooee_inv(Op* op, HalfView in, HalfView out, int dag, size_t n4) {
  if (op->Ls > kMaxLs || op->Ls < 2) {
    set_error("MooeeInv: Ls = %d outside [2, %d]", op->Ls, kMaxLs);
    return GB_ERR_UNSUPPORTED;
  }
  if (in.prec != out.prec) {
    set_error("MooeeInv: mixed field precisions");
    return GB_ERR_BAD_ARG;
  }
  InvParams p;
  p.in = in.data; p.in_n = in.norms;
  p.out = out.data; p.out_n = out.norms;
  p.n5 = n4 * op->L5;
  p.nq = n4 * op->nrhs;
  p.L5 = op->L5;
  p.Ls = op->Ls;
  if (in.prec == GB_F64) {
    LduCoef<double> c; fill_ldu(op, dag, c);
    p.nplanes = 12;
    return dag ? launch_inv_v<double2, true>(op, p, c) : launch_inv_v<double2, false>(op, p, c);
  }
  if (in.prec == GB_F32) {
    LduCoef<float> c; fill_ldu(op, dag, c);
    p.nplanes = 12;
    return dag ? launch_inv_pair<true>(op, p, c) : launch_inv_pair<false>(op, p, c);
  }
  LduCoef<float> c; fill_ldu(op, dag, c);
  p.nplanes = 1;
  const unsigned blocks = unsigned((p.nq + 127) / 128);
  if (dag) mooee_inv_half_kernel<true><<<blocks, 128, 0, op->stream>>>(p, c);
  else mooee_inv_half_kernel<false><<<blocks, 128, 0, op->stream>>>(p, c);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
