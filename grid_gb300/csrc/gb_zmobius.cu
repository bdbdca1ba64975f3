// gb_zmobius.cu -- the Cayley 5D operators with complex coefficients (ZMobiusFermion,
// Grid/qcd/action/fermion/ZMobiusFermion.h; CayleyFermion5DImplementation.h:155-271,
// 410-535; CayleyFermion5Dcache.h:41-230), FP64 and FP32 storage.
//
// A ZMobius operator has a complex omega_s per s, so bs, cs and the LDU factors of Mooee
// are complex.  As in the real case every 5D operator acts on each spin-colour component
// of each (4D site, rhs) column on its own; one thread owns one column in registers and
// runs one program:
//   ZCOL_M5D   out_s = d_s x_s + (l_s x_{s-1} | u_s x_{s+1}) [+ zc y_s]
//   ZCOL_INV   the LDU solve of MooeeInv / MooeeInvDag
//   ZCOL_DIAG  out_s = x_s + e_s y_s                      (Dminus)
// The host passes coefficients already conjugated / swapped for the dagger forms, as
// Grid assembles them; the dagger flag only selects the neighbour side and the
// chirality roles.
#include <complex>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {
namespace {

template <class R> struct Cx {
  R x, y;
};
template <class R> __device__ __forceinline__ Cx<R> cmul(Cx<R> a, Cx<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class R> __device__ __forceinline__ Cx<R> cfma(Cx<R> a, Cx<R> b, Cx<R> c) {  // a b + c
  return {fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}

template <class R, int LS> struct ZCoef {
  Cx<R> d[LS], u[LS], l[LS];                          // M5D
  Cx<R> lee[LS], leem[LS], uee[LS], ueem[LS], dinv[LS];  // LDU
  Cx<R> e[LS];                                        // DIAG
};

struct ZParams {
  const void* x;
  const void* y;
  void* out;
  size_t n5;  // 5D sites per half field
  size_t nq;  // columns (4D site, rhs)
  double zc;
};

// column I/O: FP64 = double2 planes (one site per vector), FP32 = float4 site pairs
template <class R> struct ZIO;
template <> struct ZIO<double> {
  template <int LS> static __device__ __forceinline__ void load(const void* b, size_t n5, int k, size_t q, Cx<double> (&c)[LS]) {
    const double2* p = static_cast<const double2*>(b) + size_t(k) * n5 + q * LS;
#pragma unroll
    for (int s = 0; s < LS; s++) { const double2 v = __ldg(p + s); c[s] = {v.x, v.y}; }
  }
  template <int LS> static __device__ __forceinline__ void store(void* b, size_t n5, int k, size_t q, const Cx<double> (&c)[LS]) {
    double2* p = static_cast<double2*>(b) + size_t(k) * n5 + q * LS;
#pragma unroll
    for (int s = 0; s < LS; s++) p[s] = make_double2(c[s].x, c[s].y);
  }
};
template <> struct ZIO<float> {
  template <int LS> static __device__ __forceinline__ void load(const void* b, size_t n5, int k, size_t q, Cx<float> (&c)[LS]) {
    const float4* p = static_cast<const float4*>(b) + size_t(k) * (n5 >> 1) + q * (LS / 2);
#pragma unroll
    for (int m = 0; m < LS / 2; m++) {
      const float4 v = __ldg(p + m);
      c[2 * m] = {v.x, v.z};
      c[2 * m + 1] = {v.y, v.w};
    }
  }
  template <int LS> static __device__ __forceinline__ void store(void* b, size_t n5, int k, size_t q, const Cx<float> (&c)[LS]) {
    float4* p = static_cast<float4*>(b) + size_t(k) * (n5 >> 1) + q * (LS / 2);
#pragma unroll
    for (int m = 0; m < LS / 2; m++) p[m] = make_float4(c[2 * m].x, c[2 * m + 1].x, c[2 * m].y, c[2 * m + 1].y);
  }
};

enum { ZCOL_M5D = 0, ZCOL_M5D_Y = 1, ZCOL_INV = 2, ZCOL_DIAG = 3 };

// one thread per (component k, column q); consecutive threads take consecutive columns
template <class R, int LS, bool DAG, int PROG>
__global__ void __launch_bounds__(128) zcol_kernel(const ZParams p, const ZCoef<R, LS> c) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= p.nq * 12) return;
  const int k = int(t / p.nq);
  const size_t q = t - size_t(k) * p.nq;
  const bool upper = k < 6;
  Cx<R> x[LS], o[LS];
  ZIO<R>::template load<LS>(p.x, p.n5, k, q, x);
  if (PROG == ZCOL_M5D || PROG == ZCOL_M5D_Y) {
    const bool from_minus = DAG ? !upper : upper;
#pragma unroll
    for (int s = 0; s < LS; s++) {
      const Cx<R> n = from_minus ? x[(s + LS - 1) % LS] : x[(s + 1) % LS];
      o[s] = cfma(from_minus ? c.l[s] : c.u[s], n, cmul(c.d[s], x[s]));
    }
    if (PROG == ZCOL_M5D_Y) {
      Cx<R> y[LS];
      ZIO<R>::template load<LS>(p.y, p.n5, k, q, y);
      const R zc = R(p.zc);
#pragma unroll
      for (int s = 0; s < LS; s++) { o[s].x = fma(zc, y[s].x, o[s].x); o[s].y = fma(zc, y[s].y, o[s].y); }
    }
  } else if (PROG == ZCOL_DIAG) {
    Cx<R> y[LS];
    ZIO<R>::template load<LS>(p.y, p.n5, k, q, y);
#pragma unroll
    for (int s = 0; s < LS; s++) o[s] = cfma(c.e[s], y[s], x[s]);
  } else {  // ZCOL_INV: first chirality runs the lee chain forward and the ueem column back
    const bool first = DAG ? !upper : upper;
    Cx<R> prev = {R(0), R(0)}, acc = {R(0), R(0)};
#pragma unroll
    for (int s = 0; s < LS; s++) {
      Cx<R> r = x[s];
      if (s < LS - 1) {
        if (first) {
          if (s > 0) r = cfma(Cx<R>{-c.lee[s - 1].x, -c.lee[s - 1].y}, prev, r);
        } else {
          acc = cfma(c.leem[s], r, acc);
        }
        prev = r;
      } else {
        if (first) r = cfma(Cx<R>{-c.lee[LS - 2].x, -c.lee[LS - 2].y}, prev, r);
        else { r.x -= acc.x; r.y -= acc.y; }
        r = cmul(c.dinv[LS - 1], r);
      }
      o[s] = r;
    }
    const Cx<R> last = o[LS - 1];
    Cx<R> next = last;
#pragma unroll
    for (int s = LS - 2; s >= 0; s--) {
      Cx<R> r = cmul(c.dinv[s], o[s]);
      if (!first) r = cfma(Cx<R>{-c.uee[s].x, -c.uee[s].y}, next, r);
      else r = cfma(Cx<R>{-c.ueem[s].x, -c.ueem[s].y}, last, r);
      o[s] = r;
      next = r;
    }
  }
  ZIO<R>::template store<LS>(p.out, p.n5, k, q, o);
}

template <class R, int LS>
void fill(ZCoef<R, LS>& c, const ZCoefsHost& h) {
  auto put = [](Cx<R>* dst, const std::vector<std::complex<double>>& v) {
    for (int s = 0; s < LS; s++) dst[s] = s < int(v.size()) ? Cx<R>{R(v[s].real()), R(v[s].imag())} : Cx<R>{R(0), R(0)};
  };
  put(c.d, h.d); put(c.u, h.u); put(c.l, h.l);
  put(c.lee, h.lee); put(c.leem, h.leem); put(c.uee, h.uee); put(c.ueem, h.ueem); put(c.dinv, h.dinv);
  put(c.e, h.e);
}

template <class R, int LS>
int zcol_ls(Op* op, int prog, int dag, const ZParams& p, const ZCoefsHost& h) {
  ZCoef<R, LS> c;
  fill<R, LS>(c, h);
  const unsigned blocks = unsigned((p.nq * 12 + 127) / 128);
  const int key = prog * 2 + (dag ? 1 : 0);
  switch (key) {
#define GB_Z(PROG)                                                                          \
  case PROG * 2: zcol_kernel<R, LS, false, PROG><<<blocks, 128, 0, op->stream>>>(p, c); break; \
  case PROG * 2 + 1: zcol_kernel<R, LS, true, PROG><<<blocks, 128, 0, op->stream>>>(p, c); break;
    GB_Z(ZCOL_M5D) GB_Z(ZCOL_M5D_Y) GB_Z(ZCOL_INV) GB_Z(ZCOL_DIAG)
#undef GB_Z
    default: set_error("zcol: unknown program"); return GB_ERR_BAD_ARG;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

template <class R>
int zcol_prec(Op* op, int prog, int dag, const ZParams& p, const ZCoefsHost& h) {
  switch (op->Ls) {
#define GB_ZL(L) \
  case L: return zcol_ls<R, L>(op, prog, dag, p, h);
    GB_ZL(2) GB_ZL(4) GB_ZL(6) GB_ZL(8) GB_ZL(10) GB_ZL(12) GB_ZL(14) GB_ZL(16) GB_ZL(20) GB_ZL(24) GB_ZL(32)
#undef GB_ZL
  }
  set_error("ZMobius: Ls = %d is not instantiated (2-16, 20, 24, 32)", op->Ls);
  return GB_ERR_UNSUPPORTED;
}

}  // namespace

bool zmobius_ls_supported(int Ls) {
  return (Ls >= 2 && Ls <= 16 && Ls % 2 == 0) || Ls == 20 || Ls == 24 || Ls == 32;
}

// prog: 0 M5D (zc * y when y is given), 2 INV, 3 DIAG; on one checkerboard half
int launch_zcol(Op* op, int prog, int dag, HalfView x, const HalfView* y, HalfView out, double zc, const ZCoefsHost& h) {
  if (x.prec != out.prec || (y && y->prec != x.prec)) { set_error("ZMobius: mixed field precisions"); return GB_ERR_BAD_ARG; }
  ZParams p;
  p.x = x.data;
  p.y = y ? y->data : nullptr;
  p.out = out.data;
  p.n5 = op->n5();
  p.nq = size_t(op->half4) * op->nrhs;
  p.zc = zc;
  const int pr = (prog == ZCOL_M5D && y) ? ZCOL_M5D_Y : prog;
  if (x.prec == GB_F64) return zcol_prec<double>(op, pr, dag, p, h);
  if (x.prec == GB_F32) return zcol_prec<float>(op, pr, dag, p, h);
  set_error("ZMobius: FP64 or FP32 fields");
  return GB_ERR_UNSUPPORTED;
}

}  // namespace gb
