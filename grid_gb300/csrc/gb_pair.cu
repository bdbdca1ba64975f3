// gb_pair.cu -- FP32 / FP16 (site-pair layout) versions of the 5D and linear-algebra
// kernels: one thread per pair of 5D sites (2q, 2q+1), 16-byte vector accesses only.
//
//   m5d_pair_kernel     Grid's M5D / M5Ddag (CayleyFermion5Dcache.h:41-115), with the
//                       optional fused "+ zc z" of SchurDiagMooeeOperator::Mpc
//   reduce_pair_kernel  norm2 / innerProduct / axpy_norm / the CG's r -= a Ap, |r|^2
//                       (Lattice_reduction.h:202-372, ConjugateGradient.h:160-172)
//   cg_p_pair_kernel    p = b p + r
//   cg_xp_pair_kernel   psi += a p ; p = b p + r (ConjugateGradient.h:174-183)
//   axpby_pair_kernel   z = a x + b y
// Ls is even, so both lanes of a pair sit in the same right-hand side for Moebius; for
// Wilson (Ls = 1) the two lanes are two right-hand sides, handled per lane.
#include <cuda_fp16.h>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {

struct PairShape {
  int L5, Ls, nrhs;
};

__device__ __forceinline__ float2 fma2s(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Per-rhs block sums of per-lane FP64 values.  A thread keeps one accumulator per lane; the
// grid-stride (in pairs) is a multiple of L5/2, so every thread's lanes stay on fixed right-
// hand sides.  The block sums go through shared memory as 2*blockDim "virtual threads"
// (element order), then rows of L5 are folded and each rhs sums its Ls slots.  out:
// [block][nrhs][NV].
template <int NV>
__device__ __forceinline__ void block_reduce_pairs(const double (&v0)[NV], const double (&v1)[NV], int L5, int Ls,
                                                   int nrhs, double* out) {
  extern __shared__ double red_smem[];
  const int t = threadIdx.x, B = blockDim.x, VB = 2 * B;
  if (nrhs == 1) {
    double w[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double x = v0[k] + v1[k];
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
  for (int k = 0; k < NV; k++) {
    red_smem[k * VB + 2 * t] = v0[k];
    red_smem[k * VB + 2 * t + 1] = v1[k];
  }
  __syncthreads();
  for (int stride = (VB / L5) >> 1; stride >= 1; stride >>= 1) {
    for (int vt = t; vt < L5 * stride; vt += B)
      for (int k = 0; k < NV; k++) red_smem[k * VB + vt] += red_smem[k * VB + vt + L5 * stride];
    __syncthreads();
  }
  if (t < nrhs) {
    for (int k = 0; k < NV; k++) {
      double sum = 0;
      for (int s = 0; s < Ls; s++) sum += red_smem[k * VB + t * Ls + s];
      out[(size_t(blockIdx.x) * nrhs + t) * NV + k] = sum;
    }
  }
}

// ---------------------------------------------------------------------------------------
// M5D on pairs.  Lane 0 = s (even), lane 1 = s+1.  For the upper (P+) components the
// s-1 neighbours are (previous pair lane 1, this pair lane 0); for the lower (P-) ones the
// s+1 neighbours are (this pair lane 1, next pair lane 0), with the wrap inside the
// right-hand side's block of Ls.  Dagger exchanges the roles of s-1 and s+1.
// ---------------------------------------------------------------------------------------
struct M5PairParams {
  const void* psi; const float2* psi_n;
  const void* phi; const float2* phi_n;
  void* chi; float2* chi_n;
  const void* z; const float2* z_n;
  float zc;
  size_t np;  // pairs per half field
  int L5, Ls, nrhs;
  double* norm_part;  // NORM: per-CTA sums of |chi|^2 as stored, [CTA][nrhs]
};

template <class R> struct Coef5p {
  R d[kMaxLs], u[kMaxLs], l[kMaxLs];
};

// NORM: a grid-stride loop (blockDim a multiple of L5/2) whose CTAs also sum |chi|^2 as
// stored per right-hand side, in a fixed order (block_reduce_pairs)
template <class T, bool DAG, bool ZTERM, bool SAME, bool NORM>
__global__ void __launch_bounds__(512) m5d_pair_kernel(const M5PairParams p, const Coef5p<float> c) {
  double nv0[1] = {0.0}, nv1[1] = {0.0};
  const size_t stride = NORM ? size_t(gridDim.x) * blockDim.x : p.np;
  for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; q < p.np; q += stride) {
    const int hl = p.L5 >> 1, hs = p.Ls >> 1;
    const int sp = int(q % hl);            // pair index within the 4D site
    const int s = (2 * sp) % p.Ls;         // even
    const int psb = sp % hs;               // pair index within the rhs block
    const size_t qb = q - psb;             // first pair of the rhs block
    const size_t qprev = psb == 0 ? qb + hs - 1 : q - 1;
    const size_t qnext = psb == hs - 1 ? qb : q + 1;
    Pair12 cur, prv, nxt, ph;
    PairIO<T>::load(p.psi, p.psi_n, p.np, q, cur);
    if (SAME) ph = cur; else PairIO<T>::load(p.phi, p.phi_n, p.np, q, ph);
    // neighbour chirality halves: the upper (P+) half from s-1 (non-dag) / s+1 (dag), the
    // lower (P-) half from the other side
    PairIO<T>::load6(p.psi, p.psi_n, p.np, DAG ? qnext : qprev, 0, DAG ? nxt : prv);
    PairIO<T>::load6(p.psi, p.psi_n, p.np, DAG ? qprev : qnext, 6, DAG ? prv : nxt);
    const float2 d = make_float2(c.d[s], c.d[s + 1]);
    const float2 cl = make_float2(c.l[s], c.l[s + 1]);  // coefficient of the s-1 neighbour
    const float2 cu = make_float2(c.u[s], c.u[s + 1]);  // coefficient of the s+1 neighbour
    Pair12 o;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      const bool upper = k < 6;
      // s-1 neighbours: (prev lane 1, cur lane 0); s+1 neighbours: (cur lane 1, next lane 0)
      const bool from_minus = DAG ? !upper : upper;
      float2 nr, ni;
      if (from_minus) {
        nr = make_float2(prv.re[k].y, cur.re[k].x);
        ni = make_float2(prv.im[k].y, cur.im[k].x);
      } else {
        nr = make_float2(cur.re[k].y, nxt.re[k].x);
        ni = make_float2(cur.im[k].y, nxt.im[k].x);
      }
      const float2 cc = from_minus ? cl : cu;
      o.re[k] = fma2s(cc, nr, __fmul2_rn(d, ph.re[k]));
      o.im[k] = fma2s(cc, ni, __fmul2_rn(d, ph.im[k]));
    }
    if (ZTERM) {
      Pair12 zz;
      PairIO<T>::load(p.z, p.z_n, p.np, q, zz);
      const float2 zc = make_float2(p.zc, p.zc);
#pragma unroll
      for (int k = 0; k < 12; k++) {
        o.re[k] = fma2s(zc, zz.re[k], o.re[k]);
        o.im[k] = fma2s(zc, zz.im[k], o.im[k]);
      }
    }
    if (NORM) {
      const float2 n2 = PairIO<T>::store_n2(p.chi, p.chi_n, p.np, q, o);
      nv0[0] += double(n2.x);
      nv1[0] += double(n2.y);
    } else {
      PairIO<T>::store(p.chi, p.chi_n, p.np, q, o);
    }
  }
  if (NORM) block_reduce_pairs<1>(nv0, nv1, p.L5, p.Ls, p.nrhs, p.norm_part);
}

// grid of the NORM variant: the reductions' grid (blockDim a multiple of L5/2, at most
// kRedBlocks CTAs).  Covering the field in one pass (3888 CTAs at 24^4 x 12) measured
// slower than the grid-stride loop over kRedBlocks CTAs: 102.7 against 95.4 us.
static int m5d_norm_grid(Op* op, size_t np, int* blocks, int* threads) {
  return red_grid_pair(op, np, blocks, threads);
}

template <class T, bool DAG, bool Z>
static void m5d_pair_go(Op* op, const M5PairParams& p, const Coef5p<float>& c, bool same, bool norm) {
  if constexpr (Z && !DAG) {  // the last kernel of Mpc: Mooee in - (the Dhop term)
    if (norm) {
      int g = 1, B = 256;
      m5d_norm_grid(op, p.np, &g, &B);
      const size_t smem = size_t(op->nrhs == 1 ? 32 : 2 * B) * sizeof(double);
      if (same) m5d_pair_kernel<T, DAG, Z, true, true><<<g, B, smem, op->stream>>>(p, c);
      else m5d_pair_kernel<T, DAG, Z, false, true><<<g, B, smem, op->stream>>>(p, c);
      return;
    }
  }
  const unsigned blocks = unsigned((p.np + 255) / 256);
  if (same) m5d_pair_kernel<T, DAG, Z, true, false><<<blocks, 256, 0, op->stream>>>(p, c);
  else m5d_pair_kernel<T, DAG, Z, false, false><<<blocks, 256, 0, op->stream>>>(p, c);
}

int launch_m5d_pair(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
                    const double* upper, int dag, size_t n5, const HalfView* z, double zc, int* norm_parts) {
  M5PairParams p;
  p.psi = psi.data; p.psi_n = reinterpret_cast<const float2*>(psi.norms);
  p.phi = phi.data; p.phi_n = reinterpret_cast<const float2*>(phi.norms);
  p.chi = chi.data; p.chi_n = reinterpret_cast<float2*>(chi.norms);
  p.z = z ? z->data : nullptr; p.z_n = z ? reinterpret_cast<const float2*>(z->norms) : nullptr;
  p.zc = float(zc);
  p.np = n5 >> 1;
  p.L5 = op->L5;
  p.Ls = op->Ls;
  p.nrhs = op->nrhs;
  // |chi|^2 per right-hand side on the way (Ls even: both lanes of a pair are one rhs)
  int g = 0, B = 0;
  const bool norm = norm_parts && z && !dag && m5d_norm_grid(op, p.np, &g, &B) == GB_OK;
  p.norm_part = norm ? op->d_partial : nullptr;
  if (norm_parts) *norm_parts = norm ? g : 0;
  Coef5p<float> c;
  for (int s = 0; s < op->Ls; s++) { c.d[s] = float(diag[s]); c.u[s] = float(upper[s]); c.l[s] = float(lower[s]); }
  const bool same = psi.data == phi.data;
  const bool zt = z != nullptr;
  if (psi.prec == GB_F32) {
    if (dag) { if (zt) m5d_pair_go<float, true, true>(op, p, c, same, norm); else m5d_pair_go<float, true, false>(op, p, c, same, norm); }
    else { if (zt) m5d_pair_go<float, false, true>(op, p, c, same, norm); else m5d_pair_go<float, false, false>(op, p, c, same, norm); }
  } else {
    if (dag) { if (zt) m5d_pair_go<__half, true, true>(op, p, c, same, norm); else m5d_pair_go<__half, true, false>(op, p, c, same, norm); }
    else { if (zt) m5d_pair_go<__half, false, true>(op, p, c, same, norm); else m5d_pair_go<__half, false, false>(op, p, c, same, norm); }
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Reductions on pairs (block sums: block_reduce_pairs above)
// ---------------------------------------------------------------------------------------

// KIND 0: |x|^2 ; 1: <x|y> ; 2: z = a x + y, |z|^2 ; 3: r(=y) -= a[rhs] mmp(=x), |r|^2
template <class T, int KIND>
__global__ void __launch_bounds__(512) reduce_pair_kernel(const PairShape sh, const void* x, const float2* xn,
                                                          const void* y, const float2* yn, void* z, float2* zn,
                                                          double a, const CGScalars* cg, size_t np, double* partial) {
  constexpr int NV = KIND == 1 ? 2 : 1;
  double v0[NV], v1[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) { v0[k] = 0.0; v1[k] = 0.0; }
  const size_t stride = size_t(gridDim.x) * blockDim.x;  // a multiple of L5/2 pairs
  size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float2 ar = make_float2(float(a), float(a));
  if (KIND == 3) {
    const int s5 = int((2 * q) % sh.L5);
    ar = make_float2(-float(cg[s5 / sh.Ls].a), -float(cg[(s5 + 1) / sh.Ls].a));
  }
  for (; q < np; q += stride) {
    Pair12 fx;
    PairIO<T>::load(x, xn, np, q, fx);
    if (KIND == 0) {
      float2 s = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 12; k++) s = fma2s(fx.re[k], fx.re[k], fma2s(fx.im[k], fx.im[k], s));
      v0[0] += double(s.x);
      v1[0] += double(s.y);
    } else if (KIND == 1) {
      Pair12 fy;
      PairIO<T>::load(y, yn, np, q, fy);
      float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 12; k++) {
        sr = fma2s(fx.re[k], fy.re[k], fma2s(fx.im[k], fy.im[k], sr));
        si = fma2s(fx.re[k], fy.im[k], fma2s(make_float2(-fx.im[k].x, -fx.im[k].y), fy.re[k], si));
      }
      v0[0] += double(sr.x); v1[0] += double(sr.y);
      v0[1] += double(si.x); v1[1] += double(si.y);
    } else {
      Pair12 fy;
      PairIO<T>::load(y, yn, np, q, fy);
      float2 s = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 12; k++) {
        fy.re[k] = fma2s(ar, fx.re[k], fy.re[k]);
        fy.im[k] = fma2s(ar, fx.im[k], fy.im[k]);
        s = fma2s(fy.re[k], fy.re[k], fma2s(fy.im[k], fy.im[k], s));
      }
      PairIO<T>::store(z, zn, np, q, fy);
      v0[0] += double(s.x);
      v1[0] += double(s.y);
    }
  }
  block_reduce_pairs<NV>(v0, v1, sh.L5, sh.Ls, sh.nrhs, partial);
}

// grid of the pair reductions: blockDim a multiple of L5/2 (about 256, at most 512 for
// L5 = kMaxL5), grid <= kRedBlocks
int red_grid_pair(Op* op, size_t np, int* blocks, int* threads) {
  const int h = op->L5 >> 1;
  int B = 256;
  if (op->nrhs > 1) {
    int m = 1;
    while (h * m * 2 <= 256) m *= 2;
    B = h * m;
    if (B > 512) { set_error("reduction: L5 = %d too large", op->L5); return GB_ERR_UNSUPPORTED; }
  }
  const size_t need = (np + B - 1) / B;
  int g = int(need < size_t(kRedBlocks) ? need : size_t(kRedBlocks));
  if (g < 1) g = 1;
  *blocks = g;
  *threads = B;
  return GB_OK;
}

template <class T, int KIND>
static int reduce_pair_t(Op* op, HalfView x, HalfView y, HalfView z, double a, size_t n5, double* partial) {
  int g, B;
  const size_t np = n5 >> 1;
  GB_TRY(red_grid_pair(op, np, &g, &B));
  PairShape sh{op->L5, op->Ls, op->nrhs};
  const int NV = KIND == 1 ? 2 : 1;
  const size_t smem = size_t(NV) * (op->nrhs == 1 ? 32 : 2 * B) * sizeof(double);
  reduce_pair_kernel<T, KIND><<<g, B, smem, op->stream>>>(
      sh, x.data, reinterpret_cast<const float2*>(x.norms), y.data, reinterpret_cast<const float2*>(y.norms), z.data,
      reinterpret_cast<float2*>(z.norms), a, op->d_cg, np, partial);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

int launch_reduce_pair(Op* op, int kind, HalfView x, HalfView y, HalfView z, double a, size_t n5, double* partial) {
  const bool h = x.prec == GB_F16;
  switch (kind) {
    case 0: return h ? reduce_pair_t<__half, 0>(op, x, y, z, a, n5, partial) : reduce_pair_t<float, 0>(op, x, y, z, a, n5, partial);
    case 1: return h ? reduce_pair_t<__half, 1>(op, x, y, z, a, n5, partial) : reduce_pair_t<float, 1>(op, x, y, z, a, n5, partial);
    case 2: return h ? reduce_pair_t<__half, 2>(op, x, y, z, a, n5, partial) : reduce_pair_t<float, 2>(op, x, y, z, a, n5, partial);
    case 3: return h ? reduce_pair_t<__half, 3>(op, x, y, z, a, n5, partial) : reduce_pair_t<float, 3>(op, x, y, z, a, n5, partial);
  }
  return GB_ERR_BAD_ARG;
}

// ---------------------------------------------------------------------------------------
// p = b[rhs] p + r  and  z = a x + b y on pairs
// ---------------------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) cg_p_pair_kernel(const PairShape sh, void* p, float2* pn, const void* r,
                                                        const float2* rn, const CGScalars* cg, size_t np) {
  const size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= np) return;
  const int s5 = int((2 * q) % sh.L5);
  const float2 b = make_float2(float(cg[s5 / sh.Ls].b), float(cg[(s5 + 1) / sh.Ls].b));
  Pair12 fp, fr;
  PairIO<T>::load(p, pn, np, q, fp);
  PairIO<T>::load(r, rn, np, q, fr);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    fp.re[k] = fma2s(b, fp.re[k], fr.re[k]);
    fp.im[k] = fma2s(b, fp.im[k], fr.im[k]);
  }
  PairIO<T>::store(p, pn, np, q, fp);
}

int launch_cg_p_pair(Op* op, HalfView p, HalfView r, size_t n5) {
  PairShape sh{op->L5, op->Ls, op->nrhs};
  const size_t np = n5 >> 1;
  const unsigned blocks = unsigned((np + 255) / 256);
  if (p.prec == GB_F32)
    cg_p_pair_kernel<float><<<blocks, 256, 0, op->stream>>>(sh, p.data, reinterpret_cast<float2*>(p.norms), r.data,
                                                            reinterpret_cast<const float2*>(r.norms), op->d_cg, np);
  else
    cg_p_pair_kernel<__half><<<blocks, 256, 0, op->stream>>>(sh, p.data, reinterpret_cast<float2*>(p.norms), r.data,
                                                             reinterpret_cast<const float2*>(r.norms), op->d_cg, np);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

// psi += a[rhs] p, then (PUPD) p = b[rhs] p + r: the CG's linear combination after the
// residual update, one pass over psi, p and r.  TS: storage of psi (FP32 for FP16 fields).
template <class T, class TS, bool PUPD>
__global__ void __launch_bounds__(256) cg_xp_pair_kernel(const PairShape sh, void* psi, float2* psin, void* p, float2* pn,
                                                         const void* r, const float2* rn, const CGScalars* cg,
                                                         size_t np) {
  const size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= np) return;
  const int s5 = int((2 * q) % sh.L5);
  const CGScalars& c0 = cg[s5 / sh.Ls];
  const CGScalars& c1 = cg[(s5 + 1) / sh.Ls];
  const float2 a = make_float2(float(c0.a), float(c1.a));
  Pair12 fp, fs;
  PairIO<T>::load(p, pn, np, q, fp);
  PairIO<TS>::load(psi, psin, np, q, fs);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    fs.re[k] = fma2s(a, fp.re[k], fs.re[k]);
    fs.im[k] = fma2s(a, fp.im[k], fs.im[k]);
  }
  PairIO<TS>::store(psi, psin, np, q, fs);
  if (PUPD) {
    const float2 b = make_float2(float(c0.b), float(c1.b));
    Pair12 fr;
    PairIO<T>::load(r, rn, np, q, fr);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      fp.re[k] = fma2s(b, fp.re[k], fr.re[k]);
      fp.im[k] = fma2s(b, fp.im[k], fr.im[k]);
    }
    PairIO<T>::store(p, pn, np, q, fp);
  }
}

template <class T, class TS>
static void cg_xp_pair_go(Op* op, HalfView psi, HalfView p, HalfView r, size_t np, bool pupd) {
  PairShape sh{op->L5, op->Ls, op->nrhs};
  const unsigned blocks = unsigned((np + 255) / 256);
  auto* psin = reinterpret_cast<float2*>(psi.norms);
  auto* pn = reinterpret_cast<float2*>(p.norms);
  auto* rn = reinterpret_cast<const float2*>(r.norms);
  if (pupd)
    cg_xp_pair_kernel<T, TS, true><<<blocks, 256, 0, op->stream>>>(sh, psi.data, psin, p.data, pn, r.data, rn, op->d_cg, np);
  else
    cg_xp_pair_kernel<T, TS, false><<<blocks, 256, 0, op->stream>>>(sh, psi.data, psin, p.data, pn, r.data, rn, op->d_cg, np);
}

int launch_cg_xp_pair(Op* op, HalfView psi, HalfView p, HalfView r, size_t n5, int update_p) {
  const size_t np = n5 >> 1;
  if (p.prec == GB_F32 && psi.prec == GB_F32) cg_xp_pair_go<float, float>(op, psi, p, r, np, update_p != 0);
  else if (p.prec == GB_F16 && psi.prec == GB_F32) cg_xp_pair_go<__half, float>(op, psi, p, r, np, update_p != 0);
  else if (p.prec == GB_F16 && psi.prec == GB_F16) cg_xp_pair_go<__half, __half>(op, psi, p, r, np, update_p != 0);
  else {
    set_error("CG update: solution precision %d with search-direction precision %d", psi.prec, p.prec);
    return GB_ERR_BAD_ARG;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

template <class T>
__global__ void __launch_bounds__(256) axpby_pair_kernel(void* z, float2* zn, float a, const void* x, const float2* xn,
                                                         float b, const void* y, const float2* yn, size_t np,
                                                         int use_y) {
  const size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= np) return;
  Pair12 fx, o;
  PairIO<T>::load(x, xn, np, q, fx);
  const float2 a2 = make_float2(a, a);
  if (use_y) {
    Pair12 fy;
    PairIO<T>::load(y, yn, np, q, fy);
    const float2 b2 = make_float2(b, b);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      o.re[k] = fma2s(a2, fx.re[k], __fmul2_rn(b2, fy.re[k]));
      o.im[k] = fma2s(a2, fx.im[k], __fmul2_rn(b2, fy.im[k]));
    }
  } else {
#pragma unroll
    for (int k = 0; k < 12; k++) { o.re[k] = __fmul2_rn(a2, fx.re[k]); o.im[k] = __fmul2_rn(a2, fx.im[k]); }
  }
  PairIO<T>::store(z, zn, np, q, o);
}

int launch_axpby_pair(Op* op, HalfView z, double a, HalfView x, double b, HalfView y, size_t n5, int use_y) {
  const size_t np = n5 >> 1;
  const unsigned blocks = unsigned((np + 255) / 256);
  if (z.prec == GB_F32)
    axpby_pair_kernel<float><<<blocks, 256, 0, op->stream>>>(z.data, reinterpret_cast<float2*>(z.norms), float(a), x.data,
                                                             reinterpret_cast<const float2*>(x.norms), float(b), y.data,
                                                             reinterpret_cast<const float2*>(y.norms), np, use_y);
  else
    axpby_pair_kernel<__half><<<blocks, 256, 0, op->stream>>>(z.data, reinterpret_cast<float2*>(z.norms), float(a),
                                                              x.data, reinterpret_cast<const float2*>(x.norms), float(b),
                                                              y.data, reinterpret_cast<const float2*>(y.norms), np, use_y);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
