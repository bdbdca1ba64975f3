// gb_dhop.cu -- the Wilson hopping term on one checkerboard (DhopEO / DhopOE) for
// 4D Wilson (L5 = nrhs) and 5D domain-wall fields (L5 = Ls * nrhs).
//
// Computes, for every output site x of parity p and every fifth-dimension slot s5,
//   out(x,s5) = sum_mu (1 - g_mu) Ud_mu(x) in(x+mu,s5) + (1 + g_mu) Ud_{mu+4}(x) in(x-mu,s5)
// (dagger: projector signs swapped), the kernel of Grid's
// WilsonKernels<Impl>::GenericDhopSite / GenericDhopSiteDag
// (Grid/qcd/action/fermion/implementation/WilsonKernelsImplementation.h:113-163) with the
// half-spinor projections of Grid/qcd/spin/TwoSpinor.h:75-330.
//
// GB300 structure:
//  * one CTA covers k4 whole 4D sites x all L5 slots; thread = one 5D output site with
//    the slot index fastest, so a warp's neighbour reads are contiguous runs of
//    16-byte vectors in every plane;
//  * the CTA's 8 doubled links per 4D site arrive in shared memory by one TMA bulk copy
//    (cp.async.bulk + mbarrier, bounded wait) and serve all L5 slots of the site;
//  * neighbour indices come from a per-parity table (periodic wrap; the antiperiodic
//    time boundary is already folded into the stored links, as in Grid's DoubleStore).
#include <cuda_fp16.h>

#include <atomic>
#include <type_traits>

#include "gb_device.cuh"

namespace gb {

struct DhopParams {
  const void* in;
  const float* in_norms;
  void* out;
  float* out_norms;
  const void* links;
  const int* nbr;
  int64_t n4h;
  size_t n5;
  int L5;
  int L5a;  // slots that hold right-hand sides (below L5 when an odd count is padded)
  int L5c;  // slots per CTA (L5 split over gridDim.y when above 256)
  int k4;
  int* err;
  // second checkerboard of a full-lattice Dhop, taken by the CTAs with blockIdx.z == 1
  const void* in2;
  const float* in2_norms;
  void* out2;
  float* out2_norms;
  const void* links2;
  const int* nbr2;
  // 12-real links: geometry and boundary signs to rebuild the third rows
  int L[4];
  int sgn[4];     // the (real) boundary phase of each direction
  int parity;     // output checkerboard (parity2 for blockIdx.z == 1)
  int parity2;
  // MOOEE epilogue (FP32 / FP16: the last two steps of Mpc in one launch): out = M5D x5 - (the
  // Dhop) with the Mooee coefficients, |out|^2 per CTA (and per right-hand side when there
  // are several: dpart[CTA][nrhs])
  const void* x5;
  const float* x5_norms;  // FP16: the per-5D-site norms of x5
  double* dpart;
  int Ls, nrhs;
  float md[kMaxLs], ml[kMaxLs], mu[kMaxLs];
};

// the parameters of this CTA's checkerboard (both parities of a full Dhop run in one grid)
__device__ __forceinline__ DhopParams dhop_side(const DhopParams& p) {
  DhopParams q = p;
  if (blockIdx.z) {
    q.in = p.in2; q.in_norms = p.in2_norms; q.out = p.out2; q.out_norms = p.out2_norms;
    q.links = p.links2; q.nbr = p.nbr2; q.parity = p.parity2;
  }
  return q;
}

// 12-real links: the doubled link is k V with V in SU(3) and k = -1/2 times the boundary
// sign of that leg at that site, so row 2 = conj(row 0 x row 1) / k.  Expands one leg of
// one staged 4D site from rows {0,1} (12 reals) into the full 3x3 (18 reals).
template <class R>
__device__ __forceinline__ void expand_link12(const DhopParams& p, int64_t xcb, int leg, const R* src, R* dst) {
  const int Lxh = p.L[0] >> 1;
  const int64_t row = xcb / Lxh;
  const int xh = int(xcb - row * Lxh);
  const int y = int(row % p.L[1]);
  const int64_t zt = row / p.L[1];
  const int z = int(zt % p.L[2]), t = int(zt / p.L[2]);
  const int x = 2 * xh + ((p.parity + y + z + t) & 1);
  int cm, Lm, sg;  // the coordinate, extent and boundary sign of the leg's direction
  switch (leg & 3) {
    case 0: cm = x; Lm = p.L[0]; sg = p.sgn[0]; break;
    case 1: cm = y; Lm = p.L[1]; sg = p.sgn[1]; break;
    case 2: cm = z; Lm = p.L[2]; sg = p.sgn[2]; break;
    default: cm = t; Lm = p.L[3]; sg = p.sgn[3]; break;
  }
  const bool edge = leg < 4 ? (cm == Lm - 1) : (cm == 0);
  const R inv_k = R(-2) * R(edge ? sg : 1);
#pragma unroll
  for (int e = 0; e < 12; e++) dst[e] = src[e];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
    const R ar = src[2 * j1], ai = src[2 * j1 + 1], br = src[6 + 2 * j2], bi = src[6 + 2 * j2 + 1];
    const R cr = src[2 * j2], ci = src[2 * j2 + 1], dr = src[6 + 2 * j1], di = src[6 + 2 * j1 + 1];
    const R re = (ar * br - ai * bi) - (cr * dr - ci * di);
    const R im = (ar * bi + ai * br) - (cr * di + ci * dr);
    dst[12 + 2 * j] = inv_k * re;
    dst[12 + 2 * j + 1] = -inv_k * im;
  }
}

// ---- spin projection (1 + S gamma_MU) f -> two-spinor h, Grid's spProj{X,Y,Z,T}{p,m} ----
template <int MU, int S, class R>
__device__ __forceinline__ void project(const Spinor<R>& f, R (&hr)[6], R (&hi)[6]) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const R f0r = f.re[c], f0i = f.im[c], f1r = f.re[3 + c], f1i = f.im[3 + c];
    const R f2r = f.re[6 + c], f2i = f.im[6 + c], f3r = f.re[9 + c], f3i = f.im[9 + c];
    if (MU == 0) {  // h0 = f0 + S i f3, h1 = f1 + S i f2
      hr[c] = f0r - S * f3i; hi[c] = f0i + S * f3r;
      hr[3 + c] = f1r - S * f2i; hi[3 + c] = f1i + S * f2r;
    } else if (MU == 1) {  // h0 = f0 - S f3, h1 = f1 + S f2
      hr[c] = f0r - S * f3r; hi[c] = f0i - S * f3i;
      hr[3 + c] = f1r + S * f2r; hi[3 + c] = f1i + S * f2i;
    } else if (MU == 2) {  // h0 = f0 + S i f2, h1 = f1 - S i f3
      hr[c] = f0r - S * f2i; hi[c] = f0i + S * f2r;
      hr[3 + c] = f1r + S * f3i; hi[3 + c] = f1i - S * f3r;
    } else {  // h0 = f0 + S f2, h1 = f1 + S f3
      hr[c] = f0r + S * f2r; hi[c] = f0i + S * f2i;
      hr[3 + c] = f1r + S * f3r; hi[3 + c] = f1i + S * f3i;
    }
  }
}

// ---- reconstruction, Grid's accumRecon{X,Y,Z,T}{p,m}; FIRST assigns instead of adding ----
template <int MU, int S, bool FIRST, class R>
__device__ __forceinline__ void reconstruct(Spinor<R>& r, const R (&ur)[6], const R (&ui)[6]) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const R u0r = ur[c], u0i = ui[c], u1r = ur[3 + c], u1i = ui[3 + c];
    R t2r, t2i, t3r, t3i;
    if (MU == 0) {  // r2 += -S i u1, r3 += -S i u0
      t2r = S * u1i; t2i = -S * u1r; t3r = S * u0i; t3i = -S * u0r;
    } else if (MU == 1) {  // r2 += S u1, r3 -= S u0
      t2r = S * u1r; t2i = S * u1i; t3r = -S * u0r; t3i = -S * u0i;
    } else if (MU == 2) {  // r2 += -S i u0, r3 += S i u1
      t2r = S * u0i; t2i = -S * u0r; t3r = -S * u1i; t3i = S * u1r;
    } else {  // r2 += S u0, r3 += S u1
      t2r = S * u0r; t2i = S * u0i; t3r = S * u1r; t3i = S * u1i;
    }
    if (FIRST) {
      r.re[c] = u0r; r.im[c] = u0i; r.re[3 + c] = u1r; r.im[3 + c] = u1i;
      r.re[6 + c] = t2r; r.im[6 + c] = t2i; r.re[9 + c] = t3r; r.im[9 + c] = t3i;
    } else {
      r.re[c] += u0r; r.im[c] += u0i; r.re[3 + c] += u1r; r.im[3 + c] += u1i;
      r.re[6 + c] += t2r; r.im[6 + c] += t2i; r.re[9 + c] += t3r; r.im[9 + c] += t3i;
    }
  }
}

// u = U h for both spins of the two-spinor; U is 9 complex (row-major) in shared memory
template <class R>
__device__ __forceinline__ void su3_mul(const R* __restrict__ U, const R (&hr)[6], const R (&hi)[6], R (&ur)[6],
                                        R (&ui)[6]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const R u0r = U[(a * 3 + 0) * 2], u0i = U[(a * 3 + 0) * 2 + 1];
    const R u1r = U[(a * 3 + 1) * 2], u1i = U[(a * 3 + 1) * 2 + 1];
    const R u2r = U[(a * 3 + 2) * 2], u2i = U[(a * 3 + 2) * 2 + 1];
#pragma unroll
    for (int sp = 0; sp < 2; sp++) {
      const int o = sp * 3;
      R xr = u0r * hr[o];
      R xi = u0r * hi[o];
      xr = fma(-u0i, hi[o], xr);
      xi = fma(u0i, hr[o], xi);
      xr = fma(u1r, hr[o + 1], xr);
      xi = fma(u1r, hi[o + 1], xi);
      xr = fma(-u1i, hi[o + 1], xr);
      xi = fma(u1i, hr[o + 1], xi);
      xr = fma(u2r, hr[o + 2], xr);
      xi = fma(u2r, hi[o + 2], xi);
      xr = fma(-u2i, hi[o + 2], xr);
      xi = fma(u2i, hr[o + 2], xi);
      ur[o + a] = xr;
      ui[o + a] = xi;
    }
  }
}

// The same product in double-float arithmetic: each real output is one Dot2 of six
// products (the link's real and imaginary parts against the two-spinor's).
template <>
__device__ __forceinline__ void su3_mul<dfloat>(const dfloat* __restrict__ U, const dfloat (&hr)[6],
                                                const dfloat (&hi)[6], dfloat (&ur)[6], dfloat (&ui)[6]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
#pragma unroll
    for (int sp = 0; sp < 2; sp++) {
      const int o = sp * 3;
      DfDot xr, xi;
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const dfloat vr = U[(a * 3 + b) * 2], vi = U[(a * 3 + b) * 2 + 1];
        if (b == 0) {
          xr.first(vr, hr[o]);
          xi.first(vr, hi[o]);
        } else {
          xr.mac(vr, hr[o + b]);
          xi.mac(vr, hi[o + b]);
        }
        xr.mac(-vi, hi[o + b]);
        xi.mac(vi, hr[o + b]);
      }
      ur[o + a] = xr.result();
      ui[o + a] = xi.result();
    }
  }
}

template <class T, bool DAG, int LEG>
__device__ __forceinline__ void dhop_leg(const DhopParams& p, const int (&nb)[8], int s, const typename Arith<T>::type* U,
                                         Spinor<typename Arith<T>::type>& acc) {
  using R = typename Arith<T>::type;
  constexpr int MU = LEG & 3;
  constexpr int S = (LEG < 4 ? -1 : 1) * (DAG ? -1 : 1);
  Spinor<R> f;
  SpinorIO<T>::load(p.in, p.in_norms, p.n5, size_t(nb[LEG]) * p.L5 + s, f);
  R hr[6], hi[6], ur[6], ui[6];
  project<MU, S>(f, hr, hi);
  su3_mul<R>(U + LEG * 18, hr, hi, ur, ui);
  reconstruct<MU, S, LEG == 0>(acc, ur, ui);
}

// The double-float legs as one loop: unrolled over the eight legs, the double-float
// arithmetic (about 1 200 instructions per leg) no longer fits the instruction cache.  The
// projection (in double, a switch on the leg), the split, the SU(3) product and the
// reconstruction are one body; the reconstruction adds u to spins 0, 1 and a phase
// (+-1 or +-i) times u0 or u1 to spins 2, 3, as Grid's accumRecon{X,Y,Z,T}{p,m} do.
template <bool DAG>
__device__ __forceinline__ void dhop_df64_legs(const DhopParams& p, const int* __restrict__ nbrow, int s,
                                               const dfloat* U, Spinor<dfloat>& acc) {
  constexpr int SF = DAG ? 1 : -1;  // the sign S of the forward legs 0..3 (backward: -SF)
#pragma unroll
  for (int k = 0; k < 12; k++) {
    acc.re[k] = dfloat(0);
    acc.im[k] = dfloat(0);
  }
#pragma unroll 1
  for (int leg = 0; leg < 8; leg++) {
    Spinor<double> f;
    SpinorIO<double>::load(p.in, nullptr, p.n5, size_t(__ldg(nbrow + leg)) * p.L5 + s, f);
    double dr[6], di[6];
    switch (leg) {
      case 0: project<0, SF>(f, dr, di); break;
      case 1: project<1, SF>(f, dr, di); break;
      case 2: project<2, SF>(f, dr, di); break;
      case 3: project<3, SF>(f, dr, di); break;
      case 4: project<0, -SF>(f, dr, di); break;
      case 5: project<1, -SF>(f, dr, di); break;
      case 6: project<2, -SF>(f, dr, di); break;
      default: project<3, -SF>(f, dr, di); break;
    }
    dfloat hr[6], hi[6], ur[6], ui[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      hr[k] = df::split(dr[k]);
      hi[k] = df::split(di[k]);
    }
    su3_mul<dfloat>(U + leg * 18, hr, hi, ur, ui);
    const int mu = leg & 3;
    const int S = leg < 4 ? SF : -SF;
    const bool imag = (mu & 1) == 0;               // MU = 0, 2: the phases are +-i
    const bool neg2 = imag ? S > 0 : S < 0;        // spin 2: -S i (MU 0, 2) or S (MU 1, 3)
    const bool neg3 = mu < 2 ? S > 0 : S < 0;      // spin 3: -S i, -S, S i, S for MU 0..3
#pragma unroll
    for (int c = 0; c < 3; c++) {
      acc.re[c] += ur[c];
      acc.im[c] += ui[c];
      acc.re[3 + c] += ur[3 + c];
      acc.im[3 + c] += ui[3 + c];
      // spin 2 takes u1 for MU 0, 1 and u0 for MU 2, 3; spin 3 the other one
      const dfloat v2r = mu < 2 ? ur[3 + c] : ur[c], v2i = mu < 2 ? ui[3 + c] : ui[c];
      const dfloat v3r = mu < 2 ? ur[c] : ur[3 + c], v3i = mu < 2 ? ui[c] : ui[3 + c];
      // (sign) x v, or (sign) x i v = (sign) x (-v_im, v_re)
      const dfloat a2 = imag ? -v2i : v2r, b2 = imag ? v2r : v2i;
      const dfloat a3 = imag ? -v3i : v3r, b3 = imag ? v3r : v3i;
      acc.re[6 + c] += neg2 ? -a2 : a2;
      acc.im[6 + c] += neg2 ? -b2 : b2;
      acc.re[9 + c] += neg3 ? -a3 : a3;
      acc.im[9 + c] += neg3 ? -b3 : b3;
    }
  }
}

template <class T, bool DAG, bool RECON>
__device__ __forceinline__ void dhop_body(const DhopParams& p0) {
  const DhopParams p = dhop_side(p0);
  using R = typename Arith<T>::type;
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  R* sU = reinterpret_cast<R*>(dyn_smem);  // k4 * 144
  R* sraw = sU + size_t(p.k4) * 144;        // RECON: k4 * 96 (rows 0, 1 of every leg)
  __shared__ __align__(8) uint64_t bar;

  const int t = threadIdx.x;
  const int64_t x0 = int64_t(blockIdx.x) * p.k4;
  const int nsite = int(min(int64_t(p.k4), p.n4h - x0));
  if (t == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (t == 0) {
    const uint32_t per_site = RECON ? 96u : 144u;
    const uint32_t bytes = uint32_t(nsite) * per_site * uint32_t(sizeof(R));
    mbar_expect_tx(&bar, bytes);
    bulk_g2s(RECON ? sraw : sU, static_cast<const R*>(p.links) + x0 * per_site, bytes, &bar);
  }
  // threads cover the right-hand-side slots only; the zero padding slot of an odd
  // right-hand-side count is written as zero by the site's slot-0 thread
  const int j = t / p.L5c;
  const int s = int(blockIdx.y) * p.L5c + (t - j * p.L5c);
  const bool active = j < nsite && s < p.L5a;
  int nb[8];
  if (active) {
    const int4* q = reinterpret_cast<const int4*>(p.nbr + (x0 + j) * 8);
    const int4 a = __ldg(q), b = __ldg(q + 1);
    nb[0] = a.x; nb[1] = a.y; nb[2] = a.z; nb[3] = a.w;
    nb[4] = b.x; nb[5] = b.y; nb[6] = b.z; nb[7] = b.w;
  }
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok) atomicExch(p.err, 1);
  if constexpr (std::is_same<T, DF64>::value) {
    // the staged doubles become (hi, lo) pairs in place (the same 8 bytes)
    static_assert(!RECON && sizeof(R) == sizeof(double), "double-float links: 18 reals, 8 bytes each");
    if (ok)
      for (int e = t; e < nsite * 144; e += blockDim.x) sU[e] = df::split(reinterpret_cast<const double*>(sU)[e]);
    __syncthreads();
  }
  if constexpr (RECON) {
    if (ok)
      for (int e = t; e < nsite * 8; e += blockDim.x)
        expand_link12<R>(p, x0 + (e >> 3), e & 7, sraw + (e >> 3) * 96 + (e & 7) * 12, sU + (e >> 3) * 144 + (e & 7) * 18);
    __syncthreads();
  }
  if (!ok || !active) return;
  const R* U = sU + j * 144;
  Spinor<R> acc;
  if constexpr (std::is_same<T, DF64>::value) {
    dhop_df64_legs<DAG>(p, p.nbr + (x0 + j) * 8, s, U, acc);
  } else {
    dhop_leg<T, DAG, 0>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 1>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 2>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 3>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 4>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 5>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 6>(p, nb, s, U, acc);
    dhop_leg<T, DAG, 7>(p, nb, s, U, acc);
  }
  SpinorIO<T>::store(p.out, p.out_norms, p.n5, size_t(x0 + j) * p.L5 + s, acc);
  if (s == 0 && p.L5a < p.L5) {
    Spinor<R> zero;
#pragma unroll
    for (int k = 0; k < 12; k++) { zero.re[k] = R(0); zero.im[k] = R(0); }
    for (int z = p.L5a; z < p.L5; z++) SpinorIO<T>::store(p.out, p.out_norms, p.n5, size_t(x0 + j) * p.L5 + z, zero);
  }
}

template <class T, bool DAG, bool RECON>
__global__ void __launch_bounds__(256) dhop_kernel(const DhopParams p0) {
  dhop_body<T, DAG, RECON>(p0);
}

// double-float arithmetic: two CTAs of 256 threads per SM (128 registers at most) keep
// enough warps to cover the dependent float chains
template <bool DAG>
__global__ void __launch_bounds__(256, 2) dhop_df64_kernel(const DhopParams p0) {
  dhop_body<DF64, DAG, false>(p0);
}

// 4D sites per CTA: L5 * k4 threads, about 256, at most 40 KB of staged links, and a
// multiple of 32 threads where possible
static int pick_k4(int L5, size_t link_bytes_per_site) {
  if (L5 >= 128) return 1;
  int k4 = 256 / L5;
  const int kmax = int((40 * 1024) / link_bytes_per_site);
  if (k4 > kmax) k4 = kmax;
  if (k4 < 1) k4 = 1;
  int w = k4;
  while (w > 1 && (L5 * w) % 32 != 0) w--;
  return (L5 * w) % 32 == 0 ? w : k4;
}

template <class T, bool DAG, bool RECON> static int launch_dhop_t(Op* op, const DhopParams& p) {
  using R = typename Arith<T>::type;
  const int threads = p.L5c * p.k4;
  const int64_t blocks = (p.n4h + p.k4 - 1) / p.k4;
  const unsigned ychunks = unsigned((p.L5a + p.L5c - 1) / p.L5c);
  const size_t smem = size_t(p.k4) * (RECON ? 240 : 144) * sizeof(R);
  void (*kernel)(const DhopParams);
  if constexpr (std::is_same<T, DF64>::value) kernel = dhop_df64_kernel<DAG>;
  else kernel = dhop_kernel<T, DAG, RECON>;
  static std::atomic<bool> configured{false};
  if (!configured.load()) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    configured.store(true);
  }
  kernel<<<dim3(unsigned(blocks), ychunks, p.in2 ? 2u : 1u), dim3(threads), smem, op->stream>>>(p);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

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

// legs in visiting order: +mu and -mu back to back, x and y first (the +-x and +-y
// neighbour rows of a CTA's x-rows overlap, so the second visit can hit in L1)
__device__ constexpr int kLegOrder[8] = {0, 4, 1, 5, 2, 6, 3, 7};

// neighbour spinors of GB_DHOP_PF legs ahead are in flight while a leg computes
#ifndef GB_DHOP_PF
#define GB_DHOP_PF 0
#endif

template <class T, bool DAG, int PF, int I>
__device__ __forceinline__ void dhop_pair_step(const DhopParams& p, const int (&nb)[8], int sp, size_t np, int hl,
                                               const float2* U, typename PairIO<T>::Raw (&buf)[PF + 1], Pair12& acc) {
  constexpr int LEG = kLegOrder[I];
  constexpr int MU = LEG & 3;
  constexpr int S = (LEG < 4 ? -1 : 1) * (DAG ? -1 : 1);
  if constexpr (I + PF < 8)
    PairIO<T>::load_raw(p.in, reinterpret_cast<const float2*>(p.in_norms), np, size_t(nb[kLegOrder[I + PF]]) * hl + sp,
                        buf[(I + PF) % (PF + 1)]);
  // the storage factor (FP16 site norms) is linear through projection and link: it is
  // applied by the reconstruction's fused multiply-adds
  Pair12 f;
  PairIO<T>::decode_unscaled(buf[I % (PF + 1)], f);
  float2 hr[6], hi[6], ur[6], ui[6];
  project2<MU, S>(f, hr, hi);
  su3_mul2(U + LEG * 9, hr, hi, ur, ui);
  reconstruct2<MU, S, I == 0>(acc, ur, ui, PairIO<T>::scale(buf[I % (PF + 1)]));
  if constexpr (I + 1 < 8) dhop_pair_step<T, DAG, PF, I + 1>(p, nb, sp, np, hl, U, buf, acc);
}

// resident CTAs of 128 threads per SM the register allocation targets
#ifndef GB_DHOP_MINB
#define GB_DHOP_MINB 4
#endif
// threads per CTA the site-pair kernel aims at
#ifndef GB_DHOP_THREADS
#define GB_DHOP_THREADS 128
#endif

// MOOEE epilogue of one thread: out(q) = M5D(x5)(q) - acc with the Mooee coefficients
// (the same fused multiply-adds as m5d_pair_kernel with its z term, so the result equals the
// separate Dhop and Mooee launches bit for bit); returns |out(q)|^2 per lane.  MODE 1: one
// right-hand side; 2: several, the s -+ 1 neighbours wrapping inside each rhs block.
// (p: the kernel's __grid_constant__ parameter, so the coefficient arrays are indexed in
// the parameter bank, not copied to local memory)
template <int MODE>
__device__ __forceinline__ float2 dhop_mooee_epilogue(const DhopParams& p, size_t np, size_t q, int sp,
                                                      const Pair12& acc) {
  const int hs = p.Ls >> 1;
  const int psb = MODE == 1 ? sp : sp % hs;  // pair index within the rhs block
  const int s = 2 * psb;                     // the pair's slots s, s + 1 in its rhs
  const size_t qb = q - psb;                 // the block's first pair
  const size_t qprev = psb == 0 ? qb + hs - 1 : q - 1;
  const size_t qnext = psb == hs - 1 ? qb : q + 1;
  const float4* x = static_cast<const float4*>(p.x5);
  float4* o = static_cast<float4*>(p.out);
  const float2 d = make_float2(p.md[s], p.md[s + 1]);
  const float2 cl = make_float2(p.ml[s], p.ml[s + 1]);
  const float2 cu = make_float2(p.mu[s], p.mu[s + 1]);
  const float2 zc = make_float2(-1.f, -1.f);
  float2 n2 = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const float4 cur = __ldg(x + size_t(k) * np + q);
    const float4 nb = __ldg(x + size_t(k) * np + (k < 6 ? qprev : qnext));
    float2 nr, ni, cc;
    if (k < 6) {  // P+ components from s - 1: (previous pair's lane 1, this pair's lane 0)
      nr = make_float2(nb.y, cur.x); ni = make_float2(nb.w, cur.z); cc = cl;
    } else {      // P- components from s + 1: (this pair's lane 1, next pair's lane 0)
      nr = make_float2(cur.y, nb.x); ni = make_float2(cur.w, nb.z); cc = cu;
    }
    float2 ore = __ffma2_rn(cc, nr, __fmul2_rn(d, make_float2(cur.x, cur.y)));
    float2 oim = __ffma2_rn(cc, ni, __fmul2_rn(d, make_float2(cur.z, cur.w)));
    ore = __ffma2_rn(zc, acc.re[k], ore);
    oim = __ffma2_rn(zc, acc.im[k], oim);
    o[size_t(k) * np + q] = make_float4(ore.x, ore.y, oim.x, oim.y);
    n2 = __ffma2_rn(ore, ore, __ffma2_rn(oim, oim, n2));
  }
  return n2;
}

// The same for FP16 storage: x5 is decoded with its site norms (as the Mooee kernel decodes
// it), out = M5D(x5) - acc is formed in place of acc two components at a time and stored
// through the FP16 encoder; returns |out|^2 as stored.  Unlike the separate launches, the
// Dhop result is not rounded to FP16 before the subtraction.
template <int MODE>
__device__ __forceinline__ float2 dhop_mooee_epilogue_half(const DhopParams& p, size_t np, size_t q, int sp,
                                                           Pair12& acc) {
  const int hs = p.Ls >> 1;
  const int psb = MODE == 1 ? sp : sp % hs;
  const int s = 2 * psb;
  const size_t qb = q - psb;
  const size_t qprev = psb == 0 ? qb + hs - 1 : q - 1;
  const size_t qnext = psb == hs - 1 ? qb : q + 1;
  const uint4* x = static_cast<const uint4*>(p.x5);
  const float2* xn = reinterpret_cast<const float2*>(p.x5_norms);
  const float2 ncur = __ldg(xn + q), nprv = __ldg(xn + qprev), nnxt = __ldg(xn + qnext);
  const float2 d = make_float2(p.md[s], p.md[s + 1]);
  const float2 cl = make_float2(p.ml[s], p.ml[s + 1]);
  const float2 cu = make_float2(p.mu[s], p.mu[s + 1]);
  const float2 zc = make_float2(-1.f, -1.f);
#pragma unroll
  for (int g = 0; g < 6; g++) {
    const uint4 vc = __ldg(x + size_t(g) * np + q);
    const uint4 vb = __ldg(x + size_t(g) * np + (g < 3 ? qprev : qnext));
    const __half2* hc = reinterpret_cast<const __half2*>(&vc);
    const __half2* hb = reinterpret_cast<const __half2*>(&vb);
    const float2 nb = g < 3 ? nprv : nnxt;
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int k = 2 * g + e;
      const float2 cre = __fmul2_rn(__half22float2(hc[2 * e]), ncur), cim = __fmul2_rn(__half22float2(hc[2 * e + 1]), ncur);
      const float2 bre = __fmul2_rn(__half22float2(hb[2 * e]), nb), bim = __fmul2_rn(__half22float2(hb[2 * e + 1]), nb);
      float2 nr, ni, cc;
      if (k < 6) {  // P+ from s - 1: (previous pair's lane 1, this pair's lane 0)
        nr = make_float2(bre.y, cre.x); ni = make_float2(bim.y, cim.x); cc = cl;
      } else {      // P- from s + 1: (this pair's lane 1, next pair's lane 0)
        nr = make_float2(cre.y, bre.x); ni = make_float2(cim.y, bim.x); cc = cu;
      }
      const float2 ore = __ffma2_rn(cc, nr, __fmul2_rn(d, cre));
      const float2 oim = __ffma2_rn(cc, ni, __fmul2_rn(d, cim));
      acc.re[k] = __ffma2_rn(zc, acc.re[k], ore);
      acc.im[k] = __ffma2_rn(zc, acc.im[k], oim);
    }
  }
  return PairIO<__half>::store_n2(p.out, reinterpret_cast<float2*>(p.out_norms), np, q, acc);
}

// CTA = k4 4D sites x hc pair threads.  Thread (j, sp) computes the 5D sites
// (2 sp, 2 sp + 1) of 4D site x0 + j: eight legs, +mu and -mu back to back.  MOOEE (1: one
// right-hand side, 2: several, with CTAs over 8-pair chunks that each touch at most two
// right-hand sides): the result goes through dhop_mooee_epilogue, and the CTA writes the
// sums of |out|^2, nrhs of them for MOOEE 2 (zero for the right-hand sides it does not touch).
template <class T, bool DAG, bool RECON, int MOOEE = 0>
__global__ void __launch_bounds__(GB_DHOP_THREADS, GB_DHOP_MINB) dhop_pair_kernel(const __grid_constant__ DhopParams p0) {
  const DhopParams p = dhop_side(p0);
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  float* slink = reinterpret_cast<float*>(dyn_smem);  // k4 * kLinkStride floats
  float* sraw = slink + size_t(p.k4) * kLinkStride;   // RECON: k4 * 96 floats (rows 0, 1)
  __shared__ __align__(8) uint64_t bar;

  const int t = threadIdx.x;
  const int hl = p.L5 >> 1;            // pairs per 4D site
  const int hc = p.L5c >> 1;           // pairs per 4D site in this CTA
  const int64_t x0 = int64_t(blockIdx.x) * p.k4;
  const int nsite = int(min(int64_t(p.k4), p.n4h - x0));
  if (t == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (t == 0) {
    if (RECON) {
      mbar_expect_tx(&bar, uint32_t(nsite) * 384u);
      bulk_g2s(sraw, static_cast<const float*>(p.links) + x0 * 96, uint32_t(nsite) * 384u, &bar);
    } else {
      mbar_expect_tx(&bar, uint32_t(nsite) * 576u);
      const float* src = static_cast<const float*>(p.links) + x0 * 144;
      for (int k = 0; k < nsite; k++) bulk_g2s(slink + k * kLinkStride, src + k * 144, 576u, &bar);
    }
  }
  const int j = t / hc;
  const int sp = int(blockIdx.y) * hc + (t - j * hc);
  const bool active = j < nsite && sp < hl;
  int nb[8];
  if (active) {
    const int4* q = reinterpret_cast<const int4*>(p.nbr + (x0 + j) * 8);
    const int4 a = __ldg(q), b = __ldg(q + 1);
    nb[0] = a.x; nb[1] = a.y; nb[2] = a.z; nb[3] = a.w;
    nb[4] = b.x; nb[5] = b.y; nb[6] = b.z; nb[7] = b.w;
  }
  // every thread waits for the links before it leaves.  If the bounded wait gives up,
  // the copy may still be in flight when the CTA exits: the error flag is raised and the
  // host then refuses further Dhops on this operator (Op::poisoned)
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok) atomicExch(p.err, 1);
  if (RECON) {
    if (ok)
      for (int e = t; e < nsite * 8; e += blockDim.x)
        expand_link12<float>(p, x0 + (e >> 3), e & 7, sraw + (e >> 3) * 96 + (e & 7) * 12,
                             slink + (e >> 3) * kLinkStride + (e & 7) * 18);
    __syncthreads();
  }
  if (!ok) return;  // every thread of the CTA sees the same wait result
  if (!MOOEE && !active) return;
  const size_t np = p.n5 >> 1;
  double nsum = 0.0;  // MOOEE: this thread's |out|^2
  if (active) {
    const float2* U = reinterpret_cast<const float2*>(slink + j * kLinkStride);
    Pair12 acc;
    typename PairIO<T>::Raw buf[GB_DHOP_PF + 1];
#pragma unroll
    for (int i = 0; i < GB_DHOP_PF; i++)
      PairIO<T>::load_raw(p.in, reinterpret_cast<const float2*>(p.in_norms), np, size_t(nb[kLegOrder[i]]) * hl + sp,
                          buf[i]);
    dhop_pair_step<T, DAG, GB_DHOP_PF, 0>(p, nb, sp, np, hl, U, buf, acc);
    if constexpr (MOOEE != 0) {
      float2 n2;
      if constexpr (sizeof(T) == 4) n2 = dhop_mooee_epilogue<MOOEE>(p0, np, size_t(x0 + j) * hl + sp, sp, acc);
      else n2 = dhop_mooee_epilogue_half<MOOEE>(p0, np, size_t(x0 + j) * hl + sp, sp, acc);
      nsum = double(n2.x) + double(n2.y);
    } else {
      PairIO<T>::store(p.out, reinterpret_cast<float2*>(p.out_norms), np, size_t(x0 + j) * hl + sp, acc);
    }
  }
  if constexpr (MOOEE == 1) {  // fixed-order CTA sum: warp shuffles, then the warps in order
    __shared__ double wsum[GB_DHOP_THREADS / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) nsum += __shfl_down_sync(0xffffffffu, nsum, off);
    if ((t & 31) == 0) wsum[t >> 5] = nsum;
    __syncthreads();
    if (t == 0) {
      double s = 0.0;
      for (int w = 0; w < int((blockDim.x + 31) >> 5); w++) s += wsum[w];
      p.dpart[size_t(blockIdx.y) * gridDim.x + blockIdx.x] = s;
    }
  }
  if constexpr (MOOEE == 2) {  // the chunk's first rhs and the next: two fixed-order sums
    const int rlo = (2 * int(blockIdx.y) * hc) / p.Ls;
    double lo = 0.0, hi = 0.0;
    if (active) {
      if ((2 * sp) / p.Ls == rlo) lo = nsum; else hi = nsum;
    }
    __shared__ double wlo[GB_DHOP_THREADS / 32], whi[GB_DHOP_THREADS / 32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      lo += __shfl_down_sync(0xffffffffu, lo, off);
      hi += __shfl_down_sync(0xffffffffu, hi, off);
    }
    if ((t & 31) == 0) { wlo[t >> 5] = lo; whi[t >> 5] = hi; }
    __syncthreads();
    if (t < p.nrhs) {
      double s = 0.0;
      if (t == rlo || t == rlo + 1)
        for (int w = 0; w < int((blockDim.x + 31) >> 5); w++) s += t == rlo ? wlo[w] : whi[w];
      p.dpart[(size_t(blockIdx.y) * gridDim.x + blockIdx.x) * p.nrhs + t] = s;
    }
  }
}

// CTA = k4 4D sites x (L5c/2) pair threads, about 128 threads
static int pick_k4_pair(int hc) {
  if (hc >= GB_DHOP_THREADS / 2) return 1;
  int k4 = GB_DHOP_THREADS / hc;
  while (k4 > 1 && (hc * k4) % 32 != 0) k4--;
  if ((hc * k4) % 32 != 0) k4 = GB_DHOP_THREADS / hc;
  if (k4 > 64) k4 = 64;  // shared memory: 64 x 592 B
  return k4 < 1 ? 1 : k4;
}

// the site-pair kernel's launch shape for a fifth dimension of L5 slots: pairs per CTA
// chunk (L5c / 2), 4D sites per CTA, CTAs along the sites and the L5 chunks
struct PairShapeDhop {
  int L5c, k4, threads;
  int64_t blocks;
  unsigned ychunks;
};
static PairShapeDhop dhop_pair_shape(int L5, int64_t n4h) {
  PairShapeDhop s;
  s.L5c = L5 > 256 ? 256 : L5;  // even
  // A fifth dimension of several 8-pair groups (multi-RHS operators) is split into CTAs of
  // 8 pairs: a warp then covers 4 sites x 8 pairs, whole 128-byte lines of every plane,
  // where 48 slots (3 x 128 B per site) in one CTA would straddle lines
  if (L5 > 16 && L5 % 16 == 0) s.L5c = 16;
  s.k4 = pick_k4_pair(s.L5c / 2);
  s.threads = (s.L5c / 2) * s.k4;
  s.blocks = (n4h + s.k4 - 1) / s.k4;
  s.ychunks = unsigned((L5 + s.L5c - 1) / s.L5c);
  return s;
}

size_t dhop_pair_ctas(const Op* op) {
  const PairShapeDhop s = dhop_pair_shape(op->L5, op->half4);
  return size_t(s.blocks) * s.ychunks;
}

template <class T, bool DAG, bool RECON, int MOOEE = 0> static int launch_dhop_pair_t(Op* op, DhopParams p) {
  const PairShapeDhop s = dhop_pair_shape(p.L5, p.n4h);
  p.L5c = s.L5c;
  p.k4 = s.k4;
  const size_t smem = size_t(p.k4) * (kLinkStride + (RECON ? 96 : 0)) * sizeof(float);
  static std::atomic<bool> configured{false};
  if (!configured.load()) {  // up to 64 sites x 976 B with 12-real staging
    GB_CHECK_CUDA(cudaFuncSetAttribute(dhop_pair_kernel<T, DAG, RECON, MOOEE>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
    configured.store(true);
  }
  dhop_pair_kernel<T, DAG, RECON, MOOEE>
      <<<dim3(unsigned(s.blocks), s.ychunks, p.in2 ? 2u : 1u), dim3(s.threads), smem, op->stream>>>(p);
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

static void fill_dhop_params(Op* op, HalfView in, HalfView out, int out_parity, const HalfView* in2,
                             const HalfView* out2, DhopParams& p);

static int launch_dhop_sides(Op* op, HalfView in, HalfView out, int out_parity, const HalfView* in2,
                             const HalfView* out2, int dag) {
  if (in.prec != op->prec || out.prec != op->prec || (in2 && (in2->prec != op->prec || out2->prec != op->prec))) {
    set_error("Dhop: field precision differs from the operator's");
    return GB_ERR_BAD_ARG;
  }
  if (op->L5 > kMaxL5) {
    set_error("Dhop: L5 = %d exceeds %d", op->L5, kMaxL5);
    return GB_ERR_UNSUPPORTED;
  }
  if (op->poisoned) {
    set_error("Dhop: an earlier device wait of this operator timed out; its results are untrusted, recreate it");
    return GB_ERR_TIMEOUT;
  }
  DhopParams p;
  fill_dhop_params(op, in, out, out_parity, in2, out2, p);
  if (op->df64)  // FP64 fields, double-float arithmetic (18-real links only)
    return dag ? launch_dhop_t<DF64, true, false>(op, p) : launch_dhop_t<DF64, false, false>(op, p);
  const int key = (op->prec << 2) | (dag ? 2 : 0) | (op->recon12 ? 1 : 0);
  switch (key) {
#define GB_DHOP_CASE(PREC, LAUNCH, T)                                        \
  case (PREC << 2) | 0: return LAUNCH<T, false, false>(op, p);              \
  case (PREC << 2) | 1: return LAUNCH<T, false, true>(op, p);               \
  case (PREC << 2) | 2: return LAUNCH<T, true, false>(op, p);               \
  case (PREC << 2) | 3: return LAUNCH<T, true, true>(op, p);
    GB_DHOP_CASE(GB_F64, launch_dhop_t, double)
    GB_DHOP_CASE(GB_F32, launch_dhop_pair_t, float)
    GB_DHOP_CASE(GB_F16, launch_dhop_pair_t, __half)
#undef GB_DHOP_CASE
  }
  return GB_ERR_BAD_ARG;
}

static void fill_dhop_params(Op* op, HalfView in, HalfView out, int out_parity, const HalfView* in2,
                             const HalfView* out2, DhopParams& p) {
  p.in = in.data;
  p.in_norms = in.norms;
  p.out = out.data;
  p.out_norms = out.norms;
  p.links = op->links[out_parity];
  p.nbr = op->nbr[out_parity];
  p.in2 = in2 ? in2->data : nullptr;
  p.in2_norms = in2 ? in2->norms : nullptr;
  p.out2 = out2 ? out2->data : nullptr;
  p.out2_norms = out2 ? out2->norms : nullptr;
  p.links2 = in2 ? op->links[1 - out_parity] : nullptr;
  p.nbr2 = in2 ? op->nbr[1 - out_parity] : nullptr;
  p.n4h = op->half4;
  p.n5 = op->n5();
  p.L5 = op->L5;
  // FP64 works per 5D site and skips the padding slot; the site-pair kernels keep it
  p.L5a = op->prec == GB_F64 ? op->Ls * op->nrhs_user : op->L5;
  p.L5c = p.L5a > 256 ? 256 : p.L5a;
  p.k4 = pick_k4(p.L5c, (op->prec == GB_F64 ? 1152 : 576) * (op->recon12 ? 5 : 3) / 3);  // links + 12-real staging
  p.err = op->d_err;
  for (int k = 0; k < 4; k++) {
    p.L[k] = op->dims[k];
    p.sgn[k] = op->phases[k].real() < 0 ? -1 : 1;
  }
  p.parity = out_parity;
  p.parity2 = 1 - out_parity;
  p.x5 = nullptr;
  p.x5_norms = nullptr;
  p.dpart = nullptr;
  p.Ls = op->Ls;
  p.nrhs = op->nrhs;
}

int launch_dhop_mooee(Op* op, HalfView in, HalfView x5, HalfView out, int out_parity, const double* lower,
                      const double* diag, const double* upper, int* parts) {
  *parts = 0;
  if ((op->prec != GB_F32 && op->prec != GB_F16) || in.prec != op->prec || x5.prec != op->prec ||
      out.prec != op->prec || op->Ls > kMaxLs || op->poisoned)
    return GB_OK;  // not this launch's case: the caller runs the Dhop and Mooee separately
  const PairShapeDhop s = dhop_pair_shape(op->L5, op->half4);
  int mode = 0;
  if (op->nrhs == 1 && op->L5 == op->Ls) {
    mode = 1;
  } else if (op->nrhs > 1 && s.L5c == 16 && s.ychunks > 1) {  // CTAs over 8-pair chunks
    mode = 2;
    for (unsigned c = 0; c < s.ychunks; c++)  // each chunk's 16 slots in at most two rhs blocks
      if ((16 * int(c) + 15) / op->Ls - (16 * int(c)) / op->Ls > 1) mode = 0;
  }
  if (mode == 0 || s.threads % 32 != 0 || size_t(s.blocks) * s.ychunks * op->nrhs > op->partial_doubles) return GB_OK;
  DhopParams p;
  fill_dhop_params(op, in, out, out_parity, nullptr, nullptr, p);
  p.x5 = x5.data;
  p.x5_norms = x5.norms;
  p.dpart = op->d_partial;
  for (int k = 0; k < op->Ls; k++) {
    p.md[k] = float(diag[k]);
    p.ml[k] = float(lower[k]);
    p.mu[k] = float(upper[k]);
  }
  int rc;
  if (op->prec == GB_F32) {
    if (mode == 1)
      rc = op->recon12 ? launch_dhop_pair_t<float, false, true, 1>(op, p) : launch_dhop_pair_t<float, false, false, 1>(op, p);
    else
      rc = op->recon12 ? launch_dhop_pair_t<float, false, true, 2>(op, p) : launch_dhop_pair_t<float, false, false, 2>(op, p);
  } else {
    if (mode == 1)
      rc = op->recon12 ? launch_dhop_pair_t<__half, false, true, 1>(op, p) : launch_dhop_pair_t<__half, false, false, 1>(op, p);
    else
      rc = op->recon12 ? launch_dhop_pair_t<__half, false, true, 2>(op, p) : launch_dhop_pair_t<__half, false, false, 2>(op, p);
  }
  if (rc != GB_OK) return rc;
  *parts = int(size_t(s.blocks) * s.ychunks);
  return GB_OK;
}

int launch_dhop(Op* op, HalfView in, HalfView out, int out_parity, int dag) {
  return launch_dhop_sides(op, in, out, out_parity, nullptr, nullptr, dag);
}

int launch_dhop_full(Op* op, HalfView in_odd, HalfView out_even, HalfView in_even, HalfView out_odd, int dag) {
  return launch_dhop_sides(op, in_odd, out_even, 0, &in_even, &out_odd, dag);
}

// =======================================================================================
// Force term: WilsonFermion5D::DerivInternal (WilsonFermion5DImplementation.h:212-246) with
// WilsonImpl::InsertForce5D (WilsonImpl.h:193-238).  For each output site x and direction
// mu:  mat[x][mu]_ab = sum_s sum_spin Bt(x,s)_{spin,a} conj(A(x,s)_{spin,b}),
// Bt = (1 -+ gamma_mu) U~_mu(x) B(x + mu) -- the forward leg of Dhop (dag: of Dhop^dag).
// One thread per (x, mu) walks the L5 slots (all right-hand sides are summed), so the sum
// has a fixed order; the result is FP64 in the canonical gauge layout.
// =======================================================================================
struct DerivParams {
  const void* A;
  const float* An;
  const void* B;
  const float* Bn;
  const void* links;
  const int* nbr;
  double2* mat;
  size_t n5;
  int64_t n4h;
  int L5;
  int half_out;   // 1: mat indexed by x_cb, 0: by the lexicographic site
  DhopParams geo;  // L, sgn, parity (for the 12-real link rebuild and the site index)
};

template <class T, bool DAG, int MU, bool RECON>
__device__ __forceinline__ void deriv_site(const DerivParams& q, int64_t x) {
  using R = typename Arith<T>::type;
  constexpr int S = DAG ? 1 : -1;
  R Ul[18];
  if (RECON) {
    R raw[12];
    const R* src = static_cast<const R*>(q.links) + (size_t(x) * 8 + MU) * 12;
#pragma unroll
    for (int e = 0; e < 12; e++) raw[e] = src[e];
    expand_link12<R>(q.geo, x, MU, raw, Ul);
  } else {
    const R* src = static_cast<const R*>(q.links) + (size_t(x) * 8 + MU) * 18;
#pragma unroll
    for (int e = 0; e < 18; e++) Ul[e] = src[e];
  }
  const int nb = q.nbr[size_t(x) * 8 + MU];
  double fr[9], fi[9];
#pragma unroll
  for (int e = 0; e < 9; e++) { fr[e] = 0; fi[e] = 0; }
  for (int s = 0; s < q.L5; s++) {
    Spinor<R> b, a, bt;
    SpinorIO<T>::load(q.B, q.Bn, q.n5, size_t(nb) * q.L5 + s, b);
    SpinorIO<T>::load(q.A, q.An, q.n5, size_t(x) * q.L5 + s, a);
    R hr[6], hi[6], ur[6], ui[6];
    project<MU, S>(b, hr, hi);
    su3_mul<R>(Ul, hr, hi, ur, ui);
    reconstruct<MU, S, true>(bt, ur, ui);
#pragma unroll
    for (int ca = 0; ca < 3; ca++)
#pragma unroll
      for (int cb = 0; cb < 3; cb++)
#pragma unroll
        for (int sp = 0; sp < 4; sp++) {
          const double br = bt.re[sp * 3 + ca], bi = bt.im[sp * 3 + ca];
          const double ar = a.re[sp * 3 + cb], ai = a.im[sp * 3 + cb];
          fr[ca * 3 + cb] += br * ar + bi * ai;  // b conj(a)
          fi[ca * 3 + cb] += bi * ar - br * ai;
        }
  }
  int64_t idx = x;
  if (!q.half_out) {  // lexicographic site of x_cb in the output parity
    const int Lxh = q.geo.L[0] >> 1;
    const int64_t row = x / Lxh;
    const int xh = int(x - row * Lxh);
    const int y = int(row % q.geo.L[1]);
    const int64_t zt = row / q.geo.L[1];
    const int z = int(zt % q.geo.L[2]), t = int(zt / q.geo.L[2]);
    idx = row * q.geo.L[0] + 2 * xh + ((q.geo.parity + y + z + t) & 1);
  }
  double2* o = q.mat + (size_t(idx) * 4 + MU) * 9;
#pragma unroll
  for (int e = 0; e < 9; e++) o[e] = make_double2(fr[e], fi[e]);
}

template <class T, bool DAG, bool RECON>
__global__ void __launch_bounds__(128) deriv_kernel(const DerivParams q) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= q.n4h * 4) return;
  const int64_t x = t >> 2;
  switch (int(t & 3)) {
    case 0: deriv_site<T, DAG, 0, RECON>(q, x); break;
    case 1: deriv_site<T, DAG, 1, RECON>(q, x); break;
    case 2: deriv_site<T, DAG, 2, RECON>(q, x); break;
    default: deriv_site<T, DAG, 3, RECON>(q, x); break;
  }
}

int launch_deriv(Op* op, HalfView A, HalfView B, int out_parity, int dag, double* mat, int half_out) {
  if (A.prec != op->prec || B.prec != op->prec) { set_error("DhopDeriv: field precision differs from the operator's"); return GB_ERR_BAD_ARG; }
  if (op->prec == GB_F16) { set_error("DhopDeriv: FP64 or FP32 operators"); return GB_ERR_UNSUPPORTED; }
  DerivParams q;
  q.A = A.data; q.An = A.norms; q.B = B.data; q.Bn = B.norms;
  q.links = op->links[out_parity];
  q.nbr = op->nbr[out_parity];
  q.mat = reinterpret_cast<double2*>(mat);
  q.n5 = op->n5();
  q.n4h = op->half4;
  q.L5 = op->L5;
  q.half_out = half_out;
  for (int k = 0; k < 4; k++) {
    q.geo.L[k] = op->dims[k];
    q.geo.sgn[k] = op->phases[k].real() < 0 ? -1 : 1;
  }
  q.geo.parity = out_parity;
  const unsigned blocks = unsigned((op->half4 * 4 + 127) / 128);
  const int key = (op->prec == GB_F64 ? 4 : 0) | (dag ? 2 : 0) | (op->recon12 ? 1 : 0);
  switch (key) {
    case 0: deriv_kernel<float, false, false><<<blocks, 128, 0, op->stream>>>(q); break;
    case 1: deriv_kernel<float, false, true><<<blocks, 128, 0, op->stream>>>(q); break;
    case 2: deriv_kernel<float, true, false><<<blocks, 128, 0, op->stream>>>(q); break;
    case 3: deriv_kernel<float, true, true><<<blocks, 128, 0, op->stream>>>(q); break;
    case 4: deriv_kernel<double, false, false><<<blocks, 128, 0, op->stream>>>(q); break;
    case 5: deriv_kernel<double, false, true><<<blocks, 128, 0, op->stream>>>(q); break;
    case 6: deriv_kernel<double, true, false><<<blocks, 128, 0, op->stream>>>(q); break;
    default: deriv_kernel<double, true, true><<<blocks, 128, 0, op->stream>>>(q); break;
  }
  GB_CHECK_CUDA(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb
