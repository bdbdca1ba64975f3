// gb_dhop_stream.cu -- the FP32 Wilson hopping term (DhopEO, DhopOE, or both checkerboards
// in one launch) as t-streams: the structured form of Grid's
// WilsonKernels<Impl>::DhopKernel site loop
// (Grid/qcd/action/fermion/implementation/WilsonKernelsImplementation.h:113-163, 415-487)
// for the site-pair FP32 layout, the same eight legs as gb_dhop.cu's per-site gather
// kernel summed in another order.
//
// Why a stream.  Every output site needs its eight neighbours, and one 4D site's
// fifth-dimension row is L5 x 96 B (1.5 KB at Ls = 16).  Gathering them through L1 pulls
// each input site from L2 about six times per launch.  Here a CTA owns R whole x-rows
// (consecutive y, one z) of one checkerboard and walks t, so that
//  * the input rows with the CTA's own (y, z) at slice t come into shared memory once, by
//    TMA bulk copies (cp.async.bulk + mbarrier, bounded wait), double buffered one slice
//    ahead;
//  * the thread's own input site (same checkerboard index as its output site) serves
//    three legs: the -t leg of the output one slice later (its projection is kept in
//    registers across the step), the +t leg of the output one slice earlier (read from
//    the tile of the next slice, already resident in the other buffer), and one x leg;
//  * the other x leg and the y legs inside the CTA's rows read shared memory;
//  * only the y legs that leave the rows and the z legs read global memory (L2).
// A site's links arrive with its slice (one bulk copy per site into a padded stride).
//
// Work split: units (stream, t) with stream = (side, s-chunk, z, y-block); each persistent
// CTA takes a contiguous range of units and runs it as segments of consecutive t.  A
// segment with output slices [a, b] reads input slices a-1 .. b+1 (the first step only
// projects the -t leg, the last one only loads the slice the +t legs of b need).
//
// Fault handling: every wait on a copy is bounded.  When a wait anywhere in a CTA times
// out, the whole CTA stops after that step (the decision is a barrier vote, so no thread
// is left waiting at a barrier) and raises the error flag; the host then refuses the
// operator (Op::poisoned), since a copy may still be in flight when the CTA exits.
#include <atomic>

#include "gb_spin.cuh"

namespace gb {

struct StreamParams {
  const float4* in[2];    // per side: input checkerboard (the other parity), plane 0
  float4* out[2];         // per side: output checkerboard, plane 0
  const float* links[2];  // per side: doubled links of the output parity, [x_cb][144]
  int parity[2];          // per side: output parity
  int64_t np;             // 16-byte vectors per plane (= 4D sites of a checkerboard x hl)
  int Lxh, Ly, Lz, Lt;
  int hl;      // site pairs per 4D site (L5 / 2)
  int hc;      // site pairs per CTA (hl / nchunk)
  int nchunk;
  int R;       // x-rows per CTA (consecutive y at one z)
  int nyb;     // Ly / R
  int64_t W;   // units = sides x nchunk x Lz x nyb x Lt
  int* err;
};

struct StreamStep {
  int side, chunk, y0, z;
  int a, b;   // output slices of the segment
  int t;      // input slice of the step, a-1 .. b+1 (unwrapped)
  int valid;  // 0 past the end of the CTA's range
};

// Walks the steps of a unit range [u, hi): segments of consecutive t (one stream each),
// b - a + 3 steps per segment.  One division chain per segment, none per step.
struct StreamCursor {
  int64_t u, send, hi;  // first unit of the segment, its end, the range end
  StreamStep s;
};

__device__ __forceinline__ void cursor_segment(const StreamParams& p, StreamCursor& c) {
  c.s.valid = c.u < c.hi;
  if (!c.s.valid) return;
  const int64_t st = c.u / p.Lt;
  c.s.a = int(c.u - st * p.Lt);
  c.send = min(c.hi, (st + 1) * int64_t(p.Lt));
  c.s.b = int(c.send - 1 - st * p.Lt);
  const int q = int(st);
  const int qy = q / p.nyb;
  c.s.y0 = (q - qy * p.nyb) * p.R;
  const int qz = qy / p.Lz;
  c.s.z = qy - qz * p.Lz;
  c.s.side = qz / p.nchunk;
  c.s.chunk = qz - c.s.side * p.nchunk;
  c.s.t = c.s.a - 1;
}
__device__ __forceinline__ void cursor_next(const StreamParams& p, StreamCursor& c) {
  if (!c.s.valid) return;
  if (++c.s.t > c.s.b + 1) {
    c.u = c.send;
    cursor_segment(p, c);
  }
}

__device__ __forceinline__ int wrap(int v, int L) { return v < 0 ? v + L : (v >= L ? v - L : v); }

// Warp 0 issues the copies of step k into buffer k & 1: the CTA's rows of the input slice
// (12 planes, plane stride te in the tile) and, for an output slice, the links of its sites.
__device__ __forceinline__ void stream_issue(const StreamParams& p, const StreamStep& s, int k, float4* tiles,
                                             float* slinks, uint64_t* bar, int nsite, int te) {
  if (!s.valid) return;
  const int lane = threadIdx.x & 31;
  const int nl = blockDim.x < 32 ? int(blockDim.x) : 32;  // lanes of warp 0 (a CTA may be one partial warp)
  const int buf = k & 1;
  const int tt = wrap(s.t, p.Lt);
  const int64_t xcb0 = int64_t(p.Lxh) * (s.y0 + int64_t(p.Ly) * (s.z + int64_t(p.Lz) * tt));
  const bool full = s.t >= s.a && s.t <= s.b;
  const uint32_t bytes = 12u * uint32_t(nsite * p.hc) * 16u + (full ? uint32_t(nsite) * 576u : 0u);
  if (lane == 0) mbar_expect_tx(&bar[buf], bytes);
  __syncwarp(nl == 32 ? 0xffffffffu : (1u << nl) - 1u);
  const float4* src = (s.side ? p.in[1] : p.in[0]) + xcb0 * p.hl + s.chunk * p.hc;
  float4* dst = tiles + size_t(buf) * 12 * te;
  if (p.hc == p.hl) {  // the rows are contiguous in every plane
    for (int c = lane; c < 12; c += nl)
      bulk_g2s(dst + c * te, src + c * p.np, uint32_t(nsite * p.hc) * 16u, &bar[buf]);
  } else {
    for (int c = lane; c < 12 * nsite; c += nl) {
      const int pl = c / nsite, site = c - pl * nsite;
      bulk_g2s(dst + pl * te + site * p.hc, src + pl * p.np + int64_t(site) * p.hl, uint32_t(p.hc) * 16u, &bar[buf]);
    }
  }
  if (full) {
    const float* lsrc = (s.side ? p.links[1] : p.links[0]) + xcb0 * 144;
    float* ldst = slinks + size_t(buf) * nsite * kLinkStride;
    for (int c = lane; c < nsite; c += nl) bulk_g2s(ldst + c * kLinkStride, lsrc + int64_t(c) * 144, 576u, &bar[buf]);
  }
}

// one leg whose neighbour spinor is read through src (shared or global) with plane stride ps
template <int LEG, bool DAG, bool GLOBAL>
__device__ __forceinline__ void stream_leg(const float4* src, int64_t ps, const float2* U, Pair12& acc) {
  constexpr int MU = LEG & 3;
  constexpr int S = (LEG < 4 ? -1 : 1) * (DAG ? -1 : 1);
  PairIO<float>::Raw raw;
#pragma unroll
  for (int k = 0; k < 12; k++) raw.v[k] = GLOBAL ? __ldg(src + k * ps) : src[k * ps];
  Pair12 f;
  PairIO<float>::decode(raw, f);
  float2 hr[6], hi[6], ur[6], ui[6];
  project2<MU, S>(f, hr, hi);
  su3_mul2(U + LEG * 9, hr, hi, ur, ui);
  reconstruct2<MU, S, false>(acc, ur, ui, f2(1.f));
}

// an x leg with its sign at run time (s2 = (S, S)) and its link U (9 complex)
__device__ __forceinline__ void stream_leg_x(const Pair12& f, float2 s2, const float2* U, Pair12& acc) {
  float2 hr[6], hi[6], ur[6], ui[6];
  project2_x(f, s2, hr, hi);
  su3_mul2(U, hr, hi, ur, ui);
  reconstruct2_x(acc, ur, ui, s2);
}

// Thread (j, sp): 4D site j of the CTA's rows (row r = j / Lxh, x_cb offset xh), site
// pair sp of the CTA's chunk.  blockDim = R * Lxh * hc <= MAXT.
template <bool DAG, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) dhop_stream_kernel(const StreamParams p) {
  extern __shared__ __align__(128) unsigned char dyn_smem[];
  __shared__ __align__(8) uint64_t bar[2];
  // The steps, computed by thread 0 three ahead: ring[k % 4] is step k (read by every
  // thread in step k, by warp 0 when it issues the copies of step k in step k - 2), and
  // cursor is the walk's state after the newest entry.
  __shared__ StreamStep ring[4];
  __shared__ StreamCursor cursor;
  const int nsite = p.R * p.Lxh;
  constexpr int te = MAXT;  // plane stride of a tile (>= the CTA's threads), a constant so
                            // that the 12 planes of a site are immediate offsets
  float4* tiles = reinterpret_cast<float4*>(dyn_smem);           // 2 x [12][te]
  float* slinks = reinterpret_cast<float*>(tiles + 2 * 12 * te);  // 2 x [nsite][kLinkStride]

  const int tid = threadIdx.x;
  const int j = tid / p.hc, sp = tid - j * p.hc;
  const int r = j / p.Lxh, xh = j - r * p.Lxh;
  const int64_t G = gridDim.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    StreamCursor c;
    c.u = p.W * int64_t(blockIdx.x) / G;
    c.hi = p.W * (int64_t(blockIdx.x) + 1) / G;
    cursor_segment(p, c);
    for (int q = 0; q < 3; q++) {
      ring[q] = c.s;
      cursor_next(p, c);
    }
    cursor = c;
  }
  __syncthreads();
  if (tid < 32) {
    stream_issue(p, ring[0], 0, tiles, slinks, bar, nsite, te);
    stream_issue(p, ring[1], 1, tiles, slinks, bar, nsite, te);
  }

  constexpr int SF = DAG ? 1 : -1;  // +t leg (leg 3)
  constexpr int SB = -SF;           // -t leg (leg 7)
  const float2 one = f2(1.f);
  float2 hr[6], hv[6];  // P(-t) of the own input site, for the next slice's output
#pragma unroll
  for (int c = 0; c < 6; c++) { hr[c] = f2(0.f); hv[c] = f2(0.f); }

  for (int k = 0;; k++) {
    const StreamStep s = ring[k & 3];
    if (!s.valid) break;
    if (tid == 0) {  // step k + 3 into the entry of step k - 1
      StreamCursor c = cursor;
      ring[(k + 3) & 3] = c.s;
      cursor_next(p, c);
      cursor = c;
    }
    const int buf = k & 1;
    bool ok = mbar_wait_bounded(&bar[buf], uint32_t(k >> 1) & 1u);
    if (ok && s.t <= s.b) {
      const float4* tile = tiles + size_t(buf) * 12 * te;
      const int tt = wrap(s.t, p.Lt);
      const int y = s.y0 + r;
      const int64_t pofs = int64_t(s.chunk) * p.hc + sp;  // pair index within a 4D site
      // the own input site (x_cb offset xh, row y) of a tile, read where a leg needs it
      // rather than held in registers
      auto own = [&](const float4* tl, Pair12& f) {
        PairIO<float>::Raw raw;
#pragma unroll
        for (int c = 0; c < 12; c++) raw.v[c] = tl[c * te + j * p.hc + sp];
        PairIO<float>::decode(raw, f);
      };
      if (s.t >= s.a) {  // the output at slice tt: all eight legs and its store
        float2 ur[6], ui[6];
        const float2* U = reinterpret_cast<const float2*>(slinks + (size_t(buf) * nsite + j) * kLinkStride);
        // -t leg: the neighbour's projection was taken in the previous step
        su3_mul2(U + 7 * 9, hr, hv, ur, ui);
        Pair12 acc;
        reconstruct2<3, SB, true>(acc, ur, ui, one);
        // x legs: the own site is the +x neighbour on rows of parity 0, the -x one on rows
        // of parity 1; the other x neighbour is the next / previous site of the same row
        const int rowpar = ((s.side ? p.parity[1] : p.parity[0]) + y + s.z + tt) & 1;
        const float sown = (rowpar ? 1.f : -1.f) * (DAG ? -1.f : 1.f);
        {
          const int xo = rowpar ? (xh + 1 == p.Lxh ? 0 : xh + 1) : (xh == 0 ? p.Lxh - 1 : xh - 1);
          PairIO<float>::Raw raw;
#pragma unroll
          for (int c = 0; c < 12; c++) raw.v[c] = tile[c * te + (r * p.Lxh + xo) * p.hc + sp];
          Pair12 g;
          PairIO<float>::decode(raw, g);
          stream_leg_x(g, f2(-sown), U + (rowpar ? 0 : 4) * 9, acc);
        }
        // y legs: inside the CTA's rows from shared memory, else from global memory
        const float4* gin = (s.side ? p.in[1] : p.in[0]) + pofs;
        const int64_t zt = int64_t(p.Ly) * (s.z + int64_t(p.Lz) * tt);
        {
          const int yn = wrap(y + 1, p.Ly), rn = yn - s.y0;
          const bool inside = rn >= 0 && rn < p.R;
          const float4* src = inside ? tile + (rn * p.Lxh + xh) * p.hc + sp : gin + (xh + p.Lxh * (yn + zt)) * p.hl;
          stream_leg<1, DAG, false>(src, inside ? int64_t(te) : p.np, U, acc);
        }
        {
          const int yn = wrap(y - 1, p.Ly), rn = yn - s.y0;
          const bool inside = rn >= 0 && rn < p.R;
          const float4* src = inside ? tile + (rn * p.Lxh + xh) * p.hc + sp : gin + (xh + p.Lxh * (yn + zt)) * p.hl;
          stream_leg<5, DAG, false>(src, inside ? int64_t(te) : p.np, U, acc);
        }
        // z legs: global memory
        {
          const int64_t zp = int64_t(p.Ly) * (wrap(s.z + 1, p.Lz) + int64_t(p.Lz) * tt);
          stream_leg<2, DAG, true>(gin + (xh + p.Lxh * (y + zp)) * p.hl, p.np, U, acc);
          const int64_t zm = int64_t(p.Ly) * (wrap(s.z - 1, p.Lz) + int64_t(p.Lz) * tt);
          stream_leg<6, DAG, true>(gin + (xh + p.Lxh * (y + zm)) * p.hl, p.np, U, acc);
        }
        {  // the own site's x leg
          Pair12 f;
          own(tile, f);
          stream_leg_x(f, f2(sown), U + (rowpar ? 4 : 0) * 9, acc);
        }
        // +t leg: the own site of the next slice, whose tile is in the other buffer (the
        // last step of the segment loads it and computes nothing)
        ok = mbar_wait_bounded(&bar[buf ^ 1], uint32_t((k + 1) >> 1) & 1u);
        if (ok) {
          Pair12 f;
          own(tiles + size_t(buf ^ 1) * 12 * te, f);
          float2 ph[6], pi[6];
          project2<3, SF>(f, ph, pi);
          su3_mul2(U + 3 * 9, ph, pi, ur, ui);
          reconstruct2<3, SF, false>(acc, ur, ui, one);
          const int64_t xo = xh + int64_t(p.Lxh) * (y + zt);
          PairIO<float>::store((s.side ? p.out[1] : p.out[0]), nullptr, size_t(p.np), size_t(xo * p.hl + pofs), acc);
        }
      }
      if (ok && s.t < s.b) {  // P(-t) of the own site for the next slice's output
        Pair12 f;
        own(tile, f);
        project2<3, SB>(f, hr, hv);
      }
    }
    // buffer k & 1 is free; a timed-out wait anywhere in the CTA ends it (copies of steps
    // k, k+1 may still be in flight: the host refuses the operator)
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(p.err, 1);
      break;
    }
    if (tid < 32) stream_issue(p, ring[(k + 2) & 3], k + 2, tiles, slinks, bar, nsite, te);
  }
}

namespace {
template <bool DAG, int MAXT, int MINB> int stream_occupancy(size_t smem, int threads, int* per_sm) {
  static std::atomic<size_t> allowed{0};  // dynamic shared memory the kernel may take so far
  if (smem > allowed.load()) {
    GB_CHECK_CUDA(cudaFuncSetAttribute(dhop_stream_kernel<DAG, MAXT, MINB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    allowed.store(smem);
  }
  GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, dhop_stream_kernel<DAG, MAXT, MINB>, threads, smem));
  return GB_OK;
}
template <bool DAG, int MAXT, int MINB>
int stream_launch(Op* op, const StreamParams& p, size_t smem, int threads, int nsm, int* grid_out, int* per_sm_out) {
  int per_sm = 0;
  const int orc = stream_occupancy<DAG, MAXT, MINB>(smem, threads, &per_sm);
  if (orc != GB_OK) return orc;
  if (per_sm < 1) return GB_ERR_UNSUPPORTED;
  int64_t grid = int64_t(nsm) * per_sm;
  if (grid > p.W) grid = p.W;
  dhop_stream_kernel<DAG, MAXT, MINB><<<dim3(unsigned(grid)), dim3(unsigned(threads)), smem, op->stream>>>(p);
  GB_CHECK_CUDA(cudaGetLastError());
  *grid_out = int(grid);
  *per_sm_out = per_sm;
  return GB_OK;
}
}  // namespace

// Returns GB_ERR_UNSUPPORTED (nothing launched) when the shape has no stream layout; the
// caller then uses the per-site gather kernel.
int launch_dhop_stream(Op* op, const HalfView* in, const HalfView* out, const int* parity, int nside, int dag) {
  const int Lxh = op->dims[0] / 2, Ly = op->dims[1], Lz = op->dims[2], Lt = op->dims[3];
  const int hl = op->L5 / 2;
  if (op->prec != GB_F32 || op->recon12 || hl < 1 || Lt < 2) return GB_ERR_UNSUPPORTED;
  // site pairs per CTA: the fewest chunks of the fifth dimension that keep one x-row at
  // <= 128 threads
  int nchunk = 1;
  while (nchunk <= hl && (hl % nchunk != 0 || Lxh * (hl / nchunk) > 128)) nchunk++;
  if (nchunk > hl) return GB_ERR_UNSUPPORTED;
  const int hc = hl / nchunk;
  // rows per CTA: the largest divisor of Ly that keeps a CTA at <= 160 threads
  int R = 1;
  for (int c = Ly; c >= 1; c--)
    if (Ly % c == 0 && c * Lxh * hc <= 160) { R = c; break; }
  const int nsite = R * Lxh;
  const int threads = nsite * hc;
  const int maxt = threads <= 128 ? 128 : 160;  // the kernel instance, and its tile plane stride
  if (threads > 160) return GB_ERR_UNSUPPORTED;
  const size_t smem = size_t(2) * 12 * maxt * 16 + size_t(2) * nsite * kLinkStride * 4;
  if (smem > 200 * 1024) return GB_ERR_UNSUPPORTED;

  StreamParams p;
  for (int s = 0; s < 2; s++) {
    const int k = s < nside ? s : 0;
    p.in[s] = static_cast<const float4*>(in[k].data);
    p.out[s] = static_cast<float4*>(out[k].data);
    p.links[s] = static_cast<const float*>(op->links[parity[k]]);
    p.parity[s] = parity[k];
  }
  p.np = int64_t(op->half4) * hl;
  p.Lxh = Lxh; p.Ly = Ly; p.Lz = Lz; p.Lt = Lt;
  p.hl = hl; p.hc = hc; p.nchunk = nchunk; p.R = R; p.nyb = Ly / R;
  p.W = int64_t(nside) * nchunk * Lz * (Ly / R) * Lt;
  p.err = op->d_err;

  int nsm = 0;
  GB_CHECK_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, op->device));
  int grid = 0, per_sm = 0, rc;
  if (maxt == 128)
    rc = dag ? stream_launch<true, 128, 3>(op, p, smem, threads, nsm, &grid, &per_sm)
             : stream_launch<false, 128, 3>(op, p, smem, threads, nsm, &grid, &per_sm);
  else
    rc = dag ? stream_launch<true, 160, 2>(op, p, smem, threads, nsm, &grid, &per_sm)
             : stream_launch<false, 160, 2>(op, p, smem, threads, nsm, &grid, &per_sm);
  if (rc != GB_OK) return rc;
  const int rec[8] = {1, grid, per_sm, threads, int(smem), R, nchunk, 0};
  for (int q = 0; q < 8; q++) op->dhop_cfg[q] = rec[q];
  return GB_OK;
}

}  // namespace gb
