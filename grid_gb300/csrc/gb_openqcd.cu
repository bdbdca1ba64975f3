// gb_openqcd.cu -- openQCD gauge-configuration files read into the canonical FP64 gauge
// layout (Grid/parallelIO/OpenQcdIO.h:43-170; Grid reads the format only).
//
// File: a header of four int32 (Nt, Nx, Ny, Nz) and one double (the plaquette in
// openQCD's normalisation, Nc times Grid's), then, for every odd site in openQCD's order
// (t slowest, then x, y, z; index (t Lx Ly Lz + x Ly Lz + y Lz + z) / 2), the eight SU(3)
// links T+, T-, X+, X-, Y+, Y- , Z+, Z- as 3x3 complex little-endian doubles: U_mu(x) and
// U_mu(x - mu) of that odd site.  So the link U_mu(x) of an odd site is its own mu+ entry
// and that of an even site is the mu- entry of its odd neighbour x + mu.  A read checks
// the plaquette of the field against the header's to 2e-15, as Grid does.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <fstream>
#include <vector>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {
namespace {

struct OqGeo {
  int L[4];  // Grid order x, y, z, t
  int64_t vol;
};

// one thread per (site, mu): U[site][mu] from the double-stored odd-site records
__global__ void __launch_bounds__(256) openqcd_unpack_kernel(const double2* rec, double2* U, OqGeo g) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= g.vol * 4) return;
  const int64_t site = t >> 2;
  const int mu = int(t & 3);
  int c[4];
  {
    int64_t r = site;
    for (int k = 0; k < 4; k++) { c[k] = int(r % g.L[k]); r /= g.L[k]; }
  }
  const bool odd = ((c[0] + c[1] + c[2] + c[3]) & 1) != 0;
  const int mu_o = (mu + 1) & 3;  // openQCD direction: t, x, y, z = 0, 1, 2, 3
  int slot = 2 * mu_o;
  if (!odd) {  // the backward link of the odd neighbour x + mu
    c[mu] = (c[mu] + 1) % g.L[mu];
    slot += 1;
  }
  const int Lx = g.L[0], Ly = g.L[1], Lz = g.L[2];
  const int64_t io = (int64_t(c[3]) * Lx * Ly * Lz + int64_t(c[0]) * Ly * Lz + int64_t(c[1]) * Lz + c[2]) >> 1;
  const double2* src = rec + (size_t(io) * 8 + slot) * 9;
  double2* dst = U + (size_t(site) * 4 + mu) * 9;
#pragma unroll
  for (int e = 0; e < 9; e++) dst[e] = src[e];
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gb_openqcd_read_header(const char* path, int dims[4], double* plaquette) {
  if (!path || !dims || !plaquette) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  std::ifstream f(path, std::ios::binary);
  if (!f) { set_error("openQCD: cannot open %s", path); return GB_ERR_IO; }
  unsigned char h[24];
  f.read(reinterpret_cast<char*>(h), 24);
  if (!f) { set_error("openQCD: %s is shorter than its header", path); return GB_ERR_IO; }
  int32_t n[4];
  double plaq;
  std::memcpy(n, h, 16);
  std::memcpy(&plaq, h + 16, 8);
  // Nt Nx Ny Nz -> Grid order x y z t
  dims[0] = n[1]; dims[1] = n[2]; dims[2] = n[3]; dims[3] = n[0];
  for (int k = 0; k < 4; k++)
    if (dims[k] < 2 || dims[k] > 1024 || (dims[k] & 1)) {
      set_error("openQCD: implausible extent %d in %s (byte order?)", dims[k], path);
      return GB_ERR_IO;
    }
  *plaquette = plaq / 3.0;  // openQCD normalises by 6, Grid by 18
  return GB_OK;
}

int gb_openqcd_read(const char* path, double* U, int on_device, int dims[4], double* plaquette,
                    double* plaquette_computed, int check) {
  if (!path || !U || !dims || !plaquette || !plaquette_computed) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_TRY(gb_openqcd_read_header(path, dims, plaquette));
  OqGeo g;
  g.vol = 1;
  for (int k = 0; k < 4; k++) { g.L[k] = dims[k]; g.vol *= dims[k]; }
  const size_t rec_bytes = size_t(g.vol / 2) * 8 * 9 * 16;
  const size_t out_bytes = size_t(g.vol) * 4 * 9 * 16;
  std::ifstream f(path, std::ios::binary);
  f.seekg(0, std::ios::end);
  if (int64_t(f.tellg()) < int64_t(24 + rec_bytes)) { set_error("openQCD: %s holds fewer than %zu bytes of links", path, rec_bytes); return GB_ERR_IO; }
  void* host = nullptr;
  GB_CHECK_CUDA(cudaMallocHost(&host, rec_bytes));
  struct HostFree { void* p; ~HostFree() { cudaFreeHost(p); } } hf{host};
  f.seekg(24);
  f.read(static_cast<char*>(host), std::streamsize(rec_bytes));
  if (!f) { set_error("openQCD: short read of %s", path); return GB_ERR_IO; }
  struct DevFree { void* a = nullptr; void* b = nullptr; ~DevFree() { cudaFree(a); cudaFree(b); } } df;
  double2* drec = nullptr;
  GB_CHECK_CUDA(cudaMalloc(&drec, rec_bytes));
  df.a = drec;
  double* dU = U;
  if (!on_device) {
    GB_CHECK_CUDA(cudaMalloc(&dU, out_bytes));
    df.b = dU;
  }
  GB_CHECK_CUDA(cudaMemcpy(drec, host, rec_bytes, cudaMemcpyHostToDevice));
  openqcd_unpack_kernel<<<unsigned((g.vol * 4 + 255) / 256), 256>>>(drec, reinterpret_cast<double2*>(dU), g);
  GB_CHECK_CUDA(cudaGetLastError());
  double trace = 0;
  GB_TRY(gauge_stats_device(dims, dU, nullptr, plaquette_computed, &trace));
  if (!on_device) GB_CHECK_CUDA(cudaMemcpy(U, dU, out_bytes, cudaMemcpyDeviceToHost));
  if (check && !(std::fabs(*plaquette_computed - *plaquette) < 2e-15)) {
    set_error("openQCD: plaquette %.17g of the field differs from the header's %.17g", *plaquette_computed, *plaquette);
    return GB_ERR_IO;
  }
  return GB_OK;
}

}  // extern "C"
