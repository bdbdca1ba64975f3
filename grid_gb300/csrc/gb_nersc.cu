// gb_nersc.cu -- NERSC gauge-configuration files (Grid/parallelIO/NerscIO.h) read into and
// written from the canonical FP64 gauge layout, with the byte work on the GPU.
//
// File: an ASCII header "BEGIN_HEADER ... KEY = value ... END_HEADER" followed by the
// payload, site-lexicographic (x fastest), per site the Nd = 4 links, per link either the
// first two rows (DATATYPE 4D_SU3_GAUGE; the third row is rebuilt as the conjugated cross
// product of the first two, MetaData.h:204-218) or all three (4D_SU3_GAUGE_3x3), complex
// numbers as (re, im) in IEEE32/IEEE64, big- or little-endian (FLOATING_POINT).
// CHECKSUM is the 32-bit wrapping sum of the payload's 32-bit words in host byte order
// (BinaryIO.h:109-137); PLAQUETTE and LINK_TRACE are Grid's avgPlaquette / linkTrace
// (WilsonLoops.h:88-126,203-218) and a read checks all three as Grid does
// (NerscIO.h:196-215).
//
// The payload moves to the device once; one kernel per link byte-swaps, widens,
// rebuilds the third row, accumulates the checksum and writes the canonical field, and a
// second kernel computes the plaquette and link trace.  Writing runs the same steps
// backwards.
#include <cuda_runtime.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {
namespace {

struct Geo4 {
  int L[4];
  int64_t vol;
};

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }
__device__ __forceinline__ uint64_t bswap64(uint64_t x) {
  return (uint64_t(bswap32(uint32_t(x))) << 32) | uint64_t(bswap32(uint32_t(x >> 32)));
}

// one element of the payload to double, with the checksum words of its host-order form
template <int BITS>
__device__ __forceinline__ double load_el(const unsigned char* raw, size_t e, bool swap, uint32_t& csum) {
  if (BITS == 32) {
    uint32_t w = reinterpret_cast<const uint32_t*>(raw)[e];
    if (swap) w = bswap32(w);
    csum += w;
    return double(__uint_as_float(w));
  } else {
    uint64_t w = reinterpret_cast<const uint64_t*>(raw)[e];
    if (swap) w = bswap64(w);
    csum += uint32_t(w) + uint32_t(w >> 32);
    return __longlong_as_double(static_cast<long long>(w));
  }
}

__device__ __forceinline__ void warp_csum_add(uint32_t v, uint32_t* out) {
  for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, v);  // addition mod 2^32: the order does not matter
}

// payload -> canonical U[site][mu][3][3] (complex double); one thread per link
template <int BITS>
__global__ void __launch_bounds__(256) nersc_unpack_kernel(const unsigned char* raw, double2* U, int64_t nlinks,
                                                           int rows, int swap, uint32_t* csum) {
  const int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t cs = 0;
  if (l < nlinks) {
    double2 m[3][3];
    const size_t e0 = size_t(l) * rows * 6;
    for (int i = 0; i < rows; i++)
      for (int j = 0; j < 3; j++) {
        const double re = load_el<BITS>(raw, e0 + (i * 3 + j) * 2, swap, cs);
        const double im = load_el<BITS>(raw, e0 + (i * 3 + j) * 2 + 1, swap, cs);
        m[i][j] = make_double2(re, im);
      }
    if (rows == 2) {  // row 2 = conj(row 0 x row 1)
      for (int j = 0; j < 3; j++) {
        const double2 a = m[0][(j + 1) % 3], b = m[1][(j + 2) % 3], c = m[0][(j + 2) % 3], d = m[1][(j + 1) % 3];
        const double re = (a.x * b.x - a.y * b.y) - (c.x * d.x - c.y * d.y);
        const double im = (a.x * b.y + a.y * b.x) - (c.x * d.y + c.y * d.x);
        m[2][j] = make_double2(re, -im);
      }
    }
    double2* o = U + size_t(l) * 9;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) o[i * 3 + j] = m[i][j];
  }
  warp_csum_add(cs, csum);
}

// canonical U -> payload (first `rows` rows), checksum of the host-order words
template <int BITS>
__global__ void __launch_bounds__(256) nersc_pack_kernel(const double2* U, unsigned char* raw, int64_t nlinks, int rows,
                                                         int swap, uint32_t* csum) {
  const int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t cs = 0;
  if (l < nlinks) {
    const double2* u = U + size_t(l) * 9;
    const size_t e0 = size_t(l) * rows * 6;
    for (int k = 0; k < rows * 3; k++) {
      const double v[2] = {u[k].x, u[k].y};
      for (int c = 0; c < 2; c++) {
        if (BITS == 32) {
          uint32_t w = __float_as_uint(__double2float_rn(v[c]));
          cs += w;
          reinterpret_cast<uint32_t*>(raw)[e0 + 2 * k + c] = swap ? bswap32(w) : w;
        } else {
          uint64_t w = static_cast<uint64_t>(__double_as_longlong(v[c]));
          cs += uint32_t(w) + uint32_t(w >> 32);
          reinterpret_cast<uint64_t*>(raw)[e0 + 2 * k + c] = swap ? bswap64(w) : w;
        }
      }
    }
  }
  warp_csum_add(cs, csum);
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// per site: sum over the 6 planes of Re tr(U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+) and
// sum over mu of Re tr U_mu(x); FP64 partials per block (periodic boundaries)
__global__ void __launch_bounds__(256) gauge_stats_kernel(const double2* U, Geo4 g, double* partial) {
  const int64_t x = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double plaq = 0, tr = 0;
  if (x < g.vol) {
    int c[4];
    int64_t r = x;
    for (int k = 0; k < 4; k++) { c[k] = int(r % g.L[k]); r /= g.L[k]; }
    auto shift = [&](int mu) {
      int d[4] = {c[0], c[1], c[2], c[3]};
      d[mu] = (d[mu] + 1) % g.L[mu];
      return d[0] + int64_t(g.L[0]) * (d[1] + int64_t(g.L[1]) * (d[2] + int64_t(g.L[2]) * d[3]));
    };
    for (int mu = 0; mu < 4; mu++) {
      const double2* u = U + (size_t(x) * 4 + mu) * 9;
      tr += u[0].x + u[4].x + u[8].x;
    }
    for (int mu = 1; mu < 4; mu++)
      for (int nu = 0; nu < mu; nu++) {
        const double2* A = U + (size_t(x) * 4 + mu) * 9;           // U_mu(x)
        const double2* B = U + (size_t(shift(mu)) * 4 + nu) * 9;   // U_nu(x+mu)
        const double2* C = U + (size_t(x) * 4 + nu) * 9;           // U_nu(x)
        const double2* D = U + (size_t(shift(nu)) * 4 + mu) * 9;   // U_mu(x+nu)
        // tr(M1 M2^+) = sum_ij M1_ij conj(M2_ij), M1 = A B, M2 = C D
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) {
            double2 m1 = make_double2(0, 0), m2 = make_double2(0, 0);
            for (int k = 0; k < 3; k++) {
              const double2 p = cmul(A[i * 3 + k], B[k * 3 + j]), q = cmul(C[i * 3 + k], D[k * 3 + j]);
              m1.x += p.x; m1.y += p.y;
              m2.x += q.x; m2.y += q.y;
            }
            plaq += m1.x * m2.x + m1.y * m2.y;
          }
      }
  }
  __shared__ double sp[8], st[8];
  for (int o = 16; o; o >>= 1) {
    plaq += __shfl_down_sync(0xffffffffu, plaq, o);
    tr += __shfl_down_sync(0xffffffffu, tr, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { sp[w] = plaq; st[w] = tr; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < int(blockDim.x >> 5); k++) { a += sp[k]; b += st[k]; }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

Geo4 geo4(const int dims[4]) {
  Geo4 g;
  g.vol = 1;
  for (int k = 0; k < 4; k++) { g.L[k] = dims[k]; g.vol *= dims[k]; }
  return g;
}

// avgPlaquette and linkTrace of a canonical field in device memory
int gauge_stats_dev(const int dims[4], const double* Ud, cudaStream_t s, double* plaq, double* trace) {
  const Geo4 g = geo4(dims);
  const unsigned blocks = unsigned((g.vol + 255) / 256);
  double* dpart = nullptr;
  GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dpart), size_t(blocks) * 2 * sizeof(double), s));
  gauge_stats_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const double2*>(Ud), g, dpart);
  std::vector<double> part(size_t(blocks) * 2);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), dpart, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(dpart, s);
  if (e != cudaSuccess) { set_error("gauge statistics: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
  double a = 0, b = 0;
  for (unsigned k = 0; k < blocks; k++) { a += part[2 * k]; b += part[2 * k + 1]; }
  *plaq = a / double(g.vol) / 6.0 / 3.0;
  *trace = b / double(g.vol) / 4.0 / 3.0;
  return GB_OK;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) a++;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) b--;
  return s.substr(a, b - a);
}
void copy_str(char* dst, size_t n, const std::string& s) {
  std::snprintf(dst, n, "%s", s.c_str());
}

int parse_header(const char* path, gb_nersc_header* h) {
  std::memset(h, 0, sizeof(*h));
  std::ifstream fin(path, std::ios::binary);
  if (!fin) { set_error("NERSC: cannot open %s", path); return GB_ERR_IO; }
  std::string line;
  std::getline(fin, line);
  if (trim(line) != "BEGIN_HEADER") { set_error("NERSC: %s does not start with BEGIN_HEADER", path); return GB_ERR_IO; }
  std::map<std::string, std::string> kv;
  bool end = false;
  for (int n = 0; n < 1000 && std::getline(fin, line); n++) {
    if (line.find("END_HEADER") != std::string::npos) { end = true; break; }
    const size_t eq = line.find('=');
    if (eq != std::string::npos && eq > 0) kv[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
  }
  if (!end) { set_error("NERSC: no END_HEADER in %s", path); return GB_ERR_IO; }
  h->data_start = int64_t(fin.tellg());
  auto get = [&](const char* k) { auto it = kv.find(k); return it == kv.end() ? std::string() : it->second; };
  try {
    for (int d = 0; d < 4; d++) h->dims[d] = std::stoi(get(("DIMENSION_" + std::to_string(d + 1)).c_str()));
    h->link_trace = std::stod(get("LINK_TRACE"));
    h->plaquette = std::stod(get("PLAQUETTE"));
    h->checksum = uint32_t(std::stoul(get("CHECKSUM"), nullptr, 16));
    const std::string seq = get("SEQUENCE_NUMBER");
    h->sequence_number = seq.empty() ? 0 : std::stoi(seq);
  } catch (...) {
    set_error("NERSC: malformed header values in %s", path);
    return GB_ERR_IO;
  }
  const std::string dt = get("DATATYPE"), fp = get("FLOATING_POINT");
  copy_str(h->data_type, sizeof(h->data_type), dt);
  copy_str(h->floating_point, sizeof(h->floating_point), fp);
  copy_str(h->ensemble_id, sizeof(h->ensemble_id), get("ENSEMBLE_ID"));
  copy_str(h->ensemble_label, sizeof(h->ensemble_label), get("ENSEMBLE_LABEL"));
  for (int d = 0; d < 4; d++)
    copy_str(h->boundary[d], sizeof(h->boundary[d]), get(("BOUNDARY_" + std::to_string(d + 1)).c_str()));
  if (dt == "4D_SU3_GAUGE") h->two_row = 1;
  else if (dt == "4D_SU3_GAUGE_3x3") h->two_row = 0;
  else { set_error("NERSC: DATATYPE %s is not an SU(3) gauge field", dt.c_str()); return GB_ERR_IO; }
  if (fp == "IEEE32BIG") { h->bits = 32; h->big_endian = 1; }
  else if (fp == "IEEE32") { h->bits = 32; h->big_endian = 0; }
  else if (fp == "IEEE64BIG") { h->bits = 64; h->big_endian = 1; }
  else if (fp == "IEEE64" || fp == "IEEE64LITTLE") { h->bits = 64; h->big_endian = 0; }
  else { set_error("NERSC: FLOATING_POINT %s not supported", fp.c_str()); return GB_ERR_IO; }
  for (int d = 0; d < 4; d++)
    if (h->dims[d] < 1) { set_error("NERSC: bad DIMENSION_%d", d + 1); return GB_ERR_IO; }
  return GB_OK;
}

}  // namespace

int gauge_stats_device(const int dims[4], const double* Ud, cudaStream_t s, double* plaq, double* trace) {
  return gauge_stats_dev(dims, Ud, s, plaq, trace);
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_nersc_read_header(const char* path, gb_nersc_header* h) {
  if (!path || !h) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  return parse_header(path, h);
}

int gb_gauge_stats(const int dims[4], const double* U, int on_device, double* plaquette, double* link_trace) {
  if (!dims || !U || !plaquette || !link_trace) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  const Geo4 g = geo4(dims);
  const size_t bytes = size_t(g.vol) * 36 * 16;
  const double* Ud = U;
  double* tmp = nullptr;
  if (!on_device) {
    GB_CHECK_CUDA(cudaMalloc(reinterpret_cast<void**>(&tmp), bytes));
    if (cudaMemcpy(tmp, U, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaFree(tmp);
      set_error("gauge statistics: copy to the device failed");
      return GB_ERR_CUDA;
    }
    Ud = tmp;
  }
  const int rc = gauge_stats_dev(dims, Ud, nullptr, plaquette, link_trace);
  if (tmp) cudaFree(tmp);
  return rc;
}

int gb_nersc_read(const char* path, double* U, int on_device, gb_nersc_header* h, int check) {
  if (!path || !U || !h) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_TRY(parse_header(path, h));
  const Geo4 g = geo4(h->dims);
  const int rows = h->two_row ? 2 : 3;
  const size_t nlinks = size_t(g.vol) * 4;
  const size_t raw_bytes = nlinks * rows * 6 * (h->bits / 8);
  const size_t out_bytes = nlinks * 9 * 16;
  std::ifstream fin(path, std::ios::binary);
  fin.seekg(0, std::ios::end);
  const int64_t fsize = int64_t(fin.tellg());
  if (fsize - h->data_start < int64_t(raw_bytes)) {
    set_error("NERSC: payload of %s is %lld bytes, %zu expected", path, (long long)(fsize - h->data_start), raw_bytes);
    return GB_ERR_IO;
  }
  void* host = nullptr;
  GB_CHECK_CUDA(cudaMallocHost(&host, raw_bytes));
  struct HostFree { void* p; ~HostFree() { cudaFreeHost(p); } } hf{host};
  fin.seekg(h->data_start);
  fin.read(static_cast<char*>(host), std::streamsize(raw_bytes));
  if (!fin) { set_error("NERSC: short read of %s", path); return GB_ERR_IO; }
  unsigned char* draw = nullptr;
  double* dU = nullptr;
  uint32_t* dcs = nullptr;
  GB_CHECK_CUDA(cudaMalloc(&draw, raw_bytes + 16));
  struct DevFree { void* a; void* b; void* c; ~DevFree() { cudaFree(a); cudaFree(b); cudaFree(c); } } df{draw, nullptr, nullptr};
  if (!on_device) {
    GB_CHECK_CUDA(cudaMalloc(&dU, out_bytes));
    df.b = dU;
  } else {
    dU = U;
  }
  GB_CHECK_CUDA(cudaMalloc(&dcs, sizeof(uint32_t)));
  df.c = dcs;
  GB_CHECK_CUDA(cudaMemset(dcs, 0, sizeof(uint32_t)));
  GB_CHECK_CUDA(cudaMemcpy(draw, host, raw_bytes, cudaMemcpyHostToDevice));
  const unsigned blocks = unsigned((nlinks + 255) / 256);
  if (h->bits == 32)
    nersc_unpack_kernel<32><<<blocks, 256>>>(draw, reinterpret_cast<double2*>(dU), int64_t(nlinks), rows, h->big_endian, dcs);
  else
    nersc_unpack_kernel<64><<<blocks, 256>>>(draw, reinterpret_cast<double2*>(dU), int64_t(nlinks), rows, h->big_endian, dcs);
  GB_CHECK_CUDA(cudaGetLastError());
  GB_CHECK_CUDA(cudaMemcpy(&h->checksum_computed, dcs, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  GB_TRY(gauge_stats_dev(h->dims, dU, nullptr, &h->plaquette_computed, &h->link_trace_computed));
  if (!on_device) GB_CHECK_CUDA(cudaMemcpy(U, dU, out_bytes, cudaMemcpyDeviceToHost));
  if (check) {
    if (h->checksum_computed != h->checksum) {
      set_error("NERSC: checksum %08x of the payload differs from the header's %08x", h->checksum_computed, h->checksum);
      return GB_ERR_IO;
    }
    if (std::fabs(h->plaquette_computed - h->plaquette) >= 1e-5) {
      set_error("NERSC: plaquette %.10f differs from the header's %.10f", h->plaquette_computed, h->plaquette);
      return GB_ERR_IO;
    }
    if (std::fabs(h->link_trace_computed - h->link_trace) >= 1e-6) {
      set_error("NERSC: link trace %.10f differs from the header's %.10f", h->link_trace_computed, h->link_trace);
      return GB_ERR_IO;
    }
  }
  return GB_OK;
}

int gb_nersc_write(const char* path, const double* U, int on_device, const int dims[4], int two_row, int bits,
                   int big_endian, const char* ensemble_id, const char* ensemble_label, int sequence_number) {
  if (!path || !U || !dims) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (bits != 32 && bits != 64) { set_error("NERSC: bits must be 32 or 64"); return GB_ERR_BAD_ARG; }
  const Geo4 g = geo4(dims);
  const int rows = two_row ? 2 : 3;
  const size_t nlinks = size_t(g.vol) * 4;
  const size_t raw_bytes = nlinks * rows * 6 * (bits / 8);
  const size_t in_bytes = nlinks * 9 * 16;
  const double* dU = U;
  double* tmpU = nullptr;
  unsigned char* draw = nullptr;
  uint32_t* dcs = nullptr;
  struct DevFree { void* a; void* b; void* c; ~DevFree() { cudaFree(a); cudaFree(b); cudaFree(c); } } df{nullptr, nullptr, nullptr};
  if (!on_device) {
    GB_CHECK_CUDA(cudaMalloc(&tmpU, in_bytes));
    df.a = tmpU;
    GB_CHECK_CUDA(cudaMemcpy(tmpU, U, in_bytes, cudaMemcpyHostToDevice));
    dU = tmpU;
  }
  GB_CHECK_CUDA(cudaMalloc(&draw, raw_bytes + 16));
  df.b = draw;
  GB_CHECK_CUDA(cudaMalloc(&dcs, sizeof(uint32_t)));
  df.c = dcs;
  GB_CHECK_CUDA(cudaMemset(dcs, 0, sizeof(uint32_t)));
  const unsigned blocks = unsigned((nlinks + 255) / 256);
  if (bits == 32)
    nersc_pack_kernel<32><<<blocks, 256>>>(reinterpret_cast<const double2*>(dU), draw, int64_t(nlinks), rows, big_endian, dcs);
  else
    nersc_pack_kernel<64><<<blocks, 256>>>(reinterpret_cast<const double2*>(dU), draw, int64_t(nlinks), rows, big_endian, dcs);
  GB_CHECK_CUDA(cudaGetLastError());
  uint32_t csum = 0;
  GB_CHECK_CUDA(cudaMemcpy(&csum, dcs, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  double plaq = 0, trace = 0;
  GB_TRY(gauge_stats_dev(dims, dU, nullptr, &plaq, &trace));
  void* host = nullptr;
  GB_CHECK_CUDA(cudaMallocHost(&host, raw_bytes));
  struct HostFree { void* p; ~HostFree() { cudaFreeHost(p); } } hf{host};
  GB_CHECK_CUDA(cudaMemcpy(host, draw, raw_bytes, cudaMemcpyDeviceToHost));
  // header as Grid's dump_meta_data writes it (MetaData.h:143-165)
  std::ostringstream s;
  char buf[64];
  const std::time_t now = std::time(nullptr);
  std::strftime(buf, sizeof(buf), "%c", std::gmtime(&now));
  s << "BEGIN_HEADER\n";
  s << "HDR_VERSION = 1.0\n";
  s << "DATATYPE = " << (two_row ? "4D_SU3_GAUGE" : "4D_SU3_GAUGE_3x3") << "\n";
  s << "STORAGE_FORMAT = 1.0\n";
  for (int d = 0; d < 4; d++) s << "DIMENSION_" << d + 1 << " = " << dims[d] << "\n";
  s.precision(10);
  s << "LINK_TRACE = " << trace << "\n";
  s << "PLAQUETTE  = " << plaq << "\n";
  for (int d = 0; d < 4; d++) s << "BOUNDARY_" << d + 1 << " = PERIODIC\n";
  std::snprintf(buf, sizeof(buf), "%10x", csum);
  s << "CHECKSUM = " << buf << "\n";
  s << "ENSEMBLE_ID = " << (ensemble_id ? ensemble_id : "UKQCD") << "\n";
  s << "ENSEMBLE_LABEL = " << (ensemble_label ? ensemble_label : "DWF") << "\n";
  s << "SEQUENCE_NUMBER = " << sequence_number << "\n";
  s << "CREATOR = gbdwf\n";
  s << "CREATOR_HARDWARE = GB300\n";
  std::strftime(buf, sizeof(buf), "%c", std::gmtime(&now));
  s << "CREATION_DATE = " << buf << "\n";
  s << "ARCHIVE_DATE = " << buf << "\n";
  s << "FLOATING_POINT = " << (bits == 32 ? (big_endian ? "IEEE32BIG" : "IEEE32") : (big_endian ? "IEEE64BIG" : "IEEE64"))
    << "\n";
  s << "END_HEADER\n";
  std::ofstream fout(path, std::ios::binary | std::ios::trunc);
  if (!fout) { set_error("NERSC: cannot create %s", path); return GB_ERR_IO; }
  const std::string hs = s.str();
  fout.write(hs.data(), std::streamsize(hs.size()));
  fout.write(static_cast<const char*>(host), std::streamsize(raw_bytes));
  if (!fout) { set_error("NERSC: write to %s failed", path); return GB_ERR_IO; }
  return GB_OK;
}

}  // extern "C"
