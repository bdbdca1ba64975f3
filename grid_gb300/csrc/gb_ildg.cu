// gb_ildg.cu -- ILDG / SciDAC gauge-configuration files (Grid/parallelIO/IldgIO.h:611-950,
// IldgIOtypes.h, the SciDAC checksum of BinaryIO.h:139-192) read into and written from
// the canonical FP64 gauge layout, the byte work on the GPU.
//
// Container: LIME (Lattice QCD Interchange Message Encapsulation, the c-lime library
// Grid links against; it is not part of Grid's sources).  A file is a sequence of
// records; each is a 144-byte big-endian header
//     magic 0x456789ab (4 B) | format version 1 (2 B) | flags (2 B: 0x8000 = message
//     begin, 0x4000 = message end) | data length (8 B) | record type (128 B, NUL padded)
// then the data, zero-padded to a multiple of 8 bytes.
//
// Records (the order of IldgWriter::writeConfiguration, without Grid's private
// grid-format and FieldNormMetaData records): scidac-private-file-xml [MB],
// scidac-file-xml [ME]; scidac-private-record-xml [MB], scidac-record-xml (usqcdInfo:
// plaquette and link trace), ildg-format (field su3gauge, precision 32/64, lx ly lz lt),
// ildg-data-lfn, ildg-binary-data, scidac-checksum [ME].
//
// Binary data: site-lexicographic (x fastest), per site the 4 links as full 3x3 complex
// matrices [mu][row][col], IEEE32 or IEEE64 big-endian.  SciDAC checksum: per site the
// CRC-32 (the zlib / IEEE 802.3 polynomial) of the site's bytes as stored, rotated left by
// (global site % 29) for suma and by (global site % 31) for sumb, XOR-combined; the
// checksum record holds both in lower-case hex.  A read, like Grid's
// (IldgIO.h:880-948), requires the ILDG format, LFN, binary and checksum records,
// verifies the checksums, and checks the plaquette and link trace against usqcdInfo
// (or grid-format) to 1e-5 when the file carries them.
#include <cuda_runtime.h>

#include <cctype>
#include <cinttypes>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <string>
#include <vector>

#include "gb_device.cuh"
#include "gb_ops.h"

namespace gb {
namespace {

constexpr uint32_t kLimeMagic = 0x456789abu;
constexpr int kLimeHeader = 144;

// ---- device: byte order, CRC-32, per-site conversion -------------------------------------
__device__ __forceinline__ uint32_t bswap32d(uint32_t x) { return __byte_perm(x, 0, 0x0123); }
__device__ __forceinline__ uint64_t bswap64d(uint64_t x) {
  return (uint64_t(bswap32d(uint32_t(x))) << 32) | uint64_t(bswap32d(uint32_t(x >> 32)));
}
__device__ __forceinline__ uint32_t rotl32(uint32_t x, uint32_t n) { return n ? (x << n) | (x >> (32u - n)) : x; }

// the 256-entry table of the reflected CRC-32 polynomial 0xEDB88320, built per CTA
__device__ __forceinline__ void crc_table_init(uint32_t* tab) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    uint32_t c = uint32_t(i);
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
    tab[i] = c;
  }
}
__device__ __forceinline__ uint32_t crc_bytes(const uint32_t* tab, uint32_t crc, uint64_t bytes, int n) {
  for (int b = 0; b < n; b++) crc = tab[(crc ^ uint32_t(bytes >> (8 * b))) & 0xffu] ^ (crc >> 8);
  return crc;
}

__device__ __forceinline__ void warp_xor_to(uint32_t v, uint32_t* out) {
  for (int o = 16; o; o >>= 1) v ^= __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) atomicXor(out, v);
}

// one thread per site: raw (file bytes) -> U[site][mu][3][3] complex double, with the
// SciDAC checksum of the bytes as stored; csum[0] = suma, csum[1] = sumb
template <int BITS>
__global__ void __launch_bounds__(256) ildg_unpack_kernel(const unsigned char* raw, double* U, int64_t vol,
                                                          uint32_t* csum) {
  __shared__ uint32_t tab[256];
  crc_table_init(tab);
  __syncthreads();
  const int64_t site = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t a = 0, b = 0;
  if (site < vol) {
    uint32_t crc = 0xffffffffu;
    if (BITS == 64) {
      const uint64_t* p = reinterpret_cast<const uint64_t*>(raw) + size_t(site) * 72;
      for (int e = 0; e < 72; e++) {
        const uint64_t w = p[e];  // file bytes in memory order
        crc = crc_bytes(tab, crc, w, 8);
        U[size_t(site) * 72 + e] = __longlong_as_double(static_cast<long long>(bswap64d(w)));
      }
    } else {
      const uint32_t* p = reinterpret_cast<const uint32_t*>(raw) + size_t(site) * 72;
      for (int e = 0; e < 72; e++) {
        const uint32_t w = p[e];
        crc = crc_bytes(tab, crc, w, 4);
        U[size_t(site) * 72 + e] = double(__uint_as_float(bswap32d(w)));
      }
    }
    crc ^= 0xffffffffu;
    a = rotl32(crc, uint32_t(site % 29));
    b = rotl32(crc, uint32_t(site % 31));
  }
  warp_xor_to(a, csum);
  warp_xor_to(b, csum + 1);
}

// the reverse: U -> file bytes (big-endian, 32 or 64 bit) and their checksum
template <int BITS>
__global__ void __launch_bounds__(256) ildg_pack_kernel(const double* U, unsigned char* raw, int64_t vol,
                                                        uint32_t* csum) {
  __shared__ uint32_t tab[256];
  crc_table_init(tab);
  __syncthreads();
  const int64_t site = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t a = 0, b = 0;
  if (site < vol) {
    uint32_t crc = 0xffffffffu;
    for (int e = 0; e < 72; e++) {
      const double v = U[size_t(site) * 72 + e];
      if (BITS == 64) {
        const uint64_t w = bswap64d(static_cast<uint64_t>(__double_as_longlong(v)));
        crc = crc_bytes(tab, crc, w, 8);
        reinterpret_cast<uint64_t*>(raw)[size_t(site) * 72 + e] = w;
      } else {
        const uint32_t w = bswap32d(__float_as_uint(float(v)));
        crc = crc_bytes(tab, crc, w, 4);
        reinterpret_cast<uint32_t*>(raw)[size_t(site) * 72 + e] = w;
      }
    }
    crc ^= 0xffffffffu;
    a = rotl32(crc, uint32_t(site % 29));
    b = rotl32(crc, uint32_t(site % 31));
  }
  warp_xor_to(a, csum);
  warp_xor_to(b, csum + 1);
}

// ---- host: LIME records and the XML fields Grid's reader uses ---------------------------
uint64_t be_load(const unsigned char* p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}
void be_store(unsigned char* p, uint64_t v, int n) {
  for (int i = n - 1; i >= 0; i--) { p[i] = static_cast<unsigned char>(v & 0xffu); v >>= 8; }
}

struct LimeRecord {
  std::string type;
  bool mb = false, me = false;
  int64_t offset = 0;  // of the data
  uint64_t bytes = 0;
};

int lime_scan(const char* path, std::vector<LimeRecord>& recs) {
  std::ifstream f(path, std::ios::binary);
  if (!f) { set_error("ILDG: cannot open %s", path); return GB_ERR_IO; }
  f.seekg(0, std::ios::end);
  const int64_t size = int64_t(f.tellg());
  int64_t pos = 0;
  while (pos + kLimeHeader <= size) {
    unsigned char h[kLimeHeader];
    f.seekg(pos);
    f.read(reinterpret_cast<char*>(h), kLimeHeader);
    if (!f) { set_error("ILDG: short read of a record header at %lld", (long long)pos); return GB_ERR_IO; }
    if (be_load(h, 4) != kLimeMagic) {
      set_error("ILDG: no LIME record at offset %lld of %s", (long long)pos, path);
      return GB_ERR_IO;
    }
    LimeRecord r;
    const uint32_t flags = uint32_t(be_load(h + 6, 2));
    r.mb = (flags & 0x8000u) != 0;
    r.me = (flags & 0x4000u) != 0;
    r.bytes = be_load(h + 8, 8);
    r.type.assign(reinterpret_cast<const char*>(h + 16), strnlen(reinterpret_cast<const char*>(h + 16), 128));
    r.offset = pos + kLimeHeader;
    if (r.offset + int64_t(r.bytes) > size) {
      set_error("ILDG: record %s runs past the end of %s", r.type.c_str(), path);
      return GB_ERR_IO;
    }
    recs.push_back(r);
    pos = r.offset + int64_t((r.bytes + 7) / 8 * 8);
  }
  if (recs.empty()) { set_error("ILDG: %s holds no LIME records", path); return GB_ERR_IO; }
  return GB_OK;
}

std::string read_text(const char* path, const LimeRecord& r) {
  std::ifstream f(path, std::ios::binary);
  std::string s(size_t(r.bytes), '\0');
  f.seekg(r.offset);
  f.read(&s[0], std::streamsize(r.bytes));
  const size_t z = s.find('\0');
  if (z != std::string::npos) s.resize(z);
  return s;
}

// the text of the first <tag ...>text</tag> element
bool xml_tag(const std::string& xml, const char* tag, std::string& out) {
  const std::string open = std::string("<") + tag;
  size_t p = 0;
  while ((p = xml.find(open, p)) != std::string::npos) {
    const char c = p + open.size() < xml.size() ? xml[p + open.size()] : '\0';
    if (c == '>' || c == ' ' || c == '\t' || c == '\n' || c == '\r') break;
    p += open.size();
  }
  if (p == std::string::npos) return false;
  const size_t a = xml.find('>', p);
  if (a == std::string::npos) return false;
  const size_t b = xml.find(std::string("</") + tag, a + 1);
  if (b == std::string::npos) return false;
  out = xml.substr(a + 1, b - a - 1);
  size_t i = 0, j = out.size();
  while (i < j && std::isspace(static_cast<unsigned char>(out[i]))) i++;
  while (j > i && std::isspace(static_cast<unsigned char>(out[j - 1]))) j--;
  out = out.substr(i, j - i);
  return true;
}
bool xml_int(const std::string& xml, const char* tag, int& v) {
  std::string s;
  if (!xml_tag(xml, tag, s)) return false;
  char* end = nullptr;
  const long x = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str()) return false;
  v = int(x);
  return true;
}
bool xml_double(const std::string& xml, const char* tag, double& v) {
  std::string s;
  if (!xml_tag(xml, tag, s)) return false;
  char* end = nullptr;
  v = std::strtod(s.c_str(), &end);
  return end != s.c_str();
}
bool xml_hex(const std::string& xml, const char* tag, uint32_t& v) {
  std::string s;
  if (!xml_tag(xml, tag, s)) return false;
  char* end = nullptr;
  const unsigned long long x = std::strtoull(s.c_str(), &end, 16);
  if (end == s.c_str()) return false;
  v = uint32_t(x);
  return true;
}
bool starts(const std::string& s, const char* p) { return s.compare(0, std::strlen(p), p) == 0; }

int parse(const char* path, gb_ildg_header* h, LimeRecord* binary) {
  std::memset(h, 0, sizeof(*h));
  std::vector<LimeRecord> recs;
  GB_TRY(lime_scan(path, recs));
  bool fmt = false, lfn = false, bin = false;
  for (const LimeRecord& r : recs) {
    if (starts(r.type, "ildg-binary-data")) {
      *binary = r;
      h->data_offset = r.offset;
      h->data_bytes = int64_t(r.bytes);
      bin = true;
      continue;
    }
    const std::string x = read_text(path, r);
    if (starts(r.type, "ildg-format")) {
      std::string field;
      if (xml_tag(x, "field", field)) std::snprintf(h->field, sizeof(h->field), "%s", field.c_str());
      bool ok = xml_int(x, "precision", h->precision);
      ok = ok && xml_int(x, "lx", h->dims[0]) && xml_int(x, "ly", h->dims[1]);
      ok = ok && xml_int(x, "lz", h->dims[2]) && xml_int(x, "lt", h->dims[3]);
      if (!ok) { set_error("ILDG: incomplete ildg-format record in %s", path); return GB_ERR_IO; }
      fmt = true;
    } else if (starts(r.type, "ildg-data-lfn")) {
      std::snprintf(h->lfn, sizeof(h->lfn), "%s", x.c_str());
      lfn = true;
    } else if (starts(r.type, "scidac-checksum")) {
      if (xml_hex(x, "suma", h->scidac_suma) && xml_hex(x, "sumb", h->scidac_sumb)) h->has_checksum = 1;
    } else if (starts(r.type, "scidac-record-xml") && x.find("usqcdInfo") != std::string::npos) {
      if (xml_double(x, "plaq", h->plaquette) && xml_double(x, "linktr", h->link_trace)) h->has_plaquette = 1;
    } else if (starts(r.type, "grid-format")) {
      if (xml_double(x, "plaquette", h->plaquette) && xml_double(x, "link_trace", h->link_trace)) h->has_plaquette = 1;
    }
  }
  if (!fmt) { set_error("ILDG: %s has no ildg-format record", path); return GB_ERR_IO; }
  if (!bin) { set_error("ILDG: %s has no ildg-binary-data record", path); return GB_ERR_IO; }
  if (!lfn) { set_error("ILDG: %s has no ildg-data-lfn record", path); return GB_ERR_IO; }
  if (h->precision != 32 && h->precision != 64) { set_error("ILDG: precision %d", h->precision); return GB_ERR_UNSUPPORTED; }
  if (std::strcmp(h->field, "su3gauge") != 0) { set_error("ILDG: field '%s' is not su3gauge", h->field); return GB_ERR_UNSUPPORTED; }
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) {
    if (h->dims[k] < 1) { set_error("ILDG: dimension %d = %d", k, h->dims[k]); return GB_ERR_IO; }
    vol *= h->dims[k];
  }
  if (uint64_t(vol) * 72 * uint64_t(h->precision / 8) != binary->bytes) {
    set_error("ILDG: binary record of %s holds %llu bytes, %lld sites need %llu", path, (unsigned long long)binary->bytes,
              (long long)vol, (unsigned long long)(uint64_t(vol) * 72 * uint64_t(h->precision / 8)));
    return GB_ERR_IO;
  }
  return GB_OK;
}

// one LIME record: header, data, zero padding to 8 bytes
void lime_write(std::ofstream& f, const char* type, bool mb, bool me, const void* data, uint64_t bytes) {
  unsigned char h[kLimeHeader];
  std::memset(h, 0, sizeof(h));
  be_store(h, kLimeMagic, 4);
  be_store(h + 4, 1, 2);
  be_store(h + 6, (mb ? 0x8000u : 0u) | (me ? 0x4000u : 0u), 2);
  be_store(h + 8, bytes, 8);
  std::strncpy(reinterpret_cast<char*>(h + 16), type, 127);
  f.write(reinterpret_cast<const char*>(h), kLimeHeader);
  if (bytes) f.write(static_cast<const char*>(data), std::streamsize(bytes));
  const uint64_t pad = (8 - bytes % 8) % 8;
  const char zeros[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (pad) f.write(zeros, std::streamsize(pad));
}
void lime_write_text(std::ofstream& f, const char* type, bool mb, bool me, const std::string& s) {
  lime_write(f, type, mb, me, s.data(), s.size());
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gb_ildg_read_header(const char* path, gb_ildg_header* h) {
  if (!path || !h) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  LimeRecord bin;
  return parse(path, h, &bin);
}

int gb_ildg_read(const char* path, double* U, int on_device, gb_ildg_header* h, int check) {
  if (!path || !U || !h) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  LimeRecord bin;
  GB_TRY(parse(path, h, &bin));
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= h->dims[k];
  const size_t raw_bytes = size_t(bin.bytes);
  const size_t out_bytes = size_t(vol) * 72 * sizeof(double);
  void* host = nullptr;
  GB_CHECK_CUDA(cudaMallocHost(&host, raw_bytes));
  struct HostFree { void* p; ~HostFree() { cudaFreeHost(p); } } hf{host};
  {
    std::ifstream f(path, std::ios::binary);
    f.seekg(bin.offset);
    f.read(static_cast<char*>(host), std::streamsize(raw_bytes));
    if (!f) { set_error("ILDG: short read of the binary record of %s", path); return GB_ERR_IO; }
  }
  unsigned char* draw = nullptr;
  double* dU = nullptr;
  uint32_t* dcs = nullptr;
  struct DevFree { void* a = nullptr; void* b = nullptr; void* c = nullptr; ~DevFree() { cudaFree(a); cudaFree(b); cudaFree(c); } } df;
  GB_CHECK_CUDA(cudaMalloc(&draw, raw_bytes));
  df.a = draw;
  if (on_device) {
    dU = U;
  } else {
    GB_CHECK_CUDA(cudaMalloc(&dU, out_bytes));
    df.b = dU;
  }
  GB_CHECK_CUDA(cudaMalloc(&dcs, 2 * sizeof(uint32_t)));
  df.c = dcs;
  GB_CHECK_CUDA(cudaMemset(dcs, 0, 2 * sizeof(uint32_t)));
  GB_CHECK_CUDA(cudaMemcpy(draw, host, raw_bytes, cudaMemcpyHostToDevice));
  const unsigned blocks = unsigned((vol + 255) / 256);
  if (h->precision == 64) ildg_unpack_kernel<64><<<blocks, 256>>>(draw, dU, vol, dcs);
  else ildg_unpack_kernel<32><<<blocks, 256>>>(draw, dU, vol, dcs);
  GB_CHECK_CUDA(cudaGetLastError());
  uint32_t cs[2];
  GB_CHECK_CUDA(cudaMemcpy(cs, dcs, sizeof(cs), cudaMemcpyDeviceToHost));
  h->scidac_suma_computed = cs[0];
  h->scidac_sumb_computed = cs[1];
  GB_TRY(gauge_stats_device(h->dims, dU, nullptr, &h->plaquette_computed, &h->link_trace_computed));
  if (!on_device) GB_CHECK_CUDA(cudaMemcpy(U, dU, out_bytes, cudaMemcpyDeviceToHost));
  if (check) {
    if (!h->has_checksum) { set_error("ILDG: %s has no scidac-checksum record", path); return GB_ERR_IO; }
    if (cs[0] != h->scidac_suma || cs[1] != h->scidac_sumb) {
      set_error("ILDG: SciDAC checksums %x %x of the data differ from the record's %x %x", cs[0], cs[1], h->scidac_suma,
                h->scidac_sumb);
      return GB_ERR_IO;
    }
    if (h->has_plaquette && (std::fabs(h->plaquette_computed - h->plaquette) >= 1e-5 ||
                             std::fabs(h->link_trace_computed - h->link_trace) >= 1e-5)) {
      set_error("ILDG: plaquette %.10f / link trace %.10f differ from the file's %.10f / %.10f", h->plaquette_computed,
                h->link_trace_computed, h->plaquette, h->link_trace);
      return GB_ERR_IO;
    }
  }
  return GB_OK;
}

int gb_ildg_write(const char* path, const double* U, int on_device, const int dims[4], int precision, const char* lfn) {
  if (!path || !U || !dims) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (precision != 32 && precision != 64) { set_error("ILDG: precision must be 32 or 64"); return GB_ERR_BAD_ARG; }
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) {
    if (dims[k] < 1) { set_error("ILDG: dimension %d = %d", k, dims[k]); return GB_ERR_BAD_ARG; }
    vol *= dims[k];
  }
  const size_t in_bytes = size_t(vol) * 72 * sizeof(double);
  const size_t raw_bytes = size_t(vol) * 72 * size_t(precision / 8);
  const double* dU = U;
  struct DevFree { void* a = nullptr; void* b = nullptr; void* c = nullptr; ~DevFree() { cudaFree(a); cudaFree(b); cudaFree(c); } } df;
  if (!on_device) {
    double* t = nullptr;
    GB_CHECK_CUDA(cudaMalloc(&t, in_bytes));
    df.a = t;
    GB_CHECK_CUDA(cudaMemcpy(t, U, in_bytes, cudaMemcpyHostToDevice));
    dU = t;
  }
  unsigned char* draw = nullptr;
  uint32_t* dcs = nullptr;
  GB_CHECK_CUDA(cudaMalloc(&draw, raw_bytes));
  df.b = draw;
  GB_CHECK_CUDA(cudaMalloc(&dcs, 2 * sizeof(uint32_t)));
  df.c = dcs;
  GB_CHECK_CUDA(cudaMemset(dcs, 0, 2 * sizeof(uint32_t)));
  const unsigned blocks = unsigned((vol + 255) / 256);
  if (precision == 64) ildg_pack_kernel<64><<<blocks, 256>>>(dU, draw, vol, dcs);
  else ildg_pack_kernel<32><<<blocks, 256>>>(dU, draw, vol, dcs);
  GB_CHECK_CUDA(cudaGetLastError());
  double plaq = 0, trace = 0;
  GB_TRY(gauge_stats_device(dims, dU, nullptr, &plaq, &trace));
  void* host = nullptr;
  GB_CHECK_CUDA(cudaMallocHost(&host, raw_bytes));
  struct HostFree { void* p; ~HostFree() { cudaFreeHost(p); } } hf{host};
  GB_CHECK_CUDA(cudaMemcpy(host, draw, raw_bytes, cudaMemcpyDeviceToHost));
  uint32_t cs[2];
  GB_CHECK_CUDA(cudaMemcpy(cs, dcs, sizeof(cs), cudaMemcpyDeviceToHost));

  char date[64];
  {
    const std::time_t now = std::time(nullptr);
    std::tm tmv;
    gmtime_r(&now, &tmv);
    std::strftime(date, sizeof(date), "%a %b %d %H:%M:%S %Y UTC", &tmv);
  }
  char buf[1024];
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) { set_error("ILDG: cannot create %s", path); return GB_ERR_IO; }
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\"?>\n<scidacFile><version>1.1</version><spacetime>4</spacetime>"
                "<dims>%d %d %d %d </dims><volfmt>0</volfmt></scidacFile>",
                dims[0], dims[1], dims[2], dims[3]);
  lime_write_text(f, "scidac-private-file-xml", true, false, buf);
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\"?>\n<usqcdInfo><version>1</version><plaq>%.17g</plaq><linktr>%.17g</linktr>"
                "<info>gauge configuration</info></usqcdInfo>",
                plaq, trace);
  const std::string usqcd = buf;
  lime_write_text(f, "scidac-file-xml", false, true, usqcd);
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\"?>\n<scidacRecord><version>1.1</version><date>%s</date><recordtype>0</recordtype>"
                "<datatype>QDP_%c3_ColorMatrix</datatype><precision>%c</precision><colors>3</colors><spins>4</spins>"
                "<typesize>%d</typesize><datacount>4</datacount></scidacRecord>",
                date, precision == 64 ? 'D' : 'F', precision == 64 ? 'D' : 'F', 18 * precision / 8);
  lime_write_text(f, "scidac-private-record-xml", true, false, buf);
  lime_write_text(f, "scidac-record-xml", false, false, usqcd);
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n<ildgFormat><version>1</version><field>su3gauge</field>"
                "<precision>%d</precision><lx>%d</lx><ly>%d</ly><lz>%d</lz><lt>%d</lt></ildgFormat>",
                precision, dims[0], dims[1], dims[2], dims[3]);
  lime_write_text(f, "ildg-format", false, false, buf);
  lime_write_text(f, "ildg-data-lfn", false, false, lfn ? std::string(lfn) : std::string());
  lime_write(f, "ildg-binary-data", false, false, host, raw_bytes);
  std::snprintf(buf, sizeof(buf),
                "<?xml version=\"1.0\"?>\n<scidacChecksum><version>1</version><suma>%x</suma><sumb>%x</sumb>"
                "</scidacChecksum>",
                cs[0], cs[1]);
  lime_write_text(f, "scidac-checksum", false, true, buf);
  f.close();
  if (!f) { set_error("ILDG: write to %s failed", path); return GB_ERR_IO; }
  return GB_OK;
}

}  // extern "C"
