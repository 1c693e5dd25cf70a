// formats.cpp -- on-disk formats (host only): the reference's result.bin / initial.bin, the
// ghost-slab layout of its multi-GPU programs' files, and a self-checking state snapshot.
//
// result.bin / initial.bin: nx*ny*nz float32 values, x fastest, no header
// (SingleGPU/Diffusion3d_baselineCode/tools.cpp:59-87). The reference's multi-GPU programs write
// the whole z-decomposed array including RADIUS ghost slabs at each z end, nx*ny*(Nz+2R) values
// (MultiGPU/Burgers3d_Baseline/main.c:65,79,355 with RADIUS 3 in BurgersMPI.h:50).
//
// State snapshot (for resuming a run; the reference has none): a 128-byte little-endian header
// then the state in its own precision (x fastest):
//   0  char[8]  magic "ADVSTATE"        40  double   t
//   8  int32    version (1)             48  uint64   payload bytes
//   12 int32    dtype (adv_dtype)       56  uint32   CRC-32 of the payload
//   16 int32    nx, ny, nz              60  uint32   CRC-32 of bytes 0..59
//   28 int32    reserved (0)            64  reserved (zero) up to 128
//   32 int64    step
// CRC-32 is the IEEE 802.3 polynomial (reflected 0xEDB88320, initial and final XOR 0xFFFFFFFF),
// the checksum of zlib and PNG. A truncated or altered file is rejected with an error status.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "adv_internal.h"

namespace adv {
namespace {

uint32_t crc_table_entry(uint32_t c) {
  for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
  return c;
}

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; ++i) t[i] = crc_table_entry(i);
  }
};

uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
  static const CrcTable tab;
  for (size_t i = 0; i < n; ++i) crc = tab.t[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
  return crc;
}

uint32_t crc32(const void* p, size_t n) {
  return crc32_update(0xFFFFFFFFu, static_cast<const unsigned char*>(p), n) ^ 0xFFFFFFFFu;
}

constexpr char kMagic[8] = {'A', 'D', 'V', 'S', 'T', 'A', 'T', 'E'};

size_t elem_size(int dtype) { return dtype == ADV_F32 ? 4 : 8; }

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

}  // namespace
}  // namespace adv

using namespace adv;

extern "C" {

uint32_t adv_crc32(const void* data, size_t n) { return data || n == 0 ? crc32(data, n) : 0u; }

adv_status adv_read_result_bin(const char* path, int64_t n, double* host_u) {
  if (!path || !host_u || n < 0) return set_error(ADV_ERR_INVALID_ARG, "read_result_bin: bad arguments");
  File fl;
  fl.f = std::fopen(path, "rb");
  if (!fl.f) return set_error(ADV_ERR_INVALID_ARG, std::string("read_result_bin: cannot open ") + path);
  std::fseek(fl.f, 0, SEEK_END);
  const long size = std::ftell(fl.f);
  std::fseek(fl.f, 0, SEEK_SET);
  if (size != (long)(n * 4))
    return set_error(ADV_ERR_INVALID_ARG, "read_result_bin: file holds " + std::to_string(size / 4) +
                                              " float32 values, expected " + std::to_string(n));
  std::vector<float> buf(1 << 16);
  int64_t done = 0;
  while (done < n) {
    const int64_t m = std::min<int64_t>(n - done, (int64_t)buf.size());
    if (std::fread(buf.data(), sizeof(float), (size_t)m, fl.f) != (size_t)m)
      return set_error(ADV_ERR_INVALID_ARG, "read_result_bin: short read");
    for (int64_t i = 0; i < m; ++i) host_u[done + i] = buf[i];
    done += m;
  }
  return ADV_OK;
}

adv_status adv_strip_ghost_slabs(int nx, int ny, int nz, int radius, const double* ghosted, double* interior) {
  if (nx < 1 || ny < 1 || nz < 1 || radius < 0 || !ghosted || !interior)
    return set_error(ADV_ERR_INVALID_ARG, "strip_ghost_slabs: bad arguments");
  const size_t plane = (size_t)nx * ny;
  std::memcpy(interior, ghosted + plane * radius, plane * nz * sizeof(double));
  return ADV_OK;
}

adv_status adv_pad_ghost_slabs(int nx, int ny, int nz, int radius, int periodic, const double* interior,
                               double* ghosted) {
  if (nx < 1 || ny < 1 || nz < 1 || radius < 0 || !ghosted || !interior || (periodic && radius > nz))
    return set_error(ADV_ERR_INVALID_ARG, "pad_ghost_slabs: bad arguments");
  const size_t plane = (size_t)nx * ny;
  std::memcpy(ghosted + plane * radius, interior, plane * nz * sizeof(double));
  for (int g = 0; g < radius; ++g) {
    double* lo = ghosted + plane * g;                      // z = g - radius
    double* hi = ghosted + plane * (radius + nz + g);      // z = nz + g
    if (periodic) {
      std::memcpy(lo, interior + plane * (nz - radius + g), plane * sizeof(double));
      std::memcpy(hi, interior + plane * g, plane * sizeof(double));
    } else {
      std::memset(lo, 0, plane * sizeof(double));
      std::memset(hi, 0, plane * sizeof(double));
    }
  }
  return ADV_OK;
}

adv_status adv_checkpoint_save(const char* path, int dtype, int nx, int ny, int nz, int64_t step, double t,
                               const void* host_u) {
  if (!path || !host_u || nx < 1 || ny < 1 || nz < 1 || step < 0 || (dtype != ADV_F32 && dtype != ADV_F64))
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_save: bad arguments");
  const uint64_t bytes = (uint64_t)nx * ny * nz * elem_size(dtype);
  unsigned char h[128];
  std::memset(h, 0, sizeof(h));
  const int32_t version = 1, d32 = dtype, x = nx, y = ny, z = nz;
  std::memcpy(h, kMagic, 8);
  std::memcpy(h + 8, &version, 4);
  std::memcpy(h + 12, &d32, 4);
  std::memcpy(h + 16, &x, 4);
  std::memcpy(h + 20, &y, 4);
  std::memcpy(h + 24, &z, 4);
  std::memcpy(h + 32, &step, 8);
  std::memcpy(h + 40, &t, 8);
  std::memcpy(h + 48, &bytes, 8);
  const uint32_t pc = crc32(host_u, (size_t)bytes);
  std::memcpy(h + 56, &pc, 4);
  const uint32_t hc = crc32(h, 60);
  std::memcpy(h + 60, &hc, 4);
  // write to a temporary name, then rename: a crash never leaves a half-written snapshot
  const std::string tmp = std::string(path) + ".tmp";
  {
    File fl;
    fl.f = std::fopen(tmp.c_str(), "wb");
    if (!fl.f) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_save: cannot open " + tmp);
    if (std::fwrite(h, 1, sizeof(h), fl.f) != sizeof(h) ||
        std::fwrite(host_u, 1, (size_t)bytes, fl.f) != (size_t)bytes)
      return set_error(ADV_ERR_INVALID_ARG, "checkpoint_save: short write");
    if (std::fflush(fl.f) != 0) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_save: flush failed");
  }
  if (std::rename(tmp.c_str(), path) != 0) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_save: rename failed");
  return ADV_OK;
}

adv_status adv_checkpoint_load(const char* path, adv_checkpoint_header* hdr, void* host_u, size_t capacity_bytes) {
  if (!path || !hdr) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: bad arguments");
  File fl;
  fl.f = std::fopen(path, "rb");
  if (!fl.f) return set_error(ADV_ERR_INVALID_ARG, std::string("checkpoint_load: cannot open ") + path);
  unsigned char h[128];
  if (std::fread(h, 1, sizeof(h), fl.f) != sizeof(h))
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: truncated header");
  if (std::memcmp(h, kMagic, 8) != 0) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: not a state snapshot");
  uint32_t hc;
  std::memcpy(&hc, h + 60, 4);
  if (hc != crc32(h, 60)) return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: header CRC mismatch");
  adv_checkpoint_header H{};
  std::memcpy(&H.version, h + 8, 4);
  std::memcpy(&H.dtype, h + 12, 4);
  std::memcpy(&H.nx, h + 16, 4);
  std::memcpy(&H.ny, h + 20, 4);
  std::memcpy(&H.nz, h + 24, 4);
  std::memcpy(&H.step, h + 32, 8);
  std::memcpy(&H.t, h + 40, 8);
  std::memcpy(&H.payload_bytes, h + 48, 8);
  std::memcpy(&H.payload_crc32, h + 56, 4);
  if (H.version != 1) return set_error(ADV_ERR_UNSUPPORTED, "checkpoint_load: unknown format version");
  if ((H.dtype != ADV_F32 && H.dtype != ADV_F64) || H.nx < 1 || H.ny < 1 || H.nz < 1 ||
      H.payload_bytes != (uint64_t)H.nx * H.ny * H.nz * elem_size(H.dtype))
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: inconsistent header");
  *hdr = H;
  if (!host_u) return ADV_OK;  // header only
  if (capacity_bytes < H.payload_bytes)
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: buffer smaller than the snapshot");
  if (std::fread(host_u, 1, (size_t)H.payload_bytes, fl.f) != (size_t)H.payload_bytes)
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: truncated payload");
  if (std::fgetc(fl.f) != EOF)  // a snapshot ends with its payload: appended or joined files are not one
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: data after the payload");
  if (crc32(host_u, (size_t)H.payload_bytes) != H.payload_crc32)
    return set_error(ADV_ERR_INVALID_ARG, "checkpoint_load: payload CRC mismatch");
  return ADV_OK;
}

}  // extern "C"
