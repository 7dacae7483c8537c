// Files around the occluder path: the reference demo's mesh files and a baked
// occluder file.
//
//   Mesh files (Main.cpp:56-84): IndexBuffer.bin is a raw array of u32 triangle
//   indices, VertexBuffer.bin a raw array of float4 vertices (16 bytes each),
//   both little-endian, no header; the demo sizes them from the file length.
//
//   Baked occluder file (this library's own format): the output of
//   Occluder::bake for a whole scene (Main.cpp:86-128 take about a second per
//   260k-triangle scene and ten for a 2M-triangle one), so that a program can
//   load occluders instead of decomposing, batching and quantising again.
//   Little-endian:
//     u8  magic[8]  "OCCBAKE1"
//     u32 version   1
//     u32 count     occluders
//     u64 words     packed words over all occluders (sum of 8 * packetCount)
//     count records of 96 bytes:
//       u32 packetCount (32-byte vectors, Occluder.h:20), u32 reserved[3] = 0,
//       f32 refMin[4], refMax[4], boundsMin[4], boundsMax[4], center[4]
//     the packed words of every occluder, in record order
//     u64 FNV-1a hash of every byte before it
//   A file that is short, has another magic or version, inconsistent sizes or
//   a wrong hash is refused (OCC_ERR_IO), nothing is returned from it.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rasterizer_gb300.h"

namespace occ {
int set_error(int code, const char* msg);  // capi.cu: the message of occ_last_error
}

namespace {

using occ::set_error;

constexpr char kMagic[8] = {'O', 'C', 'C', 'B', 'A', 'K', 'E', '1'};
constexpr uint32_t kVersion = 1;
constexpr size_t kHeaderBytes = 24;
constexpr size_t kRecordBytes = 96;

static_assert(sizeof(float) == 4, "32-bit float");

bool host_little_endian()
{
  const uint32_t one = 1;
  uint8_t b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

uint64_t fnv1a(const uint8_t* p, size_t n, uint64_t h = 1469598103934665603ull)
{
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

bool read_file(const char* path, std::vector<uint8_t>& out)
{
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long size = ok ? std::ftell(f) : -1;
  ok = ok && size >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    out.resize((size_t)size);
    ok = size == 0 || std::fread(out.data(), 1, (size_t)size, f) == (size_t)size;
  }
  std::fclose(f);
  return ok;
}

template <class T>
T get(const uint8_t* p)
{
  T v;
  std::memcpy(&v, p, sizeof v);
  return v;
}

template <class T>
void put(std::vector<uint8_t>& out, const T& v)
{
  const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
  out.insert(out.end(), p, p + sizeof v);
}

// Checks a whole baked file; on success `count` and `words` are its totals.
int parse_baked(const std::vector<uint8_t>& f, uint32_t& count, uint64_t& words)
{
  if (f.size() < kHeaderBytes + 8 || std::memcmp(f.data(), kMagic, 8) != 0)
    return set_error(OCC_ERR_IO, "not a baked occluder file");
  if (get<uint32_t>(f.data() + 8) != kVersion) return set_error(OCC_ERR_IO, "unknown baked occluder file version");
  count = get<uint32_t>(f.data() + 12);
  words = get<uint64_t>(f.data() + 16);
  const uint64_t body = (uint64_t)kHeaderBytes + (uint64_t)count * kRecordBytes;
  if (words > (uint64_t(1) << 40) || body + 4 * words + 8 != f.size())
    return set_error(OCC_ERR_IO, "baked occluder file: size does not match its header");
  if (fnv1a(f.data(), f.size() - 8) != get<uint64_t>(f.data() + f.size() - 8))
    return set_error(OCC_ERR_IO, "baked occluder file: hash mismatch");
  uint64_t sum = 0;
  for (uint32_t i = 0; i < count; ++i) sum += 8ull * get<uint32_t>(f.data() + kHeaderBytes + (size_t)i * kRecordBytes);
  return sum == words ? OCC_OK : set_error(OCC_ERR_IO, "baked occluder file: packet counts do not match its header");
}

}  // namespace

extern "C" {

int occ_mesh_load_bin(const char* vertexPath, const char* indexPath, float* vertices, uint32_t* numVertices,
                      uint32_t* indices, uint32_t* numIndices)
{
  if (!vertexPath || !indexPath || !numVertices || !numIndices) return set_error(OCC_ERR_INVALID_ARG, "null argument");
  if (!host_little_endian()) return set_error(OCC_ERR_UNSUPPORTED, "big-endian host");
  std::vector<uint8_t> v, i;
  if (!read_file(vertexPath, v)) return set_error(OCC_ERR_IO, "cannot read the vertex file");
  if (!read_file(indexPath, i)) return set_error(OCC_ERR_IO, "cannot read the index file");
  // the demo ignores a ragged tail (size / sizeof element); a mesh file with
  // one is refused here instead
  if (v.size() % 16 || i.size() % 4 || v.size() / 16 > 0xFFFFFFFFull || i.size() / 4 > 0xFFFFFFFFull)
    return set_error(OCC_ERR_IO, "mesh file size is not a whole number of elements");
  const uint32_t nv = (uint32_t)(v.size() / 16), ni = (uint32_t)(i.size() / 4);
  if (vertices || indices) {
    if (!vertices || !indices || *numVertices < nv || *numIndices < ni)
      return set_error(OCC_ERR_INVALID_ARG, "mesh buffers missing or too small");
    if (nv) std::memcpy(vertices, v.data(), v.size());
    if (ni) std::memcpy(indices, i.data(), i.size());
  }
  *numVertices = nv;
  *numIndices = ni;
  return OCC_OK;
}

int occ_occluders_save(const char* path, uint32_t count, const uint32_t* packetCounts, const uint32_t* const* packed,
                       const float* bounds)
{
  if (!path || (count && (!packetCounts || !packed || !bounds))) return set_error(OCC_ERR_INVALID_ARG, "null argument");
  if (!host_little_endian()) return set_error(OCC_ERR_UNSUPPORTED, "big-endian host");
  uint64_t words = 0;
  for (uint32_t k = 0; k < count; ++k) {
    if (packetCounts[k] && !packed[k]) return set_error(OCC_ERR_INVALID_ARG, "null packed data");
    words += 8ull * packetCounts[k];
  }
  std::vector<uint8_t> out;
  out.reserve(kHeaderBytes + (size_t)count * kRecordBytes + 4 * words + 8);
  out.insert(out.end(), kMagic, kMagic + 8);
  put(out, kVersion);
  put(out, count);
  put(out, words);
  for (uint32_t k = 0; k < count; ++k) {
    put(out, packetCounts[k]);
    const uint32_t reserved[3] = {0, 0, 0};
    put(out, reserved);
    const uint8_t* b = reinterpret_cast<const uint8_t*>(bounds + 20 * (size_t)k);
    out.insert(out.end(), b, b + 80);
  }
  for (uint32_t k = 0; k < count; ++k) {
    const uint8_t* p = reinterpret_cast<const uint8_t*>(packed[k]);
    out.insert(out.end(), p, p + 32 * (size_t)packetCounts[k]);
  }
  put(out, fnv1a(out.data(), out.size()));
  const std::string tmp = std::string(path) + ".part";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return set_error(OCC_ERR_IO, "cannot create the file");
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return set_error(OCC_ERR_IO, "cannot write the file");
  }
  return OCC_OK;
}

int occ_occluders_file_info(const char* path, uint32_t* count, uint64_t* words)
{
  if (!path || !count || !words) return set_error(OCC_ERR_INVALID_ARG, "null argument");
  if (!host_little_endian()) return set_error(OCC_ERR_UNSUPPORTED, "big-endian host");
  std::vector<uint8_t> f;
  if (!read_file(path, f)) return set_error(OCC_ERR_IO, "cannot read the file");
  uint32_t c = 0;
  uint64_t w = 0;
  const int st = parse_baked(f, c, w);
  if (st != OCC_OK) return st;
  *count = c;
  *words = w;
  return OCC_OK;
}

int occ_occluders_load(const char* path, uint32_t capacityCount, uint64_t capacityWords, uint32_t* packetCounts,
                       uint32_t* packed, float* bounds)
{
  if (!path || !packetCounts || !packed || !bounds) return set_error(OCC_ERR_INVALID_ARG, "null argument");
  if (!host_little_endian()) return set_error(OCC_ERR_UNSUPPORTED, "big-endian host");
  std::vector<uint8_t> f;
  if (!read_file(path, f)) return set_error(OCC_ERR_IO, "cannot read the file");
  uint32_t c = 0;
  uint64_t w = 0;
  const int st = parse_baked(f, c, w);
  if (st != OCC_OK) return st;
  if (c > capacityCount || w > capacityWords) return set_error(OCC_ERR_INVALID_ARG, "buffers too small for the file");
  for (uint32_t k = 0; k < c; ++k) {
    const uint8_t* r = f.data() + kHeaderBytes + (size_t)k * kRecordBytes;
    packetCounts[k] = get<uint32_t>(r);
    std::memcpy(bounds + 20 * (size_t)k, r + 16, 80);
  }
  if (w) std::memcpy(packed, f.data() + kHeaderBytes + (size_t)c * kRecordBytes, 4 * w);
  return OCC_OK;
}

}  // extern "C"
