// The .ffcz container: one file holding what the decoder needs besides x' --
// the field's shape and type, the bounds, the edit arrays' min/max, and the
// four Huffman+ZSTD streams with their code tables (the table layout is the
// one writeMap uses, fileIO.cpp:3-33).  Little-endian:
//
//    0  char[4] "FFCZ", uint32 version (1)
//    8  uint32 dtype (FFCZ_F32 / FFCZ_F64), uint32 flag-pack mode
//   16  uint64 nx, ny, nz
//   40  double eps, delta, freq_min, freq_max, spatial_min, spatial_max
//   88  uint32 iterations, uint32 stream mask (bit i: stream i present)
//   96  per present stream, in the order frequency codes, frequency flag
//       pack, spatial codes, spatial flag pack:
//         uint64 num_elements, bitstream_bytes, compressed_bytes
//         uint64 n, then n x (int32 symbol, uint32 code, int32 length)
//         compressed bytes (one ZSTD frame or concatenated frames)
#include <algorithm>
#include <cstring>
#include <fstream>
#include <memory>
#include <vector>

#include <string>

#include "../../include/ffcz.h"
#include "huffman_host.h"

namespace ffcz {
int fail(int code, const std::string &msg);
}
using namespace ffcz;

#define FFCZ_TRY(call)        \
  do {                        \
    int rc_ = (call);         \
    if (rc_ != FFCZ_OK) return rc_; \
  } while (0)

namespace {

constexpr char kMagic[4] = {'F', 'F', 'C', 'Z'};
constexpr uint32_t kVersion = 1;

template <typename V>
void put(std::vector<uint8_t> &b, const V &v) {
  const uint8_t *p = reinterpret_cast<const uint8_t *>(&v);
  b.insert(b.end(), p, p + sizeof(V));
}

struct Reader {
  const std::vector<uint8_t> &b;
  size_t at = 0;
  template <typename V>
  bool get(V &v) {
    if (b.size() - at < sizeof(V)) return false;
    std::memcpy(&v, b.data() + at, sizeof(V));
    at += sizeof(V);
    return true;
  }
  bool bytes(size_t n, std::vector<uint8_t> &out) {
    if (b.size() - at < n) return false;
    out.assign(b.begin() + at, b.begin() + at + n);
    at += n;
    return true;
  }
};

}  // namespace

extern "C" {

int ffcz_container_write(const char *path, const ffcz_container_header *h, ffcz_huff_result *const *in4) {
  if (!path || !h || !in4) return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::vector<uint8_t> b;
  b.insert(b.end(), kMagic, kMagic + 4);
  put(b, kVersion);
  put(b, h->dtype);
  put(b, h->pack_mode);
  put(b, h->nx);
  put(b, h->ny);
  put(b, h->nz);
  for (double v : {h->eps, h->delta, h->freq_min, h->freq_max, h->spatial_min, h->spatial_max}) put(b, v);
  put(b, h->iterations);
  uint32_t mask = 0;
  for (int i = 0; i < 4; ++i) {
    if (!in4[i]) continue;
    if (in4[i]->compressed.empty() && !in4[i]->bitstream.empty())
      return fail(FFCZ_ERR_INVALID, "stream has no ZSTD frame (encoded with FFCZ_ZSTD_NONE)");
    mask |= 1u << i;
  }
  put(b, mask);
  for (int i = 0; i < 4; ++i) {
    const ffcz_huff_result *r = in4[i];
    if (!r) continue;
    put(b, (uint64_t)r->num_elements);
    put(b, (uint64_t)r->bitstream.size());
    put(b, (uint64_t)r->compressed.size());
    put(b, (uint64_t)r->symbols.size());
    for (size_t k = 0; k < r->symbols.size(); ++k) {
      put(b, (int32_t)r->symbols[k]);
      put(b, (uint32_t)r->codes[k]);
      put(b, (int32_t)r->lengths[k]);
    }
    b.insert(b.end(), r->compressed.begin(), r->compressed.end());
  }
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(FFCZ_ERR_IO, "Could not open file for writing");
  f.write(reinterpret_cast<const char *>(b.data()), (std::streamsize)b.size());
  if (!f) return fail(FFCZ_ERR_IO, "Failed to write to file");
  return FFCZ_OK;
}

int ffcz_container_read(const char *path, ffcz_container_header *h, ffcz_huff_result **out4) {
  if (!path || !h || !out4) return fail(FFCZ_ERR_INVALID, "NULL argument");
  for (int i = 0; i < 4; ++i) out4[i] = nullptr;
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return fail(FFCZ_ERR_IO, "Error opening file");
  const std::streamsize size = f.tellg();
  f.seekg(0);
  std::vector<uint8_t> b((size_t)std::max<std::streamsize>(size, 0));
  if (size > 0 && !f.read(reinterpret_cast<char *>(b.data()), size)) return fail(FFCZ_ERR_IO, "Error reading file");
  Reader r{b};
  char magic[4];
  uint32_t version = 0, mask = 0;
  bool ok = r.get(magic) && std::memcmp(magic, kMagic, 4) == 0 && r.get(version);
  if (!ok || version != kVersion) return fail(FFCZ_ERR_IO, "not an FFCZ container (version 1)");
  ffcz_container_header hh{};
  ok = r.get(hh.dtype) && r.get(hh.pack_mode) && r.get(hh.nx) && r.get(hh.ny) && r.get(hh.nz) && r.get(hh.eps) &&
       r.get(hh.delta) && r.get(hh.freq_min) && r.get(hh.freq_max) && r.get(hh.spatial_min) &&
       r.get(hh.spatial_max) && r.get(hh.iterations) && r.get(mask);
  if (!ok) return fail(FFCZ_ERR_IO, "truncated container header");
  std::unique_ptr<ffcz_huff_result> res[4];
  for (int i = 0; i < 4; ++i) {
    if (!(mask & (1u << i))) continue;
    uint64_t ne = 0, bb = 0, cb = 0, n = 0;
    if (!(r.get(ne) && r.get(bb) && r.get(cb) && r.get(n)) || n > (b.size() - r.at) / 12)
      return fail(FFCZ_ERR_IO, "truncated container stream");
    std::unique_ptr<ffcz_huff_result> x(new ffcz_huff_result());
    x->symbols.resize(n);
    x->codes.resize(n);
    x->lengths.resize(n);
    for (uint64_t k = 0; k < n; ++k) {
      int32_t s = 0, l = 0;
      uint32_t c = 0;
      r.get(s);
      r.get(c);
      r.get(l);
      x->symbols[k] = (uint32_t)s;
      x->codes[k] = c;
      x->lengths[k] = l;
    }
    if (!r.bytes(cb, x->compressed)) return fail(FFCZ_ERR_IO, "truncated container stream");
    FFCZ_TRY(zstd_decompress(x->compressed.data(), x->compressed.size(), bb, x->bitstream));
    x->bitstream.resize(bb, 0);
    x->num_elements = ne;
    res[i] = std::move(x);
  }
  *h = hh;
  for (int i = 0; i < 4; ++i) out4[i] = res[i].release();
  return FFCZ_OK;
}

}  // extern "C"
