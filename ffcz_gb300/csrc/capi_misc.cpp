// Error reporting of the C ABI and the file formats of fileIO.h / fileIO.cpp.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "../../include/ffcz.h"

namespace ffcz {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  g_last_error = std::string("CUDA error at ") + file + ":" + std::to_string(line) + " - " +
                 cudaGetErrorString(e) + " (" + what + ")";
  return FFCZ_ERR_CUDA;
}

}  // namespace ffcz

using ffcz::fail;

extern "C" {

const char *ffcz_last_error(void) { return ffcz::g_last_error.c_str(); }

const char *ffcz_version(void) { return "ffcz-gb300 0.1.0 (sm_103a)"; }

int ffcz_read_raw(const char *path, void *dst, size_t n, size_t elem_bytes) {
  if (!path || (!dst && n)) return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return fail(FFCZ_ERR_IO, "Error opening file");
  const std::streamsize size = f.tellg();
  f.seekg(0, std::ios::beg);
  if (size != (std::streamsize)(n * elem_bytes)) return fail(FFCZ_ERR_IO, "File size does not match array size");
  if (size && !f.read(reinterpret_cast<char *>(dst), size)) return fail(FFCZ_ERR_IO, "Error reading file");
  return FFCZ_OK;
}

int ffcz_write_raw(const char *path, const void *src, size_t n, size_t elem_bytes) {
  if (!path || (!src && n)) return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(FFCZ_ERR_IO, "Could not open file for writing");
  f.write(reinterpret_cast<const char *>(src), (std::streamsize)(n * elem_bytes));
  if (!f) return fail(FFCZ_ERR_IO, "Failed to write to file");
  return FFCZ_OK;
}

int ffcz_write_map(const char *path, const int32_t *keys, const uint32_t *codes, const int32_t *lens, size_t n) {
  if (!path || (n && (!keys || !codes || !lens))) return fail(FFCZ_ERR_INVALID, "NULL argument");
  // std::map order: ascending keys, duplicates collapse to the last value.
  std::map<int32_t, std::pair<uint32_t, int32_t>> m;
  for (size_t i = 0; i < n; ++i) m[keys[i]] = {codes[i], lens[i]};
  std::ofstream f(path, std::ios::binary);
  if (!f) return fail(FFCZ_ERR_IO, "Could not open file for writing");
  const size_t size = m.size();
  f.write(reinterpret_cast<const char *>(&size), sizeof(size));
  for (const auto &kv : m) {
    f.write(reinterpret_cast<const char *>(&kv.first), sizeof(int32_t));
    f.write(reinterpret_cast<const char *>(&kv.second.first), sizeof(uint32_t));
    f.write(reinterpret_cast<const char *>(&kv.second.second), sizeof(int32_t));
  }
  if (!f) return fail(FFCZ_ERR_IO, "Failed to write to file");
  return FFCZ_OK;
}

int ffcz_read_map(const char *path, int32_t *keys, uint32_t *codes, int32_t *lens, size_t cap, size_t *n) {
  if (!path || !n) return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(FFCZ_ERR_IO, "Error opening file");
  size_t size = 0;
  if (!f.read(reinterpret_cast<char *>(&size), sizeof(size))) return fail(FFCZ_ERR_IO, "Error reading file");
  *n = size;
  if (size > cap) return fail(FFCZ_ERR_CAPACITY, "destination too small");
  if (size && (!keys || !codes || !lens)) return fail(FFCZ_ERR_INVALID, "NULL argument");
  for (size_t i = 0; i < size; ++i) {
    if (!f.read(reinterpret_cast<char *>(&keys[i]), 4) || !f.read(reinterpret_cast<char *>(&codes[i]), 4) ||
        !f.read(reinterpret_cast<char *>(&lens[i]), 4))
      return fail(FFCZ_ERR_IO, "Error reading file");
  }
  return FFCZ_OK;
}

}  // extern "C"
