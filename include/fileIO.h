// Drop-in replacement of FFCz's fileIO.h (fileIO.h:1-55, fileIO.cpp:1-85):
// headerless raw arrays and the code-table map file, byte-compatible with
// the reference.  readRawArrayBinary / readMap are implemented in
// libffcz.so (ffcz_read_raw, ffcz_read_map); the writers are header
// templates as in the reference.
#pragma once

#include <cstdint>
#include <fstream>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ffcz.h"

enum class DataType { FLOAT, DOUBLE, SIZE_T, INT };

// fileIO.cpp:3-14: size_t n, then n x (int key, uint32 code, int len).
inline void writeMap(const std::map<int, std::pair<uint32_t, int>> &m, const std::string &filename) {
  std::vector<int32_t> k;
  std::vector<uint32_t> c;
  std::vector<int32_t> l;
  for (const auto &kv : m) {
    k.push_back(kv.first);
    c.push_back(kv.second.first);
    l.push_back(kv.second.second);
  }
  ffcz_write_map(filename.c_str(), k.data(), c.data(), l.data(), k.size());
}

// fileIO.cpp:16-33
inline std::map<int, std::pair<uint32_t, int>> readMap(const std::string &filename) {
  std::map<int, std::pair<uint32_t, int>> m;
  size_t n = 0;
  ffcz_read_map(filename.c_str(), nullptr, nullptr, nullptr, 0, &n);
  std::vector<int32_t> k(n), l(n);
  std::vector<uint32_t> c(n);
  if (n && ffcz_read_map(filename.c_str(), k.data(), c.data(), l.data(), n, &n) != FFCZ_OK) return m;
  for (size_t i = 0; i < n; ++i) m[k[i]] = {c[i], l[i]};
  return m;
}

// fileIO.cpp:35-76: the file must hold exactly N elements of `type`.
inline void readRawArrayBinary(const std::string &fileName, void *data, std::size_t N, DataType type) {
  std::size_t es;
  switch (type) {
    case DataType::FLOAT: es = sizeof(float); break;
    case DataType::DOUBLE: es = sizeof(double); break;
    case DataType::SIZE_T: es = sizeof(size_t); break;
    case DataType::INT: es = sizeof(int); break;
    default: throw std::invalid_argument("Invalid data type");
  }
  if (ffcz_read_raw(fileName.c_str(), data, N, es) != FFCZ_OK) throw std::runtime_error(ffcz_last_error());
}

// fileIO.h:23-44
template <typename T>
void writeRawArrayBinary(const T *data, size_t N, const std::string &filename) {
  static_assert(std::is_trivially_copyable<T>::value, "Type must be trivially copyable.");
  if (ffcz_write_raw(filename.c_str(), data, N, sizeof(T)) != FFCZ_OK)
    std::cerr << "Error: " << ffcz_last_error() << std::endl;
}

// fileIO.h:46-55
template <typename T>
void writeVectorBinary(const std::vector<T> &vec, const std::string &filename) {
  if (ffcz_write_raw(filename.c_str(), vec.data(), vec.size(), sizeof(T)) != FFCZ_OK)
    throw std::runtime_error("Could not open file: " + filename);
}
