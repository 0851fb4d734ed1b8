// TEST INFRASTRUCTURE ONLY: runs the reference FFCz coder's host functions
// (HuffmanZSTDCoder.cuh, compiled from the reference sources with thrust on
// its CPP backend, so no GPU is needed) and fileIO.cpp, to pin the oracle
// and the library against the reference itself.
//
//   ref_harness book   <u8|u16> <symbols.bin> <table.bin>
//       cudaFrequencyCount + buildHuffmanTree + generateCodesRecursive
//       (HuffmanZSTDCoder.cuh:48-178); table = n x (u32 sym, u32 code, i32 len)
//       in ascending symbol order.
//   ref_harness decode <u8|u16> <bits.bin> <table.bin> <num_elements> <out.bin>
//       ZSTD_compress(level 3) of the bitstream, then
//       SimpleCudaHuffmanZstdCompressor<T>::decompress (:378-450).
//   ref_harness map    <table.bin> <out.map>
//       writeMap (fileIO.cpp:3-14) of {int(sym): (code, len)}.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <map>
#include <string>
#include <vector>

// thrust's sequential (CPP) sort keeps an unguarded `throw` in a
// host/device allocator that nvcc rejects; this more specialised overload
// routes the reference's thrust::sort(thrust::device, ...) of
// cudaFrequencyCount (HuffmanZSTDCoder.cuh:59) to std::sort on the same
// host-resident range.  The sorted order is the same.
#include <algorithm>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>
namespace thrust {
template <typename T, typename Policy>
void sort(const thrust::detail::execution_policy_base<Policy> &,
          thrust::detail::normal_iterator<thrust::device_ptr<T>> first,
          thrust::detail::normal_iterator<thrust::device_ptr<T>> last) {
  T *b = thrust::raw_pointer_cast(&*first);
  std::sort(b, b + (last - first));
}
}  // namespace thrust

#include "HuffmanZSTDCoder.cuh"
#include "fileIO.h"

static std::vector<char> slurp(const char *p) {
  std::ifstream f(p, std::ios::binary);
  return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

struct Entry { uint32_t sym, code; int32_t len; };

static std::vector<Entry> read_table(const char *p) {
  std::vector<char> raw = slurp(p);
  std::vector<Entry> t(raw.size() / sizeof(Entry));
  memcpy(t.data(), raw.data(), t.size() * sizeof(Entry));
  return t;
}

template <typename T>
static int book(const char *in, const char *out) {
  std::vector<char> raw = slurp(in);
  std::vector<T> data(raw.size() / sizeof(T));
  memcpy(data.data(), raw.data(), data.size() * sizeof(T));
  thrust::device_vector<T> d = data;
  thrust::device_vector<T> syms;
  thrust::device_vector<uint32_t> freqs;
  cudaFrequencyCount(d, syms, freqs);
  thrust::device_vector<HuffmanNodeGPU<T>> nodes;
  int root = -1;
  buildHuffmanTree(syms, freqs, nodes, root);
  thrust::host_vector<HuffmanNodeGPU<T>> h = nodes;
  std::unordered_map<T, std::pair<uint32_t, int>> table;
  generateCodesRecursive(h, root, table, 0, 0);
  std::map<uint32_t, std::pair<uint32_t, int>> sorted;
  for (auto &kv : table) sorted[(uint32_t)kv.first] = kv.second;
  std::ofstream f(out, std::ios::binary);
  for (auto &kv : sorted) {
    Entry e{kv.first, kv.second.first, kv.second.second};
    f.write((const char *)&e, sizeof(e));
  }
  return 0;
}

template <typename T>
static int decode(const char *bitsp, const char *tabp, size_t nel, const char *out) {
  std::vector<char> bits = slurp(bitsp);
  size_t bound = ZSTD_compressBound(bits.size());
  std::vector<uint8_t> comp(bound);
  size_t cs = ZSTD_compress(comp.data(), bound, bits.data(), bits.size(), 3);
  if (ZSTD_isError(cs)) return 2;
  comp.resize(cs);
  std::unordered_map<T, std::pair<uint32_t, int>> table;
  for (const Entry &e : read_table(tabp)) table[(T)e.sym] = {e.code, e.len};
  SimpleCudaHuffmanZstdCompressor<T> c;
  std::vector<T> dec = c.decompress(comp, table, nel, bits.size());
  std::ofstream f(out, std::ios::binary);
  f.write((const char *)dec.data(), dec.size() * sizeof(T));
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) return 1;
  const std::string mode = argv[1];
  if (mode == "book" && argc == 5) {
    return std::string(argv[2]) == "u8" ? book<uint8_t>(argv[3], argv[4]) : book<uint16_t>(argv[3], argv[4]);
  }
  if (mode == "decode" && argc == 7) {
    const size_t nel = std::strtoull(argv[5], nullptr, 10);
    return std::string(argv[2]) == "u8" ? decode<uint8_t>(argv[3], argv[4], nel, argv[6])
                                        : decode<uint16_t>(argv[3], argv[4], nel, argv[6]);
  }
  if (mode == "map" && argc == 4) {
    std::map<int, std::pair<uint32_t, int>> m;
    for (const Entry &e : read_table(argv[2])) m[(int)e.sym] = {e.code, e.len};
    writeMap(m, argv[3]);
    return 0;
  }
  return 1;
}
