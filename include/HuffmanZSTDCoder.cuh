// Drop-in replacement of FFCz's HuffmanZSTDCoder.cuh (HuffmanZSTDCoder.cuh:
// 1-470): SimpleCudaHuffmanZstdCompressor<T>, its CompressionResult, the
// free functions cudaHuffmanZstdCompress / cudaHuffmanZstdDecompress and,
// for nvcc translation units, the helper templates HuffmanNodeGPU,
// cudaFrequencyCount, buildHuffmanTree, generateCodesRecursive and
// packBitsKernel, backed by libffcz.so.  Histogram, code lengths, bit
// offsets and bit packing run on the GPU; the codebook and ZSTD run on the
// host, as in the reference.
//
// Symbol types: 8- and 16-bit integers, signed or unsigned (the reference
// CLI uses uint16_t and uint8_t, projection_example.cu:235-244).  Signed
// symbols are coded through an order-preserving map to the unsigned type,
// so the codebook (whose ties break by ascending symbol) is the one the
// reference builds.  Errors throw std::runtime_error with the reference's
// messages where it has one ("Empty data", "ZSTD compression failed: ...").
// Codes longer than 32 bits, which the reference's uint32 codes cannot
// represent (HuffmanZSTDCoder.cuh:175-176), throw instead of producing an
// undecodable stream.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "ffcz.h"

namespace ffcz_coder_detail {
// Order-preserving map of an 8/16-bit symbol type onto its unsigned type.
template <typename T>
struct SymbolMap {
  static_assert(std::is_integral<T>::value && (sizeof(T) == 1 || sizeof(T) == 2),
                "symbols are 8- or 16-bit integers");
  using U = typename std::conditional<sizeof(T) == 1, uint8_t, uint16_t>::type;
  static constexpr U flip = std::is_signed<T>::value ? (U)(U(1) << (8 * sizeof(T) - 1)) : U(0);
  static U to_u(T v) { return (U)((U)v ^ flip); }
  static T from_u(uint32_t u) { return (T)(U)((U)u ^ flip); }
};
}  // namespace ffcz_coder_detail

template <typename T>
class SimpleCudaHuffmanZstdCompressor {
  using Map = ffcz_coder_detail::SymbolMap<T>;
  using U = typename Map::U;

 public:
  // HuffmanZSTDCoder.cuh:240-246
  struct CompressionResult {
    std::vector<uint8_t> compressed_data;
    std::unordered_map<T, std::pair<uint32_t, int>> code_table;
    size_t original_bitstream_size;
    size_t num_elements;
  };

  // HuffmanZSTDCoder.cuh:248-376
  CompressionResult compress(const std::vector<T> &data, int zstd_level = 3) {
    if (data.empty()) throw std::runtime_error("Empty data");
    ffcz_huff_result *r = nullptr;
    std::vector<U> mapped;
    const U *src = reinterpret_cast<const U *>(data.data());
    if (Map::flip) {
      mapped.resize(data.size());
      for (size_t i = 0; i < data.size(); ++i) mapped[i] = Map::to_u(data[i]);
      src = mapped.data();
    }
    int rc = sizeof(T) == 2 ? ffcz_huff_compress_u16((const uint16_t *)src, data.size(), zstd_level, &r)
                            : ffcz_huff_compress_u8((const uint8_t *)src, data.size(), zstd_level, &r);
    if (rc != FFCZ_OK) throw std::runtime_error(ffcz_last_error());
    CompressionResult out;
    size_t comp = 0, bits = 0, nel = 0, nsym = 0;
    ffcz_huff_result_sizes(r, &comp, &bits, &nel, &nsym);
    out.compressed_data.resize(comp);
    ffcz_huff_result_compressed(r, out.compressed_data.data(), comp);
    std::vector<uint32_t> sym(nsym), code(nsym);
    std::vector<int32_t> len(nsym);
    if (nsym) ffcz_huff_result_codes(r, sym.data(), code.data(), len.data(), nsym);
    for (size_t i = 0; i < nsym; ++i) out.code_table[Map::from_u(sym[i])] = {code[i], (int)len[i]};
    out.original_bitstream_size = bits;
    out.num_elements = nel;
    ffcz_huff_result_free(r);
    return out;
  }

  // HuffmanZSTDCoder.cuh:378-450
  std::vector<T> decompress(const std::vector<uint8_t> &compressed_data,
                            const std::unordered_map<T, std::pair<uint32_t, int>> &code_table, size_t num_elements,
                            size_t original_bitstream_size) {
    std::vector<uint32_t> sym, code;
    std::vector<int32_t> len;
    for (const auto &kv : code_table) {
      sym.push_back(Map::to_u(kv.first));
      code.push_back(kv.second.first);
      len.push_back(kv.second.second);
    }
    std::vector<T> out(num_elements);
    size_t got = 0;
    int rc = sizeof(T) == 2
                 ? ffcz_huff_decompress_u16(compressed_data.data(), compressed_data.size(), sym.data(), code.data(),
                                            len.data(), sym.size(), num_elements, original_bitstream_size,
                                            (uint16_t *)out.data(), &got)
                 : ffcz_huff_decompress_u8(compressed_data.data(), compressed_data.size(), sym.data(), code.data(),
                                           len.data(), sym.size(), num_elements, original_bitstream_size,
                                           (uint8_t *)out.data(), &got);
    if (rc != FFCZ_OK) throw std::runtime_error(ffcz_last_error());
    out.resize(got);
    if (Map::flip)
      for (T &v : out) v = Map::from_u((uint32_t)(U)v);
    return out;
  }
};

// HuffmanZSTDCoder.cuh:454-470
template <typename T>
typename SimpleCudaHuffmanZstdCompressor<T>::CompressionResult cudaHuffmanZstdCompress(const std::vector<T> &data,
                                                                                      int zstd_level = 3) {
  SimpleCudaHuffmanZstdCompressor<T> c;
  return c.compress(data, zstd_level);
}

template <typename T>
std::vector<T> cudaHuffmanZstdDecompress(const std::vector<uint8_t> &compressed_data,
                                         const std::unordered_map<T, std::pair<uint32_t, int>> &code_table,
                                         size_t num_elements, size_t original_bitstream_size) {
  SimpleCudaHuffmanZstdCompressor<T> c;
  return c.decompress(compressed_data, code_table, num_elements, original_bitstream_size);
}

#ifdef __CUDACC__
#include <thrust/device_vector.h>
#include <thrust/host_vector.h>

// HuffmanZSTDCoder.cuh:32-46: a node of the Huffman tree (leaves hold a
// symbol; -1 marks a missing child).
template <typename T>
struct HuffmanNodeGPU {
  T value;
  uint32_t freq;
  int left, right;
  __host__ __device__ HuffmanNodeGPU() : value(), freq(0), left(-1), right(-1) {}
  __host__ __device__ HuffmanNodeGPU(T val, uint32_t f) : value(val), freq(f), left(-1), right(-1) {}
  __host__ __device__ bool is_leaf() const { return left == -1 && right == -1; }
};

// HuffmanZSTDCoder.cuh:48-83: the distinct symbols of `data` in ascending
// order and their counts, from the GPU histogram (ffcz_huff_histogram_device)
// instead of a device sort.
template <typename T>
void cudaFrequencyCount(const thrust::device_vector<T> &data, thrust::device_vector<T> &unique_values,
                        thrust::device_vector<uint32_t> &frequencies) {
  using Map = ffcz_coder_detail::SymbolMap<T>;
  if (data.empty()) return;
  const size_t nbins = sizeof(T) == 1 ? 256 : 65536;
  std::vector<uint32_t> hist(nbins);
  const void *d = thrust::raw_pointer_cast(data.data());
  thrust::device_vector<T> aligned;
  if (((uintptr_t)d) & 15) {  // the histogram reads 16-byte vectors
    aligned = data;
    d = thrust::raw_pointer_cast(aligned.data());
  }
  if (ffcz_huff_histogram_device(d, data.size(), (int)sizeof(T), nullptr, hist.data()) != FFCZ_OK)
    throw std::runtime_error(ffcz_last_error());
  // bins in the order of the symbols' values (signed types start at the
  // bin of their most negative value)
  std::vector<T> vals;
  std::vector<uint32_t> cnts;
  for (size_t u = 0; u < nbins; ++u) {
    const T v = Map::from_u((uint32_t)u);
    const size_t bin = (size_t)(typename Map::U)v;
    if (hist[bin]) {
      vals.push_back(v);
      cnts.push_back(hist[bin]);
    }
  }
  unique_values.assign(vals.begin(), vals.end());
  frequencies.assign(cnts.begin(), cnts.end());
}

// HuffmanZSTDCoder.cuh:85-152: the tree with the reference's node numbering
// and tie-breaking (ffcz_huff_tree); leaves 0..n-1 are the given symbols.
template <typename T>
void buildHuffmanTree(const thrust::device_vector<T> &symbols, const thrust::device_vector<uint32_t> &frequencies,
                      thrust::device_vector<HuffmanNodeGPU<T>> &nodes, int &root_idx) {
  thrust::host_vector<T> h_sym = symbols;
  thrust::host_vector<uint32_t> h_freq = frequencies;
  const size_t n = h_sym.size();
  if (n == 0) {
    root_idx = -1;
    return;
  }
  const size_t m = 2 * n - 1;
  std::vector<int32_t> left(m), right(m);
  std::vector<uint64_t> wt(m);
  std::vector<uint32_t> f(h_freq.begin(), h_freq.end());
  int32_t root = -1;
  if (ffcz_huff_tree(f.data(), n, left.data(), right.data(), wt.data(), &root) != FFCZ_OK)
    throw std::runtime_error(ffcz_last_error());
  thrust::host_vector<HuffmanNodeGPU<T>> h(m);
  for (size_t i = 0; i < m; ++i) {
    h[i].value = i < n ? h_sym[i] : T();
    h[i].freq = (uint32_t)wt[i];
    h[i].left = left[i];
    h[i].right = right[i];
  }
  nodes = h;
  root_idx = root;
}

// HuffmanZSTDCoder.cuh:154-178: codes read from the root, 0 for the left
// branch, MSB first; a lone leaf gets code 0 of length 1.
template <typename T>
void generateCodesRecursive(const thrust::host_vector<HuffmanNodeGPU<T>> &nodes, int node_idx,
                            std::unordered_map<T, std::pair<uint32_t, int>> &code_table, uint32_t code,
                            int length) {
  if (node_idx < 0) return;
  const HuffmanNodeGPU<T> &nd = nodes[node_idx];
  if (nd.is_leaf()) {
    code_table[nd.value] = {code, length ? length : 1};
    return;
  }
  generateCodesRecursive(nodes, nd.left, code_table, code << 1, length + 1);
  generateCodesRecursive(nodes, nd.right, code_table, (code << 1) | 1u, length + 1);
}

// HuffmanZSTDCoder.cuh:180-233: ORs the code of data[i] into the u64 words
// of `output` MSB first from bit bit_positions[i] (a code may straddle two
// words).  The symbol is found by binary search when `symbols` ascends (as
// cudaFrequencyCount returns them), else by a linear scan, as the reference
// does; a symbol missing from the table packs code 0 of length 1.
template <typename T>
__global__ void packBitsKernel(const T *data, size_t data_size, const T *symbols, const uint32_t *codes,
                               const int *lengths, size_t num_symbols, uint64_t *output, size_t *bit_positions) {
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (tid >= data_size) return;
  const T value = data[tid];
  size_t lo = 0, hi = num_symbols;
  while (lo < hi) {
    const size_t mid = (lo + hi) / 2;
    if (symbols[mid] < value) lo = mid + 1;
    else hi = mid;
  }
  size_t at = num_symbols;
  if (lo < num_symbols && symbols[lo] == value) {
    at = lo;
  } else {
    for (size_t i = 0; i < num_symbols; ++i)
      if (symbols[i] == value) {
        at = i;
        break;
      }
  }
  const uint32_t code = at < num_symbols ? codes[at] : 0u;
  const int length = at < num_symbols ? lengths[at] : 1;
  const size_t bit_pos = bit_positions[tid];
  const size_t word = bit_pos / 64;
  const int off = (int)(bit_pos % 64);
  if (length <= 0 || length > 64) return;
  if (off + length <= 64) {
    atomicOr((unsigned long long *)&output[word], (unsigned long long)code << (64 - off - length));
  } else {
    const int first = 64 - off, second = length - first;
    atomicOr((unsigned long long *)&output[word], (unsigned long long)(second >= 32 ? 0u : code >> second));
    atomicOr((unsigned long long *)&output[word + 1],
             ((unsigned long long)code & ((1ull << second) - 1ull)) << (64 - second));
  }
}
#endif  // __CUDACC__
