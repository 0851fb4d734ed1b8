// Drop-in replacement of FFCz's HuffmanZSTDCoder.cuh (HuffmanZSTDCoder.cuh:
// 1-470): SimpleCudaHuffmanZstdCompressor<T>, its CompressionResult and the
// free functions cudaHuffmanZstdCompress / cudaHuffmanZstdDecompress, backed
// by libffcz.so.  Histogram, code lengths, bit offsets and bit packing run on
// the GPU; the codebook and ZSTD run on the host, as in the reference.
//
// Supported symbol types: uint8_t and uint16_t (the two the reference CLI
// uses, projection_example.cu:235-244).  Errors throw std::runtime_error
// with the reference's messages where it has one ("Empty data", "ZSTD
// compression failed: ...").  Codes longer than 32 bits, which the
// reference's uint32 codes cannot represent (HuffmanZSTDCoder.cuh:175-176),
// throw instead of producing an undecodable stream.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "ffcz.h"

template <typename T>
class SimpleCudaHuffmanZstdCompressor {
  static_assert(std::is_same<T, uint8_t>::value || std::is_same<T, uint16_t>::value,
                "symbols are uint8_t or uint16_t");

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
    int rc = sizeof(T) == 2 ? ffcz_huff_compress_u16((const uint16_t *)data.data(), data.size(), zstd_level, &r)
                            : ffcz_huff_compress_u8((const uint8_t *)data.data(), data.size(), zstd_level, &r);
    if (rc != FFCZ_OK) throw std::runtime_error(ffcz_last_error());
    CompressionResult out;
    size_t comp = 0, bits = 0, nel = 0, nsym = 0;
    ffcz_huff_result_sizes(r, &comp, &bits, &nel, &nsym);
    out.compressed_data.resize(comp);
    ffcz_huff_result_compressed(r, out.compressed_data.data(), comp);
    std::vector<uint32_t> sym(nsym), code(nsym);
    std::vector<int32_t> len(nsym);
    if (nsym) ffcz_huff_result_codes(r, sym.data(), code.data(), len.data(), nsym);
    for (size_t i = 0; i < nsym; ++i) out.code_table[(T)sym[i]] = {code[i], (int)len[i]};
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
      sym.push_back(kv.first);
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
