// Runs the reference coder's helper pipeline through the drop-in header
// include/HuffmanZSTDCoder.cuh, the way SimpleCudaHuffmanZstdCompressor::
// compress composes it (HuffmanZSTDCoder.cuh:248-357): cudaFrequencyCount,
// buildHuffmanTree, generateCodesRecursive, bit positions by a host scan of
// the code lengths, packBitsKernel, and the u64 words split big-endian into
// ceil(bits/8) bytes.  Also round-trips the stream through
// cudaHuffmanZstdCompress / cudaHuffmanZstdDecompress.
//
//   coder_helpers_driver <u8|u16|i8|i16> <symbols.bin> <out.bin>
//
// out.bin: u64 table entries, then entries x (i64 symbol, u32 code, i32
// length) in ascending symbol order, u64 root index, u64 byte count, the
// packed bytes, u8 round-trip flag.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <string>
#include <vector>

#include "HuffmanZSTDCoder.cuh"

template <typename T>
static int run(const std::vector<char> &raw, FILE *out) {
  std::vector<T> data(raw.size() / sizeof(T));
  std::memcpy(data.data(), raw.data(), data.size() * sizeof(T));
  thrust::device_vector<T> d = data;
  thrust::device_vector<T> syms;
  thrust::device_vector<uint32_t> freqs;
  cudaFrequencyCount(d, syms, freqs);
  thrust::device_vector<HuffmanNodeGPU<T>> nodes;
  int root = -1;
  buildHuffmanTree(syms, freqs, nodes, root);
  thrust::host_vector<HuffmanNodeGPU<T>> h_nodes = nodes;
  std::unordered_map<T, std::pair<uint32_t, int>> table;
  generateCodesRecursive(h_nodes, root, table, 0u, 0);
  // device code arrays in the order of the ascending symbols
  thrust::host_vector<T> h_syms = syms;
  std::vector<uint32_t> h_codes(h_syms.size());
  std::vector<int> h_lens(h_syms.size());
  for (size_t i = 0; i < h_syms.size(); ++i) {
    h_codes[i] = table[h_syms[i]].first;
    h_lens[i] = table[h_syms[i]].second;
  }
  std::vector<size_t> pos(data.size());
  size_t total = 0;
  for (size_t i = 0; i < data.size(); ++i) {
    pos[i] = total;
    total += (size_t)table[data[i]].second;
  }
  thrust::device_vector<uint32_t> d_codes(h_codes.begin(), h_codes.end());
  thrust::device_vector<int> d_lens(h_lens.begin(), h_lens.end());
  thrust::device_vector<size_t> d_pos(pos.begin(), pos.end());
  thrust::device_vector<uint64_t> d_words((total + 63) / 64, 0ull);
  const unsigned grid = (unsigned)((data.size() + 255) / 256);
  packBitsKernel<T><<<grid, 256>>>(thrust::raw_pointer_cast(d.data()), data.size(),
                                   thrust::raw_pointer_cast(syms.data()), thrust::raw_pointer_cast(d_codes.data()),
                                   thrust::raw_pointer_cast(d_lens.data()), h_syms.size(),
                                   thrust::raw_pointer_cast(d_words.data()), thrust::raw_pointer_cast(d_pos.data()));
  if (cudaDeviceSynchronize() != cudaSuccess) return 3;
  thrust::host_vector<uint64_t> words = d_words;
  std::vector<uint8_t> bytes;
  const size_t nbytes = (total + 7) / 8;
  for (size_t w = 0; w < words.size() && bytes.size() < nbytes; ++w)
    for (int j = 7; j >= 0 && bytes.size() < nbytes; --j) bytes.push_back((uint8_t)(words[w] >> (8 * j)));
  std::map<long long, std::pair<uint32_t, int>> sorted;
  for (auto &kv : table) sorted[(long long)kv.first] = kv.second;
  const uint64_t ne = sorted.size();
  fwrite(&ne, 8, 1, out);
  for (auto &kv : sorted) {
    const int64_t s = kv.first;
    const uint32_t c = kv.second.first;
    const int32_t l = kv.second.second;
    fwrite(&s, 8, 1, out);
    fwrite(&c, 4, 1, out);
    fwrite(&l, 4, 1, out);
  }
  const uint64_t r64 = (uint64_t)root, nb = bytes.size();
  fwrite(&r64, 8, 1, out);
  fwrite(&nb, 8, 1, out);
  fwrite(bytes.data(), 1, bytes.size(), out);
  // the drop-in class on the same stream
  auto res = cudaHuffmanZstdCompress(data, 3);
  std::vector<T> back =
      cudaHuffmanZstdDecompress(res.compressed_data, res.code_table, res.num_elements, res.original_bitstream_size);
  const uint8_t ok = (back == data && res.code_table == table && res.original_bitstream_size == nbytes) ? 1 : 0;
  fwrite(&ok, 1, 1, out);
  return 0;
}

int main(int argc, char **argv) {
  if (argc != 4) return 1;
  std::ifstream f(argv[2], std::ios::binary);
  std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  FILE *out = fopen(argv[3], "wb");
  if (!out) return 1;
  const std::string t = argv[1];
  int rc = t == "u8" ? run<uint8_t>(raw, out)
         : t == "u16" ? run<uint16_t>(raw, out)
         : t == "i8" ? run<int8_t>(raw, out)
         : t == "i16" ? run<int16_t>(raw, out) : 1;
  fclose(out);
  return rc;
}
