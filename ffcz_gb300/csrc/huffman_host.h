// Host parts of the Huffman + ZSTD coder: codebook construction with the
// reference's tie-breaking, prefix decoding with the reference's stop and
// skip rules, and libzstd access (loaded at run time).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

struct ffcz_huff_result {
  std::vector<uint8_t> compressed;   // ZSTD frame(s)
  std::vector<uint8_t> bitstream;    // MSB-first Huffman bits, zero padded
  std::vector<uint32_t> symbols;     // ascending
  std::vector<uint32_t> codes;
  std::vector<int32_t> lengths;
  size_t num_elements = 0;
};

namespace ffcz {

struct Codebook {
  std::vector<uint32_t> sym, freq, code;
  std::vector<int32_t> len;
  int max_len = 0;
};

// Codebook of HuffmanZSTDCoder.cuh:48-178 from a dense histogram: symbols
// with non-zero count in ascending order are the leaves 0..n-1; internal
// nodes n.. are created in merge order; the two smallest (freq, node index)
// pairs are merged, the first becoming the 0 branch; codes are read from
// the root MSB-first in 32-bit words (longer codes keep their low 32 bits,
// as the reference's uint32 shift does); one symbol gets code 0, length 1.
void build_codebook(const uint32_t *hist, size_t nbins, Codebook &cb);
// The tree of that codebook in the reference's node numbering
// (HuffmanZSTDCoder.cuh:85-152): leaves 0..n-1 with weights freq[0..n-1],
// internal nodes n..2n-2 in merge order, left = the first of the two
// popped nodes, -1 for no child; the root is 2n-2 (0 for one leaf).
void build_tree(const uint32_t *freq, int n, std::vector<int> &left, std::vector<int> &right,
                std::vector<uint64_t> &wt);

// Prefix decode of HuffmanZSTDCoder.cuh:394-449 over `bits` bytes: stops at
// num_elements symbols or at the end of the stream; where no code of length
// 1..32 matches, one bit is skipped.  A stored code of 2^L or more never
// matches (the reference keys on length << 32 | code); of entries with the
// same (length, code) the first wins (the reference leaves this to its hash
// map's iteration order).  Returns the decoded symbols.
std::vector<uint32_t> huffman_decode(const uint8_t *bits, size_t nbytes, const uint32_t *symbols,
                                     const uint32_t *codes, const int32_t *lengths, size_t nsym,
                                     size_t num_elements);

// libzstd entry points, resolved with dlopen("libzstd.so.1").
bool zstd_available(std::string *why);
// ZSTD_compress(level) of the whole buffer, or (chunked) independent frames
// of about size/threads bytes compressed on host threads and concatenated.
int zstd_compress(const uint8_t *src, size_t n, int level, bool chunked, std::vector<uint8_t> &out);
// Upper bound of zstd_compress's output in either mode (0 without libzstd).
size_t zstd_bound(size_t n);
// ZSTD_decompress into exactly `expect` bytes.
int zstd_decompress(const uint8_t *src, size_t n, size_t expect, std::vector<uint8_t> &out);

}  // namespace ffcz
