// Device side of the Huffman encoder and its host driver.
#pragma once

#include "common.cuh"
#include "huffman_host.h"

namespace ffcz {

// Grow-only device/host scratch of one encoder instance.
struct HuffWorkspace {
  int device = -1;
  unsigned *d_hist = nullptr;               // 65536 bins
  unsigned long long *d_lut = nullptr;      // (len << 32) | code per symbol
  unsigned long long *d_blk = nullptr;      // per-block bit counts / offsets
  size_t blk_cap = 0;
  unsigned *d_out = nullptr;                // packed words
  size_t out_cap = 0;                       // words
  unsigned *h_hist = nullptr;               // pinned
  unsigned long long *h_lut = nullptr;      // pinned
  uint8_t *h_bits = nullptr;                // pinned
  size_t hbits_cap = 0;
  long long launches = 0;
  ~HuffWorkspace();
};

// Encodes n symbols (symbol_bytes = 1 or 2) resident on the device into
// `res` (codebook + bitstream, ZSTD when level >= 0).  Runs on `stream`;
// returns after the bitstream is on the host.
int huff_encode_device(HuffWorkspace &ws, const void *d_data, size_t n, int symbol_bytes,
                       cudaStream_t stream, ffcz_huff_result &res);
// ZSTD stage of an encoded result (res.bitstream -> res.compressed).
int huff_zstd(ffcz_huff_result &res, int level, int mode);

}  // namespace ffcz
