// Decoder side: GPU prefix decoding of the Huffman bitstreams, and the
// kernels that turn decoded edit streams back into a corrected field:
// flag pack + uint16 codes -> dequantised edits at their flat indices, the
// frequency edits scattered straight into the padded half spectrum, and the
// final sum x^ = x' + (C2R(freq edits)/N + spatial edits).
#pragma once

#include "common.cuh"

namespace ffcz {

// ------------------------------------------------------ Huffman decoding --
// Segmented self-synchronising decode.  The bitstream is cut into segments
// of kSegBits bits (one thread each); each segment is decoded from an entry bit position up
// to the first step boundary at or past the next segment's start.  Entry
// positions are iterated to the fixed point of "entry[k] = end[k-1]"
// (entry[0] = 0), which is the sequential decoder's path; a segment whose
// entry did not change is not decoded again.  Each decode step is the
// sequential decoder's: walk the code trie MSB-first from the step's first
// bit; at the first leaf emit its symbol; where a bit has no child, the
// stream ends, or 32 bits pass without a leaf, skip one bit.
constexpr int kLutBitsMax = 14;   // up to 2^14 table entries (64 KB of shared memory)
constexpr int kSegBits = 512;

// Device image of a code table: trie nodes (children for bit 0 / bit 1, -1
// when absent), the symbol index of each node that ends a code (-1
// otherwise), and a 2^lut_bits table of the walk over the next lut_bits
// bits: EMIT (symbol index, length), SKIP, or CONT (node reached after
// lut_bits bits, no leaf on the way).  lut_bits = the longest code, within
// [8, kLutBitsMax], so that codes longer than the table are rare.
struct DecodeTables {
  int nnodes = 0;
  int lut_bits = 8;
  int2 *child = nullptr;
  int *leaf = nullptr;
  unsigned *lut = nullptr;
  uint32_t *symbols = nullptr;
};

// Grow-only device scratch of a decoder (tables, staged bitstream, segment
// state), so that repeated decodes allocate nothing once warm.
struct DecodeWorkspace {
  DecodeTables t;
  size_t child_cap = 0, leaf_cap = 0, sym_cap = 0;  // elements
  uint32_t *bits = nullptr;                          // staged bitstream
  size_t bits_cap = 0;                               // bytes
  long long *entry = nullptr, *end = nullptr;
  unsigned long long *cnt = nullptr;
  unsigned char *dirty = nullptr;
  size_t seg_cap = 0;
  int *changed = nullptr, *h_changed = nullptr;
  unsigned long long *h_total = nullptr;
  ~DecodeWorkspace();
};

// Builds the tables of (symbols, codes, lengths) on the host and uploads
// them into ws, with the host decoder's rules (codes of length 1..32 below
// 2^length; the first of equal codes wins).
int decode_tables_build(DecodeWorkspace &ws, const uint32_t *symbols, const uint32_t *codes, const int32_t *lengths,
                        size_t nsym, cudaStream_t st);

// Decodes up to num_elements symbols of the nbytes-byte bitstream ws.bits
// into d_out (symbol_bytes 1 or 2).  *decoded receives the count (fewer
// than num_elements when the stream ends first).  Runs on `st`;
// synchronises it.
int huff_decode_gpu(DecodeWorkspace &ws, size_t nbytes, size_t num_elements, int symbol_bytes, void *d_out,
                    size_t *decoded, cudaStream_t st);

// Table build + staging + decode of a bitstream in host (kind
// cudaMemcpyHostToDevice) or device memory; returns after the stream
// finished.
int huff_decode_bits(DecodeWorkspace &ws, const uint8_t *bits, size_t nbytes, cudaMemcpyKind kind,
                     const uint32_t *symbols, const uint32_t *codes, const int32_t *lengths, size_t nsym,
                     size_t num_elements, int symbol_bytes, void *d_out, size_t *decoded, void *stream);

// -------------------------------------------------- edits from streams --
constexpr int UP_THREADS = 128;              // one 32-bit flag word per thread
constexpr int UP_CHUNK = UP_THREADS * 32;    // 4096 elements per block

// Set flags per 4096-element chunk (bits past n ignored).
__global__ void k_unpack_count(const unsigned *__restrict__ flags, long long n,
                               unsigned long long *__restrict__ blk);
// Exclusive scan in place (one block of 1024 threads).
__global__ void k_unpack_scan(unsigned long long *__restrict__ v, long long n);

// Dequantisation of a uint16 code (the inverse of the quantiser, following
// projection_algorithm.cu:638): q / 65535 * (max - min) + min in T, each
// operation rounded on its own (no contraction).
template <typename T>
__device__ __forceinline__ T dequant(unsigned q, T mn, T mx);
template <>
__device__ __forceinline__ float dequant<float>(unsigned q, float mn, float mx) {
  return __fadd_rn(__fmul_rn(__fdiv_rn((float)q, 65535.0f), __fsub_rn(mx, mn)), mn);
}
template <>
__device__ __forceinline__ double dequant<double>(unsigned q, double mn, double mx) {
  return __dadd_rn(__dmul_rn(__ddiv_rn((double)q, 65535.0), __dsub_rn(mx, mn)), mn);
}

// The r-th set flag (ascending flat index i) receives dequant(quant[r]).
// Frequency edits (spec != nullptr): i < H is the real part, H <= i < 2H the
// imaginary part of coefficient i mod H, written into the half spectrum of
// row pitch Hzp; spatial edits: dense[i].
template <typename T>
__global__ void __launch_bounds__(UP_THREADS) k_unpack_scatter(const unsigned *__restrict__ flags, long long n,
                                                               const unsigned long long *__restrict__ blk_off,
                                                               const uint16_t *__restrict__ quant,
                                                               long long count, T mn, T mx,
                                                               T *__restrict__ dense, c2<T> *__restrict__ spec,
                                                               long long H, int Hz, int Hzp) {
  __shared__ unsigned wsum[UP_THREADS / 32];
  const long long w = (long long)blockIdx.x * UP_THREADS + threadIdx.x;
  const long long i0 = w * 32;
  unsigned bits = 0;
  if (i0 < n) {
    bits = flags[w];
    const long long left = n - i0;
    if (left < 32) bits &= (1u << left) - 1u;
  }
  // block-exclusive prefix of the popcounts
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned c = __popc(bits);
  unsigned x = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  unsigned before = 0;
  for (int k = 0; k < warp; ++k) before += wsum[k];
  long long r = (long long)blk_off[blockIdx.x] + before + x - c;
  while (bits) {
    const int j = __ffs(bits) - 1;
    bits &= bits - 1u;
    const long long i = i0 + j;
    if (r < count) {
      const T v = dequant<T>(quant[r], mn, mx);
      if (spec) {
        const bool im = i >= H;
        const long long k = im ? i - H : i;
        const long long row = k / Hz;
        T *p = reinterpret_cast<T *>(spec + row * Hzp + (k - row * Hz));
        p[im ? 1 : 0] = v;
      } else {
        dense[i] = v;
      }
    }
    ++r;
  }
}

// out = x' + (e + s), T arithmetic.
template <typename T>
__global__ void k_recon_sum(const T *__restrict__ xp, const T *__restrict__ e, const T *__restrict__ s,
                            T *__restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = xp[i] + (e[i] + s[i]);
}

}  // namespace ffcz
