// GPU prefix decoder of the Huffman bitstreams (HuffmanZSTDCoder.cuh:394-449
// rules, decoded in parallel segments) and the flag/code unpacking kernels of
// the reconstruction.
#include <algorithm>
#include <memory>
#include <vector>

#include "decode.cuh"
#include "huffman_host.h"

namespace ffcz {

namespace {

constexpr unsigned kEmit = 0u, kSkip = 1u, kCont = 2u;

__device__ __forceinline__ unsigned bswap32d(unsigned x) { return __byte_perm(x, 0u, 0x0123); }

// 64 stream bits starting at bit `pos` (MSB-first), most significant first.
__device__ __forceinline__ unsigned long long window64(const unsigned *__restrict__ W, long long pos) {
  const long long wi = pos >> 5;
  const unsigned sh = (unsigned)(pos & 31);
  const unsigned long long a = ((unsigned long long)bswap32d(W[wi]) << 32) | bswap32d(W[wi + 1]);
  const unsigned b = bswap32d(W[wi + 2]);
  return sh ? ((a << sh) | (b >> (32 - sh))) : a;
}

struct DevTables {
  const int2 *child;
  const int *leaf;
  const uint32_t *symbols;
};

// One step of the sequential decoder from bit `pos`; sym = symbol index or -1.
__device__ __forceinline__ long long dec_step(const unsigned *__restrict__ W, const uint8_t *__restrict__ B,
                                              long long total, const unsigned *lut, const DevTables &t,
                                              long long pos, int &sym) {
  if (pos + 32 <= total) {
    const unsigned long long w = window64(W, pos);
    const unsigned e = lut[w >> (64 - kLutBits)];
    const unsigned type = e >> 30;
    if (type == kEmit) {
      sym = (int)(e & 0xFFFFFFu);
      return pos + ((e >> 24) & 63u);
    }
    if (type == kSkip) {
      sym = -1;
      return pos + 1;
    }
    int node = (int)(e & 0xFFFFFFu);
    for (int d = kLutBits; d < 32; ++d) {
      const int bit = (int)((w >> (63 - d)) & 1ull);
      const int2 ch = t.child[node];
      node = bit ? ch.y : ch.x;
      if (node < 0) break;
      const int lf = t.leaf[node];
      if (lf >= 0) {
        sym = lf;
        return pos + d + 1;
      }
    }
    sym = -1;
    return pos + 1;
  }
  // the last 32 bits: bit by bit, stopping at the end of the stream
  int node = 0;
  long long p = pos;
  int depth = 0;
  while (p < total && depth < 32) {
    const int bit = (B[p >> 3] >> (7 - (p & 7))) & 1;
    const int2 ch = t.child[node];
    node = bit ? ch.y : ch.x;
    ++p;
    ++depth;
    if (node < 0) break;
    const int lf = t.leaf[node];
    if (lf >= 0) {
      sym = lf;
      return p;
    }
  }
  sym = -1;
  return pos + 1;
}

__device__ __forceinline__ void load_lut(unsigned *lut, const unsigned *__restrict__ g) {
  for (int i = threadIdx.x; i < (1 << kLutBits); i += blockDim.x) lut[i] = g[i];
  __syncthreads();
}

// Decode of every dirty segment from its entry to its end.
__global__ void __launch_bounds__(256) k_dec_round(const unsigned *__restrict__ W, long long total,
                                                   const unsigned *__restrict__ lut_g, DevTables t, int nseg,
                                                   const long long *__restrict__ entry,
                                                   const unsigned char *__restrict__ dirty,
                                                   long long *__restrict__ end,
                                                   unsigned long long *__restrict__ cnt) {
  __shared__ unsigned lut[1 << kLutBits];
  load_lut(lut, lut_g);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg || !dirty[k]) return;
  const uint8_t *B = reinterpret_cast<const uint8_t *>(W);
  const long long lim = min((long long)(k + 1) * kSegBits, total);
  long long pos = entry[k];
  unsigned long long c = 0;
  while (pos < lim) {
    int sym;
    pos = dec_step(W, B, total, lut, t, pos, sym);
    c += sym >= 0;
  }
  end[k] = pos;
  cnt[k] = c;
}

// entry[k] = end[k-1]; a segment whose entry moved is decoded again.
__global__ void k_dec_check(int nseg, long long *__restrict__ entry, const long long *__restrict__ end,
                            unsigned char *__restrict__ dirty, int *__restrict__ changed) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg) return;
  if (k == 0) {
    dirty[0] = 0;
    return;
  }
  const long long e = end[k - 1];
  if (e != entry[k]) {
    entry[k] = e;
    dirty[k] = 1;
    *changed = 1;
  } else {
    dirty[k] = 0;
  }
}

template <typename S>
__global__ void __launch_bounds__(256) k_dec_write(const unsigned *__restrict__ W, long long total,
                                                   const unsigned *__restrict__ lut_g, DevTables t, int nseg,
                                                   const long long *__restrict__ entry,
                                                   const unsigned long long *__restrict__ off, long long nmax,
                                                   S *__restrict__ out) {
  __shared__ unsigned lut[1 << kLutBits];
  load_lut(lut, lut_g);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg) return;
  const uint8_t *B = reinterpret_cast<const uint8_t *>(W);
  const long long lim = min((long long)(k + 1) * kSegBits, total);
  long long pos = entry[k];
  long long o = (long long)off[k];
  while (pos < lim && o < nmax) {
    int sym;
    pos = dec_step(W, B, total, lut, t, pos, sym);
    if (sym >= 0) out[o++] = (S)t.symbols[sym];
  }
}

__global__ void k_dec_init(int nseg, long long *__restrict__ entry, unsigned char *__restrict__ dirty) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg) return;
  entry[k] = (long long)k * kSegBits;
  dirty[k] = 1;
}

}  // namespace

// ------------------------------------------------------------ unpacking --
__global__ void __launch_bounds__(UP_THREADS) k_unpack_count(const unsigned *__restrict__ flags, long long n,
                                                             unsigned long long *__restrict__ blk) {
  __shared__ unsigned ws[UP_THREADS / 32];
  const long long w = (long long)blockIdx.x * UP_THREADS + threadIdx.x;
  const long long i0 = w * 32;
  unsigned bits = 0;
  if (i0 < n) {
    bits = flags[w];
    const long long left = n - i0;
    if (left < 32) bits &= (1u << left) - 1u;
  }
  unsigned c = __popc(bits);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int k = 0; k < UP_THREADS / 32; ++k) s += ws[k];
    blk[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(1024) k_unpack_scan(unsigned long long *__restrict__ v, long long n) {
  __shared__ unsigned long long wsum[32];
  __shared__ unsigned long long carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (long long b0 = 0; b0 < n; b0 += 1024) {
    const long long i = b0 + threadIdx.x;
    const unsigned long long a = (i < n) ? v[i] : 0ull;
    unsigned long long x = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned long long s = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      wsum[lane] = s;
    }
    __syncthreads();
    const unsigned long long pre = carry + (warp ? wsum[warp - 1] : 0ull) + x - a;
    if (i < n) v[i] = pre;
    __syncthreads();
    if (threadIdx.x == 0) carry += wsum[31];
    __syncthreads();
  }
}

// ---------------------------------------------------------------- tables --
int decode_tables_build(const uint32_t *symbols, const uint32_t *codes, const int32_t *lengths, size_t nsym,
                        DecodeTables &t) {
  if (nsym >= (1u << 24)) return fail(FFCZ_ERR_UNSUPPORTED, "code table larger than 2^24 symbols");
  std::vector<int2> child(1, make_int2(-1, -1));
  std::vector<int> leaf(1, -1);
  for (size_t s = 0; s < nsym; ++s) {
    const int L = lengths[s];
    if (L < 1 || L > 32) continue;
    int node = 0;
    for (int d = L - 1; d >= 0; --d) {
      const int bit = (codes[s] >> d) & 1u;
      int c = bit ? child[node].y : child[node].x;
      if (c < 0) {
        c = (int)leaf.size();
        if (bit) child[node].y = c;
        else child[node].x = c;
        leaf.push_back(-1);
        child.push_back(make_int2(-1, -1));
      }
      node = c;
    }
    if (leaf[node] < 0) leaf[node] = (int)s;
  }
  if (child.size() >= (1u << 24)) return fail(FFCZ_ERR_UNSUPPORTED, "code trie too large");
  std::vector<unsigned> lut(1u << kLutBits);
  for (unsigned v = 0; v < (1u << kLutBits); ++v) {
    int node = 0;
    unsigned e = 0;
    bool done = false;
    for (int d = 0; d < kLutBits && !done; ++d) {
      const int bit = (v >> (kLutBits - 1 - d)) & 1u;
      node = bit ? child[node].y : child[node].x;
      if (node < 0) {
        e = kSkip << 30;
        done = true;
      } else if (leaf[node] >= 0) {
        e = (kEmit << 30) | ((unsigned)(d + 1) << 24) | (unsigned)leaf[node];
        done = true;
      }
    }
    if (!done) e = (kCont << 30) | (unsigned)node;
    lut[v] = e;
  }
  std::vector<uint32_t> sym(symbols, symbols + nsym);
  if (sym.empty()) sym.push_back(0);
  decode_tables_free(t);
  t.nnodes = (int)child.size();
  FFCZ_CUDA(cudaMalloc(&t.child, child.size() * sizeof(int2)));
  FFCZ_CUDA(cudaMalloc(&t.leaf, leaf.size() * sizeof(int)));
  FFCZ_CUDA(cudaMalloc(&t.lut, lut.size() * sizeof(unsigned)));
  FFCZ_CUDA(cudaMalloc(&t.symbols, sym.size() * sizeof(uint32_t)));
  FFCZ_CUDA(cudaMemcpy(t.child, child.data(), child.size() * sizeof(int2), cudaMemcpyHostToDevice));
  FFCZ_CUDA(cudaMemcpy(t.leaf, leaf.data(), leaf.size() * sizeof(int), cudaMemcpyHostToDevice));
  FFCZ_CUDA(cudaMemcpy(t.lut, lut.data(), lut.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
  FFCZ_CUDA(cudaMemcpy(t.symbols, sym.data(), sym.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  return FFCZ_OK;
}

void decode_tables_free(DecodeTables &t) {
  if (t.child) cudaFree(t.child);
  if (t.leaf) cudaFree(t.leaf);
  if (t.lut) cudaFree(t.lut);
  if (t.symbols) cudaFree(t.symbols);
  t = DecodeTables{};
}

// ---------------------------------------------------------------- driver --
int huff_decode_gpu(const uint32_t *d_bits, size_t nbytes, const DecodeTables &t, size_t num_elements,
                    int symbol_bytes, void *d_out, size_t *decoded, cudaStream_t st) {
  *decoded = 0;
  const long long total = (long long)nbytes * 8;
  if (num_elements == 0 || total == 0) return FFCZ_OK;
  const int nseg = (int)((total + kSegBits - 1) / kSegBits);
  long long *entry = nullptr, *end = nullptr;
  unsigned long long *cnt = nullptr;
  unsigned char *dirty = nullptr;
  int *changed = nullptr, *h_changed = nullptr;
  auto release = [&]() {
    if (entry) cudaFree(entry);
    if (end) cudaFree(end);
    if (cnt) cudaFree(cnt);
    if (dirty) cudaFree(dirty);
    if (changed) cudaFree(changed);
    if (h_changed) cudaFreeHost(h_changed);
  };
  struct Guard {
    decltype(release) &f;
    ~Guard() { f(); }
  } guard{release};
  FFCZ_CUDA(cudaMalloc(&entry, nseg * sizeof(long long)));
  FFCZ_CUDA(cudaMalloc(&end, nseg * sizeof(long long)));
  FFCZ_CUDA(cudaMalloc(&cnt, (nseg + 1) * sizeof(unsigned long long)));
  FFCZ_CUDA(cudaMalloc(&dirty, nseg));
  FFCZ_CUDA(cudaMalloc(&changed, sizeof(int)));
  FFCZ_CUDA(cudaMallocHost(&h_changed, sizeof(int)));
  const DevTables dt{t.child, t.leaf, t.symbols};
  const unsigned g = (unsigned)((nseg + 255) / 256);
  k_dec_init<<<g, 256, 0, st>>>(nseg, entry, dirty);
  // Each round fixes at least the next segment's entry, so nseg rounds
  // always reach the fixed point; self-synchronising codes take two or three.
  for (int round = 0; round <= nseg; ++round) {
    k_dec_round<<<g, 256, 0, st>>>(reinterpret_cast<const unsigned *>(d_bits), total, t.lut, dt, nseg, entry, dirty,
                                   end, cnt);
    FFCZ_CUDA(cudaMemsetAsync(changed, 0, sizeof(int), st));
    k_dec_check<<<g, 256, 0, st>>>(nseg, entry, end, dirty, changed);
    FFCZ_CUDA(cudaMemcpyAsync(h_changed, changed, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFCZ_CUDA(cudaStreamSynchronize(st));
    if (!*h_changed) break;
  }
  FFCZ_CUDA(cudaMemsetAsync(cnt + nseg, 0, sizeof(unsigned long long), st));
  k_unpack_scan<<<1, 1024, 0, st>>>(cnt, nseg + 1);
  unsigned long long total_syms = 0;
  FFCZ_CUDA(cudaMemcpyAsync(&total_syms, cnt + nseg, sizeof(total_syms), cudaMemcpyDeviceToHost, st));
  if (symbol_bytes == 2)
    k_dec_write<uint16_t><<<g, 256, 0, st>>>(reinterpret_cast<const unsigned *>(d_bits), total, t.lut, dt, nseg,
                                             entry, cnt, (long long)num_elements, (uint16_t *)d_out);
  else
    k_dec_write<uint8_t><<<g, 256, 0, st>>>(reinterpret_cast<const unsigned *>(d_bits), total, t.lut, dt, nseg,
                                            entry, cnt, (long long)num_elements, (uint8_t *)d_out);
  FFCZ_CUDA(cudaGetLastError());
  FFCZ_CUDA(cudaStreamSynchronize(st));
  *decoded = (size_t)std::min<unsigned long long>(total_syms, num_elements);
  return FFCZ_OK;
}

}  // namespace ffcz

namespace ffcz {

namespace {

// Copies a bitstream (host or device) into a 4-byte aligned device buffer
// with 16 zero bytes after it, as the decode kernels read.
int stage_bits(const uint8_t *src, size_t nbytes, cudaMemcpyKind kind, uint32_t **out, cudaStream_t st) {
  const size_t cap = (nbytes + 3) / 4 * 4 + 16;
  FFCZ_CUDA(cudaMalloc(out, cap));
  FFCZ_CUDA(cudaMemsetAsync(*out, 0, cap, st));
  if (nbytes) FFCZ_CUDA(cudaMemcpyAsync(*out, src, nbytes, kind, st));
  return FFCZ_OK;
}

}  // namespace

int huff_decode_bits(const uint8_t *bits, size_t nbytes, cudaMemcpyKind kind, const uint32_t *symbols,
                     const uint32_t *codes, const int32_t *lengths, size_t nsym, size_t num_elements,
                     int symbol_bytes, void *d_out, size_t *decoded, void *stream) {
  if (!decoded || (!bits && nbytes) || (!symbols && nsym) || (!codes && nsym) || (!lengths && nsym) ||
      (!d_out && num_elements))
    return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (symbol_bytes != 1 && symbol_bytes != 2) return fail(FFCZ_ERR_INVALID, "symbol_bytes must be 1 or 2");
  cudaStream_t st = (cudaStream_t)stream;
  DecodeTables t;
  uint32_t *d_bits = nullptr;
  int rc = decode_tables_build(symbols, codes, lengths, nsym, t);
  if (rc == FFCZ_OK) rc = stage_bits(bits, nbytes, kind, &d_bits, st);
  if (rc == FFCZ_OK) rc = huff_decode_gpu(d_bits, nbytes, t, num_elements, symbol_bytes, d_out, decoded, st);
  cudaStreamSynchronize(st);
  if (d_bits) cudaFree(d_bits);
  decode_tables_free(t);
  return rc;
}

}  // namespace ffcz

using namespace ffcz;

extern "C" {

int ffcz_huff_decode_device(const uint8_t *d_bits, size_t nbytes, const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols, size_t num_elements, int symbol_bytes,
                            void *d_out, size_t *decoded, void *stream) {
  return huff_decode_bits(d_bits, nbytes, cudaMemcpyDeviceToDevice, symbols, codes, lengths, num_symbols, num_elements,
                    symbol_bytes, d_out, decoded, stream);
}

int ffcz_huff_zstd_decompress_device(const uint8_t *comp, size_t comp_len, const uint32_t *symbols,
                                     const uint32_t *codes, const int32_t *lengths, size_t num_symbols,
                                     size_t num_elements, size_t bitstream_bytes, int symbol_bytes, void *d_out,
                                     size_t *decoded, void *stream) {
  if (!comp && comp_len) return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::vector<uint8_t> bits;
  FFCZ_TRY(zstd_decompress(comp, comp_len, bitstream_bytes, bits));
  bits.resize(bitstream_bytes, 0);
  return huff_decode_bits(bits.data(), bits.size(), cudaMemcpyHostToDevice, symbols, codes, lengths, num_symbols,
                    num_elements, symbol_bytes, d_out, decoded, stream);
}

}  // extern "C"
