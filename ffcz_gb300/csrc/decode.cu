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
// The staged stream is zero past its end and readable for 12 bytes, so the
// window is always loaded; `rem` keeps the walk inside the stream.
__device__ __forceinline__ long long dec_step(const unsigned *__restrict__ W, long long total, const unsigned *lut,
                                              int lut_bits, const DevTables &t, long long pos, int &sym) {
  const unsigned long long w = window64(W, pos);
  const long long rem = total - pos;
  const unsigned e = lut[w >> (64 - lut_bits)];
  const unsigned type = e >> 30;
  sym = -1;
  if (type == kEmit) {
    const int len = (int)((e >> 24) & 63u);
    if (len <= rem) {
      sym = (int)(e & 0xFFFFFFu);
      return pos + len;
    }
    return pos + 1;
  }
  if (type == kSkip) return pos + 1;
  int node = (int)(e & 0xFFFFFFu);
  for (int d = lut_bits; d < 32 && d < rem; ++d) {
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
  return pos + 1;
}

__device__ __forceinline__ void load_lut(unsigned *lut, const unsigned *__restrict__ g, int lut_bits) {
  const uint4 *src = reinterpret_cast<const uint4 *>(g);
  uint4 *dst = reinterpret_cast<uint4 *>(lut);
  for (int i = threadIdx.x; i < (1 << lut_bits) / 4; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
}

// Decode of every dirty segment from its entry to its end.
__global__ void __launch_bounds__(256) k_dec_round(const unsigned *__restrict__ W, long long total,
                                                   const unsigned *__restrict__ lut_g, int lut_bits, DevTables t,
                                                   int nseg,
                                                   const long long *__restrict__ entry,
                                                   const unsigned char *__restrict__ dirty,
                                                   long long *__restrict__ end,
                                                   unsigned long long *__restrict__ cnt) {
  extern __shared__ __align__(16) unsigned lut[];
  load_lut(lut, lut_g, lut_bits);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg || !dirty[k]) return;
  const long long lim = min((long long)(k + 1) * kSegBits, total);
  long long pos = entry[k];
  unsigned long long c = 0;
  while (pos < lim) {
    int sym;
    pos = dec_step(W, total, lut, lut_bits, t, pos, sym);
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
                                                   const unsigned *__restrict__ lut_g, int lut_bits, DevTables t,
                                                   int nseg,
                                                   const long long *__restrict__ entry,
                                                   const unsigned long long *__restrict__ off, long long nmax,
                                                   S *__restrict__ out) {
  extern __shared__ __align__(16) unsigned lut[];
  load_lut(lut, lut_g, lut_bits);
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nseg) return;
  const long long lim = min((long long)(k + 1) * kSegBits, total);
  long long pos = entry[k];
  long long o = (long long)off[k];
  while (pos < lim && o < nmax) {
    int sym;
    pos = dec_step(W, total, lut, lut_bits, t, pos, sym);
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
namespace {

template <typename V>
int grow(V **p, size_t &cap, size_t need) {
  if (need <= cap) return FFCZ_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  cap = 0;
  FFCZ_CUDA(cudaMalloc(p, need * sizeof(V)));
  cap = need;
  return FFCZ_OK;
}

}  // namespace

DecodeWorkspace::~DecodeWorkspace() {
  void *dev[] = {t.child, t.leaf, t.lut, t.symbols, bits, entry, end, cnt, dirty, changed};
  for (void *p : dev)
    if (p) cudaFree(p);
  if (h_changed) cudaFreeHost(h_changed);
  if (h_total) cudaFreeHost(h_total);
}

int decode_tables_build(DecodeWorkspace &ws, const uint32_t *symbols, const uint32_t *codes, const int32_t *lengths,
                        size_t nsym, cudaStream_t st) {
  if (nsym >= (1u << 24)) return fail(FFCZ_ERR_UNSUPPORTED, "code table larger than 2^24 symbols");
  // Codes in (length, index) order: where one code is a prefix of another
  // or two are equal, the walk meets the shorter / earlier one first.
  std::vector<std::vector<int>> by_len(33);
  int maxlen = 1;
  for (size_t s = 0; s < nsym; ++s) {
    const int L = lengths[s];
    // (length, code) keys: a stored code of 2^L or more never matches
    if (L < 1 || L > 32 || (L < 32 && (codes[s] >> L) != 0)) continue;
    by_len[L].push_back((int)s);
    maxlen = std::max(maxlen, L);
  }
  const int lb = std::min(std::max(8, maxlen), kLutBitsMax);
  const unsigned kEmpty = 0xFFFFFFFFu;
  std::vector<unsigned> lut(1u << lb, kEmpty);
  auto low = [](uint32_t c, int) { return c; };  // codes below 2^L (checked above)
  // codes of at most lb bits fill their range of the table (EMIT); the
  // ranges of a prefix code are disjoint, so this touches each entry once
  for (int L = 1; L <= lb; ++L)
    for (int s : by_len[L]) {
      const unsigned base = low(codes[s], L) << (lb - L), span = 1u << (lb - L);
      for (unsigned v = base; v < base + span; ++v)
        if (lut[v] == kEmpty) lut[v] = (kEmit << 30) | ((unsigned)L << 24) | (unsigned)s;
    }
  // longer codes: a trie below their first lb bits, reached through CONT
  std::vector<int2> child;
  std::vector<int> leaf;
  auto new_node = [&]() {
    child.push_back(make_int2(-1, -1));
    leaf.push_back(-1);
    return (int)leaf.size() - 1;
  };
  for (int L = lb + 1; L <= 32; ++L)
    for (int s : by_len[L]) {
      const uint32_t c = low(codes[s], L);
      const unsigned p = (unsigned)(c >> (L - lb));
      unsigned &e = lut[p];
      if (e != kEmpty && (e >> 30) == kEmit) continue;  // a shorter code is met first
      if (e == kEmpty) e = (kCont << 30) | (unsigned)new_node();
      int node = (int)(e & 0xFFFFFFu);
      bool blocked = false;
      for (int d = L - lb - 1; d >= 0; --d) {
        if (leaf[node] >= 0) {  // a shorter long code ends on this path
          blocked = true;
          break;
        }
        const int bit = (c >> d) & 1u;
        int nx = bit ? child[node].y : child[node].x;
        if (nx < 0) {
          nx = new_node();
          if (bit) child[node].y = nx;
          else child[node].x = nx;
        }
        node = nx;
      }
      if (!blocked && leaf[node] < 0) leaf[node] = s;
      if (child.size() >= (1u << 24)) return fail(FFCZ_ERR_UNSUPPORTED, "code trie too large");
    }
  for (unsigned &e : lut)
    if (e == kEmpty) e = kSkip << 30;
  if (child.empty()) new_node();  // keep the device arrays non-empty
  DecodeTables &t = ws.t;
  t.nnodes = (int)child.size();
  t.lut_bits = lb;
  FFCZ_TRY(grow(&t.child, ws.child_cap, child.size()));
  FFCZ_TRY(grow(&t.leaf, ws.leaf_cap, leaf.size()));
  FFCZ_TRY(grow(&t.symbols, ws.sym_cap, std::max<size_t>(nsym, 1)));
  if (!t.lut) FFCZ_CUDA(cudaMalloc(&t.lut, ((size_t)1 << kLutBitsMax) * sizeof(unsigned)));
  FFCZ_CUDA(cudaMemcpyAsync(t.child, child.data(), child.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
  FFCZ_CUDA(cudaMemcpyAsync(t.leaf, leaf.data(), leaf.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  FFCZ_CUDA(cudaMemcpyAsync(t.lut, lut.data(), lut.size() * sizeof(unsigned), cudaMemcpyHostToDevice, st));
  if (nsym) FFCZ_CUDA(cudaMemcpyAsync(t.symbols, symbols, nsym * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  // the host vectors go out of scope: finish the copies first
  FFCZ_CUDA(cudaStreamSynchronize(st));
  return FFCZ_OK;
}

// ---------------------------------------------------------------- driver --
int huff_decode_gpu(DecodeWorkspace &ws, size_t nbytes, size_t num_elements, int symbol_bytes, void *d_out,
                    size_t *decoded, cudaStream_t st) {
  *decoded = 0;
  const long long total = (long long)nbytes * 8;
  if (num_elements == 0 || total == 0) return FFCZ_OK;
  const int nseg = (int)((total + kSegBits - 1) / kSegBits);
  if ((size_t)nseg + 1 > ws.seg_cap) {
    size_t cap = 0;
    FFCZ_TRY(grow(&ws.entry, cap, (size_t)nseg + 1));
    cap = 0;
    FFCZ_TRY(grow(&ws.end, cap, (size_t)nseg + 1));
    cap = 0;
    FFCZ_TRY(grow(&ws.cnt, cap, (size_t)nseg + 1));
    cap = 0;
    FFCZ_TRY(grow(&ws.dirty, cap, (size_t)nseg + 1));
    ws.seg_cap = (size_t)nseg + 1;
  }
  if (!ws.changed) FFCZ_CUDA(cudaMalloc(&ws.changed, sizeof(int)));
  if (!ws.h_changed) FFCZ_CUDA(cudaMallocHost(&ws.h_changed, sizeof(int)));
  if (!ws.h_total) FFCZ_CUDA(cudaMallocHost(&ws.h_total, sizeof(unsigned long long)));
  const DecodeTables &t = ws.t;
  const DevTables dt{t.child, t.leaf, t.symbols};
  const unsigned *W = ws.bits;
  const unsigned g = (unsigned)((nseg + 255) / 256);
  const size_t lut_smem = ((size_t)1 << t.lut_bits) * sizeof(unsigned);
  // the table may take up to 64 KB (set on the current device every call)
  FFCZ_CUDA(cudaFuncSetAttribute(k_dec_round, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536));
  FFCZ_CUDA(cudaFuncSetAttribute(k_dec_write<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536));
  FFCZ_CUDA(cudaFuncSetAttribute(k_dec_write<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 65536));
  k_dec_init<<<g, 256, 0, st>>>(nseg, ws.entry, ws.dirty);
  // Each round fixes at least the next segment's entry, so nseg rounds
  // always reach the fixed point; self-synchronising codes take a few.
  for (int round = 0; round <= nseg; ++round) {
    k_dec_round<<<g, 256, lut_smem, st>>>(W, total, t.lut, t.lut_bits, dt, nseg, ws.entry, ws.dirty, ws.end,
                                          ws.cnt);
    FFCZ_CUDA(cudaMemsetAsync(ws.changed, 0, sizeof(int), st));
    k_dec_check<<<g, 256, 0, st>>>(nseg, ws.entry, ws.end, ws.dirty, ws.changed);
    FFCZ_CUDA(cudaMemcpyAsync(ws.h_changed, ws.changed, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFCZ_CUDA(cudaStreamSynchronize(st));
    if (!*ws.h_changed) break;
  }
  FFCZ_CUDA(cudaMemsetAsync(ws.cnt + nseg, 0, sizeof(unsigned long long), st));
  k_unpack_scan<<<1, 1024, 0, st>>>(ws.cnt, nseg + 1);
  FFCZ_CUDA(cudaMemcpyAsync(ws.h_total, ws.cnt + nseg, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  if (symbol_bytes == 2)
    k_dec_write<uint16_t><<<g, 256, lut_smem, st>>>(W, total, t.lut, t.lut_bits, dt, nseg, ws.entry, ws.cnt,
                                                    (long long)num_elements, (uint16_t *)d_out);
  else
    k_dec_write<uint8_t><<<g, 256, lut_smem, st>>>(W, total, t.lut, t.lut_bits, dt, nseg, ws.entry, ws.cnt,
                                                   (long long)num_elements, (uint8_t *)d_out);
  FFCZ_CUDA(cudaGetLastError());
  FFCZ_CUDA(cudaStreamSynchronize(st));
  *decoded = (size_t)std::min<unsigned long long>(*ws.h_total, num_elements);
  return FFCZ_OK;
}

int huff_decode_bits(DecodeWorkspace &ws, const uint8_t *bits, size_t nbytes, cudaMemcpyKind kind,
                     const uint32_t *symbols, const uint32_t *codes, const int32_t *lengths, size_t nsym,
                     size_t num_elements, int symbol_bytes, void *d_out, size_t *decoded, void *stream) {
  if (!decoded || (!bits && nbytes) || (!symbols && nsym) || (!codes && nsym) || (!lengths && nsym) ||
      (!d_out && num_elements))
    return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (symbol_bytes != 1 && symbol_bytes != 2) return fail(FFCZ_ERR_INVALID, "symbol_bytes must be 1 or 2");
  cudaStream_t st = (cudaStream_t)stream;
  FFCZ_TRY(decode_tables_build(ws, symbols, codes, lengths, nsym, st));
  // staged copy: 4-byte aligned, 16 zero bytes after it (the window reads)
  const size_t cap = (nbytes + 3) / 4 * 4 + 16;
  size_t words = ws.bits_cap / 4;
  FFCZ_TRY(grow(&ws.bits, words, cap / 4));
  ws.bits_cap = words * 4;
  FFCZ_CUDA(cudaMemsetAsync((uint8_t *)ws.bits + (nbytes & ~(size_t)3), 0, cap - (nbytes & ~(size_t)3), st));
  if (nbytes) FFCZ_CUDA(cudaMemcpyAsync(ws.bits, bits, nbytes, kind, st));
  return huff_decode_gpu(ws, nbytes, num_elements, symbol_bytes, d_out, decoded, st);
}

}  // namespace ffcz

using namespace ffcz;

extern "C" {

int ffcz_huff_decode_device(const uint8_t *d_bits, size_t nbytes, const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols, size_t num_elements, int symbol_bytes,
                            void *d_out, size_t *decoded, void *stream) {
  DecodeWorkspace ws;
  return huff_decode_bits(ws, d_bits, nbytes, cudaMemcpyDeviceToDevice, symbols, codes, lengths, num_symbols, num_elements,
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
  DecodeWorkspace ws;
  return huff_decode_bits(ws, bits.data(), bits.size(), cudaMemcpyHostToDevice, symbols, codes, lengths, num_symbols,
                    num_elements, symbol_bytes, d_out, decoded, stream);
}

}  // extern "C"
