// Huffman encoder of HuffmanZSTDCoder.cuh:248-376 on the GPU.
//
//   k_hist_u8 / k_hist_u16 : shared-memory-privatised symbol histogram
//                            (u16: 65536 packed 16-bit counters = 128 KB per
//                            block, flushed with one global atomic per
//                            non-empty bin)                        R n*b
//   host                   : codebook (reference tie-breaking), LUT upload,
//                            total bits = sum(count * length)
//   k_huff_bits            : code-length sum per 2048-symbol block R n*b
//   k_scan_u64             : exclusive scan of the block sums (1 block)
//   k_huff_pack            : per block: thread bit offsets by block scan,
//                            codes OR-ed MSB-first into a shared bit
//                            buffer, words stored big-endian (byte stream
//                            order); the two edge words of a block use
//                            atomicOr, every other word a plain store.
//                                                          R n*b  W bits/8
// The word->byte order equals the reference's u64 word split (:344-357):
// an MSB-first bitstream zero padded to whole bytes.
#include <cstring>
#include <mutex>
#include <thread>

#include "huffman.cuh"

namespace ffcz {

constexpr int HB_THREADS = 256;
constexpr int HB_PER_THREAD = 8;
constexpr int HB_CHUNK = HB_THREADS * HB_PER_THREAD;  // 2048 symbols per block
constexpr int H16_CHUNK = 32768;                      // symbols per u16 histogram block

__global__ void __launch_bounds__(256) k_hist_u8(const uint8_t *__restrict__ d, long long n,
                                                 unsigned *__restrict__ hist) {
  __shared__ unsigned sh[256];
  sh[threadIdx.x] = 0;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&sh[d[i]], 1u);
  __syncthreads();
  const unsigned v = sh[threadIdx.x];
  if (v) atomicAdd(&hist[threadIdx.x], v);
}

// `chunk` symbols per block (a multiple of 8, at most 32768, so every packed
// 16-bit counter stays < 65536).
__global__ void __launch_bounds__(256) k_hist_u16(const uint16_t *__restrict__ d, long long n, int chunk,
                                                  unsigned *__restrict__ hist) {
  extern __shared__ __align__(16) unsigned sh16[];  // 32768 words
  for (int w = threadIdx.x; w < 32768; w += blockDim.x) sh16[w] = 0u;
  __syncthreads();
  const long long base = (long long)blockIdx.x * chunk;
  const long long end = min(base + (long long)chunk, n);
  if (base + chunk <= n) {
    const uint4 *v4 = reinterpret_cast<const uint4 *>(d + base);
    for (int j = threadIdx.x; j < chunk / 8; j += blockDim.x) {
      const uint4 q = v4[j];
      const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const unsigned s0 = w[t] & 0xffffu, s1 = w[t] >> 16;
        atomicAdd(&sh16[s0 >> 1], 1u << ((s0 & 1u) * 16));
        atomicAdd(&sh16[s1 >> 1], 1u << ((s1 & 1u) * 16));
      }
    }
  } else {
    for (long long i = base + threadIdx.x; i < end; i += blockDim.x) {
      const unsigned s = d[i];
      atomicAdd(&sh16[s >> 1], 1u << ((s & 1u) * 16));
    }
  }
  __syncthreads();
  for (int w = threadIdx.x; w < 32768; w += blockDim.x) {
    const unsigned v = sh16[w];
    if (v & 0xffffu) atomicAdd(&hist[2 * w], v & 0xffffu);
    if (v >> 16) atomicAdd(&hist[2 * w + 1], v >> 16);
  }
}

template <typename S>
__device__ __forceinline__ void load_syms(const S *__restrict__ d, long long n, long long i0,
                                          unsigned (&s)[HB_PER_THREAD], int &cnt) {
  if (i0 + HB_PER_THREAD <= n) {
    cnt = HB_PER_THREAD;
    if (sizeof(S) == 2) {
      const uint4 q = *reinterpret_cast<const uint4 *>(d + i0);
      const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        s[2 * t] = w[t] & 0xffffu;
        s[2 * t + 1] = w[t] >> 16;
      }
    } else {
      const uint2 q = *reinterpret_cast<const uint2 *>(d + i0);
      const unsigned w[2] = {q.x, q.y};
#pragma unroll
      for (int t = 0; t < 2; ++t)
#pragma unroll
        for (int b = 0; b < 4; ++b) s[4 * t + b] = (w[t] >> (8 * b)) & 0xffu;
    }
  } else {
    cnt = (int)max(0ll, n - i0);
#pragma unroll
    for (int t = 0; t < HB_PER_THREAD; ++t) s[t] = (t < cnt) ? (unsigned)d[i0 + t] : 0u;
  }
}

template <typename S>
__global__ void __launch_bounds__(HB_THREADS) k_huff_bits(const S *__restrict__ d, long long n,
                                                          const unsigned long long *__restrict__ lut,
                                                          unsigned long long *__restrict__ blk) {
  const long long i0 = (long long)blockIdx.x * HB_CHUNK + threadIdx.x * HB_PER_THREAD;
  unsigned s[HB_PER_THREAD];
  int cnt;
  load_syms<S>(d, n, i0, s, cnt);
  unsigned long long bits = 0;
#pragma unroll
  for (int t = 0; t < HB_PER_THREAD; ++t)
    if (t < cnt) bits += __ldg(lut + s[t]) >> 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) bits += __shfl_xor_sync(0xffffffffu, bits, o);
  __shared__ unsigned long long ws[HB_THREADS / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = bits;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < HB_THREADS / 32; ++w) t += ws[w];
    blk[blockIdx.x] = t;
  }
}

// Exclusive scan in place (one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_scan_u64(unsigned long long *__restrict__ v, long long n) {
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
      unsigned long long w = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;
    }
    __syncthreads();
    const unsigned long long pre = carry + (warp ? wsum[warp - 1] : 0ull) + x - a;
    if (i < n) v[i] = pre;
    __syncthreads();
    if (threadIdx.x == 0) carry += wsum[31];
    __syncthreads();
  }
}

__device__ __forceinline__ unsigned bswap32(unsigned x) { return __byte_perm(x, 0u, 0x0123); }

template <typename S>
__global__ void __launch_bounds__(HB_THREADS) k_huff_pack(const S *__restrict__ d, long long n,
                                                          const unsigned long long *__restrict__ lut,
                                                          const unsigned long long *__restrict__ blk_off,
                                                          unsigned *__restrict__ out) {
  __shared__ unsigned sbits[HB_CHUNK + 2];  // <= 32 bits per symbol
  __shared__ unsigned long long ws[HB_THREADS / 32];
  const long long i0 = (long long)blockIdx.x * HB_CHUNK + threadIdx.x * HB_PER_THREAD;
  unsigned s[HB_PER_THREAD];
  int cnt;
  load_syms<S>(d, n, i0, s, cnt);
  unsigned long long e[HB_PER_THREAD];
  unsigned mybits = 0;
#pragma unroll
  for (int t = 0; t < HB_PER_THREAD; ++t) {
    e[t] = (t < cnt) ? __ldg(lut + s[t]) : 0ull;
    mybits += (unsigned)(e[t] >> 32);
  }
  // block exclusive scan of mybits
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = mybits;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  for (int w = threadIdx.x; w < HB_CHUNK + 2; w += HB_THREADS) sbits[w] = 0u;
  __syncthreads();
  unsigned wpre = 0, tot = 0;
#pragma unroll
  for (int w = 0; w < HB_THREADS / 32; ++w) {
    const unsigned c = (unsigned)ws[w];
    wpre += (w < warp) ? c : 0u;
    tot += c;
  }
  const unsigned long long bit0 = blk_off[blockIdx.x];
  const unsigned lead = (unsigned)(bit0 & 31ull);
  unsigned p = lead + wpre + x - mybits;  // local bit position of my first code
#pragma unroll
  for (int t = 0; t < HB_PER_THREAD; ++t) {
    const unsigned L = (unsigned)(e[t] >> 32);
    if (L == 0) continue;
    const unsigned code = (unsigned)e[t];
    const unsigned wi = p >> 5, o = p & 31u;
    if (o + L <= 32u) {
      atomicOr(&sbits[wi], code << (32u - o - L));
    } else {
      atomicOr(&sbits[wi], code >> (o + L - 32u));
      atomicOr(&sbits[wi + 1], code << (64u - o - L));
    }
    p += L;
  }
  __syncthreads();
  const unsigned nloc = (lead + tot + 31u) >> 5;
  const unsigned long long w0 = bit0 >> 5;
  for (unsigned i = threadIdx.x; i < nloc; i += HB_THREADS) {
    const unsigned v = bswap32(sbits[i]);
    if (i == 0 || i == nloc - 1) {
      if (v) atomicOr(&out[w0 + i], v);
    } else {
      out[w0 + i] = v;
    }
  }
}

// --------------------------------------------------------------- driver --
HuffWorkspace::~HuffWorkspace() {
  cudaFree(d_hist);
  cudaFree(d_lut);
  cudaFree(d_blk);
  cudaFree(d_out);
  cudaFreeHost(h_hist);
  cudaFreeHost(h_lut);
  cudaFreeHost(h_bits);
}

static int ws_prepare(HuffWorkspace &ws) {
  if (ws.d_hist) return FFCZ_OK;
  FFCZ_CUDA(cudaGetDevice(&ws.device));
  FFCZ_CUDA(cudaMalloc(&ws.d_hist, 65536 * sizeof(unsigned)));
  FFCZ_CUDA(cudaMalloc(&ws.d_lut, 65536 * sizeof(unsigned long long)));
  FFCZ_CUDA(cudaMallocHost(&ws.h_hist, 65536 * sizeof(unsigned)));
  FFCZ_CUDA(cudaMallocHost(&ws.h_lut, 65536 * sizeof(unsigned long long)));
  FFCZ_CUDA(cudaFuncSetAttribute(k_hist_u16, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 32768 * (int)sizeof(unsigned)));
  return FFCZ_OK;
}

// Dense histogram of n symbols (256 or 65536 bins) into ws.d_hist.
static int launch_histogram(HuffWorkspace &ws, const void *d_data, size_t n, int symbol_bytes, cudaStream_t stream) {
  const size_t nbins = symbol_bytes == 1 ? 256 : 65536;
  FFCZ_CUDA(cudaMemsetAsync(ws.d_hist, 0, nbins * sizeof(unsigned), stream));
  if (symbol_bytes == 1) {
    const int grid = (int)std::min<size_t>(ceil_div(n, 256 * 16), 1024);
    k_hist_u8<<<grid, 256, 0, stream>>>((const uint8_t *)d_data, (long long)n, ws.d_hist);
  } else {
    // enough blocks to fill the SMs (the zeroing and flushing of a block's
    // 128 KB of counters runs on every SM at once), at most H16_CHUNK each
    const size_t chunk = std::min<size_t>(H16_CHUNK, std::max<size_t>(4096, round_up(ceil_div(n, (size_t)152), 8)));
    const size_t grid = ceil_div(n, chunk);
    k_hist_u16<<<(unsigned)grid, 256, 32768 * sizeof(unsigned), stream>>>((const uint16_t *)d_data,
                                                                           (long long)n, (int)chunk, ws.d_hist);
  }
  ws.launches++;
  FFCZ_CUDA(cudaGetLastError());
  return FFCZ_OK;
}

int huff_encode_device(HuffWorkspace &ws, const void *d_data, size_t n, int symbol_bytes,
                       cudaStream_t stream, ffcz_huff_result &res) {
  if (n == 0) return fail(FFCZ_ERR_EMPTY, "Empty data");
  if (symbol_bytes != 1 && symbol_bytes != 2) return fail(FFCZ_ERR_INVALID, "symbol_bytes must be 1 or 2");
  if (((uintptr_t)d_data) & 15) return fail(FFCZ_ERR_INVALID, "device symbols must be 16-byte aligned");
  FFCZ_TRY(ws_prepare(ws));
  const size_t nbins = symbol_bytes == 1 ? 256 : 65536;
  ws.launches = 0;
  FFCZ_TRY(launch_histogram(ws, d_data, n, symbol_bytes, stream));
  FFCZ_CUDA(cudaMemcpyAsync(ws.h_hist, ws.d_hist, nbins * sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
  FFCZ_CUDA(cudaStreamSynchronize(stream));

  Codebook cb;
  build_codebook(ws.h_hist, nbins, cb);
  if (cb.sym.empty()) return fail(FFCZ_ERR_EMPTY, "No symbols found");
  if (cb.max_len > 32)
    return fail(FFCZ_ERR_CODE_TOO_LONG, "Huffman code longer than 32 bits (" + std::to_string(cb.max_len) + ")");
  std::memset(ws.h_lut, 0, nbins * sizeof(unsigned long long));
  unsigned long long total_bits = 0;
  for (size_t i = 0; i < cb.sym.size(); ++i) {
    ws.h_lut[cb.sym[i]] = ((unsigned long long)cb.len[i] << 32) | cb.code[i];
    total_bits += (unsigned long long)cb.freq[i] * (unsigned long long)cb.len[i];
  }
  FFCZ_CUDA(cudaMemcpyAsync(ws.d_lut, ws.h_lut, nbins * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                            stream));
  const size_t nblk = ceil_div(n, HB_CHUNK);
  if (nblk > ws.blk_cap) {
    cudaFree(ws.d_blk);
    ws.d_blk = nullptr;
    FFCZ_CUDA(cudaMalloc(&ws.d_blk, nblk * sizeof(unsigned long long)));
    ws.blk_cap = nblk;
  }
  const size_t nwords = (size_t)((total_bits + 31) / 32) + 1;
  if (nwords > ws.out_cap) {
    cudaFree(ws.d_out);
    ws.d_out = nullptr;
    FFCZ_CUDA(cudaMalloc(&ws.d_out, nwords * sizeof(unsigned)));
    ws.out_cap = nwords;
  }
  FFCZ_CUDA(cudaMemsetAsync(ws.d_out, 0, nwords * sizeof(unsigned), stream));
  if (symbol_bytes == 1) {
    k_huff_bits<uint8_t><<<(unsigned)nblk, HB_THREADS, 0, stream>>>((const uint8_t *)d_data, (long long)n,
                                                                     ws.d_lut, ws.d_blk);
    k_scan_u64<<<1, 1024, 0, stream>>>(ws.d_blk, (long long)nblk);
    k_huff_pack<uint8_t><<<(unsigned)nblk, HB_THREADS, 0, stream>>>((const uint8_t *)d_data, (long long)n,
                                                                     ws.d_lut, ws.d_blk, ws.d_out);
  } else {
    k_huff_bits<uint16_t><<<(unsigned)nblk, HB_THREADS, 0, stream>>>((const uint16_t *)d_data, (long long)n,
                                                                      ws.d_lut, ws.d_blk);
    k_scan_u64<<<1, 1024, 0, stream>>>(ws.d_blk, (long long)nblk);
    k_huff_pack<uint16_t><<<(unsigned)nblk, HB_THREADS, 0, stream>>>((const uint16_t *)d_data, (long long)n,
                                                                      ws.d_lut, ws.d_blk, ws.d_out);
  }
  ws.launches += 3;
  FFCZ_CUDA(cudaGetLastError());
  const size_t nbytes = (size_t)((total_bits + 7) / 8);
  if (nbytes > ws.hbits_cap) {
    cudaFreeHost(ws.h_bits);
    ws.h_bits = nullptr;
    FFCZ_CUDA(cudaMallocHost(&ws.h_bits, nbytes ? nbytes : 1));
    ws.hbits_cap = nbytes;
  }
  if (nbytes)
    FFCZ_CUDA(cudaMemcpyAsync(ws.h_bits, ws.d_out, nbytes, cudaMemcpyDeviceToHost, stream));
  FFCZ_CUDA(cudaStreamSynchronize(stream));
  res.bitstream.assign(ws.h_bits, ws.h_bits + nbytes);
  res.symbols = cb.sym;
  res.codes = cb.code;
  res.lengths = cb.len;
  res.num_elements = n;
  res.compressed.clear();
  return FFCZ_OK;
}

int huff_zstd(ffcz_huff_result &res, int level, int mode) {
  if (mode == FFCZ_ZSTD_NONE) {
    res.compressed.clear();
    return FFCZ_OK;
  }
  return zstd_compress(res.bitstream.data(), res.bitstream.size(), level, mode == FFCZ_ZSTD_CHUNKED,
                       res.compressed);
}

// Process-wide encoder state for the standalone entry points (one per
// device, serialised by a mutex).
namespace {
std::mutex g_ws_mu;
HuffWorkspace *g_ws[64];
cudaStream_t g_stream[64];
}  // namespace

static int global_encode(const void *data, size_t n, int sb, bool host_data, int level, int mode,
                         cudaStream_t user_stream, ffcz_huff_result **out) {
  if (!out) return fail(FFCZ_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (n == 0) return fail(FFCZ_ERR_EMPTY, "Empty data");
  if (!data) return fail(FFCZ_ERR_INVALID, "data is NULL");
  int dev = 0;
  FFCZ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FFCZ_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_ws_mu);
  if (!g_ws[dev]) {
    g_ws[dev] = new HuffWorkspace();
    FFCZ_CUDA(cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking));
  }
  cudaStream_t st = host_data ? g_stream[dev] : user_stream;
  const void *d = data;
  void *tmp = nullptr;
  if (host_data) {
    FFCZ_CUDA(cudaMallocAsync(&tmp, n * sb + 16, st));
    FFCZ_CUDA(cudaMemcpyAsync(tmp, data, n * sb, cudaMemcpyHostToDevice, st));
    d = tmp;
  }
  ffcz_huff_result *r = new ffcz_huff_result();
  int rc = huff_encode_device(*g_ws[dev], d, n, sb, st, *r);
  if (tmp) cudaFreeAsync(tmp, st);
  if (rc == FFCZ_OK) rc = huff_zstd(*r, level, mode);
  if (rc != FFCZ_OK) {
    delete r;
    return rc;
  }
  *out = r;
  return FFCZ_OK;
}

}  // namespace ffcz

using namespace ffcz;

extern "C" {

int ffcz_huff_compress_u16(const uint16_t *h_data, size_t n, int zstd_level, ffcz_huff_result **out) {
  return global_encode(h_data, n, 2, true, zstd_level, FFCZ_ZSTD_SINGLE, nullptr, out);
}
int ffcz_huff_compress_u8(const uint8_t *h_data, size_t n, int zstd_level, ffcz_huff_result **out) {
  return global_encode(h_data, n, 1, true, zstd_level, FFCZ_ZSTD_SINGLE, nullptr, out);
}
int ffcz_huff_compress_device(const void *d_data, size_t n, int symbol_bytes, int zstd_level, int zstd_mode,
                              void *stream, ffcz_huff_result **out) {
  if (symbol_bytes != 1 && symbol_bytes != 2) return fail(FFCZ_ERR_INVALID, "symbol_bytes must be 1 or 2");
  if (zstd_mode < FFCZ_ZSTD_SINGLE || zstd_mode > FFCZ_ZSTD_NONE) return fail(FFCZ_ERR_INVALID, "unknown ZSTD mode");
  return global_encode(d_data, n, symbol_bytes, false, zstd_level, zstd_mode, (cudaStream_t)stream, out);
}
void ffcz_huff_result_free(ffcz_huff_result *r) { delete r; }

int ffcz_huff_histogram_device(const void *d_data, size_t n, int symbol_bytes, void *stream, uint32_t *h_hist) {
  if (!d_data || !h_hist) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (symbol_bytes != 1 && symbol_bytes != 2) return fail(FFCZ_ERR_INVALID, "symbol_bytes must be 1 or 2");
  if (((uintptr_t)d_data) & 15) return fail(FFCZ_ERR_INVALID, "device symbols must be 16-byte aligned");
  const size_t nbins = symbol_bytes == 1 ? 256 : 65536;
  if (n == 0) {
    std::memset(h_hist, 0, nbins * sizeof(uint32_t));
    return FFCZ_OK;
  }
  int dev = 0;
  FFCZ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(FFCZ_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lk(g_ws_mu);
  if (!g_ws[dev]) {
    g_ws[dev] = new HuffWorkspace();
    FFCZ_CUDA(cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking));
  }
  HuffWorkspace &ws = *g_ws[dev];
  FFCZ_TRY(ws_prepare(ws));
  cudaStream_t st = (cudaStream_t)stream;
  FFCZ_TRY(launch_histogram(ws, d_data, n, symbol_bytes, st));
  FFCZ_CUDA(cudaMemcpyAsync(ws.h_hist, ws.d_hist, nbins * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  FFCZ_CUDA(cudaStreamSynchronize(st));
  std::memcpy(h_hist, ws.h_hist, nbins * sizeof(uint32_t));
  return FFCZ_OK;
}

int ffcz_huff_tree(const uint32_t *freqs, size_t n, int32_t *left, int32_t *right, uint64_t *weights,
                   int32_t *root) {
  if (!root || (n && (!freqs || !left || !right || !weights))) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (n > (size_t)1 << 30) return fail(FFCZ_ERR_INVALID, "too many symbols");
  if (n == 0) {
    *root = -1;
    return FFCZ_OK;
  }
  std::vector<int> l, r;
  std::vector<uint64_t> w;
  build_tree(freqs, (int)n, l, r, w);
  const size_t nodes = 2 * n - 1;
  for (size_t i = 0; i < nodes; ++i) {
    left[i] = l[i];
    right[i] = r[i];
    weights[i] = w[i];
  }
  *root = (int32_t)(nodes - 1);
  return FFCZ_OK;
}

int ffcz_huff_codebook(const uint32_t *hist, size_t nbins, uint32_t *symbols, uint32_t *codes, int32_t *lengths,
                       size_t cap, size_t *n) {
  if (!n || (nbins && !hist)) return fail(FFCZ_ERR_INVALID, "NULL argument");
  Codebook cb;
  build_codebook(hist, nbins, cb);
  *n = cb.sym.size();
  if (cb.sym.size() > cap) return fail(FFCZ_ERR_CAPACITY, "more symbols than the arrays hold");
  if (!cb.sym.empty() && (!symbols || !codes || !lengths)) return fail(FFCZ_ERR_INVALID, "NULL argument");
  for (size_t i = 0; i < cb.sym.size(); ++i) {
    symbols[i] = cb.sym[i];
    codes[i] = cb.code[i];
    lengths[i] = cb.len[i];
  }
  return FFCZ_OK;
}

size_t ffcz_zstd_bound(size_t n) { return zstd_bound(n); }

int ffcz_zstd_compress(const uint8_t *src, size_t n, int level, int mode, uint8_t *dst, size_t cap,
                       size_t *out_len) {
  if ((!src && n) || !dst || !out_len) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (mode != FFCZ_ZSTD_SINGLE && mode != FFCZ_ZSTD_CHUNKED) return fail(FFCZ_ERR_INVALID, "unknown ZSTD mode");
  std::vector<uint8_t> out;
  FFCZ_TRY(zstd_compress(src, n, level, mode == FFCZ_ZSTD_CHUNKED, out));
  *out_len = out.size();
  if (cap < out.size()) return fail(FFCZ_ERR_CAPACITY, "destination too small");
  if (!out.empty()) std::memcpy(dst, out.data(), out.size());
  return FFCZ_OK;
}

int ffcz_huff_result_create(const uint8_t *compressed, size_t comp_len, const uint8_t *bitstream,
                            size_t bitstream_bytes, const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols, size_t num_elements,
                            ffcz_huff_result **out) {
  if (!out) return fail(FFCZ_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if ((!compressed && comp_len) || (num_symbols && (!symbols || !codes || !lengths)))
    return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::unique_ptr<ffcz_huff_result> r(new ffcz_huff_result());
  r->compressed.assign(compressed, compressed + comp_len);
  if (bitstream) {
    r->bitstream.assign(bitstream, bitstream + bitstream_bytes);
  } else {
    FFCZ_TRY(zstd_decompress(compressed, comp_len, bitstream_bytes, r->bitstream));
    r->bitstream.resize(bitstream_bytes, 0);
  }
  r->symbols.assign(symbols, symbols + num_symbols);
  r->codes.assign(codes, codes + num_symbols);
  r->lengths.assign(lengths, lengths + num_symbols);
  r->num_elements = num_elements;
  *out = r.release();
  return FFCZ_OK;
}

int ffcz_huff_result_sizes(const ffcz_huff_result *r, size_t *compressed_bytes, size_t *bitstream_bytes,
                           size_t *num_elements, size_t *num_symbols) {
  if (!r) return fail(FFCZ_ERR_INVALID, "result is NULL");
  if (compressed_bytes) *compressed_bytes = r->compressed.size();
  if (bitstream_bytes) *bitstream_bytes = r->bitstream.size();
  if (num_elements) *num_elements = r->num_elements;
  if (num_symbols) *num_symbols = r->symbols.size();
  return FFCZ_OK;
}
int ffcz_huff_result_compressed(const ffcz_huff_result *r, uint8_t *dst, size_t cap) {
  if (!r || (!dst && !r->compressed.empty())) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (cap < r->compressed.size()) return fail(FFCZ_ERR_CAPACITY, "destination too small");
  if (!r->compressed.empty()) std::memcpy(dst, r->compressed.data(), r->compressed.size());
  return FFCZ_OK;
}
int ffcz_huff_result_view(const ffcz_huff_result *r, int which, const void **ptr, size_t *count) {
  if (!r || !ptr || !count) return fail(FFCZ_ERR_INVALID, "NULL argument");
  switch (which) {
    case 0: *ptr = r->compressed.data(); *count = r->compressed.size(); break;
    case 1: *ptr = r->bitstream.data(); *count = r->bitstream.size(); break;
    case 2: *ptr = r->symbols.data(); *count = r->symbols.size(); break;
    case 3: *ptr = r->codes.data(); *count = r->codes.size(); break;
    case 4: *ptr = r->lengths.data(); *count = r->lengths.size(); break;
    default: return fail(FFCZ_ERR_INVALID, "unknown buffer");
  }
  return FFCZ_OK;
}

int ffcz_huff_result_bitstream(const ffcz_huff_result *r, uint8_t *dst, size_t cap) {
  if (!r || (!dst && !r->bitstream.empty())) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (cap < r->bitstream.size()) return fail(FFCZ_ERR_CAPACITY, "destination too small");
  if (!r->bitstream.empty()) std::memcpy(dst, r->bitstream.data(), r->bitstream.size());
  return FFCZ_OK;
}
int ffcz_huff_result_codes(const ffcz_huff_result *r, uint32_t *symbols, uint32_t *codes, int32_t *lengths,
                           size_t cap) {
  if (!r || !symbols || !codes || !lengths) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (cap < r->symbols.size()) return fail(FFCZ_ERR_CAPACITY, "destination too small");
  for (size_t i = 0; i < r->symbols.size(); ++i) {
    symbols[i] = r->symbols[i];
    codes[i] = r->codes[i];
    lengths[i] = r->lengths[i];
  }
  return FFCZ_OK;
}

static int decompress_any(const uint8_t *comp, size_t comp_len, const uint32_t *symbols, const uint32_t *codes,
                          const int32_t *lengths, size_t nsym, size_t num_elements, size_t bitstream_bytes,
                          void *out, int sb, size_t *out_len) {
  if ((!comp && comp_len) || (!symbols && nsym) || !out_len || (!out && num_elements))
    return fail(FFCZ_ERR_INVALID, "NULL argument");
  std::vector<uint8_t> bits;
  FFCZ_TRY(zstd_decompress(comp, comp_len, bitstream_bytes, bits));
  bits.resize(bitstream_bytes, 0);
  std::vector<uint32_t> dec =
      huffman_decode(bits.data(), bits.size(), symbols, codes, lengths, nsym, num_elements);
  for (size_t i = 0; i < dec.size(); ++i) {
    if (sb == 2) ((uint16_t *)out)[i] = (uint16_t)dec[i];
    else ((uint8_t *)out)[i] = (uint8_t)dec[i];
  }
  *out_len = dec.size();
  return FFCZ_OK;
}

int ffcz_huff_decompress_u16(const uint8_t *comp, size_t comp_len, const uint32_t *symbols, const uint32_t *codes,
                             const int32_t *lengths, size_t num_symbols, size_t num_elements,
                             size_t bitstream_bytes, uint16_t *out, size_t *out_len) {
  return decompress_any(comp, comp_len, symbols, codes, lengths, num_symbols, num_elements, bitstream_bytes, out,
                        2, out_len);
}
int ffcz_huff_decompress_u8(const uint8_t *comp, size_t comp_len, const uint32_t *symbols, const uint32_t *codes,
                            const int32_t *lengths, size_t num_symbols, size_t num_elements,
                            size_t bitstream_bytes, uint8_t *out, size_t *out_len) {
  return decompress_any(comp, comp_len, symbols, codes, lengths, num_symbols, num_elements, bitstream_bytes, out,
                        1, out_len);
}

}  // extern "C"
