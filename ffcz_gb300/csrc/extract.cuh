// Edit compaction (projection_algorithm_impl.cuh:371-456 and
// projection_algorithm.cu:365-379, 382-405, 427-457, 459-550) instead of the
// reference's flag kernels, two CUB reductions, a CUB scan, the scatter
// kernel and two bool-pack kernels.  The solver uses the single-read form
// further down (k_ex_part, k_ex_scan_rec, k_ex_place); the two-read form
// below serves the no-allocation entry point, whose caller-provided scratch
// has no room for the compacted values:
//   k_ex_stats   : per 4096-element chunk: #(|v| > thr), min, max   (R n*s)
//   k_ex_scan    : one block: chunk offsets (exclusive scan), global
//                  min/max, active count                        (tiny)
//   k_ex_compact : chunk re-read; per-thread flag bits + one block scan give
//                  the positions; scatter of the active values and their
//                  uint16 quantisation; LSB-first flag words from thread
//                  pairs                                   (R n*s, W 2*cnt*s + n/8)
#pragma once

#include "common.cuh"

namespace ffcz {

constexpr int EX_THREADS = 256;
constexpr int EX_ROUNDS = 16;
constexpr int EX_CHUNK = EX_THREADS * EX_ROUNDS;  // 4096

template <typename T> __device__ __forceinline__ T dev_inf();
template <> __device__ __forceinline__ float dev_inf<float>() { return __int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double dev_inf<double>() {
  return __longlong_as_double(0x7ff0000000000000ll);
}

template <typename T> __device__ __forceinline__ T div_rn(T a, T b);
template <> __device__ __forceinline__ float div_rn<float>(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ double div_rn<double>(double a, double b) { return __ddiv_rn(a, b); }
template <typename T> __device__ __forceinline__ T mul_rn(T a, T b);
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T sub_rn(T a, T b);
template <> __device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }

// uint16 quantiser of projection_algorithm.cu:447-455:
// n = (v - mn)/(mx - mn) in T; q = n > 0.5 ? ceil(n*65535) : floor(n*65535).
template <typename T>
__device__ __forceinline__ uint16_t quantize16(T v, T mn, T mx) {
  const T nrm = div_rn<T>(sub_rn<T>(v, mn), sub_rn<T>(mx, mn));
  const T s = mul_rn<T>(nrm, T(65535));
  const T q = (nrm > T(0.5)) ? ceil(s) : floor(s);
  if (!(q == q)) return 0;  // 0/0 when every entry is equal: cvt of NaN gives 0
  return (uint16_t)(unsigned)q;
}

// Thread t of a block owns the 16 consecutive values [base + 16t, +16) of
// its 4096-value chunk: 16-byte vector loads, thread-order = element order.
constexpr int EX_PER = EX_CHUNK / EX_THREADS;  // 16

template <typename T>
__device__ __forceinline__ int load16(const T *__restrict__ a, long long n, long long i0, T (&v)[EX_PER]) {
  if (i0 + EX_PER <= n) {
    if (sizeof(T) == 4) {
      const float4 *p = reinterpret_cast<const float4 *>(a + i0);
#pragma unroll
      for (int q = 0; q < EX_PER / 4; ++q) {
        const float4 f = p[q];
        v[4 * q] = (T)f.x;
        v[4 * q + 1] = (T)f.y;
        v[4 * q + 2] = (T)f.z;
        v[4 * q + 3] = (T)f.w;
      }
    } else {
      const double2 *p = reinterpret_cast<const double2 *>(a + i0);
#pragma unroll
      for (int q = 0; q < EX_PER / 2; ++q) {
        const double2 f = p[q];
        v[2 * q] = (T)f.x;
        v[2 * q + 1] = (T)f.y;
      }
    }
    return EX_PER;
  }
  const int cnt = (int)max(0ll, min((long long)EX_PER, n - i0));
#pragma unroll
  for (int t = 0; t < EX_PER; ++t) v[t] = (t < cnt) ? a[i0 + t] : T(0);
  return cnt;
}

template <typename T>
__global__ void __launch_bounds__(EX_THREADS) k_ex_stats(const T *__restrict__ a, long long n, T thr,
                                                         unsigned *__restrict__ blk_cnt,
                                                         T *__restrict__ blk_mn,
                                                         T *__restrict__ blk_mx) {
  const long long i0 = (long long)blockIdx.x * EX_CHUNK + (long long)threadIdx.x * EX_PER;
  T v[EX_PER];
  const int cnt_valid = load16<T>(a, n, i0, v);
  unsigned cnt = 0;
  T mn = dev_inf<T>(), mx = -dev_inf<T>();
#pragma unroll
  for (int t = 0; t < EX_PER; ++t) {
    if (t < cnt_valid) {
      cnt += (fabs(v[t]) > thr) ? 1u : 0u;
      mn = (v[t] < mn) ? v[t] : mn;
      mx = (v[t] > mx) ? v[t] : mx;
    }
  }
  __shared__ unsigned sc[EX_THREADS / 32];
  __shared__ T smn[EX_THREADS / 32], smx[EX_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    const T a1 = __shfl_xor_sync(0xffffffffu, mn, o);
    const T b1 = __shfl_xor_sync(0xffffffffu, mx, o);
    mn = (a1 < mn) ? a1 : mn;
    mx = (b1 > mx) ? b1 : mx;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sc[warp] = cnt;
    smn[warp] = mn;
    smx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned c = 0;
    T lo = smn[0], hi = smx[0];
    for (int w = 0; w < EX_THREADS / 32; ++w) {
      c += sc[w];
      lo = (smn[w] < lo) ? smn[w] : lo;
      hi = (smx[w] > hi) ? smx[w] : hi;
    }
    blk_cnt[blockIdx.x] = c;
    blk_mn[blockIdx.x] = lo;
    blk_mx[blockIdx.x] = hi;
  }
}

// One block of 1024 threads.  Exclusive scan of blk_cnt in place, global
// min/max into mnmx[0..1] (T) and the count / min / max into ctl slot
// `which` (0 = frequency, 1 = spatial).
template <typename T>
__global__ void __launch_bounds__(1024) k_ex_scan(unsigned *__restrict__ blk_cnt, long long nblk,
                                                  const T *__restrict__ blk_mn,
                                                  const T *__restrict__ blk_mx,
                                                  T *__restrict__ mnmx, LoopCtl *ctl, int which) {
  __shared__ unsigned long long wsum[32];
  __shared__ T wmn[32], wmx[32];
  __shared__ unsigned long long carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  T mn = dev_inf<T>(), mx = -dev_inf<T>();
  __syncthreads();
  for (long long b0 = 0; b0 < nblk; b0 += 1024) {
    const long long i = b0 + threadIdx.x;
    unsigned long long v = 0;
    if (i < nblk) {
      v = blk_cnt[i];
      const T a1 = blk_mn[i], b1 = blk_mx[i];
      mn = (a1 < mn) ? a1 : mn;
      mx = (b1 > mx) ? b1 : mx;
    }
    unsigned long long x = v;
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
      wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const unsigned long long wpre = warp ? wsum[warp - 1] : 0ull;
    const unsigned long long excl = carry + wpre + x - v;
    if (i < nblk) blk_cnt[i] = (unsigned)excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += wsum[31];
    __syncthreads();
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T a1 = __shfl_xor_sync(0xffffffffu, mn, o);
    const T b1 = __shfl_xor_sync(0xffffffffu, mx, o);
    mn = (a1 < mn) ? a1 : mn;
    mx = (b1 > mx) ? b1 : mx;
  }
  if (lane == 0) {
    wmn[warp] = mn;
    wmx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 32; ++w) {
      mn = (wmn[w] < mn) ? wmn[w] : mn;
      mx = (wmx[w] > mx) ? wmx[w] : mx;
    }
    mn = (wmn[0] < mn) ? wmn[0] : mn;
    mx = (wmx[0] > mx) ? wmx[0] : mx;
    mnmx[0] = mn;
    mnmx[1] = mx;
    ctl->count[which] = carry;
    ctl->mn[which] = (double)mn;
    ctl->mx[which] = (double)mx;
  }
}

// Positions: per-thread count of active values -> block exclusive scan
// (one barrier) -> each thread writes its active values in order.  Flag
// words: thread pairs (2u, 2u+1) hold the 32 flags of word base/32 + u.
template <typename T>
__global__ void __launch_bounds__(EX_THREADS) k_ex_compact(
    const T *__restrict__ a, long long n, T thr, const unsigned *__restrict__ blk_off,
    const T *__restrict__ mnmx, T *__restrict__ compact, uint16_t *__restrict__ quant,
    unsigned *__restrict__ pack_words, int write_pack) {
  __shared__ unsigned wsum[EX_THREADS / 32];
  const long long i0 = (long long)blockIdx.x * EX_CHUNK + (long long)threadIdx.x * EX_PER;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T v[EX_PER];
  const int cnt_valid = load16<T>(a, n, i0, v);
  unsigned bits = 0;
#pragma unroll
  for (int t = 0; t < EX_PER; ++t)
    if (t < cnt_valid && fabs(v[t]) > thr) bits |= 1u << t;
  const unsigned mine = __popc(bits);
  unsigned x = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  const unsigned partner = __shfl_down_sync(0xffffffffu, bits, 1);
  if (write_pack && !(lane & 1) && i0 < n) pack_words[i0 >> 5] = bits | (partner << 16);
  __syncthreads();
  unsigned wpre = 0;
#pragma unroll
  for (int w = 0; w < EX_THREADS / 32; ++w) wpre += (w < warp) ? wsum[w] : 0u;
  if (!bits) return;
  const T mn = mnmx[0], mx = mnmx[1];
  unsigned pos = blk_off[blockIdx.x] + wpre + x - mine;
#pragma unroll
  for (int t = 0; t < EX_PER; ++t) {
    if (bits & (1u << t)) {
      compact[pos] = v[t];
      quant[pos] = quantize16<T>(v[t], mn, mx);
      ++pos;
    }
  }
}

// ---------------------------------------------------------------------------
// Single-read compaction (the solver's path): three launches per
// accumulator, the edit array read once.  A chunk is the span of one warp (8
// coalesced 16-byte loads per lane: 1024 FP32 / 512 FP64 values), a group
// the 8 chunks of one block.
//   k_ex_part     : warp = chunk: flag words (shuffles), lane offsets of the
//                   active values (three ballots of the per-lane counts),
//                   the active values compacted into scratch at the chunk's
//                   own start, the chunk's count; per block a group record
//                   (count, min and max as order-preserving integer keys)
//                                                  (R n*s, W cnt*s + n/8)
//                   With a clean flag that reads 0 (an accumulator nothing
//                   has written since it was cleared) it writes zero flag
//                   words and zero records without reading the array (W n/8).
//   k_ex_scan_rec : one block: exclusive offsets of the groups, whole-array
//                   count, min and max
//   k_ex_place    : one warp per chunk moves the chunk's values to their
//                   final positions and quantises them (R cnt*s, W cnt*(s+2))
// Group records are struct-of-arrays padded to a multiple of XP_PAD groups;
// the padding keeps its initial neutral values (count 0, min key ~0, max
// key 0), so the scan reads whole 16-byte vectors.
constexpr int XP_NQ = 8;                 // 16-byte loads per lane
constexpr int XP_WPG = EX_THREADS / 32;  // chunks (warps) per group (block)
template <typename T> __host__ __device__ constexpr int xp_vec() { return 16 / (int)sizeof(T); }
template <typename T> __host__ __device__ constexpr int xp_chunk() { return 32 * XP_NQ * xp_vec<T>(); }
template <typename T> __host__ __device__ constexpr int xp_group() { return XP_WPG * xp_chunk<T>(); }
constexpr int XP_PAD = 4096;

struct ExRec {
  unsigned *wcnt;                       // per chunk
  unsigned *cnt;                        // per group
  unsigned long long *kmn, *kmx, *off;  // per group
};

template <typename T> __device__ __forceinline__ unsigned long long ord_key(T v);
template <> __device__ __forceinline__ unsigned long long ord_key<float>(float v) {
  const unsigned u = __float_as_uint(v);
  return (unsigned long long)(u ^ ((u >> 31) ? 0xffffffffu : 0x80000000u));
}
template <> __device__ __forceinline__ unsigned long long ord_key<double>(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return u ^ ((u >> 63) ? ~0ull : 0x8000000000000000ull);
}
template <typename T> __device__ __forceinline__ T key_val(unsigned long long k);
template <> __device__ __forceinline__ float key_val<float>(unsigned long long k) {
  const unsigned u = (unsigned)k;
  return __uint_as_float(u ^ ((u >> 31) ? 0x80000000u : 0xffffffffu));
}
template <> __device__ __forceinline__ double key_val<double>(unsigned long long k) {
  return __longlong_as_double((long long)(k ^ ((k >> 63) ? 0x8000000000000000ull : ~0ull)));
}

// One chunk of one warp; FULL: every value of the chunk lies below n.
// Returns the chunk's active count (the same in every lane).
template <typename T, bool FULL>
__device__ __forceinline__ unsigned ex_chunk(const T *__restrict__ a, long long n, long long base, T thr,
                                             T *__restrict__ dst, unsigned *__restrict__ pack_words,
                                             int write_pack, T &mn, T &mx, bool &any) {
  constexpr int VEC = xp_vec<T>(), SPAN = 32 * VEC;
  constexpr int LPW = 32 / VEC;  // lanes per 32-bit flag word
  const int lane = threadIdx.x & 31;
  T v[XP_NQ][VEC];
  unsigned f[XP_NQ];
#pragma unroll
  for (int q = 0; q < XP_NQ; ++q) {
    const long long i = base + q * SPAN + lane * VEC;
    if (FULL || i + VEC <= n) {
      if constexpr (VEC == 4) {
        const float4 t = *reinterpret_cast<const float4 *>(a + i);
        v[q][0] = t.x;
        v[q][1] = t.y;
        v[q][2] = t.z;
        v[q][3] = t.w;
      } else {
        const double2 t = *reinterpret_cast<const double2 *>(a + i);
        v[q][0] = t.x;
        v[q][1] = t.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < VEC; ++j) v[q][j] = (i + j < n) ? a[i + j] : T(0);
    }
  }
#pragma unroll
  for (int q = 0; q < XP_NQ; ++q) {
    const long long i = base + q * SPAN + lane * VEC;
    unsigned bits = 0;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      const T x = v[q][j];
      if (FULL || i + j < n) {
        bits |= (fabs(x) > thr) ? 1u << j : 0u;
        mn = fmin(mn, x);
        mx = fmax(mx, x);
      }
    }
    if (!FULL && i < n) any = true;
    f[q] = bits;
    // flag word of the 32 values [base + q*SPAN + 32*(lane/LPW), +32)
    unsigned w = bits << (VEC * (lane % LPW));
#pragma unroll
    for (int o = 1; o < LPW; o <<= 1) w |= __shfl_xor_sync(0xffffffffu, w, o);
    if (write_pack && lane % LPW == 0 && (FULL || i < n)) pack_words[i >> 5] = w;
  }
  if (FULL) any = true;
  // offsets: values of the chunk in element order (q, lane, j)
  const unsigned lt = (1u << lane) - 1u;
  unsigned run = 0;
#pragma unroll
  for (int q = 0; q < XP_NQ; ++q) {
    const unsigned k = __popc(f[q]);  // 0 .. VEC (<= 4)
    const unsigned b0 = __ballot_sync(0xffffffffu, k & 1u), b1 = __ballot_sync(0xffffffffu, k & 2u),
                   b2 = __ballot_sync(0xffffffffu, k & 4u);
    if (b0 | b1 | b2) {
      if (f[q]) {
        T *d = dst + run + __popc(b0 & lt) + 2u * __popc(b1 & lt) + 4u * __popc(b2 & lt);
#pragma unroll
        for (int j = 0; j < VEC; ++j)
          if (f[q] & (1u << j)) *d++ = v[q][j];
      }
      run += __popc(b0) + 2u * __popc(b1) + 4u * __popc(b2);
    }
  }
  return run;
}

// State of an accumulator's compaction outputs (xst[0]): 1 while its records
// and flag words hold the results of the untouched (all-zero) array, apart
// from the flag words listed in xst[2 .. 2 + xst[1]) that the last listed fold
// set bits in.  While the accumulator is untouched (dirty flag 0) a
// compaction then needs no pass: no active value, min = max = 0.
__device__ __forceinline__ bool ex_known_clean(const unsigned *dirty, const unsigned *xst) {
  return xst && dirty && *dirty == 0u && xst[0] != 0u;
}

template <typename T>
__global__ void __launch_bounds__(EX_THREADS, 3) k_ex_part(const T *__restrict__ a, long long n, long long nchunk, T thr,
                                                           const unsigned *__restrict__ dirty,
                                                           const unsigned *__restrict__ xst,
                                                           T *__restrict__ scratch, ExRec rec,
                                                           unsigned *__restrict__ pack_words, int write_pack) {
  constexpr int CH = xp_chunk<T>(), SPAN = 32 * xp_vec<T>();
  if (ex_known_clean(dirty, xst)) return;
  __shared__ unsigned scnt[XP_WPG];
  __shared__ unsigned long long smn[XP_WPG], smx[XP_WPG];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long c = (long long)blockIdx.x * XP_WPG + warp;
  T mn = dev_inf<T>(), mx = -dev_inf<T>();
  bool any = false;
  unsigned run = 0;
  if (dirty && *dirty == 0u) {
    // the accumulator is all zeros (nothing written since it was cleared):
    // zero flag words, no active value, min = max = 0, nothing read
    if (c < nchunk) {
      any = true;
      mn = mx = T(0);
      if (write_pack)
        for (int q = 0; q < XP_NQ; ++q) {
          const long long i = c * CH + (long long)q * SPAN + 32 * lane;
          if (32 * lane < SPAN && i < n) pack_words[i >> 5] = 0u;
        }
    }
  } else if (c < nchunk) {
    const long long base = c * CH;
    if (base + CH <= n)
      run = ex_chunk<T, true>(a, n, base, thr, scratch + base, pack_words, write_pack, mn, mx, any);
    else
      run = ex_chunk<T, false>(a, n, base, thr, scratch + base, pack_words, write_pack, mn, mx, any);
  }
  unsigned long long kmn = any ? ord_key<T>(mn) : ~0ull, kmx = any ? ord_key<T>(mx) : 0ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long p = __shfl_xor_sync(0xffffffffu, kmn, o);
    const unsigned long long q = __shfl_xor_sync(0xffffffffu, kmx, o);
    kmn = p < kmn ? p : kmn;
    kmx = q > kmx ? q : kmx;
  }
  if (lane == 0) {
    if (c < nchunk) rec.wcnt[c] = run;
    scnt[warp] = run;
    smn[warp] = kmn;
    smx[warp] = kmx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = 0;
    for (int w = 0; w < XP_WPG; ++w) {
      t += scnt[w];
      kmn = smn[w] < kmn ? smn[w] : kmn;
      kmx = smx[w] > kmx ? smx[w] : kmx;
    }
    rec.cnt[blockIdx.x] = t;
    rec.kmn[blockIdx.x] = kmn;
    rec.kmx[blockIdx.x] = kmx;
  }
}

// One block of XS_THREADS: thread t scans the group records [t*K, (t+1)*K)
// (K a multiple of 4, 16-byte vector loads) into exclusive offsets; the
// whole-array count, min and max go to mnmx and ctl slot `which`.
constexpr int XS_THREADS = 1024;
template <typename T>
__global__ void __launch_bounds__(XS_THREADS) k_ex_scan_rec(long long ngroup, ExRec rec, T *__restrict__ mnmx,
                                                            LoopCtl *__restrict__ ctl, int which,
                                                            const unsigned *__restrict__ dirty,
                                                            unsigned *__restrict__ xst) {
  constexpr int NW = XS_THREADS / 32;
  __shared__ unsigned long long wa[NW], wb[NW], wc[NW];
  if (ex_known_clean(dirty, xst)) {  // no active value, min = max = 0
    if (threadIdx.x == 0) {
      mnmx[0] = T(0);
      mnmx[1] = T(0);
      ctl->count[which] = 0ull;
      ctl->mn[which] = 0.0;
      ctl->mx[which] = 0.0;
    }
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long K = (ngroup + XP_PAD - 1) / XP_PAD * (XP_PAD / XS_THREADS);
  const long long r0 = threadIdx.x * K;
  unsigned long long sum = 0, kmn = ~0ull, kmx = 0ull;
#pragma unroll 4
  for (long long r = r0; r < r0 + K; r += 4) {
    const uint4 c4 = *reinterpret_cast<const uint4 *>(rec.cnt + r);
    const ulonglong2 m0 = *reinterpret_cast<const ulonglong2 *>(rec.kmn + r);
    const ulonglong2 m1 = *reinterpret_cast<const ulonglong2 *>(rec.kmn + r + 2);
    const ulonglong2 x0 = *reinterpret_cast<const ulonglong2 *>(rec.kmx + r);
    const ulonglong2 x1 = *reinterpret_cast<const ulonglong2 *>(rec.kmx + r + 2);
    sum += (unsigned long long)c4.x + c4.y + c4.z + c4.w;
    kmn = min(kmn, min(min(m0.x, m0.y), min(m1.x, m1.y)));
    kmx = max(kmx, max(max(x0.x, x0.y), max(x1.x, x1.y)));
  }
  unsigned long long xs = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, xs, o);
    if (lane >= o) xs += y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long p = __shfl_xor_sync(0xffffffffu, kmn, o);
    const unsigned long long q = __shfl_xor_sync(0xffffffffu, kmx, o);
    kmn = p < kmn ? p : kmn;
    kmx = q > kmx ? q : kmx;
  }
  if (lane == 31) wc[warp] = xs;
  if (lane == 0) {
    wa[warp] = kmn;
    wb[warp] = kmx;
  }
  __syncthreads();
  unsigned long long off = xs - sum, tot = 0;
  for (int w = 0; w < NW; ++w) {
    off += w < warp ? wc[w] : 0ull;
    tot += wc[w];
  }
#pragma unroll 4
  for (long long r = r0; r < r0 + K; r += 4) {
    const uint4 c4 = *reinterpret_cast<const uint4 *>(rec.cnt + r);
    ulonglong2 o0, o1;
    o0.x = off;
    o0.y = o0.x + c4.x;
    o1.x = o0.y + c4.y;
    o1.y = o1.x + c4.z;
    off = o1.y + c4.w;
    *reinterpret_cast<ulonglong2 *>(rec.off + r) = o0;
    *reinterpret_cast<ulonglong2 *>(rec.off + r + 2) = o1;
  }
  if (threadIdx.x == 0) {
    kmn = wa[0];
    kmx = wb[0];
    for (int w = 1; w < NW; ++w) {
      kmn = wa[w] < kmn ? wa[w] : kmn;
      kmx = wb[w] > kmx ? wb[w] : kmx;
    }
    const T gmn = key_val<T>(kmn), gmx = key_val<T>(kmx);
    mnmx[0] = gmn;
    mnmx[1] = gmx;
    ctl->count[which] = tot;
    ctl->mn[which] = (double)gmn;
    ctl->mx[which] = (double)gmx;
    // k_ex_part rewrote the records and the flag words: they hold the
    // untouched array's results exactly when it was untouched
    if (xst) {
      xst[0] = (dirty && *dirty == 0u) ? 1u : 0u;
      xst[1] = 0u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(EX_THREADS) k_ex_place(const T *__restrict__ scratch, long long nchunk, ExRec rec,
                                                         T *__restrict__ compact, uint16_t *__restrict__ quant,
                                                         const T *__restrict__ mnmx,
                                                         const unsigned *__restrict__ dirty,
                                                         const unsigned *__restrict__ xst) {
  constexpr int CH = xp_chunk<T>();
  if (ex_known_clean(dirty, xst)) return;  // nothing to place
  const int lane = threadIdx.x & 31;
  const long long wpb = EX_THREADS / 32;
  const T mn = mnmx[0], mx = mnmx[1];
  for (long long c = blockIdx.x * wpb + (threadIdx.x >> 5); c < nchunk; c += gridDim.x * wpb) {
    const long long g = c / XP_WPG;
    const int me = (int)(c - g * XP_WPG);
    // lane l < XP_WPG holds the count of chunk g*XP_WPG + l (chunks past the
    // end count 0)
    const unsigned wc = (lane < XP_WPG && g * XP_WPG + lane < nchunk) ? rec.wcnt[g * XP_WPG + lane] : 0u;
    unsigned before = lane < me ? wc : 0u;
#pragma unroll
    for (int o = 1; o < XP_WPG; o <<= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    before = __shfl_sync(0xffffffffu, before, 0);  // the sum sits in lanes 0 .. XP_WPG-1
    const long long cnt = (long long)__shfl_sync(0xffffffffu, wc, me);
    if (!cnt) continue;
    const unsigned long long off = rec.off[g] + before;
    const T *src = scratch + c * CH;
    // four loads in flight per lane
    for (long long r = lane; r < cnt; r += 128) {
      T v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (r + 32 * k < cnt) v[k] = src[r + 32 * k];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (r + 32 * k < cnt) {
          compact[off + r + 32 * k] = v[k];
          quant[off + r + 32 * k] = quantize16<T>(v[k], mn, mx);
        }
    }
  }
}

// ---------------------------------------------------------------------------
// Listed accumulators.  An edit accumulator whose dirty flag reads 0 but
// whose index list (slist[0] = count, slist[4..] = indices, at most
// EX_LIST_MAX) is non-empty holds zeros everywhere except at the listed
// indices (a list may repeat an index).  k_ex_part treats it as untouched
// (zero flag words and records, nothing read); this one block then folds
// the listed values into the results the full compaction gives for the
// array: the active values in ascending index order with their uint16
// codes, their flag bits, the count and the whole-array min and max (the
// zeros of the unlisted entries included).
constexpr int EX_LIST_MAX = 4096;
constexpr int EX_LIST_THREADS = 1024;

template <typename T>
__global__ void __launch_bounds__(EX_LIST_THREADS) k_ex_listed(const T *__restrict__ a, long long n, T thr,
                                                                const unsigned *__restrict__ dirty,
                                                                const unsigned *__restrict__ slist,
                                                                T *__restrict__ compact, uint16_t *__restrict__ quant,
                                                                unsigned *__restrict__ pack_words, int write_pack,
                                                                T *__restrict__ mnmx, LoopCtl *__restrict__ ctl,
                                                                int which, unsigned *__restrict__ xst) {
  constexpr int PER = EX_LIST_MAX / EX_LIST_THREADS;
  __shared__ unsigned key[EX_LIST_MAX];
  __shared__ unsigned wsum[EX_LIST_THREADS / 32];
  __shared__ unsigned long long wmn[EX_LIST_THREADS / 32], wmx[EX_LIST_THREADS / 32];
  if (*dirty != 0u) return;  // written throughout: the full compaction stands
  {
    // the flag words the last fold set bits in go back to zero (the other
    // words are zero: k_ex_part wrote them, or left them from a compaction
    // of the untouched array)
    const unsigned nw = min(xst[1], (unsigned)EX_LIST_MAX);
    for (unsigned i = threadIdx.x; i < nw; i += EX_LIST_THREADS) pack_words[xst[2 + i]] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) xst[1] = 0u;
    __syncthreads();
  }
  const unsigned cnt = slist[0];
  if (cnt == 0u) return;     // untouched
  if (cnt > (unsigned)EX_LIST_MAX) {  // (an overflowing recorder marks the array written throughout)
    if (threadIdx.x == 0) ctl->err = 2;
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if ((long long)cnt < n) {
    // with no listed value active (the strict finish's rounding-size
    // clamps) the results need no order and no deduplication: count 0, min
    // and max over the listed values and the zeros of the unlisted entries
    bool act = false;
    T mn0 = T(0), mx0 = T(0);
    for (unsigned i = tid; i < cnt; i += EX_LIST_THREADS) {
      const T v = a[slist[4 + i]];
      act |= fabs(v) > thr;
      mn0 = fmin(mn0, v);
      mx0 = fmax(mx0, v);
    }
    if (!__syncthreads_or(act)) {
      unsigned long long kmn = ord_key<T>(mn0), kmx = ord_key<T>(mx0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long p = __shfl_xor_sync(0xffffffffu, kmn, o), q = __shfl_xor_sync(0xffffffffu, kmx, o);
        kmn = p < kmn ? p : kmn;
        kmx = q > kmx ? q : kmx;
      }
      if (lane == 0) {
        wmn[warp] = kmn;
        wmx[warp] = kmx;
      }
      __syncthreads();
      if (tid == 0) {
        for (int w = 1; w < EX_LIST_THREADS / 32; ++w) {
          kmn = wmn[w] < kmn ? wmn[w] : kmn;
          kmx = wmx[w] > kmx ? wmx[w] : kmx;
        }
        const T gmn = key_val<T>(kmn), gmx = key_val<T>(kmx);
        mnmx[0] = gmn;
        mnmx[1] = gmx;
        ctl->count[which] = 0ull;
        ctl->mn[which] = (double)gmn;
        ctl->mx[which] = (double)gmx;
      }
      return;
    }
  }
  int P = 1;
  while (P < (int)cnt) P <<= 1;
  for (int i = tid; i < P; i += EX_LIST_THREADS) key[i] = i < (int)cnt ? slist[4 + i] : 0xffffffffu;
  __syncthreads();
  // bitonic sort, ascending
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += EX_LIST_THREADS) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned x = key[i], y = key[l];
          if (((i & k) == 0) == (x > y)) {
            key[i] = y;
            key[l] = x;
          }
        }
      }
      __syncthreads();
    }
  // thread t owns sorted slots [t*PER, t*PER + PER)
  T v[PER];
  unsigned act = 0, uniq = 0;
  T mn = dev_inf<T>(), mx = -dev_inf<T>();
#pragma unroll
  for (int q = 0; q < PER; ++q) {
    const int i = tid * PER + q;
    v[q] = T(0);
    if (i < (int)cnt && (i == 0 || key[i] != key[i - 1])) {
      v[q] = a[key[i]];
      ++uniq;
      mn = fmin(mn, v[q]);
      mx = fmax(mx, v[q]);
      if (fabs(v[q]) > thr) act |= 1u << q;
    }
  }
  // block sums of the unique and active counts, min and max as keys
  unsigned na = __popc(act), xs = na;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, xs, o);
    if (lane >= o) xs += y;
  }
  unsigned long long kmn = uniq ? ord_key<T>(mn) : ~0ull, kmx = uniq ? ord_key<T>(mx) : 0ull;
  unsigned u = uniq;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    u += __shfl_xor_sync(0xffffffffu, u, o);
    const unsigned long long p = __shfl_xor_sync(0xffffffffu, kmn, o), q = __shfl_xor_sync(0xffffffffu, kmx, o);
    kmn = p < kmn ? p : kmn;
    kmx = q > kmx ? q : kmx;
  }
  __shared__ unsigned wu[EX_LIST_THREADS / 32];
  if (lane == 31) wsum[warp] = xs;
  if (lane == 0) {
    wu[warp] = u;
    wmn[warp] = kmn;
    wmx[warp] = kmx;
  }
  __syncthreads();
  unsigned off = xs - na, total = 0, utot = 0;
  for (int w = 0; w < EX_LIST_THREADS / 32; ++w) {
    off += w < warp ? wsum[w] : 0u;
    total += wsum[w];
    utot += wu[w];
    kmn = wmn[w] < kmn ? wmn[w] : kmn;
    kmx = wmx[w] > kmx ? wmx[w] : kmx;
  }
  T gmn = key_val<T>(kmn), gmx = key_val<T>(kmx);
  if ((long long)utot < n) {  // the unlisted entries are zeros
    gmn = fmin(gmn, T(0));
    gmx = fmax(gmx, T(0));
  }
  // the full compaction's keys of the same values
  gmn = key_val<T>(ord_key<T>(gmn));
  gmx = key_val<T>(ord_key<T>(gmx));
#pragma unroll
  for (int q = 0; q < PER; ++q)
    if (act & (1u << q)) {
      const unsigned idx = key[tid * PER + q];
      compact[off] = v[q];
      quant[off] = quantize16<T>(v[q], gmn, gmx);
      ++off;
      if (write_pack) {
        atomicOr(pack_words + (idx >> 5), 1u << (idx & 31u));
        xst[2 + atomicAdd(&xst[1], 1u)] = idx >> 5;
      }
    }
  if (tid == 0) {
    mnmx[0] = gmn;
    mnmx[1] = gmx;
    ctl->count[which] = total;
    ctl->mn[which] = (double)gmn;
    ctl->mx[which] = (double)gmx;
  }
}

// Records element i of an accumulator that a clamp just wrote: while the
// accumulator's dirty flag reads 0 the index joins its list; a full list
// marks the accumulator written throughout instead.
__device__ __forceinline__ void ex_list_record(unsigned *dirty, unsigned *slist, long long i) {
  if (*(volatile unsigned *)dirty != 0u) return;
  const unsigned k = atomicAdd(slist, 1u);
  if (k < (unsigned)EX_LIST_MAX) slist[4 + k] = (unsigned)i;
  else atomicExch(dirty, 1u);
}

// Flag pack of projection_algorithm.cu:382-405 as launched by
// projection_algorithm_impl.cuh:429-449 (nbytes = ceil(n/8)): byte b <
// ceil(nbytes/8) holds the flags of elements [8b, 8b+8) ∩ [0, nbytes);
// all later bytes are zero.
template <typename T>
__global__ void k_pack_reference(const T *__restrict__ a, long long n, T thr,
                                 uint8_t *__restrict__ pack, long long pack_bytes) {
  const long long nbytes = (n + 7) / 8;
  const long long written = (nbytes + 7) / 8;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < pack_bytes;
       b += (long long)gridDim.x * blockDim.x) {
    unsigned byte = 0;
    if (b < written) {
      for (int i = 0; i < 8; ++i) {
        const long long idx = 8 * b + i;
        if (idx < nbytes && fabs(a[idx]) > thr) byte |= 1u << i;
      }
    }
    pack[b] = (uint8_t)byte;
  }
}

}  // namespace ffcz
