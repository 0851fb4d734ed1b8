// Edit compaction (projection_algorithm_impl.cuh:371-456 and
// projection_algorithm.cu:365-379, 382-405, 427-457, 459-550), in three
// launches per accumulator instead of the reference's flag kernels, two CUB
// reductions, a CUB scan, the scatter kernel and two bool-pack kernels:
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
