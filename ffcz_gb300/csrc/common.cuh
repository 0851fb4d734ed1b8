// Shared definitions of the FFCz GB300 library: complex arithmetic for
// float/double, error plumbing of the C ABI, and the loop-control block the
// iteration kernels share.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/ffcz.h"

namespace ffcz {

// ---------------------------------------------------------------- errors --
// Thread-local message behind ffcz_last_error().
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define FFCZ_CUDA(call)                                                     \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) return ::ffcz::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define FFCZ_TRY(call)                                                      \
  do {                                                                      \
    int rc_ = (call);                                                       \
    if (rc_ != FFCZ_OK) return rc_;                                         \
  } while (0)

// --------------------------------------------------------------- complex --
template <typename T> struct C2;
template <> struct C2<float> { using type = float2; };
template <> struct C2<double> { using type = double2; };
template <typename T> using c2 = typename C2<T>::type;

template <typename T>
__host__ __device__ __forceinline__ c2<T> mkc(T x, T y) {
  c2<T> r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename V>
__host__ __device__ __forceinline__ V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <typename V>
__host__ __device__ __forceinline__ V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename V>
__host__ __device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a * conj(b)
template <typename V>
__host__ __device__ __forceinline__ V cmulc(V a, V b) {
  V r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = a.y * b.x - a.x * b.y;
  return r;
}
template <typename V>
__host__ __device__ __forceinline__ V cconj(V a) { a.y = -a.y; return a; }
// multiply by -i (DIR = -1, forward) or +i (DIR = +1, inverse)
template <int DIR, typename V>
__host__ __device__ __forceinline__ V cmul_i(V a) {
  V r;
  if (DIR < 0) { r.x = a.y; r.y = -a.x; }
  else         { r.x = -a.y; r.y = a.x; }
  return r;
}
template <typename V, typename S>
__host__ __device__ __forceinline__ V cscale(V a, S s) { a.x *= s; a.y *= s; return a; }

// ---------------------------------------------------------- loop control --
// Device-resident state of one solve.  viol_bits holds the bit pattern of
// the non-negative spatial violation (as a 64-bit integer so that float and
// double patterns both order like their values under atomicMax).
struct LoopCtl {
  unsigned long long viol_bits;  // max(|e|-eps, 0) of the running iteration
  double last_viol;              // metric of the last finished iteration
  int iterations;                // finished iterations (impl:843)
  int converged;                 // last metric < tol (impl:845)
  int cont;                      // loop continues
  int pad;
  // compaction results
  unsigned long long count[2];   // active freq / spatial edits
  double mn[2], mx[2];           // whole-array min / max (as double)
  unsigned long long total_bits; // Huffman bitstream length
  int err;                       // device-side error word (0 = none)
  int pad2;
};

template <typename T> __device__ __forceinline__ unsigned long long to_bits(T v);
template <> __device__ __forceinline__ unsigned long long to_bits<float>(float v) {
  return (unsigned long long)__float_as_uint(v);
}
template <> __device__ __forceinline__ unsigned long long to_bits<double>(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
template <typename T> __device__ __forceinline__ T from_bits(unsigned long long b);
template <> __device__ __forceinline__ float from_bits<float>(unsigned long long b) {
  return __uint_as_float((unsigned)b);
}
template <> __device__ __forceinline__ double from_bits<double>(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }
inline size_t round_up(size_t a, size_t b) { return ceil_div(a, b) * b; }

}  // namespace ffcz
