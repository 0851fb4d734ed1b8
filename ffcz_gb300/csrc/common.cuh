// Shared definitions of the FFCz GB300 library: complex arithmetic for
// float/double, error plumbing of the C ABI, and the loop-control block the
// iteration kernels share.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <type_traits>

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

// ------------------------------------------------------- float-float --
// Split-precision scalar for FP64 data computed on the FP32 pipes: value =
// hi + lo, |lo| <= ulp(hi)/2, a 48-bit significand (relative rounding about
// 2^-47 per operation instead of 2^-53).  Error-free transformations of
// Knuth (two-sum) and Dekker (fast two-sum), products through one rounded
// product and FMAs for the error term; every step rounded on its own (no
// contraction, no reassociation).
struct ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  // from a double (a literal folds at compile time)
  __host__ __device__ constexpr ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr ff(int i) : ff((double)i) {}
};
__host__ __device__ __forceinline__ float ff_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;
  return r;
#endif
}
__host__ __device__ __forceinline__ float ff_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
__host__ __device__ __forceinline__ float ff_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
__host__ __device__ __forceinline__ float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}
// s + e = a + b exactly, |e| <= ulp(s)/2 (needs |a| >= |b| or a == 0)
__host__ __device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
  const float s = ff_add(a, b);
  return ff(s, ff_sub(b, ff_sub(s, a)));
}
__host__ __device__ __forceinline__ ff operator+(ff a, ff b) {
  const float s = ff_add(a.hi, b.hi);
  const float bb = ff_sub(s, a.hi);
  float e = ff_add(ff_sub(a.hi, ff_sub(s, bb)), ff_sub(b.hi, bb));  // two-sum error
  e = ff_add(e, ff_add(a.lo, b.lo));
  return ff_fast_two_sum(s, e);
}
__host__ __device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__host__ __device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__host__ __device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = ff_mul(a.hi, b.hi);
  float e = ff_fma(a.hi, b.hi, -p);  // exact error of the rounded product
  e = ff_fma(a.hi, b.lo, e);
  e = ff_fma(a.lo, b.hi, e);
  return ff_fast_two_sum(p, e);
}
__host__ __device__ __forceinline__ ff &operator+=(ff &a, ff b) { return a = a + b; }
__host__ __device__ __forceinline__ ff &operator-=(ff &a, ff b) { return a = a - b; }
__host__ __device__ __forceinline__ ff &operator*=(ff &a, ff b) { return a = a * b; }
__host__ __device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

struct ffc {
  ff x, y;
};
template <> struct C2<ff> { using type = ffc; };

// Conversions without the FP64 pipe (GB300's FP64 rate is a small fraction
// of its FP32 rate): the fields of a double split by integer operations.
// double -> ff: hi = the top 24 significand bits, lo = the other 29 bits
// (rounded to 24) scaled by the exponent, then renormalised; exact for 48
// significant bits.  Only doubles whose hi and scaled lo are normal floats
// (2^-74 <= |d| < 2^127) take this path; zeros and the rest are converted by
// the FP64 path.
__device__ __forceinline__ ff ff_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex < 949 || ex > 1150) return ff(d);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long mant = b & 0xfffffffffffffull;
  const float hi = __uint_as_float(sign | ((unsigned)(ex - 1023 + 127) << 23) | (unsigned)(mant >> 29));
  const float scale = __uint_as_float((unsigned)(ex - 1075 + 127) << 23);  // 2^(ex - 1075)
  // the 29 low bits as a float without a conversion instruction: the top 23
  // and the last 6 placed in float significands (2^23 + v - 2^23 is exact),
  // then one rounding (the same as converting the 29-bit integer)
  const unsigned r = (unsigned)(mant & 0x1fffffffull);
  const float r1 = __fsub_rn(__uint_as_float(0x4b000000u | (r >> 6)), 8388608.0f);
  const float r0 = __fsub_rn(__uint_as_float(0x4b000000u | (r & 63u)), 8388608.0f);
  float lo = __fmul_rn(__fmaf_rn(r1, 64.0f, r0), scale);
  if (sign) lo = -lo;
  return ff_fast_two_sum(hi, lo);
}
// Exact widening of a float by its fields (normal floats; others through
// the conversion instruction).
__device__ __forceinline__ double f2d_fields(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) |
                                          ((unsigned long long)(e - 127u + 1023u) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}
__device__ __forceinline__ double ff_to_double_fast(ff a) { return f2d_fields(a.hi) + f2d_fields(a.lo); }

// Complex conversions between a storage type and a compute type (identity
// unless one side is ff).
template <typename To, typename VF>
__host__ __device__ __forceinline__ c2<To> cvt(const VF &a) {
  using From = std::remove_cv_t<decltype(a.x)>;
  if constexpr (std::is_same<To, From>::value) {
    return a;
  } else if constexpr (std::is_same<To, ff>::value) {
    c2<To> r;
#ifdef __CUDA_ARCH__
    r.x = ff_from_double((double)a.x);
    r.y = ff_from_double((double)a.y);
#else
    r.x = ff((double)a.x);
    r.y = ff((double)a.y);
#endif
    return r;
  } else {
    c2<To> r;
#ifdef __CUDA_ARCH__
    r.x = (To)ff_to_double_fast(a.x);
    r.y = (To)ff_to_double_fast(a.y);
#else
    r.x = (To)ff_to_double(a.x);
    r.y = (To)ff_to_double(a.y);
#endif
    return r;
  }
}

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
  // max over the spectrum of max(|Re|, |Im|) after the all-abs frequency
  // clamp, as the bits of an FP32 value rounded up: of the running
  // iteration, and of the last finished one
  unsigned fmax_cur, fmax_last;
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
