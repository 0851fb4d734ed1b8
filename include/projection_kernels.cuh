// Definitions of the kernels FFCz's projection_algorithm.cuh declares
// (projection_algorithm.cuh:111-235), with the reference's per-element
// semantics (projection_algorithm.cu:85-673), in a header so that code
// launching them instantiates them in its own translation units (the
// reference compiles them into its own library with separable compilation;
// a kernel template's launch stub is local to the translation unit that
// instantiates it).  Included by projection_algorithm.cuh in nvcc
// translation units.  The library's own passes fuse this work and never
// launch these kernels.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstddef>
#include <cstdint>

namespace ffcz_kernels_detail {

// uint16 quantiser of projection_algorithm.cu:447-455: n = (v - mn)/(mx -
// mn) in T, q = n > 0.5 ? ceil(n*65535) : floor(n*65535), each operation
// rounded to nearest (no contraction); 0/0 (every entry equal) gives 0.
__device__ __forceinline__ float q_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double q_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float q_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double q_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float q_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double q_mul(double a, double b) { return __dmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ uint16_t quantize16(T v, T mn, T mx) {
  const T nrm = q_div(q_sub(v, mn), q_sub(mx, mn));
  const T s = q_mul(nrm, T(65535));
  const T q = (nrm > T(0.5)) ? ceil(s) : floor(s);
  if (!(q == q)) return 0;
  return (uint16_t)(unsigned)q;
}

template <typename T>
__device__ __forceinline__ void clamp_into(T &v, T bound, T *edit) {
  if (v > bound) {
    atomicAdd(edit, bound - v);
    v = bound;
  } else if (v < -bound) {
    atomicAdd(edit, -bound - v);
    v = -bound;
  }
}

// Pointwise-relative box of the power spectrum: DC is reset to the original
// when its error leaves [x0(1/sqrt(1+d)-1), x0(1/sqrt(1-d)-1)]; other
// coefficients whose |F+E|^2/|F|^2 leaves [sqrt(1-d), sqrt(1+d)] are clamped
// componentwise to min(1-sqrt(1-d), sqrt(1+d)-1)/sqrt(2).
template <typename T>
__device__ __forceinline__ void ptw_one(typename CufftTraits<T>::ComplexType *err,
                                        const typename CufftTraits<T>::ComplexType *orig, size_t k, T dp,
                                        T *freq_edits, size_t H) {
  if (k == 0) {
    const T lo = orig[0].x * (1 / sqrt(1 + dp) - 1);
    const T hi = orig[0].x * (1 / sqrt(1 - dp) - 1);
    const T e = err[0].x;
    if (e > hi || e < lo) {
      atomicAdd(&freq_edits[0], -e);
      err[0].x = 0;
    }
    return;
  }
  const T om = orig[k].x * orig[k].x + orig[k].y * orig[k].y;
  const T cx = orig[k].x + err[k].x, cy = orig[k].y + err[k].y;
  const T ratio = (cx * cx + cy * cy) / om;
  if (ratio <= sqrt(1 + dp) && ratio >= sqrt(1 - dp)) return;
  // The reference divides by sqrt_val(2.0f), a float square root for both T.
  const T d = fmin(1 - sqrt(1 - dp), sqrt(1 + dp) - 1) / (T)sqrtf(2.0f);
  clamp_into(err[k].x, d, &freq_edits[k]);
  clamp_into(err[k].y, d, &freq_edits[k + H]);
}

}  // namespace ffcz_kernels_detail

template <typename T>
__global__ void normalize_kernel(T *data, T factor, size_t size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < size) data[i] *= factor;
}

template <typename T>
__global__ void project_frequency_constraints_direct(typename CufftTraits<T>::ComplexType *curr_freq_err,
                                                     const size_t *freq_constraint_indices, const T *delta_k,
                                                     T *freq_edits, size_t, size_t, size_t, size_t max_freq_size,
                                                     size_t num_constraints) {
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= 2 * num_constraints) return;
  const size_t c = id % num_constraints;
  const bool imag = id >= num_constraints;
  const size_t k = freq_constraint_indices[c];
  const T d = delta_k[c];
  if (imag) ffcz_kernels_detail::clamp_into(curr_freq_err[k].y, d, &freq_edits[k + max_freq_size]);
  else ffcz_kernels_detail::clamp_into(curr_freq_err[k].x, d, &freq_edits[k]);
}

template <typename T>
__global__ void project_frequency_constraints_all_abs(typename CufftTraits<T>::ComplexType *curr_freq_err,
                                                      const T delta, T *freq_edits, size_t, size_t, size_t,
                                                      size_t max_freq_size) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= max_freq_size) return;
  ffcz_kernels_detail::clamp_into(curr_freq_err[k].x, delta, &freq_edits[k]);
  ffcz_kernels_detail::clamp_into(curr_freq_err[k].y, delta, &freq_edits[k + max_freq_size]);
}

template <typename T>
__global__ void project_frequency_constraints_all_ptw(typename CufftTraits<T>::ComplexType *curr_freq_err,
                                                      const typename CufftTraits<T>::ComplexType *orig_freq,
                                                      const T delta_ptw, T *freq_edits, size_t, size_t, size_t,
                                                      size_t max_freq_size) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= max_freq_size) return;
  ffcz_kernels_detail::ptw_one<T>(curr_freq_err, orig_freq, k, delta_ptw, freq_edits, max_freq_size);
}

template <typename T>
__global__ void project_frequency_constraints_partial_ptw(
    typename CufftTraits<T>::ComplexType *curr_freq_err, const typename CufftTraits<T>::ComplexType *orig_freq,
    const size_t *freq_constraint_indices, const T delta_ptw, T *freq_edits, size_t, size_t, size_t,
    size_t max_freq_size, size_t num_constraints) {
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= num_constraints) return;
  // Constraint 0 always addresses the DC coefficient (projection_algorithm.cu:277-289).
  const size_t k = id == 0 ? 0 : freq_constraint_indices[id];
  ffcz_kernels_detail::ptw_one<T>(curr_freq_err, orig_freq, k, delta_ptw, freq_edits, max_freq_size);
}

template <typename T>
__global__ void project_spatial_constraints_direct(T *spatial_error, T spatial_epsilon, T *spatial_edits,
                                                   size_t total_size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  const T v = spatial_error[i];
  if (v > spatial_epsilon) {
    spatial_edits[i] += spatial_epsilon - v;
    spatial_error[i] = spatial_epsilon;
  } else if (v < -spatial_epsilon) {
    spatial_edits[i] += -spatial_epsilon - v;
    spatial_error[i] = -spatial_epsilon;
  }
}

template <typename T>
__global__ void extract_active_flags(const T *edit_array, bool *flag_array, int *int_flag_array, size_t total_size,
                                     T threshold = T(0)) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  const bool f = fabs(edit_array[i]) > threshold;
  flag_array[i] = f;
  int_flag_array[i] = f ? 1 : 0;
}

// Same observable effect as projection_algorithm.cu:382-405: thread b with
// 8b < num_bytes writes byte b from the flags [8b, 8b+8) that lie below
// num_bytes, LSB first; other bytes are left untouched.
// (static: a non-template kernel defined in a header gets one copy per
// translation unit)
static __global__ void pack_bools(const bool *__restrict__ flag, uint8_t *__restrict__ flag_pack,
                                  size_t num_bytes) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (8 * b >= num_bytes) return;
  unsigned v = 0;
  for (int i = 0; i < 8; ++i) {
    const size_t idx = 8 * b + i;
    if (idx < num_bytes && flag[idx]) v |= 1u << i;
  }
  flag_pack[b] = (uint8_t)v;
}

template <typename T>
__global__ void compact_with_prefix_positions(const T *edit_array, const bool *flag_array,
                                              const int *prefix_positions, T *compact_values, size_t total_size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < total_size && flag_array[i]) compact_values[prefix_positions[i]] = edit_array[i];
}

template <typename T>
__global__ void compact_and_quantize_with_prefix_positions(const T *edit_array, const bool *flag_array,
                                                           const int *prefix_positions, T *compact_values,
                                                           T *min_edit, T *max_edit, uint16_t *quant_values,
                                                           size_t total_size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size || !flag_array[i]) return;
  const int p = prefix_positions[i];
  compact_values[p] = edit_array[i];
  quant_values[p] = ffcz_kernels_detail::quantize16<T>(edit_array[i], *min_edit, *max_edit);
}

template <typename T>
__global__ void reset_accumulators(T *freq_edits, T *spatial_edits, size_t freq_size, size_t spatial_size) {
  const size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t st = (size_t)blockDim.x * gridDim.x;
  for (size_t i = i0; i < 2 * freq_size; i += st) freq_edits[i] = T(0);
  for (size_t i = i0; i < spatial_size; i += st) spatial_edits[i] = T(0);
}

template <typename T>
__global__ void compute_convergence_metric(const T *spatial_error, T spatial_epsilon, T *convergence_result,
                                           size_t total_size) {
  __shared__ T red[1024];
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  T v = 0;
  if (i < total_size) {
    const T a = fabs(spatial_error[i]);
    if (a > spatial_epsilon) v = a - spatial_epsilon;
  }
  red[threadIdx.x] = v;
  __syncthreads();
  for (unsigned s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) convergence_result[blockIdx.x] = red[0];
}

template <typename T>
__global__ void quantize_and_dequantize(const T *org_arr, T *dequant_arr, T min_val, T max_val, size_t total_size,
                                        T threshold = T(1e-7)) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  const T v = org_arr[i];
  if (fabs(v) > threshold) {
    const T q = (T)ffcz_kernels_detail::quantize16<T>(v, min_val, max_val);
    dequant_arr[i] = q / ((1u << 16) - 1) * (max_val - min_val) + min_val;
  } else {
    dequant_arr[i] = 0;
  }
}

template <typename T>
__global__ void frequency_float_to_complex(const T *freq_split, typename CufftTraits<T>::ComplexType *freq_complex,
                                           size_t total_size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  freq_complex[i].x = freq_split[i];
  freq_complex[i].y = freq_split[i + total_size];
}

template <typename T>
__global__ void add_two_arrays(const T *arr1, T *arr2, size_t total_size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < total_size) arr2[i] += arr1[i];
}

