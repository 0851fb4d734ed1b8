// Definitions of the kernels projection_algorithm.cuh declares
// (projection_algorithm.cuh:111-235) with the float/double instantiations
// of projection_algorithm.cu:675-761, so that code written against the
// reference header links and launches them unchanged.  They are plain
// elementwise kernels with the reference's per-element semantics; the
// solver itself never launches them (its passes fuse this work, see
// passes.cuh and extract.cuh).
#include <projection_algorithm.cuh>

#include "extract.cuh"

template <typename T>
__global__ void normalize_kernel(T *data, T factor, size_t size) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < size) data[i] *= factor;
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
  if (imag) clamp_into(curr_freq_err[k].y, d, &freq_edits[k + max_freq_size]);
  else clamp_into(curr_freq_err[k].x, d, &freq_edits[k]);
}

template <typename T>
__global__ void project_frequency_constraints_all_abs(typename CufftTraits<T>::ComplexType *curr_freq_err,
                                                      const T delta, T *freq_edits, size_t, size_t, size_t,
                                                      size_t max_freq_size) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= max_freq_size) return;
  clamp_into(curr_freq_err[k].x, delta, &freq_edits[k]);
  clamp_into(curr_freq_err[k].y, delta, &freq_edits[k + max_freq_size]);
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

template <typename T>
__global__ void project_frequency_constraints_all_ptw(typename CufftTraits<T>::ComplexType *curr_freq_err,
                                                      const typename CufftTraits<T>::ComplexType *orig_freq,
                                                      const T delta_ptw, T *freq_edits, size_t, size_t, size_t,
                                                      size_t max_freq_size) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= max_freq_size) return;
  ptw_one<T>(curr_freq_err, orig_freq, k, delta_ptw, freq_edits, max_freq_size);
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
  ptw_one<T>(curr_freq_err, orig_freq, k, delta_ptw, freq_edits, max_freq_size);
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
                                     T threshold) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  const bool f = fabs(edit_array[i]) > threshold;
  flag_array[i] = f;
  int_flag_array[i] = f ? 1 : 0;
}

// Same observable effect as projection_algorithm.cu:382-405: thread b with
// 8b < num_bytes writes byte b from the flags [8b, 8b+8) that lie below
// num_bytes, LSB first; other bytes are left untouched.
__global__ void pack_bools(const bool *__restrict__ flag, uint8_t *__restrict__ flag_pack, size_t num_bytes) {
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
  quant_values[p] = ffcz::quantize16<T>(edit_array[i], *min_edit, *max_edit);
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
                                        T threshold) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= total_size) return;
  const T v = org_arr[i];
  if (fabs(v) > threshold) {
    const T q = (T)ffcz::quantize16<T>(v, min_val, max_val);
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

// ---------------------------------------------------------------------------
// projection_algorithm.cu:459-550: whole-array min/max, exclusive scan of
// the int flags, scatter + quantisation of the bool-flagged entries.
template <typename T>
__global__ void k_legacy_stats(const T *a, const int *iflag, long long n, unsigned *blk_cnt, T *blk_mn, T *blk_mx) {
  const long long base = (long long)blockIdx.x * ffcz::EX_CHUNK;
  unsigned cnt = 0;
  T mn = ffcz::dev_inf<T>(), mx = -ffcz::dev_inf<T>();
  for (int r = 0; r < ffcz::EX_ROUNDS; ++r) {
    const long long i = base + r * ffcz::EX_THREADS + threadIdx.x;
    if (i < n) {
      const T v = a[i];
      cnt += iflag[i] ? 1u : 0u;
      mn = v < mn ? v : mn;
      mx = v > mx ? v : mx;
    }
  }
  __shared__ unsigned sc[ffcz::EX_THREADS];
  __shared__ T smn[ffcz::EX_THREADS], smx[ffcz::EX_THREADS];
  sc[threadIdx.x] = cnt;
  smn[threadIdx.x] = mn;
  smx[threadIdx.x] = mx;
  __syncthreads();
  for (int s = ffcz::EX_THREADS / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sc[threadIdx.x] += sc[threadIdx.x + s];
      smn[threadIdx.x] = smn[threadIdx.x + s] < smn[threadIdx.x] ? smn[threadIdx.x + s] : smn[threadIdx.x];
      smx[threadIdx.x] = smx[threadIdx.x + s] > smx[threadIdx.x] ? smx[threadIdx.x + s] : smx[threadIdx.x];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    blk_cnt[blockIdx.x] = sc[0];
    blk_mn[blockIdx.x] = smn[0];
    blk_mx[blockIdx.x] = smx[0];
  }
}

template <typename T>
__global__ void k_legacy_scatter(const T *a, const bool *flag, const int *iflag, long long n, const unsigned *blk_off,
                                 const T *mnmx, T *compact, uint16_t *quant) {
  __shared__ unsigned wc[ffcz::EX_THREADS / 32];
  const long long base = (long long)blockIdx.x * ffcz::EX_CHUNK;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned running = blk_off[blockIdx.x];
  for (int r = 0; r < ffcz::EX_ROUNDS; ++r) {
    const long long i = base + r * ffcz::EX_THREADS + threadIdx.x;
    const bool counted = i < n && iflag[i];
    const unsigned bal = __ballot_sync(0xffffffffu, counted);
    if (lane == 0) wc[warp] = __popc(bal);
    __syncthreads();
    unsigned woff = 0, tot = 0;
    for (int w = 0; w < ffcz::EX_THREADS / 32; ++w) {
      woff += w < warp ? wc[w] : 0u;
      tot += wc[w];
    }
    if (i < n && flag[i]) {
      const unsigned pos = running + woff + __popc(bal & ((1u << lane) - 1u));
      compact[pos] = a[i];
      quant[pos] = ffcz::quantize16<T>(a[i], mnmx[0], mnmx[1]);
    }
    running += tot;
    __syncthreads();
  }
}

template <typename T>
void compact_and_quantize_active_elements(const T *edit_array, const bool *flag_array, const int *int_flag_array,
                                          T *compact_values, uint16_t *quant_values, T *h_min_edit, T *h_max_edit,
                                          size_t total_size, size_t *h_num_active) {
  const size_t nblk = (total_size + ffcz::EX_CHUNK - 1) / ffcz::EX_CHUNK;
  unsigned *blk = nullptr;
  T *bmn = nullptr, *bmx = nullptr, *mnmx = nullptr;
  ffcz::LoopCtl *ctl = nullptr;
  CHECK_CUDA(cudaMalloc(&blk, nblk * sizeof(unsigned)));
  CHECK_CUDA(cudaMalloc(&bmn, nblk * sizeof(T)));
  CHECK_CUDA(cudaMalloc(&bmx, nblk * sizeof(T)));
  CHECK_CUDA(cudaMalloc(&mnmx, 2 * sizeof(T)));
  CHECK_CUDA(cudaMalloc(&ctl, sizeof(ffcz::LoopCtl)));
  k_legacy_stats<T><<<(unsigned)nblk, ffcz::EX_THREADS>>>(edit_array, int_flag_array, (long long)total_size, blk, bmn,
                                                          bmx);
  ffcz::k_ex_scan<T><<<1, 1024>>>(blk, (long long)nblk, bmn, bmx, mnmx, ctl, 0);
  k_legacy_scatter<T><<<(unsigned)nblk, ffcz::EX_THREADS>>>(edit_array, flag_array, int_flag_array,
                                                            (long long)total_size, blk, mnmx, compact_values,
                                                            quant_values);
  CHECK_CUDA(cudaGetLastError());
  ffcz::LoopCtl h;
  CHECK_CUDA(cudaMemcpy(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost));
  T mm[2];
  CHECK_CUDA(cudaMemcpy(mm, mnmx, sizeof(mm), cudaMemcpyDeviceToHost));
  *h_min_edit = mm[0];
  *h_max_edit = mm[1];
  *h_num_active = (size_t)h.count[0];
  cudaFree(blk);
  cudaFree(bmn);
  cudaFree(bmx);
  cudaFree(mnmx);
  cudaFree(ctl);
}

#define INST(T, C)                                                                                                 \
  template __global__ void normalize_kernel<T>(T *, T, size_t);                                                    \
  template __global__ void project_frequency_constraints_direct<T>(C *, const size_t *, const T *, T *, size_t,    \
                                                                   size_t, size_t, size_t, size_t);                \
  template __global__ void project_frequency_constraints_all_abs<T>(C *, const T, T *, size_t, size_t, size_t,     \
                                                                    size_t);                                       \
  template __global__ void project_frequency_constraints_all_ptw<T>(C *, const C *, const T, T *, size_t, size_t,  \
                                                                    size_t, size_t);                               \
  template __global__ void project_frequency_constraints_partial_ptw<T>(C *, const C *, const size_t *, const T,   \
                                                                        T *, size_t, size_t, size_t, size_t,       \
                                                                        size_t);                                   \
  template __global__ void project_spatial_constraints_direct<T>(T *, T, T *, size_t);                             \
  template __global__ void extract_active_flags<T>(const T *, bool *, int *, size_t, T);                           \
  template __global__ void compact_with_prefix_positions<T>(const T *, const bool *, const int *, T *, size_t);    \
  template __global__ void compact_and_quantize_with_prefix_positions<T>(const T *, const bool *, const int *,    \
                                                                         T *, T *, T *, uint16_t *, size_t);       \
  template void compact_and_quantize_active_elements<T>(const T *, const bool *, const int *, T *, uint16_t *,     \
                                                        T *, T *, size_t, size_t *);                               \
  template __global__ void reset_accumulators<T>(T *, T *, size_t, size_t);                                       \
  template __global__ void compute_convergence_metric<T>(const T *, T, T *, size_t);                               \
  template __global__ void quantize_and_dequantize<T>(const T *, T *, T, T, size_t, T);                            \
  template __global__ void frequency_float_to_complex<T>(const T *, C *, size_t);                                  \
  template __global__ void add_two_arrays<T>(const T *, T *, size_t);

INST(float, cufftComplex)
INST(double, cufftDoubleComplex)
