// The float/double instantiations of the kernels projection_algorithm.cuh
// declares (their definitions: include/projection_kernels.cuh), as
// projection_algorithm.cu:675-761 instantiates them, and the host
// compaction driver compact_and_quantize_active_elements
// (projection_algorithm.cu:459-550).  The solver itself never launches these
// kernels (its passes fuse this work, see passes.cuh and extract.cuh).
#include <projection_algorithm.cuh>

#include "extract.cuh"

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
