// Drop-in replacement of FFCz's projection_algorithm.cuh
// (projection_algorithm.cuh:1-336): same types, kernel declarations and
// ProjectionSolver<T> interface, implemented by the GB300 library
// (libffcz.so) through the C ABI of ffcz.h.  cufft.h is included for its
// type definitions only (cufftComplex, cufftDoubleComplex, cufftHandle);
// nothing links cuFFT.
//
// Behaviour kept from the reference:
//   * CUDA failures print "CUDA error at <file>:<line> - <msg>" and exit(1)
//     (projection_algorithm.cuh:11-31);
//   * solve*/solve_all_* throw std::runtime_error("Solver not initialized")
//     before initialisation (projection_algorithm_impl.cuh:822-825) and print
//     "Total number of iterations: %d" (impl:854);
//   * host arrays are borrowed for the call, results come back as
//     std::vector copies (impl:458-595).
// Other failures (unsupported sizes, bad arguments) throw std::runtime_error.
// The solver is non-copyable (the reference's implicit copy double-frees).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

// The reference header reaches <cstring>, <algorithm> and friends through
// <cub/cub.cuh>; code written against it (projection_example.cu uses
// std::strcmp) relies on that, so they are included here explicitly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ffcz.h"

// Error checking macros (projection_algorithm.cuh:11-31)
#define CHECK_CUDA(call)                                                                       \
  do {                                                                                         \
    cudaError_t error = call;                                                                  \
    if (error != cudaSuccess) {                                                                \
      std::cerr << "CUDA error at " << __FILE__ << ":" << __LINE__ << " - "                    \
                << cudaGetErrorString(error) << std::endl;                                     \
      exit(1);                                                                                 \
    }                                                                                          \
  } while (0)

#define CHECK_CUFFT(call)                                                                      \
  do {                                                                                         \
    cufftResult error = call;                                                                  \
    if (error != CUFFT_SUCCESS) {                                                              \
      std::cerr << "CUFFT error at " << __FILE__ << ":" << __LINE__ << " - " << error          \
                << std::endl;                                                                  \
      exit(1);                                                                                 \
    }                                                                                          \
  } while (0)

template <typename T>
struct CufftTraits {};

template <>
struct CufftTraits<float> {
  using ComplexType = cufftComplex;
  static const cufftType R2C = CUFFT_R2C;
  static const cufftType C2R = CUFFT_C2R;
};

template <>
struct CufftTraits<double> {
  using ComplexType = cufftDoubleComplex;
  static const cufftType R2C = CUFFT_D2Z;
  static const cufftType C2R = CUFFT_Z2D;
};

// projection_algorithm.cuh:56-72
template <typename T>
struct ProjectionParams {
  T *d_orig_data;
  T *d_spatial_error;
  typename CufftTraits<T>::ComplexType *d_orig_freq;
  typename CufftTraits<T>::ComplexType *d_freq_error;
  size_t *d_freq_indices;
  T *d_delta_k;
  T delta;
  T delta_ptw;
  T spatial_epsilon;
  size_t Nx, Ny, Nz;
  size_t num_freq_constraints;
  cufftHandle fft_plan_forward;
  cufftHandle fft_plan_inverse;
};

// projection_algorithm.cuh:75-108
template <typename T>
struct IterationResults {
  T *d_freq_edits;
  T *d_spatial_edits;
  bool *d_freq_flag;
  bool *d_spatial_flag;
  uint8_t *d_freq_flag_pack;
  uint8_t *d_spatial_flag_pack;
  T *d_freq_edit_compact;
  T *d_spatial_edit_compact;
  uint16_t *d_freq_edit_compact_quantized;
  uint16_t *d_spatial_edit_compact_quantized;
  T h_freq_min_edit;
  T h_spatial_min_edit;
  T h_freq_max_edit;
  T h_spatial_max_edit;
  size_t h_num_active_freq;
  size_t h_num_active_spatial;
  T convergence_metric;
  int iteration_count;
  size_t max_freq_size;
  size_t max_spatial_size;
};

#ifdef __CUDACC__
// The kernels of projection_algorithm.cuh:111-235, defined in a header (see
// there) with the float/double instantiations also in libffcz.so.
#include "projection_kernels.cuh"
#endif  // __CUDACC__

// projection_algorithm.cu:459-550 (device arrays; min, max and count to
// host pointers).
template <typename T>
void compact_and_quantize_active_elements(const T *edit_array, const bool *flag_array, const int *int_flag_array,
                                          T *compact_values, uint16_t *quant_values, T *h_min_edit, T *h_max_edit,
                                          size_t total_size, size_t *h_num_active);

namespace ffcz_detail {
inline void check(int rc) {
  if (rc == FFCZ_OK) return;
  if (rc == FFCZ_ERR_CUDA) {
    std::cerr << ffcz_last_error() << std::endl;
    exit(1);
  }
  throw std::runtime_error(ffcz_last_error());
}
template <typename T>
constexpr int dtype() {
  static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double");
  return std::is_same<T, float>::value ? FFCZ_F32 : FFCZ_F64;
}
}  // namespace ffcz_detail

// projection_algorithm.cuh:238-333
template <typename T>
class ProjectionSolver {
 public:
  ProjectionSolver(size_t Nx, size_t Ny, size_t Nz) : Nx_(Nx), Ny_(Ny), Nz_(Nz) {
    ffcz_detail::check(ffcz_solver_create(Nx, Ny, Nz, ffcz_detail::dtype<T>(), &h_));
  }
  ~ProjectionSolver() { ffcz_solver_destroy(h_); }
  ProjectionSolver(const ProjectionSolver &) = delete;
  ProjectionSolver &operator=(const ProjectionSolver &) = delete;

  // initialize -- impl:598-637 (per-index bounds delta_k)
  void initialize(const T *h_orig_data, const size_t *h_freq_indices, const T *h_delta_k, T spatial_epsilon,
                  size_t num_freq_constraints) {
    ffcz_detail::check(ffcz_init_direct(h_, h_orig_data, h_freq_indices, h_delta_k, (double)spatial_epsilon,
                                        num_freq_constraints));
  }
  void initialize_all_abs(const T *h_orig_data, T spatial_epsilon, T delta) {
    ffcz_detail::check(ffcz_init_all_abs(h_, h_orig_data, (double)spatial_epsilon, (double)delta));
  }
  // initialize_all_ptw -- impl:670-697 (pointwise power-spectrum box)
  void initialize_all_ptw(const T *h_orig_data, T spatial_epsilon, T delta_ptw) {
    ffcz_detail::check(ffcz_init_all_ptw(h_, h_orig_data, (double)spatial_epsilon, (double)delta_ptw));
  }
  // initialize_partial_ptw -- impl:699-738
  void initialize_partial_ptw(const T *h_orig_data, const size_t *h_freq_indices, const T delta_ptw,
                              T spatial_epsilon, size_t num_freq_constraints) {
    ffcz_detail::check(ffcz_init_partial_ptw(h_, h_orig_data, h_freq_indices, (double)delta_ptw,
                                             (double)spatial_epsilon, num_freq_constraints));
  }
  // solve -- impl:772-814
  void solve(T *h_spatial_error, int max_iterations, T convergence_tolerance) {
    ffcz_detail::check(ffcz_solve(h_, h_spatial_error, max_iterations, (double)convergence_tolerance));
    print_iterations_();
  }
  void solve_all_abs(T *h_spatial_error, int max_iterations, T convergence_tolerance) {
    ffcz_detail::check(ffcz_solve_all_abs(h_, h_spatial_error, max_iterations, (double)convergence_tolerance));
    print_iterations_();
  }
  // solve_all_ptw -- impl:860-902
  void solve_all_ptw(T *h_spatial_error, int max_iterations, T convergence_tolerance) {
    ffcz_detail::check(ffcz_solve_all_ptw(h_, h_spatial_error, max_iterations, (double)convergence_tolerance));
    print_iterations_();
  }

  void get_results(T *h_spatial_error) { ffcz_detail::check(ffcz_get_results(h_, h_spatial_error)); }

  void extract_compact_representation() { ffcz_detail::check(ffcz_extract(h_)); }
  std::vector<bool> get_freq_flags() { return flags_(true); }
  std::vector<bool> get_spatial_flags() { return flags_(false); }
  std::vector<uint8_t> get_freq_flags_pack() {
    return bytes_(2 * freq_size_(), &ffcz_get_freq_flags_pack);
  }
  std::vector<uint8_t> get_spatial_flags_pack() { return bytes_(Nx_ * Ny_ * Nz_, &ffcz_get_spatial_flags_pack); }
  std::vector<uint16_t> get_active_freq_quant_edit_distances() { return quant_(true); }
  std::vector<uint16_t> get_active_spatial_quant_edit_distances() { return quant_(false); }
  std::vector<T> get_active_freq_edit_distances() { return compact_(true); }
  std::vector<T> get_active_spatial_edit_distances() { return compact_(false); }

  std::vector<T> get_freq_edits_full() {
    std::vector<T> v(2 * freq_size_());
    ffcz_detail::check(ffcz_get_freq_edits_full(h_, v.data(), v.size()));
    return v;
  }
  std::vector<T> get_spatial_edits_full() {
    std::vector<T> v(Nx_ * Ny_ * Nz_);
    ffcz_detail::check(ffcz_get_spatial_edits_full(h_, v.data(), v.size()));
    return v;
  }

  T get_min_freq_edit() { return (T)minmax_(0); }
  T get_max_freq_edit() { return (T)minmax_(1); }
  T get_min_spatial_edit() { return (T)minmax_(2); }
  T get_max_spatial_edit() { return (T)minmax_(3); }

  void reset_edit_accumulators() { ffcz_detail::check(ffcz_reset_edit_accumulators(h_)); }

  // Handle of the underlying C ABI object (for mixing both interfaces).
  ffcz_solver *handle() const { return h_; }

 private:
  ffcz_solver *h_ = nullptr;
  size_t Nx_, Ny_, Nz_;

  size_t freq_size_() const { return Nx_ * Ny_ * (Nz_ / 2 + 1); }
  void print_iterations_() {
    int it = 0;
    ffcz_get_iterations(h_, &it);
    printf("Total number of iterations: %d\n", it);
  }
  double minmax_(int i) {
    double v[4] = {0, 0, 0, 0};
    ffcz_detail::check(ffcz_get_minmax(h_, &v[0], &v[1], &v[2], &v[3]));
    return v[i];
  }
  std::vector<bool> flags_(bool freq) {
    const size_t n = freq ? 2 * freq_size_() : Nx_ * Ny_ * Nz_;
    std::vector<uint8_t> raw(n);
    size_t len = 0;
    ffcz_detail::check(freq ? ffcz_get_freq_flags(h_, raw.data(), n, &len)
                            : ffcz_get_spatial_flags(h_, raw.data(), n, &len));
    return std::vector<bool>(raw.begin(), raw.end());
  }
  std::vector<uint8_t> bytes_(size_t nflags, int (*fn)(ffcz_solver *, uint8_t *, size_t, size_t *)) {
    std::vector<uint8_t> v((nflags + 7) / 8);
    size_t len = 0;
    ffcz_detail::check(fn(h_, v.data(), v.size(), &len));
    return v;
  }
  std::vector<uint16_t> quant_(bool freq) {
    size_t nf = 0, ns = 0;
    ffcz_detail::check(ffcz_get_active_counts(h_, &nf, &ns));
    std::vector<uint16_t> v(freq ? nf : ns);
    size_t len = 0;
    ffcz_detail::check(freq ? ffcz_get_freq_quant(h_, v.data(), v.size(), &len)
                            : ffcz_get_spatial_quant(h_, v.data(), v.size(), &len));
    return v;
  }
  std::vector<T> compact_(bool freq) {
    size_t nf = 0, ns = 0;
    ffcz_detail::check(ffcz_get_active_counts(h_, &nf, &ns));
    std::vector<T> v(freq ? nf : ns);
    size_t len = 0;
    ffcz_detail::check(freq ? ffcz_get_freq_compact(h_, v.data(), v.size(), &len)
                            : ffcz_get_spatial_compact(h_, v.data(), v.size(), &len));
    return v;
  }
};
