// A uniform scalar quantiser as the base compressor in front of the
// corrector (no counterpart in the reference, which reads x' from a file):
//   q_i = rint(x_i / (2E)) (round half to even),  x'_i = T(2E * q_i)
// in FP64, so that |x'_i - x_i| <= E up to the final rounding to T.
#include <algorithm>

#include "common.cuh"

namespace ffcz {
namespace {

template <typename T>
__global__ void k_base_quantize(const T *__restrict__ x, T *__restrict__ xp, long long n, double step,
                                int *__restrict__ q) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double k = rint(__ddiv_rn((double)x[i], step));
    xp[i] = (T)__dmul_rn(step, k);
    if (q) q[i] = (int)k;
  }
}

}  // namespace
}  // namespace ffcz

using namespace ffcz;

extern "C" {

int ffcz_base_quantize_device(const void *d_x, size_t n, int dtype, double eps, void *d_xprime, int32_t *d_index,
                              void *stream) {
  if ((!d_x || !d_xprime) && n) return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (dtype != FFCZ_F32 && dtype != FFCZ_F64) return fail(FFCZ_ERR_INVALID, "dtype must be FFCZ_F32 or FFCZ_F64");
  if (!(eps > 0.0)) return fail(FFCZ_ERR_INVALID, "eps must be positive");
  if (n == 0) return FFCZ_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned g = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (dtype == FFCZ_F32)
    k_base_quantize<float><<<g, 256, 0, st>>>((const float *)d_x, (float *)d_xprime, (long long)n, 2.0 * eps, d_index);
  else
    k_base_quantize<double><<<g, 256, 0, st>>>((const double *)d_x, (double *)d_xprime, (long long)n, 2.0 * eps,
                                               d_index);
  FFCZ_CUDA(cudaGetLastError());
  FFCZ_CUDA(cudaStreamSynchronize(st));
  return FFCZ_OK;
}

}  // extern "C"
