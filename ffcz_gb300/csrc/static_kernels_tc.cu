// Instantiations of the tensor-core strided passes (passes_tc.cuh) for the
// FP32 axis lengths 256 and 512, in a translation unit of their own.
#include "passes_tc.cuh"
#include "static_kernels.h"

namespace ffcz {

template <int L>
static bool tc_for(int mode, StridedFn<float> &fn, StaticGeom &g) {
  switch (mode) {
    case MODE_FWD: fn = ks_strided_tc<MODE_FWD, L>; break;
    case MODE_INV: fn = ks_strided_tc<MODE_INV, L>; break;
    case MODE_FC: fn = ks_strided_tc<MODE_FC, L>; break;
    case MODE_FCI: fn = ks_strided_tc<MODE_FCI, L>; break;
    default: return false;
  }
  g.TW = kTcTW;
  g.threads = kTcThreads;
  g.smem = tc_smem_bytes(L);
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem) == cudaSuccess;
}

bool tc_strided(int L, int mode, StridedFn<float> &fn, StaticGeom &g) {
  if (L == 256) return tc_for<256>(mode, fn, g);
  if (L == 512) return tc_for<512>(mode, fn, g);
  return false;
}

}  // namespace ffcz
