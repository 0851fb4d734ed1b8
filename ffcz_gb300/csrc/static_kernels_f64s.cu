// Float-float instantiations of the FP64 pass kernels (FP64 storage,
// registers and shared memory in float-float on the FP32 pipes) for the
// power-of-two lengths 128..512, and their lookup.
#include "static_inst.cuh"

namespace ffcz {

template <>
bool split_zfwd<double>(int M, int pro, ZfwdFn<double> &fn, StaticGeom &g, int var) {
  switch (M) {
    CASES_SPLIT(ZFS)
    default: return false;
  }
}
template <>
bool split_zinv<double>(int M, ZinvFn<double> &fn, StaticGeom &g, int var) {
  switch (M) {
    CASES_SPLIT(ZIS)
    default: return false;
  }
}
template <>
bool split_strided<double>(int L, int mode, StridedFn<double> &fn, StaticGeom &g, int var) {
  switch (L) {
    CASES_SPLIT(STS)
    default: return false;
  }
}

}  // namespace ffcz
