// Instantiations of the compile-time-sized pass kernels for power-of-two
// lengths 16..1024 (FP32) and 16..512 (FP64), and their lookup.
#include "passes_static.cuh"
#include "static_kernels.h"

namespace ffcz {

namespace {

template <typename T, int L>
struct Cfg {
  static constexpr int LGTW = sizeof(T) == 4 ? (L <= 512 ? 4 : 3) : (L <= 256 ? 3 : 3);
  static constexpr int TW = 1 << LGTW;
  static constexpr int NT0 = L * TW / 8;
  static constexpr int NT = NT0 < 64 ? 64 : (NT0 > 1024 ? 1024 : NT0);
};

template <typename F>
int set_smem(F fn, size_t smem) {
  if (smem > 48 * 1024)
    FFCZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  return FFCZ_OK;
}

template <typename T, int M>
bool zfwd_for(int pro, ZfwdFn<T> &fn, StaticGeom &g) {
  using C = Cfg<T, M>;
  if (pro == PRO_PLAIN) fn = ks_zfwd<T, PRO_PLAIN, M, C::LGTW, C::NT>;
  else if (pro == PRO_DIFF) fn = ks_zfwd<T, PRO_DIFF, M, C::LGTW, C::NT>;
  else fn = ks_zfwd<T, PRO_CLAMP, M, C::LGTW, C::NT>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)(M + 1) * (C::TW + 1) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}

template <typename T, int M>
bool zinv_for(ZinvFn<T> &fn, StaticGeom &g) {
  using C = Cfg<T, M>;
  fn = ks_zinv<T, M, C::LGTW, C::NT>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)(M + 1) * (C::TW + 1) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}

template <typename T, int L>
bool strided_for(int mode, StridedFn<T> &fn, StaticGeom &g) {
  using C = Cfg<T, L>;
  if (mode == MODE_FWD) fn = ks_strided<T, MODE_FWD, L, C::LGTW, C::NT>;
  else if (mode == MODE_INV) fn = ks_strided<T, MODE_INV, L, C::LGTW, C::NT>;
  else fn = ks_strided<T, MODE_FCI, L, C::LGTW, C::NT>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)L * (C::TW + 1) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}

}  // namespace

#define CASES_F32(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)
#define CASES_F64(X) X(16) X(32) X(64) X(128) X(256) X(512)

template <>
bool static_zfwd<float>(int M, int pro, ZfwdFn<float> &fn, StaticGeom &g) {
  switch (M) {
#define X(n) case n: return zfwd_for<float, n>(pro, fn, g);
    CASES_F32(X)
#undef X
    default: return false;
  }
}
template <>
bool static_zfwd<double>(int M, int pro, ZfwdFn<double> &fn, StaticGeom &g) {
  switch (M) {
#define X(n) case n: return zfwd_for<double, n>(pro, fn, g);
    CASES_F64(X)
#undef X
    default: return false;
  }
}
template <>
bool static_zinv<float>(int M, ZinvFn<float> &fn, StaticGeom &g) {
  switch (M) {
#define X(n) case n: return zinv_for<float, n>(fn, g);
    CASES_F32(X)
#undef X
    default: return false;
  }
}
template <>
bool static_zinv<double>(int M, ZinvFn<double> &fn, StaticGeom &g) {
  switch (M) {
#define X(n) case n: return zinv_for<double, n>(fn, g);
    CASES_F64(X)
#undef X
    default: return false;
  }
}
template <>
bool static_strided<float>(int L, int mode, StridedFn<float> &fn, StaticGeom &g) {
  switch (L) {
#define X(n) case n: return strided_for<float, n>(mode, fn, g);
    CASES_F32(X)
#undef X
    default: return false;
  }
}
template <>
bool static_strided<double>(int L, int mode, StridedFn<double> &fn, StaticGeom &g) {
  switch (L) {
#define X(n) case n: return strided_for<double, n>(mode, fn, g);
    CASES_F64(X)
#undef X
    default: return false;
  }
}

}  // namespace ffcz
