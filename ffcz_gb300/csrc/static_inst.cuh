// Instantiation helpers of the register-resident pass kernels: tile
// geometry per length (Cfg), the typed lookups and the length lists.  Each
// element type is instantiated in its own translation unit.
#pragma once

#include "passes_static.cuh"
#include "static_kernels.h"

namespace ffcz {

#ifndef FFCZ_TILE_THREADS
#define FFCZ_TILE_THREADS 512
#endif
#ifndef FFCZ_Z_TILE_THREADS
#define FFCZ_Z_TILE_THREADS 256
#endif
#ifndef FFCZ_Z_MIXED_TILE
#define FFCZ_Z_MIXED_TILE 0
#endif

// VAR 0: the default tile; VAR 1: the autotuner's alternative (half or
// double the thread budget), compiled beside it.
template <typename T, int L, int CAP = 16, int VAR = 0>
struct Cfg {
  static constexpr int E = rp_elems(L, CAP);
  static constexpr int TC = L / E;
  static constexpr int TWMAX = sizeof(T) == 4 ? 16 : 8;
  // 16 values per thread take ~80-100 registers: at most 512 threads; 20-30
  // values (~130-170 registers): 256; 8-12 values may use FFCZ_TILE_THREADS.
  // The power-of-two z passes run 256-thread blocks (8 rows of 256 complex
  // values at 512^3: z inverse 283 -> 230 us, z forward 278 -> 264 us).
  static constexpr int BUDGET0 = E > 16 ? 256 : E == 16 ? 512
                               : (CAP == 8 && (FFCZ_Z_MIXED_TILE || !mx_list(L))) ? FFCZ_Z_TILE_THREADS
                                                                                   : FFCZ_TILE_THREADS;
  static constexpr int BUDGET = VAR == 0 ? BUDGET0 : (BUDGET0 >= 512 ? BUDGET0 / 2 : BUDGET0 * 2);
  static constexpr int TW0 = BUDGET / TC;
  static constexpr int TW1 = TW0 < 1 ? 1 : (TW0 > TWMAX ? TWMAX : TW0);
  static constexpr int LGTW = ilog2(TW1);  // tile widths are powers of two
  static constexpr int TW = 1 << LGTW;
  static constexpr int NT = TC * TW;
};

template <typename F>
int set_smem(F fn, size_t smem) {
  if (smem > 48 * 1024)
    FFCZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  return FFCZ_OK;
}

template <typename T, int M, int VAR, bool SPLIT = false>
bool zfwd_for(int pro, ZfwdFn<T> &fn, StaticGeom &g) {
  using C = Cfg<T, M, 8, VAR>;
  if (VAR && C::TW == Cfg<T, M, 8, 0>::TW) return false;  // same tile as the default
  if (pro == PRO_PLAIN) fn = ks_zfwd<T, PRO_PLAIN, M, C::LGTW, SPLIT>;
  else if (pro == PRO_DIFF) fn = ks_zfwd<T, PRO_DIFF, M, C::LGTW, SPLIT>;
  else fn = ks_zfwd<T, PRO_CLAMP, M, C::LGTW, SPLIT>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)C::TW * row_pitch(M, sizeof(T)) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}

template <typename T, int M, int VAR, bool SPLIT = false>
bool zinv_for(ZinvFn<T> &fn, StaticGeom &g) {
  using C = Cfg<T, M, 8, VAR>;
  if (VAR && C::TW == Cfg<T, M, 8, 0>::TW) return false;
  fn = ks_zinv<T, M, C::LGTW, SPLIT>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)C::TW * row_pitch(M, sizeof(T)) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}

// The plain passes (forward, inverse) take the plain_cap(L) stage list, the
// fused ones (forward + clamp + inverse) the CAP 16 list.
// (Float-float kernels take the CAP 16 lists for every pass: 8 values per
// thread fit them in 118 registers, the 16 of [16,16,2] spill.)
template <typename T, int L, int VAR, bool FUSED, bool SPLIT = false>
bool strided_for_family(int mode, StridedFn<T> &fn, StaticGeom &g) {
  constexpr int CAP = (FUSED || SPLIT) ? 16 : plain_cap(L);
  using C = Cfg<T, L, CAP, VAR>;
  if (VAR && C::TW == Cfg<T, L, CAP, 0>::TW) return false;
  if constexpr (FUSED) {
    if (mode == MODE_FCI) fn = ks_strided<T, MODE_FCI, L, C::LGTW, CAP, SPLIT>;
    else fn = ks_strided<T, MODE_FCIX, L, C::LGTW, CAP, SPLIT>;
  } else {
    if (mode == MODE_FWD) fn = ks_strided<T, MODE_FWD, L, C::LGTW, CAP, SPLIT>;
    else fn = ks_strided<T, MODE_INV, L, C::LGTW, CAP, SPLIT>;
  }
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)sl_size(L, C::TW, sizeof(T), CAP) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}
template <typename T, int L, int VAR>
bool strided_fc_for(StridedFn<T> &fn, StaticGeom &g) {
  constexpr int CAP = plain_cap(L);
  using C = Cfg<T, L, CAP, VAR>;
  if (VAR && C::TW == Cfg<T, L, CAP, 0>::TW) return false;
  fn = ks_strided<T, MODE_FC, L, C::LGTW, CAP, false>;
  g.TW = C::TW;
  g.threads = C::NT;
  g.smem = (size_t)sl_size(L, C::TW, sizeof(T), CAP) * sizeof(c2<T>);
  return set_smem(fn, g.smem) == FFCZ_OK;
}
template <typename T, int L, int VAR, bool SPLIT = false>
bool strided_for(int mode, StridedFn<T> &fn, StaticGeom &g) {
  return (mode == MODE_FWD || mode == MODE_INV) ? strided_for_family<T, L, VAR, false, SPLIT>(mode, fn, g)
                                                : strided_for_family<T, L, VAR, true, SPLIT>(mode, fn, g);
}

// The float-float kernels (FP64 storage) are instantiated in their own
// translation unit for the power-of-two lengths 128..512 (their fully
// unrolled float-float butterflies grow the code about tenfold; compiling
// longer or mixed-radix lists takes minutes each).
template <typename T> bool split_zfwd(int M, int pro, ZfwdFn<T> &fn, StaticGeom &g, int var);
template <typename T> bool split_zinv(int M, ZinvFn<T> &fn, StaticGeom &g, int var);
template <typename T> bool split_strided(int L, int mode, StridedFn<T> &fn, StaticGeom &g, int var);

#define CASES_F32(X)                                                                                      \
  X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(96) X(100) X(192) X(200) X(250) X(384)  \
  X(400) X(500) X(768) X(900) X(1000) X(1800)
#define CASES_F64(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(96) X(100) X(192) X(250) X(500) X(1000)

#define DEFINE_LOOKUPS(T, CASES)                                                  \
  template <>                                                                     \
  bool static_zfwd<T>(int M, int pro, ZfwdFn<T> &fn, StaticGeom &g, int var, int split) { \
    if (split) return split_zfwd<T>(M, pro, fn, g, var);                          \
    switch (M) {                                                                  \
      CASES(ZF)                                                                   \
      default: return false;                                                      \
    }                                                                             \
  }                                                                               \
  template <>                                                                     \
  bool static_zinv<T>(int M, ZinvFn<T> &fn, StaticGeom &g, int var, int split) {  \
    if (split) return split_zinv<T>(M, fn, g, var);                               \
    switch (M) {                                                                  \
      CASES(ZI)                                                                   \
      default: return false;                                                      \
    }                                                                             \
  }                                                                               \
  template <>                                                                     \
  bool static_strided<T>(int L, int mode, StridedFn<T> &fn, StaticGeom &g, int var, int split) { \
    if (split) return split_strided<T>(L, mode, fn, g, var);                      \
    switch (L) {                                                                  \
      CASES(ST)                                                                   \
      default: return false;                                                      \
    }                                                                             \
  }

#define DEFINE_FC_LOOKUP(T, CASES)                                                \
  template <>                                                                     \
  bool static_strided_fc<T>(int L, StridedFn<T> &fn, StaticGeom &g, int var) {    \
    switch (L) {                                                                  \
      CASES(SFC)                                                                  \
      default: return false;                                                      \
    }                                                                             \
  }
#define SFC(n) case n: return var ? strided_fc_for<TT, n, 1>(fn, g) : strided_fc_for<TT, n, 0>(fn, g);

#define ZF(n) case n: return var ? zfwd_for<TT, n, 1>(pro, fn, g) : zfwd_for<TT, n, 0>(pro, fn, g);
#define ZI(n) case n: return var ? zinv_for<TT, n, 1>(fn, g) : zinv_for<TT, n, 0>(fn, g);
#define ST(n) case n: return var ? strided_for<TT, n, 1>(mode, fn, g) : strided_for<TT, n, 0>(mode, fn, g);

#define CASES_SPLIT(X) X(128) X(256) X(512)
#define ZFS(n) case n: return var ? zfwd_for<double, n, 1, true>(pro, fn, g) : zfwd_for<double, n, 0, true>(pro, fn, g);
#define ZIS(n) case n: return var ? zinv_for<double, n, 1, true>(fn, g) : zinv_for<double, n, 0, true>(fn, g);
#define STS(n)                                                                 \
  case n:                                                                      \
    return var ? strided_for<double, n, 1, true>(mode, fn, g) : strided_for<double, n, 0, true>(mode, fn, g);

}  // namespace ffcz
