// Lookup of the compile-time-sized pass kernels (passes_static.cuh).
#pragma once

#include "passes.cuh"

namespace ffcz {

template <typename T>
using ZfwdFn = void (*)(const T *, const T *, T *, T, c2<T> *, ZArgs, AxisPlan, const c2<T> *);
template <typename T>
using ZinvFn = void (*)(const c2<T> *, T *, T, T, LoopCtl *, ZArgs, AxisPlan, const c2<T> *);
template <typename T>
using StridedFn = void (*)(c2<T> *, SArgs, AxisPlan, T, T *, long long);

struct StaticGeom {
  int TW = 0;        // tile width (columns or rows)
  int threads = 0;   // block size
  size_t smem = 0;   // dynamic shared memory bytes
};

// Kernel for a power-of-two length, or false when none is compiled in.
// z passes: M = Nz/2 (even Nz only); pro is PRO_PLAIN/PRO_DIFF/PRO_CLAMP.
template <typename T> bool static_zfwd(int M, int pro, ZfwdFn<T> &fn, StaticGeom &g);
template <typename T> bool static_zinv(int M, ZinvFn<T> &fn, StaticGeom &g);
template <typename T> bool static_strided(int L, int mode, StridedFn<T> &fn, StaticGeom &g);

}  // namespace ffcz
