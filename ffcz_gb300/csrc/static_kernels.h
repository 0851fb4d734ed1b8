// Lookup of the compile-time-sized register-resident pass kernels
// (passes_static.cuh) and construction of their twiddle tables.
#pragma once

#include <cuda.h>

#include <complex>
#include <vector>

#include "passes.cuh"

namespace ffcz {

template <typename T>
using ZfwdFn = void (*)(const T *, const T *, T *, T, c2<T> *, ZArgs, AxisPlan, const c2<T> *);
template <typename T>
using ZinvFn = void (*)(const c2<T> *, T *, T, T, LoopCtl *, double *, ZArgs, AxisPlan, const c2<T> *);
template <typename T>
using StridedFn = void (*)(c2<T> *, SArgs, AxisPlan, ClampArgs<T>, T *, long long);

struct StaticGeom {
  int TW = 0;        // tile width (columns or rows)
  int threads = 0;   // block size
  size_t smem = 0;   // dynamic shared memory bytes
};

// True when a compile-time kernel exists for this length (power of two,
// 16..4096 for FP32, 16..2048 for FP64).
bool static_length(int L, bool fp64);
// Appends the forward and inverse stage twiddles of length L to `table`
// and fills p.twoff (forward at [s], inverse at [12 + s]); p.tw left null.
// cap = 16 for the strided passes' stage lists (17: the plain passes'
// family, static_plain_cap), 8 for the z passes'.
void build_static_plan(int L, int cap, AxisPlan &p, std::vector<std::complex<double>> &table);
// Stage-list family (the cap argument above) of the plain forward / inverse
// strided passes of length L; the fused passes use 16.
int static_plain_cap(int L);

// Kernel for a length static_length() accepts (false otherwise).
// z passes: M = Nz/2; pro is PRO_PLAIN/PRO_DIFF/PRO_CLAMP.
// var 0: the default tile; var 1: the autotuner's alternative tile width
// (false when it equals the default's).  split (FP64 only): the kernels that
// compute in float-float on the FP32 pipes.
template <typename T> bool static_zfwd(int M, int pro, ZfwdFn<T> &fn, StaticGeom &g, int var = 0, int split = 0);
template <typename T> bool static_zinv(int M, ZinvFn<T> &fn, StaticGeom &g, int var = 0, int split = 0);
template <typename T>
bool static_strided(int L, int mode, StridedFn<T> &fn, StaticGeom &g, int var = 0, int split = 0);
// The plain form's forward pass with the all-abs clamp in its epilogue
// (MODE_FC): the plain stage-list family and tile of MODE_FWD, so it shares
// that pass's geometry.  No float-float variant.
template <typename T> bool static_strided_fc(int L, StridedFn<T> &fn, StaticGeom &g, int var = 0);
// The FP32 passes whose radix-16 stages run on the tensor cores
// (passes_tc.cuh), L = 256 or 512, modes MODE_FWD, MODE_INV, MODE_FC and
// MODE_FCI, all on the plain stage list (static_plain_cap); false otherwise.
bool tc_strided(int L, int mode, StridedFn<float> &fn, StaticGeom &g);

// TMA-staged persistent variant of an FP32 strided pass (passes_pipe.cuh):
// the tile geometry of the register kernel of the same mode and variant,
// tiles read through a rank-4 tensor map over the padded spectrum
// (kz: Hz, q: Q, position: L, batch: B; 8-byte elements), nbuf tile slots
// per block; grid = resident blocks, at most one per tile.  False where
// no such kernel exists.
using PipeFn = void (*)(const CUtensorMap, c2<float> *, SArgs, AxisPlan, ClampArgs<float>, float *, long long,
                        long long, int *);
bool pipe_strided(int L, int mode, PipeFn &fn, StaticGeom &g, int var, int &nbuf);
// Positions per box of that tensor map for length L and tile width TW.
int pipe_box_positions(int L, int TW);

}  // namespace ffcz
