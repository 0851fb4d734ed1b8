// Host-side planning of the mixed-radix Stockham transforms: factorisation of
// each axis length, per-stage twiddle tables (computed in double, rounded to
// the element type on upload) and the launch geometry of every pass.
#pragma once

#include <complex>
#include <vector>

namespace ffcz {

constexpr int kMaxStages = 24;

// One axis transform of length L = prod(R[s]).  Stage s (radix R[s]) works
// on sub-transforms of span Ns[s] = R[0]*...*R[s-1]; its twiddles
// exp(-2*pi*i*r*k/(Ns*R)), k < Ns, 1 <= r < R, start at twoff[s] in the
// device table `tw` (k-major, r-minor).  Passed to kernels by value.
// Radices other than 2, 3, 4, 5, 7, 8 (the primes above 7) run through a
// generic stage whose R roots exp(-2*pi*i*m/R) start at rootoff[s].
struct AxisPlan {
  int L;
  int nst;
  int R[kMaxStages];
  int Ns[kMaxStages];
  int twoff[kMaxStages];
  int rootoff[kMaxStages];
  const void *tw;
};

// Radices with an unrolled register butterfly.
bool specialised_radix(int r);

// Largest prime factor handled by the generic stage.
constexpr int kMaxGenericRadix = 4093;
// Factorises L into radices: powers of two as 8/4/2, then 5, 3, 7, then
// the remaining primes (generic stage).  Returns false when a prime factor
// exceeds kMaxGenericRadix or there are more than kMaxStages stages.
bool factorize(int L, std::vector<int> &radices);
// Fills `p` (tw left null) and appends its twiddles to `table`.
bool build_axis_plan(int L, AxisPlan &p, std::vector<std::complex<double>> &table);

}  // namespace ffcz
