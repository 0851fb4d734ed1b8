#include "fft_plan.h"

#include <cmath>

namespace ffcz {

bool specialised_radix(int r) {
  return r == 2 || r == 3 || r == 4 || r == 5 || r == 7 || r == 8;
}

bool factorize(int L, std::vector<int> &radices) {
  radices.clear();
  if (L < 1) return false;
  int n = L;
  while (n % 8 == 0) { radices.push_back(8); n /= 8; }
  if (n % 4 == 0) { radices.push_back(4); n /= 4; }
  if (n % 2 == 0) { radices.push_back(2); n /= 2; }
  const int odd[] = {5, 3, 7};
  for (int p : odd) {
    while (n % p == 0) { radices.push_back(p); n /= p; }
  }
  for (int p = 11; p <= kMaxGenericRadix && n > 1; p += 2) {
    while (n % p == 0) { radices.push_back(p); n /= p; }
  }
  return n == 1 && (int)radices.size() <= kMaxStages;
}

// exp(-2*pi*i*a/d) with the argument reduced to [0, d) first.
static std::complex<double> root(long long a, long long d) {
  a %= d;
  if (a < 0) a += d;
  const double th = -2.0 * M_PI * (double)a / (double)d;
  return {std::cos(th), std::sin(th)};
}

bool build_axis_plan(int L, AxisPlan &p, std::vector<std::complex<double>> &table) {
  std::vector<int> rad;
  if (!factorize(L, rad)) return false;
  p.L = L;
  p.nst = (int)rad.size();
  p.tw = nullptr;
  int Ns = 1;
  for (int s = 0; s < p.nst; ++s) {
    const int R = rad[s];
    p.R[s] = R;
    p.Ns[s] = Ns;
    p.twoff[s] = (int)table.size();
    if (Ns > 1) {
      for (int k = 0; k < Ns; ++k)
        for (int r = 1; r < R; ++r) table.push_back(root((long long)r * k, (long long)Ns * R));
    }
    p.rootoff[s] = -1;
    if (!specialised_radix(R)) {
      p.rootoff[s] = (int)table.size();
      for (int m = 0; m < R; ++m) table.push_back(root(m, R));
    }
    Ns *= R;
  }
  return true;
}

}  // namespace ffcz
