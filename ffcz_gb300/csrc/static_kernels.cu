// Instantiations of the register-resident pass kernels (FP32 lengths
// 16..4096, FP64 16..2048, and the 2^a 3^b 5^c lengths with a stage list),
// their lookup, and their twiddle tables.
#include <cmath>

#include "static_inst.cuh"

namespace ffcz {

bool static_length(int L, bool fp64) {
  if (mx_list(L)) return mx_E(L) <= (fp64 ? 12 : 30);
  return L >= 16 && (L & (L - 1)) == 0 && L <= (fp64 ? 2048 : 4096);
}

int static_plain_cap(int L) { return plain_cap(L); }

void build_static_plan(int L, int cap, AxisPlan &p, std::vector<std::complex<double>> &table) {
  p.L = L;
  p.nst = rp_nst(L, cap);
  p.tw = nullptr;
  for (int dir : {-1, +1}) {
    long long Ns = 1;
    for (int s = 0; s < rp_nst(L, cap); ++s) {
      const int R = rp_rad(L, dir, s, cap);
      // paired stages: R entries per k from a 16-byte aligned start
      const bool vec = tw_paired(cap, R);
      while (vec && table.size() % 2) table.push_back({1.0, 0.0});
      p.twoff[(dir < 0 ? 0 : kInvBase) + s] = (int)table.size();
      if (Ns > 1)
        for (long long k = 0; k < Ns; ++k)
          for (int r = vec ? 0 : 1; r < R; ++r) {
            const long long d = Ns * R, a = (r * k) % d;
            const double th = -2.0 * M_PI * (double)a / (double)d;
            table.push_back({std::cos(th), std::sin(th)});
          }
      Ns *= R;
    }
  }
}

template <> bool split_zfwd<float>(int, int, ZfwdFn<float> &, StaticGeom &, int) { return false; }
template <> bool split_zinv<float>(int, ZinvFn<float> &, StaticGeom &, int) { return false; }
template <> bool split_strided<float>(int, int, StridedFn<float> &, StaticGeom &, int) { return false; }

#define TT float
DEFINE_LOOKUPS(float, CASES_F32)
#undef TT

}  // namespace ffcz
