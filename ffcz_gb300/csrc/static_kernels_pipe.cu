// Instantiations of the TMA-staged strided passes (passes_pipe.cuh) for the
// FP32 compile-time lengths, in a translation unit of their own.  Each mode
// and tile variant takes the stage list, tile width and block size of the
// register kernel it stands in for (static_inst.cuh's Cfg), so the two share
// their pass arguments and plan.
#include "passes_pipe.cuh"
#include "static_inst.cuh"

namespace ffcz {

template <int L, int VAR, int MODE>
static bool pipe_one(PipeFn &fn, StaticGeom &g, int &nbuf) {
  constexpr bool FUSED = MODE == MODE_FCI || MODE == MODE_FCIX;
  constexpr int CAP = FUSED ? 16 : plain_cap(L);
  using C = Cfg<float, L, CAP, VAR>;
  if (VAR && C::TW == Cfg<float, L, CAP, 0>::TW) return false;  // same tile as the default
  constexpr int MINB = strided_minb(4, C::NT, rp_elems(L, CAP));
  constexpr int NBUF = pipe_nbuf(L, C::TW, CAP, MINB);
  if constexpr (NBUF < 2 || C::LGTW < 1 || pipe_nbox(L, C::TW) == 0) {
    return false;
  } else {
    fn = ks_strided_pipe<MODE, L, C::LGTW, CAP, NBUF, MINB>;
    g.TW = C::TW;
    g.threads = C::NT;
    g.smem = pipe_smem_bytes(L, C::TW, CAP, NBUF);
    nbuf = NBUF;
    return set_smem(fn, g.smem) == FFCZ_OK;
  }
}

template <int L, int VAR>
static bool pipe_for(int mode, PipeFn &fn, StaticGeom &g, int &nbuf) {
  switch (mode) {
    case MODE_FWD: return pipe_one<L, VAR, MODE_FWD>(fn, g, nbuf);
    case MODE_INV: return pipe_one<L, VAR, MODE_INV>(fn, g, nbuf);
    case MODE_FC: return pipe_one<L, VAR, MODE_FC>(fn, g, nbuf);
    case MODE_FCI: return pipe_one<L, VAR, MODE_FCI>(fn, g, nbuf);
    case MODE_FCIX: return pipe_one<L, VAR, MODE_FCIX>(fn, g, nbuf);
    default: return false;
  }
}

#define CASES_PIPE(X) X(64) X(128) X(256) X(512) X(1024) X(2048) X(100) X(200) X(250) X(400) X(500) X(1000) X(1800)
#define PP(n) \
  case n: return var ? pipe_for<n, 1>(mode, fn, g, nbuf) : pipe_for<n, 0>(mode, fn, g, nbuf);

bool pipe_strided(int L, int mode, PipeFn &fn, StaticGeom &g, int var, int &nbuf) {
  switch (L) {
    CASES_PIPE(PP)
    default: return false;
  }
}

int pipe_box_positions(int L, int TW) { return pipe_nbox(L, TW) ? L / pipe_nbox(L, TW) : 0; }

}  // namespace ffcz
