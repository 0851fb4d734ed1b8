// Strided passes whose radix-16 stages run as dense 16-point DFT matmuls on
// the tensor cores (mma.sync m16n8k8, TF32 operands, FP32 accumulation),
// for the axis lengths whose plain stage list is made of radix-16 stages
// and at most one small stage: 256 = [16,16], 512 = [16,16,2].
//
// A tile of TW columns x L positions is staged in shared memory (two
// buffers, Stockham ping-pong).  A radix-16 stage of span Ns computes, for
// each butterfly j (and column c),
//   Y[m] = sum_k W16^(mk) * (x[j + k L/16] * w_j^k),  W16 = exp(-+2 pi i/16),
//   w_j^k = twiddle (j mod Ns, k) of the stage (conjugated inverse),
// and stores Y[m] at (j / Ns) Ns 16 + j mod Ns + m Ns -- the arithmetic of
// the register kernels' rstage + Dft<16>, as a matrix product per group of
// eight butterflies (the eight columns of one j): in real form
//   Yr = Wr Xr + Wi (-Xi),  Yi = Wi Xr + Wr Xi,
// each a (16 x 16)(16 x 8) product = two m16n8k8 MMAs.  Precision: every
// operand is split into two TF32 terms, x = hi + lo (hi = x rounded to TF32,
// lo = the rest rounded to TF32), and the product is hi*hi + hi*lo + lo*hi
// (the "3xTF32" scheme), so a product keeps ~21 of FP32's 24 bits; the
// twiddle multiply stays in FP32 before the split.  24 MMAs per group of 8
// butterflies.  The radix-2 stage of 512 runs on the FP32 pipes.
//
// Modes: MODE_FWD, MODE_INV, MODE_FC (forward, all-abs clamp) and MODE_FCI
// (forward, clamp, inverse in the same tile), all on the plain stage list
// and its twiddle plan.
#pragma once

#include "passes_static.cuh"

namespace ffcz {

constexpr int kTcTW = 8;       // columns per tile (one MMA N dimension)
constexpr int kTcThreads = 256;

// Column pitch: room for L positions plus the largest skew (8 * 15 slots),
// and 2 mod 16 slots, so that consecutive columns start 4 banks apart.
__host__ __device__ constexpr int tc_pitch(int L) { return L + 130; }
// Shared-memory slot of (position, column): positions skew by 8 slots per
// L/16 block, so that the eight columns and four rows an MMA fragment
// touches spread over all banks.  Slots of a column stay below the next
// column's first slot: L - 1 + 8 * 15 < tc_pitch(L).
template <int L>
__device__ __forceinline__ int tc_slot(int pos, int c) {
  return c * tc_pitch(L) + pos + 8 * (pos / (L / 16));
}

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo) {
  hi = tf32_bits(x);
  lo = tf32_bits(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// cos and sin of 2 pi q / 16
__device__ __forceinline__ void w16(int q, float &c, float &s) {
  constexpr float C1 = 0.92387953251128674f, C2 = 0.70710678118654752f, C3 = 0.38268343236508977f;
  q &= 15;
  const int a = q & 7;  // angle within a half turn: cos(a pi/8), sin(a pi/8)
  auto cs = [&](int i) { return i == 0 ? 1.0f : i == 1 ? C1 : i == 2 ? C2 : i == 3 ? C3 : 0.0f; };
  const float ca = a <= 4 ? cs(a) : -cs(8 - a);
  const float sa = a <= 4 ? cs(4 - a) : cs(a - 4);
  c = q < 8 ? ca : -ca;
  s = q < 8 ? sa : -sa;
}

// The DFT matrix fragments of one lane: A(m, k) = W16^(m k) for the two
// K-tiles (k < 8, k >= 8), m16n8k8 row layout (a0: (g, t), a1: (g+8, t),
// a2: (g, t+4), a3: (g+8, t+4); g = lane / 4, t = lane % 4); split hi/lo.
// Forward: W = cos - i sin; the inverse flips the sign of the Wi terms.
struct TcFrag {
  uint32_t wr_hi[2][4], wr_lo[2][4], wi_hi[2][4], wi_lo[2][4];
};
__device__ __forceinline__ void tc_frag(TcFrag &f, int lane) {
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kt = 0; kt < 2; ++kt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int m = g + ((e & 1) ? 8 : 0), k = 8 * kt + t + ((e & 2) ? 4 : 0);
      float c, s;
      w16(m * k, c, s);
      tf32_split(c, f.wr_hi[kt][e], f.wr_lo[kt][e]);
      tf32_split(-s, f.wi_hi[kt][e], f.wi_lo[kt][e]);  // forward: Wi = -sin
    }
}

// One radix-16 stage on the tensor cores, in -> out.  DIR -1 forward, +1
// inverse; tw: the stage's twiddles (R = 16 entries per k, entry 0 unused)
// or null for the first stage (Ns = 1).
template <int L, int DIR>
__device__ __forceinline__ void tc_stage16(const float2 *__restrict__ in, float2 *__restrict__ out, int Ns,
                                           const float2 *__restrict__ tw, const TcFrag &f, int warp, int lane) {
  const int g = lane >> 2, t = lane & 3;
  constexpr int NB = L / 16;  // butterflies per column
  const uint32_t flip = DIR > 0 ? 0x80000000u : 0u;  // inverse: Wi -> -Wi
  for (int j = warp; j < NB; j += kTcThreads / 32) {
    const int jm = j % Ns;
    // B fragments: rows k = 8 kt + t (+4), column n = g
    uint32_t xr_hi[2][2], xr_lo[2][2], xi_hi[2][2], xi_lo[2][2];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int k = 8 * kt + t + 4 * h;
        float2 x = in[tc_slot<L>(j + k * NB, g)];
        if (tw != nullptr && k > 0) {
          const float2 w = tw[jm * 16 + k];
          x = DIR < 0 ? cmul(x, w) : cmulc(x, w);
        }
        tf32_split(x.x, xr_hi[kt][h], xr_lo[kt][h]);
        tf32_split(x.y, xi_hi[kt][h], xi_lo[kt][h]);
      }
    float yr[4] = {0.f, 0.f, 0.f, 0.f}, yi[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      uint32_t wih[4], wil[4], nwih[4], nwil[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        wih[e] = f.wi_hi[kt][e] ^ flip;
        wil[e] = f.wi_lo[kt][e] ^ flip;
        nwih[e] = wih[e] ^ 0x80000000u;  // -Wi, for Yr = Wr Xr - Wi Xi
        nwil[e] = wil[e] ^ 0x80000000u;
      }
      // Yr = Wr Xr - Wi Xi
      mma_tf32(yr, f.wr_hi[kt], xr_hi[kt][0], xr_hi[kt][1]);
      mma_tf32(yr, f.wr_hi[kt], xr_lo[kt][0], xr_lo[kt][1]);
      mma_tf32(yr, f.wr_lo[kt], xr_hi[kt][0], xr_hi[kt][1]);
      mma_tf32(yr, nwih, xi_hi[kt][0], xi_hi[kt][1]);
      mma_tf32(yr, nwih, xi_lo[kt][0], xi_lo[kt][1]);
      mma_tf32(yr, nwil, xi_hi[kt][0], xi_hi[kt][1]);
      // Yi = Wi Xr + Wr Xi
      mma_tf32(yi, wih, xr_hi[kt][0], xr_hi[kt][1]);
      mma_tf32(yi, wih, xr_lo[kt][0], xr_lo[kt][1]);
      mma_tf32(yi, wil, xr_hi[kt][0], xr_hi[kt][1]);
      mma_tf32(yi, f.wr_hi[kt], xi_hi[kt][0], xi_hi[kt][1]);
      mma_tf32(yi, f.wr_hi[kt], xi_lo[kt][0], xi_lo[kt][1]);
      mma_tf32(yi, f.wr_lo[kt], xi_hi[kt][0], xi_hi[kt][1]);
    }
    // D fragments: (m = g (+8), n = 2t (+1))
    const int base = (j / Ns) * Ns * 16 + jm;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int m = g + ((e & 2) ? 8 : 0), n = 2 * t + (e & 1);
      out[tc_slot<L>(base + m * Ns, n)] = make_float2(yr[e], yi[e]);
    }
  }
}

// Radix-2 stage on the FP32 pipes (butterfly j: inputs j, j + L/2).
template <int L, int DIR>
__device__ __forceinline__ void tc_stage2(const float2 *__restrict__ in, float2 *__restrict__ out, int Ns,
                                          const float2 *__restrict__ tw, int tid) {
  for (int i = tid; i < (L / 2) * kTcTW; i += kTcThreads) {
    const int j = i / kTcTW, c = i % kTcTW;
    const int jm = j % Ns;
    float2 a = in[tc_slot<L>(j, c)], b = in[tc_slot<L>(j + L / 2, c)];
    if (tw != nullptr) {
      const float2 w = tw[jm * 2 + 1];
      b = DIR < 0 ? cmul(b, w) : cmulc(b, w);
    }
    const int base = (j / Ns) * Ns * 2 + jm;
    out[tc_slot<L>(base, c)] = cadd(a, b);
    out[tc_slot<L>(base + Ns, c)] = csub(a, b);
  }
}

// Runs the plain stage list of L in direction DIR from buffer `cur`;
// returns the buffer that holds the result.
template <int L, int DIR>
__device__ __forceinline__ float2 *tc_transform(float2 *cur, float2 *other, const AxisPlan &p, const TcFrag &f,
                                                int tid) {
  constexpr int CAP = plain_cap(L);
  constexpr int NST = rp_nst(L, CAP);
  const int warp = tid >> 5, lane = tid & 31;
  int Ns = 1;
#pragma unroll
  for (int st = 0; st < NST; ++st) {
    const int R = rp_rad(L, DIR, st, CAP);
    const float2 *tw = st == 0 ? nullptr : (const float2 *)p.tw + p.twoff[(DIR < 0 ? 0 : kInvBase) + st];
    if (R == 16) tc_stage16<L, DIR>(cur, other, Ns, tw, f, warp, lane);
    else tc_stage2<L, DIR>(cur, other, Ns, tw, tid);
    __syncthreads();
    float2 *t = cur;
    cur = other;
    other = t;
    Ns *= R;
  }
  return cur;
}

template <int MODE, int L>
__global__ void __launch_bounds__(kTcThreads) ks_strided_tc(float2 *__restrict__ spec, SArgs s, AxisPlan p,
                                                            ClampArgs<float> ca, float *__restrict__ fedits,
                                                            long long H) {
  static_assert(L == 256 || L == 512, "tensor-core passes: L = 256 or 512");
  static_assert((L - 1) + 8 * 15 < tc_pitch(L) && tc_pitch(L) % 16 == 2, "slot layout");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *b0 = reinterpret_cast<float2 *>(smem_raw);
  float2 *b1 = b0 + kTcTW * tc_pitch(L) + 16;
  const int tid = threadIdx.x;
  const long long tile = blockIdx.x;
  const long long per_b = (long long)s.Q * s.tpq;
  const long long bb = tile / per_b;
  const int rem = (int)(tile - bb * per_b);
  const int q = rem / s.tpq;
  const int kz0 = (rem - q * s.tpq) * kTcTW;
  const int ncol = min(kTcTW, s.Hz - kz0);
  float2 *g = spec + bb * (long long)L * s.Wtot + (long long)q * s.Hzp + kz0;
  for (int i = tid; i < L * kTcTW; i += kTcThreads) {
    const int pos = i / kTcTW, c = i % kTcTW;
    b0[tc_slot<L>(pos, c)] = c < ncol ? g[(long long)pos * s.Wtot + c] : make_float2(0.f, 0.f);
  }
  TcFrag f;
  tc_frag(f, tid & 31);
  __syncthreads();
  float2 *res;
  if (MODE == MODE_INV) res = tc_transform<L, +1>(b0, b1, p, f, tid);
  else res = tc_transform<L, -1>(b0, b1, p, f, tid);
  if (MODE == MODE_FC || MODE == MODE_FCI) {
    bool hit = false;
    float fm = 0.0f;
    for (int i = tid; i < L * kTcTW; i += kTcThreads) {
      const int pos = i / kTcTW, c = i % kTcTW;
      if (c < ncol) {
        const long long k = ((bb * L + pos) * (long long)s.Q + q) * s.Hz + kz0 + c;
        const float2 w = freq_clamp<float>(res[tc_slot<L>(pos, c)], ca.delta, fedits, k, H, hit);
        res[tc_slot<L>(pos, c)] = w;
        fm = fmaxf(fm, fmaxf(fabsf(w.x), fabsf(w.y)));
      }
    }
    mark_dirty(ca.fdirty, hit);
    record_fmax(ca.fmax, fm);
    __syncthreads();
    if (MODE == MODE_FCI) res = tc_transform<L, +1>(res, res == b0 ? b1 : b0, p, f, tid);
  }
  for (int i = tid; i < L * kTcTW; i += kTcThreads) {
    const int pos = i / kTcTW, c = i % kTcTW;
    if (c < ncol) g[(long long)pos * s.Wtot + c] = res[tc_slot<L>(pos, c)];
  }
}

// Shared memory of ks_strided_tc<L>: two staged tiles.
__host__ __device__ constexpr size_t tc_smem_bytes(int L) {
  return (size_t)(2 * (kTcTW * tc_pitch(L) + 16)) * sizeof(float2);
}

}  // namespace ffcz
