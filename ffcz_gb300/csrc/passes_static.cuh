// Compile-time-sized, register-resident pass kernels for power-of-two axis
// lengths L = 16 .. 4096 and a table of 2^a 3^b 5^c lengths.
//
// Each column (strided passes) or row (z passes) of length L is handled by
// TC = L/E threads holding E elements each (E = a multiple of every radix of
// the stage list).  A stage of radix R runs E/R butterflies per thread in
// registers; butterfly j = t + m*TC reads Stockham positions j + r*L/R and
// writes (j/Ns)*Ns*R + j%Ns + r*Ns.  Stages exchange data through shared
// memory, but the first stage reads its inputs straight from HBM into
// registers and the last stage writes straight to HBM, so a transform of
// S stages makes S-1 shared-memory round trips (one for L = 256 = 16*16).
// In the fused pass (forward, frequency clamp, inverse) the inverse's
// first radix equals the forward's last, so the clamped coefficients feed
// the inverse without an exchange.
//
// The inverse runs the forward stage list in reverse order.
// Twiddles come from a table built on the host for the same lists:
// AxisPlan.twoff[s] for forward stage s, twoff[kInvBase + s] for inverse
// stage s.
#pragma once

#include "passes.cuh"

namespace ffcz {

constexpr int kInvBase = 12;

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// Stage lists of the non-power-of-two lengths (the same for every pass),
// packed as E | nst << 8 | r0 << 16 | r1 << 24 | r2 << 32 | r3 << 40
// (forward order; every radix divides E; composite radices are prime-factor
// butterflies).  0: no list.
__host__ __device__ constexpr unsigned long long mx_pack(int E, int r0, int r1 = 0, int r2 = 0, int r3 = 0) {
  return (unsigned long long)E | (unsigned long long)((r1 ? 1 : 0) + (r2 ? 1 : 0) + (r3 ? 1 : 0) + 1) << 8 |
         (unsigned long long)r0 << 16 | (unsigned long long)r1 << 24 | (unsigned long long)r2 << 32 |
         (unsigned long long)r3 << 40;
}
__host__ __device__ constexpr unsigned long long mx_list(int L) {
  return L == 96 ? mx_pack(12, 12, 4, 2)
       : L == 100 ? mx_pack(10, 10, 10)
       : L == 192 ? mx_pack(12, 12, 4, 4)
       : L == 200 ? mx_pack(20, 20, 10)
       : L == 250 ? mx_pack(10, 10, 5, 5)
       : L == 384 ? mx_pack(24, 24, 8, 2)
       : L == 400 ? mx_pack(20, 20, 20)
       : L == 500 ? mx_pack(10, 10, 10, 5)
       : L == 768 ? mx_pack(24, 24, 8, 4)
       : L == 900 ? mx_pack(30, 30, 30)
       : L == 1000 ? mx_pack(10, 10, 10, 10)
       : L == 1800 ? mx_pack(30, 30, 30, 2)
       : 0;
}
__host__ __device__ constexpr int mx_E(int L) { return (int)(mx_list(L) & 0xff); }
__host__ __device__ constexpr int mx_nst(int L) { return (int)((mx_list(L) >> 8) & 0xff); }
__host__ __device__ constexpr int mx_r(int L, int s) { return (int)((mx_list(L) >> (16 + 8 * s)) & 0xff); }

// Power-of-two stage lists.  Strided passes (CAP 16): 16:[16] 32:[8,4]
// 64:[8,8] 128:[16,8] 256:[16,16] 512:[8,8,8] 1024:[16,8,8] 2048:[16,16,8]
// 4096:[16,16,16].  CAP 17, the plain forward / inverse strided passes: the
// same except 512:[16,16,2] (16 values per thread, 16-column tiles: y passes
// at 512^3 0.286 -> 0.242 ms, while the fused pass, two transforms per
// tile, is faster on [8,8,8]: 0.451 vs 0.483 ms).  z passes (CAP 8, 16+
// threads per row): radix-8 stages then one radix 4 or 2 stage for the
// remainder.
__host__ __device__ constexpr int rp_nst(int L, int cap = 16) {
  return mx_list(L) ? mx_nst(L)
       : cap == 8 ? (ilog2(L) / 3 + (ilog2(L) % 3 ? 1 : 0))
#ifdef FFCZ_L256_R8
       : (L == 16 ? 1 : (L < 256 ? 2 : 3));
#else
       : (L == 16 ? 1 : (L <= 256 ? 2 : 3));
#endif
}
__host__ __device__ constexpr int rp_radix(int L, int s, int cap = 16) {
  return mx_list(L) ? mx_r(L, s)
       : cap == 8 ? (s < ilog2(L) / 3 ? 8 : (ilog2(L) % 3 == 2 ? 4 : 2))
       : L == 16 ? 16
       : L == 32 ? (s == 0 ? 8 : 4)
       : L == 64 ? 8
       : L == 128 ? (s == 0 ? 16 : 8)
#ifdef FFCZ_L256_R8
       : L == 256 ? (s < 2 ? 8 : 4)
#else
       : L == 256 ? 16
#endif
       : L == 512 ? (cap == 17 ? (s < 2 ? 16 : 2) : 8)
       : L == 1024 ? (s == 0 ? 16 : 8)
       : L == 2048 ? (s < 2 ? 16 : 8)
       : 16;
}
__host__ __device__ constexpr int rp_elems(int L, int cap = 16) {
#ifdef FFCZ_L256_R8
  return mx_list(L) ? mx_E(L) : cap == 8 ? 8 : ((L == 32 || L == 64 || L == 256 || L == 512) ? 8 : 16);
#else
  return mx_list(L) ? mx_E(L) : cap == 8 ? 8 : ((L == 32 || L == 64 || (L == 512 && cap != 17)) ? 8 : 16);
#endif
}
// radix of stage s in direction DIR (inverse = reversed list)
__host__ __device__ constexpr int rp_rad(int L, int dir, int s, int cap = 16) {
  return dir < 0 ? rp_radix(L, s, cap) : rp_radix(L, rp_nst(L, cap) - 1 - s, cap);
}
// span Ns before stage s in direction dir
__host__ __device__ constexpr int rp_ns(int L, int dir, int s, int cap = 16) {
  return s == 0 ? 1 : rp_ns(L, dir, s - 1, cap) * rp_rad(L, dir, s - 1, cap);
}
// Strided passes' even radices store R twiddles per k (entry 0 unused) so
// that a butterfly's R-1 twiddles are 16-byte aligned and read in pairs:
// there a warp's lanes share few twiddle rows.  Odd radices and the z
// passes (whose lanes each need a different row) keep R-1 per k.
__host__ __device__ constexpr bool tw_paired(int cap, int R) { return cap != 8 && R % 2 == 0; }
// Stage-list family of the plain (forward / inverse) strided passes.
__host__ __device__ constexpr int plain_cap(int L) { return L == 512 ? 17 : 16; }

// Prime-factor butterfly of length N1*N2 (coprime): input n = (N2 n1 + N1 n2)
// mod N, N2 transforms of length N1, N1 of length N2, output at
// k = (k1 e1 + k2 e2) mod N with e1 = 1 mod N1, 0 mod N2 and e2 = 0 mod N1,
// 1 mod N2 -- no twiddles between the two layers (Good-Thomas).
__host__ __device__ constexpr int crt_unit(int a, int b) {  // x = 0 mod b, x = 1 mod a
  int x = 0;
  while ((x * b) % a != 1) ++x;
  return x * b;
}
template <int N1, int N2, int DIR, typename V>
struct DftPfa {
  __device__ __forceinline__ static void run(V *v);
};

// Radix 16 = 4 x 4 with the w16 twiddles between the two radix-4 layers.
template <int DIR, typename V> struct Dft<16, DIR, V> {
  __device__ __forceinline__ static void run(V *v) {
    using S = decltype(v[0].x);
    const S c1 = S(0.9238795325112867), s1 = S(0.3826834323650898), h = S(0.7071067811865476);
    // layer 1: for each n2, radix-4 over n1 (elements 4*n1 + n2)
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) bfly4<DIR>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
    // twiddle w16^(n2*k1): element (k1, n2) at v[4*k1 + n2]
    auto tw = [&](V &a, S c, S s) {  // a *= (c, DIR*s)
      V r;
      const S sd = DIR < 0 ? -s : s;
      r.x = a.x * c - a.y * sd;
      r.y = a.x * sd + a.y * c;
      a = r;
    };
    tw(v[4 + 1], c1, s1);   // k1=1,n2=1 : w^1
    tw(v[4 + 2], h, h);     // k1=1,n2=2 : w^2
    tw(v[4 + 3], s1, c1);   // k1=1,n2=3 : w^3
    v[8 + 1] = (DIR < 0) ? mkc<S>((v[9].x + v[9].y) * h, (v[9].y - v[9].x) * h)
                         : mkc<S>((v[9].x - v[9].y) * h, (v[9].x + v[9].y) * h);  // w^2
    v[8 + 2] = cmul_i<DIR>(v[8 + 2]);                                              // w^4
    tw(v[8 + 3], -h, h);    // w^6
    tw(v[12 + 1], s1, c1);  // w^3
    tw(v[12 + 2], -h, h);   // w^6
    tw(v[12 + 3], -c1, -s1);  // w^9
    // layer 2: for each k1, radix-4 over n2 -> outputs k1 + 4*k2
    V out[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      V a0 = v[4 * k1], a1 = v[4 * k1 + 1], a2 = v[4 * k1 + 2], a3 = v[4 * k1 + 3];
      bfly4<DIR>(a0, a1, a2, a3);
      out[k1] = a0;
      out[k1 + 4] = a1;
      out[k1 + 8] = a2;
      out[k1 + 12] = a3;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = out[k];
  }
};

template <int N1, int N2, int DIR, typename V>
__device__ __forceinline__ void DftPfa<N1, N2, DIR, V>::run(V *v) {
  constexpr int N = N1 * N2, E1 = crt_unit(N1, N2), E2 = crt_unit(N2, N1);
  V a[N2][N1];
#pragma unroll
  for (int n2 = 0; n2 < N2; ++n2)
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) a[n2][n1] = v[(N2 * n1 + N1 * n2) % N];
#pragma unroll
  for (int n2 = 0; n2 < N2; ++n2) Dft<N1, DIR, V>::run(a[n2]);
  V b[N1][N2];
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1)
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2) b[k1][n2] = a[n2][k1];
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1) Dft<N2, DIR, V>::run(b[k1]);
#pragma unroll
  for (int k1 = 0; k1 < N1; ++k1)
#pragma unroll
    for (int k2 = 0; k2 < N2; ++k2) v[(k1 * E1 + k2 * E2) % N] = b[k1][k2];
}
template <int DIR, typename V> struct Dft<6, DIR, V> : DftPfa<2, 3, DIR, V> {};
template <int DIR, typename V> struct Dft<10, DIR, V> : DftPfa<2, 5, DIR, V> {};
template <int DIR, typename V> struct Dft<12, DIR, V> : DftPfa<4, 3, DIR, V> {};
template <int DIR, typename V> struct Dft<15, DIR, V> : DftPfa<3, 5, DIR, V> {};
template <int DIR, typename V> struct Dft<20, DIR, V> : DftPfa<4, 5, DIR, V> {};
template <int DIR, typename V> struct Dft<24, DIR, V> : DftPfa<8, 3, DIR, V> {};
template <int DIR, typename V> struct Dft<30, DIR, V> : DftPfa<2, 15, DIR, V> {};

// Butterflies of one stage on the thread's registers: v[m*R + r] is input
// r of butterfly m (j = t + m*TC) and becomes output r.
// Twiddles of one stage's butterflies for thread t (a stage of radix R and
// span NS; none when NS == 1): w[m][r], r >= 1, of butterfly j = t + m*TC,
// row j % NS of the stage's table (R entries per row when VEC -- read as
// aligned pairs --, R - 1 otherwise).
template <typename T, int R, int NS, int L, int E, bool VEC, typename TS>
struct StageTw {
  c2<T> w[E / R][R];
  __device__ __forceinline__ void load(int t, const c2<TS> *__restrict__ tw) {
    if constexpr (NS > 1) {
      constexpr int TC = L / E;
#pragma unroll
      for (int m = 0; m < E / R; ++m) {
        const unsigned row = (unsigned)(t + m * TC) % (unsigned)NS;
        if constexpr (VEC) {
          const c2<TS> *p = tw + row * R;
          if constexpr (sizeof(TS) == 4) {
#pragma unroll
            for (int r = 0; r < R; r += 2) {
              const float4 q = *reinterpret_cast<const float4 *>(p + r);
              w[m][r] = mkc<T>((T)q.x, (T)q.y);
              w[m][r + 1] = mkc<T>((T)q.z, (T)q.w);
            }
          } else {
#pragma unroll
            for (int r = 1; r < R; ++r) w[m][r] = cvt<T>(p[r]);
          }
        } else {
          const c2<TS> *p = tw + row * (R - 1);
#pragma unroll
          for (int r = 1; r < R; ++r) w[m][r] = cvt<T>(p[r - 1]);
        }
      }
    }
  }
};

// Butterflies of one stage on the thread's registers: v[m*R + r] is input
// r of butterfly m (j = t + m*TC) and becomes output r; twiddles read from
// the stage's table as each butterfly needs them (the z passes' form).
template <typename T, int DIR, int R, int NS, int L, int E, bool VEC, typename TS = T>
__device__ __forceinline__ void rstage(c2<T> (&v)[E], int t, const c2<TS> *__restrict__ tw) {
  using V = c2<T>;
  constexpr int TC = L / E;
#pragma unroll
  for (int m = 0; m < E / R; ++m) {
    if (NS > 1) {
      const int j = t + m * TC;
      if constexpr (VEC) {
        const c2<TS> *w = tw + (j % NS) * R;
        V ww[R];
        if constexpr (sizeof(TS) == 4) {
#pragma unroll
          for (int r = 0; r < R; r += 2) {
            const float4 q = *reinterpret_cast<const float4 *>(w + r);
            ww[r] = mkc<T>((T)q.x, (T)q.y);
            ww[r + 1] = mkc<T>((T)q.z, (T)q.w);
          }
        } else {
#pragma unroll
          for (int r = 1; r < R; ++r) ww[r] = cvt<T>(w[r]);
        }
#pragma unroll
        for (int r = 1; r < R; ++r) v[m * R + r] = (DIR < 0) ? cmul(v[m * R + r], ww[r]) : cmulc(v[m * R + r], ww[r]);
      } else {
        const c2<TS> *w = tw + (j % NS) * (R - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const V ww = cvt<T>(w[r - 1]);
          v[m * R + r] = (DIR < 0) ? cmul(v[m * R + r], ww) : cmulc(v[m * R + r], ww);
        }
      }
    }
    Dft<R, DIR, V>::run(&v[m * R]);
  }
}

// The same with the stage's twiddles for this thread loaded beforehand (tw;
// the strided passes' form).
template <typename T, int DIR, int R, int NS, int L, int E, bool VEC, typename TS>
__device__ __forceinline__ void rstage_tw(c2<T> (&v)[E], const StageTw<T, R, NS, L, E, VEC, TS> &tw) {
  using V = c2<T>;
#pragma unroll
  for (int m = 0; m < E / R; ++m) {
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r)
        v[m * R + r] = (DIR < 0) ? cmul(v[m * R + r], tw.w[m][r]) : cmulc(v[m * R + r], tw.w[m][r]);
    }
    Dft<R, DIR, V>::run(&v[m * R]);
  }
}

// Shared-memory layouts of a tile of positions x columns, chosen per length
// from a bank model of every stage exchange (64-bit accesses served in
// 128-byte wavefronts) and kept where they measured faster: the mixed-radix
// z passes' pads cut their modelled wavefronts from 2.4-4.6x to 1.3-1.4x of
// the minimum (z forward at 250: 100 -> 91 us, z inverse 84 -> 66 us).
//
// Strided passes (lanes along columns): element (pos, c) at
// pos*P + c + (pos/B)*TW, i.e. rows of P slots with one extra row of TW
// slots after every B positions (B = 0: none).  The FP32 tiles take P = TW
// and the B for which a bank model of every stage exchange of the length's
// forward and inverse stage lists (64-bit accesses, a half-warp's distinct
// words per bank) reaches or nears the minimum wavefront count; tiles of 16
// columns are conflict-free dense.  Against the earlier P = TW + 1 layouts
// the modelled wavefronts per warp and tile fall, e.g. for the fused
// 512-point pass of 8 columns from 224 to the minimum 128 (the profile of
// that kernel counted 227 with 42% bank conflicts), for the plain 512-point
// passes of 8 columns from 512 to 288, for 1024 from 480 to 288, for 500
// from 296 to 176 and for 1800 from 840 to 568.  z passes (lanes along
// positions): row-major with pitch RP and one pad slot every B positions.
// FP64 tiles keep P = TW + 1, B = 0 (strided) and B = 16 (z).
// cap: the stage-list family (17: the plain 512-point passes' [16,16,2]).
__host__ __device__ constexpr int sl_p(int L, int TW, int es, int cap) { return es != 4 ? TW + 1 : TW; }
__host__ __device__ constexpr int sl_b(int L, int TW, int es, int cap) {
  return (es != 4 || TW >= 16) ? 0
       : L == 512 ? (cap == 17 ? 16 : 8)
       : (L == 1024 || L == 2048 || L == 4096 || L == 400) ? 16
       : L == 500 ? (TW == 8 ? 16 : 0)
       : L == 1000 ? (TW == 4 ? 32 : 0)
       : L == 1800 ? 32
       : L == 768 ? 8
       : L == 900 ? 2
       : 0;
}
// elements of a strided tile
__host__ __device__ constexpr int sl_size(int L, int TW, int es, int cap) {
  return (L - 1) * sl_p(L, TW, es, cap) + TW + (sl_b(L, TW, es, cap) ? (L - 1) / sl_b(L, TW, es, cap) * TW : 0);
}
__host__ __device__ constexpr int zl_b(int M, int es) {
  return (es == 4 && mx_list(M))
             ? (M == 250 ? 0 : M == 500 ? 100 : M == 1800 ? 60 : M == 900 ? 90 : M == 100 ? 10 : M == 1000 ? 100
                : M == 96 ? 8 : M == 192 ? 8 : M == 384 ? 16 : M == 768 ? 16 : M == 200 ? 40 : M == 400 ? 20 : 16)
             : 16;
}
__host__ __device__ constexpr int row_pitch(int M, int es) {
  return (es == 4 && mx_list(M))
             ? (M == 250 ? 265 : M == 500 ? 514 : M == 1800 ? 1836 : M == 900 ? 926 : M == 100 ? 122
                : M == 1000 ? 1012 : M == 96 ? 116 : M == 192 ? 232 : M == 384 ? 424 : M == 768 ? 817
                : M == 200 ? 218 : M == 400 ? 436 : M + M / 16 + 1)
             : M + M / 16 + 1;
}
// (Positions are never negative: unsigned division by the compile-time B
// is a plain shift or multiply-high, without the signed rounding fix-up.)
template <int P, int B, int PAD>
struct ColLayout {
  static __host__ __device__ __forceinline__ constexpr int idx(int pos, int c) {
    return pos * P + c + (B ? (int)((unsigned)pos / (unsigned)B) * PAD : 0);
  }
};
template <int RP, int B>
struct RowLayout {
  static_assert(B == 0 || RP > 0, "pitch");
  static __host__ __device__ __forceinline__ constexpr int idx(int pos, int c) {
    return c * RP + pos + (B ? (int)((unsigned)pos / (unsigned)B) : 0);
  }
};

template <int L, int E, int R>
__host__ __device__ __forceinline__ constexpr int in_pos(int t, int m, int r) {
  return t + m * (L / E) + r * (L / R);
}
template <int L, int E, int R, int NS>
__host__ __device__ __forceinline__ constexpr int out_pos(int t, int m, int r) {
  const unsigned j = (unsigned)(t + m * (L / E));
  return (int)((j / NS) * NS * R + j % NS + r * NS);
}

// Shared-memory offset of slot (m, r) of a thread's exchange accesses from
// its slot (0, 0): the writes of a stage of radix R and span NS (OUT), or
// the reads of a stage of radix R.  Layouts add the column (row) linearly,
// so the offset does not depend on it.
template <typename LY, int L, int E, int R, int NS, bool OUT>
__host__ __device__ constexpr int xoff(int t, int m, int r) {
  return OUT ? LY::idx(out_pos<L, E, R, NS>(t, m, r), 0) - LY::idx(out_pos<L, E, R, NS>(t, 0, 0), 0)
             : LY::idx(in_pos<L, E, R>(t, m, r), 0) - LY::idx(in_pos<L, E, R>(t, 0, 0), 0);
}
// True when those offsets are the same for every thread of a column (row):
// the accesses then address one base register with compile-time offsets.
template <typename LY, int L, int E, int R, int NS, bool OUT>
__host__ __device__ constexpr bool xaffine() {
  for (int t = 1; t < L / E; ++t)
    for (int m = 0; m < E / R; ++m)
      for (int r = 0; r < R; ++r)
        if (xoff<LY, L, E, R, NS, OUT>(t, m, r) != xoff<LY, L, E, R, NS, OUT>(0, m, r)) return false;
  return true;
}

// Runs stages S..end of direction DIR; v holds stage S's inputs.  Between
// stages the data goes through shared memory (layout LY).  On return v
// holds the last stage's outputs (positions out_pos of that stage).
// T: register / shared-memory type; TS: type of the twiddle table.
template <typename T, int DIR, int L, typename LY, int S, int CAP = 16, typename TS = T>
struct RRun {
  static constexpr int E = rp_elems(L, CAP);
  static constexpr int NST = rp_nst(L, CAP);
  static constexpr int R = S < NST ? rp_rad(L, DIR, S, CAP) : 1;
  static constexpr int LG = S < NST ? rp_ns(L, DIR, S, CAP) : 1;
  using Tw = StageTw<T, R, LG, L, E, tw_paired(CAP, R), TS>;
  static __device__ __forceinline__ const c2<TS> *table(const AxisPlan &p) {
    return (const c2<TS> *)p.tw + p.twoff[(DIR < 0 ? 0 : kInvBase) + S];
  }
  static __device__ __forceinline__ void run(c2<T> (&v)[E], c2<T> *buf, int t, int c, const AxisPlan &p) {
    if constexpr (S < NST) {
      Tw tw;
      if constexpr (CAP != 8) tw.load(t, table(p));
      run_with(v, buf, t, c, p, tw);
    }
  }
  // The same with stage S's twiddles already loaded: each stage of a
  // strided pass loads the next one's before the exchange barrier, so that
  // their latency overlaps the wait (fused 512-point pass at 512^3 0.356 ->
  // 0.338 ms, y passes 0.215 / 0.225 -> 0.205 / 0.210 ms).
  static __device__ __forceinline__ void run_with(c2<T> (&v)[E], c2<T> *buf, int t, int c, const AxisPlan &p,
                                                  const Tw &tw) {
    if constexpr (S < NST) {
      if constexpr (CAP == 8) rstage<T, DIR, R, LG, L, E, tw_paired(CAP, R), TS>(v, t, table(p));
      else rstage_tw<T, DIR, R, LG, L, E, tw_paired(CAP, R), TS>(v, tw);
      if constexpr (S + 1 < NST) {
        using Next = RRun<T, DIR, L, LY, S + 1, CAP, TS>;
        constexpr int R2 = Next::R;
        if constexpr (xaffine<LY, L, E, R, LG, true>()) {
          c2<T> *w = buf + LY::idx(out_pos<L, E, R, LG>(t, 0, 0), c);
#pragma unroll
          for (int m = 0; m < E / R; ++m)
#pragma unroll
            for (int r = 0; r < R; ++r) w[xoff<LY, L, E, R, LG, true>(0, m, r)] = v[m * R + r];
        } else {
#pragma unroll
          for (int m = 0; m < E / R; ++m)
#pragma unroll
            for (int r = 0; r < R; ++r) buf[LY::idx(out_pos<L, E, R, LG>(t, m, r), c)] = v[m * R + r];
        }
        typename Next::Tw nt;
        // (the z passes, CAP 8, read their twiddles in rstage as each
        // butterfly needs them: loaded beforehand they measured slower, z
        // inverse at 512^3 0.223 -> 0.253 ms)
        if constexpr (CAP != 8) nt.load(t, Next::table(p));
        __syncthreads();
        if constexpr (xaffine<LY, L, E, R2, 1, false>()) {
          const c2<T> *rd = buf + LY::idx(in_pos<L, E, R2>(t, 0, 0), c);
#pragma unroll
          for (int m = 0; m < E / R2; ++m)
#pragma unroll
            for (int r = 0; r < R2; ++r) v[m * R2 + r] = rd[xoff<LY, L, E, R2, 1, false>(0, m, r)];
        } else {
#pragma unroll
          for (int m = 0; m < E / R2; ++m)
#pragma unroll
            for (int r = 0; r < R2; ++r) v[m * R2 + r] = buf[LY::idx(in_pos<L, E, R2>(t, m, r), c)];
        }
        __syncthreads();
        Next::run_with(v, buf, t, c, p, nt);
      }
    }
  }
};

// Position of v[i] after the last stage of direction DIR.
template <int L, int DIR, int CAP = 16>
__device__ __forceinline__ int last_pos(int t, int i) {
  constexpr int S = rp_nst(L, CAP) - 1, E = rp_elems(L, CAP), R = rp_rad(L, DIR, S, CAP),
                LG = rp_ns(L, DIR, S, CAP);
  return out_pos<L, E, R, LG>(t, i / R, i % R);
}
// Position of v[i] as input of the first stage of direction DIR.
template <int L, int DIR, int CAP = 16>
__device__ __forceinline__ int first_pos(int t, int i) {
  constexpr int E = rp_elems(L, CAP), R = rp_rad(L, DIR, 0, CAP);
  return in_pos<L, E, R>(t, i / R, i % R);
}

// Resident blocks the FP32 strided tiles are compiled for: three for the
// 256-thread radix-16 tiles (35 KB tiles, 24 warps resident), two for tiles
// of 384+ threads with at most 12 values per thread (the 512-thread L = 512
// tile at 71 registers would otherwise fit once per SM: 647 vs 460 us for
// the fused pass at 512^3); others: one (two blocks of the 30-value lists
// would cap them at 128 registers, and their spills cost more than the
// occupancy gains: 63 vs 48 us at 1800).
#ifndef FFCZ_MINB16
#define FFCZ_MINB16 3
#endif
__host__ __device__ constexpr int strided_minb(int es, int nt, int E) {
  return (es == 4 && nt == 256 && E == 16) ? FFCZ_MINB16 : (es == 4 && nt >= 384 && E <= 12) ? 2 : 1;
}

// Frequency projection of the modes MODE_FCI / MODE_FCIX / MODE_FC on the
// forward result of a strided tile: thread t's values v of column c of the
// tile (batch bb, row q, first column kz0), recording clamps in fedits,
// hits in ca.fdirty and, for the all-abs box, the maximum |Re|, |Im| after
// the clamp.  SPLIT (FP64 data in float-float registers): the box decided
// in FP64.
template <typename T, int MODE, int L, int CAP, bool SPLIT, typename V>
__device__ __forceinline__ void tile_clamp(V (&v)[rp_elems(L, CAP)], int t, int c, long long bb, int q, int kz0,
                                           bool live, const SArgs &s, const ClampArgs<T> &ca,
                                           T *__restrict__ fedits, long long H) {
  using C = std::conditional_t<SPLIT, ff, T>;
  using VG = c2<T>;
  constexpr int E = rp_elems(L, CAP);
  constexpr bool ABS = MODE == MODE_FCI || MODE == MODE_FC;  // the all-abs box
  bool hit = false;
  T fm = T(0);  // max(|Re|, |Im|) after the all-abs clamp
  // SPLIT: the same as an upper bound of the float-float values,
  // |hi| + |lo| rounded up
  float fms = 0.0f;
  auto ffmag = [](const V &w) {
    if constexpr (SPLIT)
      return fmaxf(__fadd_ru(fabsf(w.x.hi), fabsf(w.x.lo)), __fadd_ru(fabsf(w.y.hi), fabsf(w.y.lo)));
    else
      return 0.0f;
  };
  // split FCI: |hi| below this is inside the box (0 when delta is too small
  // for the margin to mean anything: every coefficient decides in FP64)
  const float dlo = SPLIT ? (float)((double)ca.delta * (1.0 - 0x1p-20)) : 0.0f;
  bool any = live;
  if constexpr (ABS && !SPLIT) {
    // Branch-free look first: a thread none of whose coefficients leaves the
    // box (|Re|, |Im| <= delta; NaN compares false, as in the clamp) has
    // nothing to clamp and its maximum is that of its values; the others
    // run the per-coefficient clamp below.
    any = false;
    if (live) {
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const T ax = fabs((T)v[i].x), ay = fabs((T)v[i].y);
        any |= (ax > ca.delta) | (ay > ca.delta);
        fm = fmax(fm, fmax(ax, ay));
      }
    }
    if (any) fm = T(0);
  }
  if (any) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int l = last_pos<L, -1, CAP>(t, i);
      const long long k = ((bb * L + l) * (long long)s.Q + q) * s.Hz + kz0 + c;
      if constexpr (SPLIT) {  // the box in FP64; unclamped values keep their split form
        // hi is within 2^-23 of the value: well inside the box, nothing to
        // decide in FP64 (the pointwise box always decides in FP64)
        if (ABS && fabsf(v[i].x.hi) < dlo && fabsf(v[i].y.hi) < dlo) {
          fms = fmaxf(fms, ffmag(v[i]));
          continue;
        }
        const VG g = cvt<T>(v[i]);
        VG h;
        if (ABS) {
          h = freq_clamp<T>(g, ca.delta, fedits, k, H, hit);
        } else {
          const long long pad = (bb * L + l) * s.Wtot + (long long)q * s.Hzp + kz0 + c;
          h = freq_project<T>(g, ca, fedits, k, pad, H, hit);
        }
        if (h.x != g.x) v[i].x = C((double)h.x);
        if (h.y != g.y) v[i].y = C((double)h.y);
        if (ABS) fms = fmaxf(fms, ffmag(v[i]));
      } else if (ABS) {
        v[i] = freq_clamp<T>(v[i], ca.delta, fedits, k, H, hit);
        fm = fmax(fm, fmax(fabs((T)v[i].x), fabs((T)v[i].y)));
      } else {
        const long long pad = (bb * L + l) * s.Wtot + (long long)q * s.Hzp + kz0 + c;
        v[i] = freq_project<T>(v[i], ca, fedits, k, pad, H, hit);
      }
    }
  }
  mark_dirty(ca.fdirty, hit);
  if constexpr (ABS && !SPLIT) record_fmax(ca.fmax, fm);
  if constexpr (ABS && SPLIT) record_fmax(ca.fmax, fms);
}

// ---------------------------------------------------------------------------
// Strided C2C pass.  Block = TC threads per column x TW columns (c fastest
// across lanes, so each row access is TW contiguous complex values).
// SPLIT (FP64 data): registers and shared memory in float-float, loads,
// stores, twiddle table and clamps in FP64.
template <typename T, int MODE, int L, int LGTW, int CAP = 16, bool SPLIT = false>
__global__ void __launch_bounds__((L / rp_elems(L, CAP)) << LGTW,
                                  strided_minb(sizeof(T), (L / rp_elems(L, CAP)) << LGTW, rp_elems(L, CAP)))
    ks_strided(c2<T> *__restrict__ spec, SArgs s, AxisPlan p, ClampArgs<T> ca, T *__restrict__ fedits, long long H) {
  using C = std::conditional_t<SPLIT, ff, T>;
  using V = c2<C>;
  using VG = c2<T>;
  constexpr int E = rp_elems(L, CAP), TW = 1 << LGTW;
  using LY = ColLayout<sl_p(L, TW, sizeof(T), CAP), sl_b(L, TW, sizeof(T), CAP), TW>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  const int c = threadIdx.x & (TW - 1);
  const int t = threadIdx.x >> LGTW;
  // tile -> (batch, row, first column) in 32-bit arithmetic (a pass has
  // fewer than 2^31 tiles; a 64-bit division costs dozens of instructions)
  const unsigned tile = blockIdx.x;
  const unsigned per_b = (unsigned)s.Q * (unsigned)s.tpq;
  const unsigned bbu = tile / per_b;
  const unsigned rem = tile - bbu * per_b;
  const int q = (int)(rem / (unsigned)s.tpq);
  const int kb = (int)rem - q * s.tpq;
  const long long bb = bbu;
  const int kz0 = kb * TW;
  const bool live = c < s.Hz - kz0;
  const VG *src = spec + bb * (long long)L * s.Wtot + (long long)q * s.Hzp + kz0 + c;
  constexpr int D0 = (MODE == MODE_INV) ? +1 : -1;
  V v[E];
#pragma unroll
  for (int i = 0; i < E; ++i)
    v[i] = live ? cvt<C>(src[(long long)first_pos<L, D0, CAP>(t, i) * s.Wtot]) : mkc<C>(C(0), C(0));
  RRun<C, D0, L, LY, 0, CAP, C>::run(v, buf, t, c, p);  // split: p.tw is the float-float table
  if (MODE == MODE_FCI || MODE == MODE_FCIX || MODE == MODE_FC) {
    tile_clamp<T, MODE, L, CAP, SPLIT>(v, t, c, bb, q, kz0, live, s, ca, fedits, H);
    // The inverse's first stage reads the positions the forward's last
    // stage wrote, so the same registers continue.  A barrier separates the
    // forward's last shared reads from the inverse's first shared writes.
    if constexpr (MODE != MODE_FC) {
      __syncthreads();
      RRun<C, +1, L, LY, 0, CAP, C>::run(v, buf, t, c, p);
    }
  }
  constexpr int DL = (MODE == MODE_FWD || MODE == MODE_FC) ? -1 : +1;
  VG *dst = spec + bb * (long long)L * s.Wtot + (long long)q * s.Hzp + kz0 + c;
  if (live) {
#pragma unroll
    for (int i = 0; i < E; ++i) dst[(long long)last_pos<L, DL, CAP>(t, i) * s.Wtot] = cvt<T>(v[i]);
  }
}

// ---------------------------------------------------------------------------
// R2C along z (Nz = 2M): TC = M/E threads per row x TW rows (t fastest
// across lanes: each load is a run of consecutive complex values of one row).
template <typename T, int PRO, int M, int LGTW, bool SPLIT = false>
__global__ void __launch_bounds__((M / rp_elems(M, 8)) << LGTW) ks_zfwd(const T *__restrict__ a, const T *__restrict__ b,
                                                          T *__restrict__ sedits, T eps,
                                                          c2<T> *__restrict__ spec, ZArgs z, AxisPlan p,
                                                          const c2<T> *__restrict__ post) {
  using C = std::conditional_t<SPLIT, ff, T>;  // float-float for split FP64
  using V = c2<C>;
  using VG = c2<T>;
  constexpr int E = rp_elems(M, 8), TC = M / E;
  using LY = RowLayout<row_pitch(M, sizeof(T)), zl_b(M, sizeof(T))>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  const int t = threadIdx.x % TC;
  const int c = threadIdx.x / TC;
  const long long row = (long long)blockIdx.x * (1 << LGTW) + c;
  const bool live = row < z.rows;
  const long long rbase = row * (long long)(2 * M);
  VG g[E];  // prologue in the storage type
#pragma unroll
  for (int i = 0; i < E; ++i) {
    g[i] = mkc<T>(T(0), T(0));
    if (live) {
      const long long gi = rbase + 2 * first_pos<M, -1, 8>(t, i);
      g[i] = *reinterpret_cast<const VG *>(a + gi);
      if (PRO == PRO_DIFF) {
        const VG w = *reinterpret_cast<const VG *>(b + gi);
        g[i].x -= w.x;
        g[i].y -= w.y;
      }
    }
  }
  if (PRO == PRO_CLAMP && live) {
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const long long gi = rbase + 2 * first_pos<M, -1, 8>(t, i);
      g[i].x = spatial_clamp(g[i].x, eps, sedits, gi);
      g[i].y = spatial_clamp(g[i].y, eps, sedits, gi + 1);
    }
  }
  V v[E];
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = cvt<C>(g[i]);
  RRun<C, -1, M, LY, 0, 8, C>::run(v, buf, t, c, p);  // split: p.tw, post: float-float tables
  // Z in natural order to shared memory, then the real-to-complex split of
  // row c: X[k] = (Z[k] + conj Z[M-k])/2 - i W^k (Z[k] - conj Z[M-k])/2.
  if (rp_nst(M, 8) > 1) __syncthreads();
#pragma unroll
  for (int i = 0; i < E; ++i) buf[LY::idx(last_pos<M, -1, 8>(t, i), c)] = v[i];
  __syncthreads();
  if (!live) return;
  VG *out = spec + row * (long long)z.Hzp;
  for (int k = t; k <= M; k += TC) {
    const int k1 = (k == M) ? 0 : k;
    const int k2 = (k == 0) ? 0 : M - k;
    const V A = buf[LY::idx(k1, c)];
    const V B = cconj(buf[LY::idx(k2, c)]);
    const V w = reinterpret_cast<const V *>(post)[k];
    const V sm = cadd(A, B);
    const V d = csub(A, B);
    const V tt = cmul(mkc<C>(-w.y, w.x), d);
    V X;
    X.x = C(0.5) * (sm.x - tt.x);
    X.y = C(0.5) * (sm.y - tt.y);
    out[k] = cvt<T>(X);
  }
}

// C2R along z (Nz = 2M) + normalisation + violation max.  Each thread reads
// X[k] and X[M-k] for its first-stage positions straight from global memory
// (the row is read by the block, so the second read mostly hits L1) and
// forms Z[k] = (X[k] + conj X[M-k]) + i W^-k (X[k] - conj X[M-k]) in
// registers (imaginary parts of X[0] and X[M] ignored).
template <typename T, int M, int LGTW, bool SPLIT = false>
__global__ void __launch_bounds__((M / rp_elems(M, 8)) << LGTW) ks_zinv(const c2<T> *__restrict__ spec, T *__restrict__ e,
                                                          T eps, T factor, LoopCtl *ctl, double *zpart,
                                                          ZArgs z, AxisPlan p, const c2<T> *__restrict__ post) {
  using C = std::conditional_t<SPLIT, ff, T>;  // float-float for split FP64
  using V = c2<C>;
  using VG = c2<T>;
  constexpr int E = rp_elems(M, 8), TC = M / E;
  static_assert(2 * E <= ZS_TERMS, "a thread sums at most ZS_TERMS squares in T");
  using LY = RowLayout<row_pitch(M, sizeof(T)), zl_b(M, sizeof(T))>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  const int t = threadIdx.x % TC;
  const int c = threadIdx.x / TC;
  const long long row = (long long)blockIdx.x * (1 << LGTW) + c;
  const bool live = row < z.rows;
  const VG *in = spec + row * (long long)z.Hzp;
  V v[E];
  if (live) {
    V xa[E], xb[E];
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int k = first_pos<M, +1, 8>(t, i);
      xa[i] = cvt<C>(in[k]);
      xb[i] = cvt<C>(in[M - k]);
    }
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const int k = first_pos<M, +1, 8>(t, i);
      if (k == 0) {
        v[i] = mkc<C>(xa[i].x + xb[i].x, xa[i].x - xb[i].x);
      } else {
        const V w = reinterpret_cast<const V *>(post)[k];
        const V s1 = cadd(xa[i], cconj(xb[i]));
        const V d1 = csub(xa[i], cconj(xb[i]));
        v[i] = cadd(s1, cmul(mkc<C>(w.y, w.x), d1));
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = mkc<C>(C(0), C(0));
  }
  RRun<C, +1, M, LY, 0, 8, C>::run(v, buf, t, c, p);
  T amax = T(0), ssq = T(0);
  if constexpr (SPLIT) {
    // no statistics (they would need FP64 arithmetic on every value): a sum
    // that is not a number tells the strict finish to make its own pass
    T vmax = T(0);
    if (live) {
      // float-float normalisation; the violation in FP64 only where an FP32
      // look at hi cannot rule it out (|o| <= |hi|(1 + 2^-23) < eps below elo)
      T *out = e + row * (long long)(2 * M);
      const C F = cvt<C>(mkc<T>(factor, T(0))).x;
      const float elo = (float)((double)eps * (1.0 - 0x1p-20));
#pragma unroll
      for (int i = 0; i < E; ++i) {
        V w;
        w.x = v[i].x * F;
        w.y = v[i].y * F;
        const VG o = cvt<T>(w);
        *reinterpret_cast<VG *>(out + 2 * last_pos<M, +1, 8>(t, i)) = o;
        if (fabsf(w.x.hi) >= elo) {
          const T a0 = fabs(o.x);
          if (a0 > eps) vmax = max(vmax, a0 - eps);
        }
        if (fabsf(w.y.hi) >= elo) {
          const T a1 = fabs(o.y);
          if (a1 > eps) vmax = max(vmax, a1 - eps);
        }
      }
    }
    block_stats_to_ctl<T, true>(T(0), __longlong_as_double(0x7ff8000000000000ll), eps, ctl, zpart, vmax);
  } else if (live) {
    T *out = e + row * (long long)(2 * M);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const VG u = cvt<T>(v[i]);
      VG o;
      o.x = u.x * factor;
      o.y = u.y * factor;
      *reinterpret_cast<VG *>(out + 2 * last_pos<M, +1, 8>(t, i)) = o;
      zs_note<T>(o.x, amax, ssq);
      zs_note<T>(o.y, amax, ssq);
    }
  }
  if constexpr (!SPLIT) block_stats_to_ctl<T>(amax, ssq, eps, ctl, zpart);
}

}  // namespace ffcz
