// Device FFT engine: mixed-radix Stockham autosort transforms over a tile
// of TW independent columns held in shared memory.
//
// Tile layout: element l (0 <= l < L) of column c (0 <= c < TW) lives at
// buf[l*P + c] with an odd pitch P = TW + 1, so that both the column-wise
// global<->shared copies and the butterfly reads/writes of a half warp hit
// distinct banks.  Each stage reads R strided elements of one column into
// registers, applies the stage twiddles, runs a radix-R butterfly and, after
// a barrier, writes the results to their autosorted positions (in place).
// Work item = (butterfly j, column c) with c fastest, so a warp's accesses
// are contiguous in shared memory.
#pragma once

#include "common.cuh"
#include "fft_plan.h"

namespace ffcz {

// cos / sin of 2*pi*j/R for j = 1..(R-1)/2 (literals, folded at compile time
// once the butterfly loops are unrolled).
__host__ __device__ __forceinline__ constexpr double root_cos(int R, int j) {
  return R == 3 ? -0.5
       : R == 5 ? (j == 1 ? 0.30901699437494745 : -0.8090169943749473)
       : R == 7 ? (j == 1 ? 0.6234898018587336 : j == 2 ? -0.22252093395631434 : -0.900968867902419)
       : R == 11 ? (j == 1 ? 0.8412535328311812 : j == 2 ? 0.41541501300188644 : j == 3 ? -0.142314838273285
                    : j == 4 ? -0.654860733945285 : -0.9594929736144974)
       : (j == 1 ? 0.8854560256532099 : j == 2 ? 0.5680647467311559 : j == 3 ? 0.120536680255323
          : j == 4 ? -0.35460488704253545 : j == 5 ? -0.7485107481711012 : -0.970941817426052);
}
__host__ __device__ __forceinline__ constexpr double root_sin(int R, int j) {
  return R == 3 ? 0.8660254037844386
       : R == 5 ? (j == 1 ? 0.9510565162951535 : 0.5877852522924732)
       : R == 7 ? (j == 1 ? 0.7818314824680298 : j == 2 ? 0.9749279121818236 : 0.43388373911755823)
       : R == 11 ? (j == 1 ? 0.5406408174555976 : j == 2 ? 0.9096319953545183 : j == 3 ? 0.9898214418809328
                    : j == 4 ? 0.7557495743542583 : 0.28173255684142967)
       : (j == 1 ? 0.4647231720437685 : j == 2 ? 0.8229838658936564 : j == 3 ? 0.992708874098054
          : j == 4 ? 0.9350162426854148 : j == 5 ? 0.6631226582407952 : 0.23931566428755768);
}

// ---------------------------------------------------------------------------
// Butterflies.  DIR = -1: forward, y_k = sum_n v_n exp(-2*pi*i*n*k/R);
// DIR = +1: inverse (unnormalised).  In place on v[0..R-1].
template <int DIR, typename V>
__device__ __forceinline__ void bfly2(V &a, V &b) {
  V t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int DIR, typename V>
__device__ __forceinline__ void bfly4(V &a0, V &a1, V &a2, V &a3) {
  V t0 = cadd(a0, a2), t1 = csub(a0, a2);
  V t2 = cadd(a1, a3), t3 = cmul_i<DIR>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <int R, int DIR, typename V> struct Dft;

template <int DIR, typename V> struct Dft<2, DIR, V> {
  __device__ __forceinline__ static void run(V *v) { bfly2<DIR>(v[0], v[1]); }
};
template <int DIR, typename V> struct Dft<4, DIR, V> {
  __device__ __forceinline__ static void run(V *v) { bfly4<DIR>(v[0], v[1], v[2], v[3]); }
};
template <int DIR, typename V> struct Dft<8, DIR, V> {
  __device__ __forceinline__ static void run(V *v) {
    using S = decltype(v[0].x);
    const S h = S(0.7071067811865476);
    V a0 = cadd(v[0], v[4]), b0 = csub(v[0], v[4]);
    V a1 = cadd(v[1], v[5]), b1 = csub(v[1], v[5]);
    V a2 = cadd(v[2], v[6]), b2 = csub(v[2], v[6]);
    V a3 = cadd(v[3], v[7]), b3 = csub(v[3], v[7]);
    // b_r *= w8^r, w8 = exp(DIR*2*pi*i/8)
    V t;
    if (DIR < 0) {
      t.x = (b1.x + b1.y) * h; t.y = (b1.y - b1.x) * h; b1 = t;
      t.x = (b3.y - b3.x) * h; t.y = -(b3.x + b3.y) * h; b3 = t;
    } else {
      t.x = (b1.x - b1.y) * h; t.y = (b1.x + b1.y) * h; b1 = t;
      t.x = -(b3.x + b3.y) * h; t.y = (b3.x - b3.y) * h; b3 = t;
    }
    b2 = cmul_i<DIR>(b2);
    bfly4<DIR>(a0, a1, a2, a3);
    bfly4<DIR>(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
  }
};
// Odd radices: y_k = A_k + (-/+ i) B_k, y_{R-k} = A_k - (-/+ i) B_k with
// A_k = v0 + sum_m cos(2 pi m k/R) (v_m + v_{R-m}),
// B_k = sum_m sin(2 pi m k/R) (v_m - v_{R-m}).
template <int R, int DIR, typename V> struct Dft {
  static_assert(R % 2 == 1, "odd radix");
  __device__ __forceinline__ static void run(V *v) {
    using S = decltype(v[0].x);
    constexpr int H = (R - 1) / 2;
    V p[H], q[H];
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      p[m - 1] = cadd(v[m], v[R - m]);
      q[m - 1] = csub(v[m], v[R - m]);
    }
    V y0 = v[0];
#pragma unroll
    for (int m = 0; m < H; ++m) y0 = cadd(y0, p[m]);
    V out[R];
    out[0] = y0;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      V A = v[0];
      V B;
      B.x = S(0);
      B.y = S(0);
#pragma unroll
      for (int m = 1; m <= H; ++m) {
        const int j = (m * k) % R;
        const S c = (j <= H) ? S(root_cos(R, j)) : S(root_cos(R, R - j));
        const S s = (j <= H) ? S(root_sin(R, j)) : -S(root_sin(R, R - j));
        A.x += c * p[m - 1].x;
        A.y += c * p[m - 1].y;
        B.x += s * q[m - 1].x;
        B.y += s * q[m - 1].y;
      }
      V iB = cmul_i<DIR>(B);
      out[k] = cadd(A, iB);
      out[R - k] = csub(A, iB);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = out[k];
  }
};

// ---------------------------------------------------------------------------
// One Stockham stage of radix R over the tile.  EPT = elements per thread
// the caller sized the block for (nthr >= L*TW/EPT).
template <typename T, int DIR, int R, int EPT>
__device__ __forceinline__ void fft_stage(c2<T> *buf, int L, int P, int log2TW, int Ns,
                                          const c2<T> *__restrict__ tw, int tid, int nthr) {
  using V = c2<T>;
  constexpr int K = (EPT + R - 1) / R;
  const int TW = 1 << log2TW;
  const int m = L / R;
  const int nitems = m << log2TW;
  V v[K][R];
  int jj[K];
#pragma unroll
  for (int kk = 0; kk < K; ++kk) {
    const int item = tid + kk * nthr;
    jj[kk] = -1;
    if (item < nitems) {
      const int j = item >> log2TW;
      const int c = item & (TW - 1);
      jj[kk] = j;
#pragma unroll
      for (int r = 0; r < R; ++r) v[kk][r] = buf[(j + r * m) * P + c];
      if (Ns > 1) {
        const int k = j % Ns;
        const V *t = tw + k * (R - 1);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const V w = t[r - 1];
          v[kk][r] = (DIR < 0) ? cmul(v[kk][r], w) : cmulc(v[kk][r], w);
        }
      }
      Dft<R, DIR, V>::run(v[kk]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int kk = 0; kk < K; ++kk) {
    if (jj[kk] >= 0) {
      const int item = tid + kk * nthr;
      const int c = item & (TW - 1);
      const int j = jj[kk];
      const int q = j / Ns;
      const int base = q * Ns * R + (j - q * Ns);
#pragma unroll
      for (int r = 0; r < R; ++r) buf[(base + r * Ns) * P + c] = v[kk][r];
    }
  }
  __syncthreads();
}

// Generic stage for a prime radix R > 7: each work item produces one output
// y[r] = sum_t v[t] w^(t k) roots[(t r) mod R] of butterfly j directly from
// shared memory (O(R) reads per output), held in registers until the
// barrier, then stored in place.
template <typename T, int DIR, int EPT>
__device__ __noinline__ void fft_stage_generic(c2<T> *buf, int L, int P, int log2TW, int R, int Ns,
                                               const c2<T> *__restrict__ tw,
                                               const c2<T> *__restrict__ roots, int tid, int nthr) {
  using V = c2<T>;
  const int TW = 1 << log2TW;
  const int m = L / R;
  const int nitems = L << log2TW;
  V out[EPT];
#pragma unroll
  for (int kk = 0; kk < EPT; ++kk) {
    const int item = tid + kk * nthr;
    if (item < nitems) {
      const int o = item >> log2TW;
      const int c = item & (TW - 1);
      const int q0 = o / (Ns * R);
      const int rem = o - q0 * Ns * R;
      const int r = rem / Ns;
      const int k = rem - r * Ns;
      const int j = q0 * Ns + k;
      V acc;
      acc.x = T(0);
      acc.y = T(0);
      int tr = 0;  // (t*r) mod R
      for (int t = 0; t < R; ++t) {
        V v = buf[(j + t * m) * P + c];
        if (t > 0 && Ns > 1) {
          const V w = tw[k * (R - 1) + t - 1];
          v = (DIR < 0) ? cmul(v, w) : cmulc(v, w);
        }
        const V w2 = roots[tr];
        const V u = (DIR < 0) ? cmul(v, w2) : cmulc(v, w2);
        acc.x += u.x;
        acc.y += u.y;
        tr += r;
        if (tr >= R) tr -= R;
      }
      out[kk] = acc;
    }
  }
  __syncthreads();
#pragma unroll
  for (int kk = 0; kk < EPT; ++kk) {
    const int item = tid + kk * nthr;
    if (item < nitems) buf[(item >> log2TW) * P + (item & (TW - 1))] = out[kk];
  }
  __syncthreads();
}

// Full transform of length p.L along the tile (all stages).  Must be called
// by all threads of the block; returns after a barrier.
template <typename T, int DIR, int EPT>
__device__ __forceinline__ void fft_tile(c2<T> *buf, const AxisPlan &p, int P, int log2TW, int tid,
                                         int nthr) {
  const c2<T> *tw = (const c2<T> *)p.tw;
  for (int s = 0; s < p.nst; ++s) {
    const int R = p.R[s];
    const int Ns = p.Ns[s];
    const c2<T> *t = tw + p.twoff[s];
    switch (R) {
      case 8: fft_stage<T, DIR, 8, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      case 4: fft_stage<T, DIR, 4, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      case 2: fft_stage<T, DIR, 2, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      case 3: fft_stage<T, DIR, 3, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      case 5: fft_stage<T, DIR, 5, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      case 7: fft_stage<T, DIR, 7, EPT>(buf, p.L, P, log2TW, Ns, t, tid, nthr); break;
      default:
        fft_stage_generic<T, DIR, EPT>(buf, p.L, P, log2TW, R, Ns, t, tw + p.rootoff[s], tid, nthr);
        break;
    }
  }
}

}  // namespace ffcz
