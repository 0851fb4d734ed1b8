// Compile-time-sized pass kernels for power-of-two axis lengths.
//
// Same kernels, arguments, layouts and arithmetic as passes.cuh, with the
// axis length L, the tile width TW and the block size NT fixed at compile
// time, so that:
//   * the stage sequence (radix 8 stages, then one radix 4 or 2 stage, the
//     factorisation fft_plan.cpp uses) is unrolled, with shifts in place of
//     the divisions by the sub-transform span;
//   * each block needs no register-heavy radix switch (fewer registers,
//     more resident blocks per SM);
//   * every thread issues all of its global loads before its first shared
//     store, so a tile's loads are in flight together.
// The twiddle table offsets still come from the runtime AxisPlan.
#pragma once

#include "passes.cuh"

namespace ffcz {

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// Radix of stage s for L = 2^lg: 8, 8, ..., then 4 or 2 for the remainder.
__host__ __device__ constexpr int p2_nst(int lg) { return lg / 3 + (lg % 3 ? 1 : 0); }
__host__ __device__ constexpr int p2_radix(int lg, int s) { return s < lg / 3 ? 8 : (lg % 3 == 2 ? 4 : 2); }
__host__ __device__ constexpr int p2_lgns(int lg, int s) { return 3 * (s < lg / 3 ? s : lg / 3); }

template <typename T, int DIR, int R, int LGNS, int L, int LGTW, int NT>
__device__ __forceinline__ void sstage(c2<T> *buf, const c2<T> *__restrict__ tw, int tid) {
  using V = c2<T>;
  constexpr int TW = 1 << LGTW, P = TW + 1, M = L / R, NITEMS = M * TW;
  constexpr int K = (NITEMS + NT - 1) / NT;
  constexpr int NS = 1 << LGNS;
  V v[K][R];
#pragma unroll
  for (int kk = 0; kk < K; ++kk) {
    const int item = tid + kk * NT;
    if (NITEMS % NT == 0 || item < NITEMS) {
      const int j = item >> LGTW;
      const int c = item & (TW - 1);
#pragma unroll
      for (int r = 0; r < R; ++r) v[kk][r] = buf[(j + r * M) * P + c];
      if (NS > 1) {
        const int k = j & (NS - 1);
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
    const int item = tid + kk * NT;
    if (NITEMS % NT == 0 || item < NITEMS) {
      const int j = item >> LGTW;
      const int c = item & (TW - 1);
      const int base = ((j >> LGNS) << (LGNS + ilog2(R))) + (j & (NS - 1));
#pragma unroll
      for (int r = 0; r < R; ++r) buf[(base + r * NS) * P + c] = v[kk][r];
    }
  }
  __syncthreads();
}

template <typename T, int DIR, int L, int LGTW, int NT, int S>
struct SFft {
  static __device__ __forceinline__ void run(c2<T> *buf, const AxisPlan &p, int tid) {
    constexpr int lg = ilog2(L);
    if constexpr (S < p2_nst(lg)) {
      sstage<T, DIR, p2_radix(lg, S), p2_lgns(lg, S), L, LGTW, NT>(buf, (const c2<T> *)p.tw + p.twoff[S], tid);
      SFft<T, DIR, L, LGTW, NT, S + 1>::run(buf, p, tid);
    }
  }
};

template <typename T, int DIR, int L, int LGTW, int NT>
__device__ __forceinline__ void sfft(c2<T> *buf, const AxisPlan &p, int tid) {
  SFft<T, DIR, L, LGTW, NT, 0>::run(buf, p, tid);
}

// ---------------------------------------------------------------------------
// R2C along z (even Nz = 2M, M = 2^k) for TW rows; see k_zfwd.
template <typename T, int PRO, int M, int LGTW, int NT>
__global__ void __launch_bounds__(NT) ks_zfwd(const T *__restrict__ a, const T *__restrict__ b,
                                             T *__restrict__ sedits, T eps, c2<T> *__restrict__ spec, ZArgs z,
                                             AxisPlan p, const c2<T> *__restrict__ post) {
  using V = c2<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  constexpr int TW = 1 << LGTW, P = TW + 1, LGM = ilog2(M);
  constexpr int NLD = M * TW, KLD = (NLD + NT - 1) / NT;
  const int tid = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * TW;
  const int nrows = (int)min((long long)TW, z.rows - row0);
  V v[KLD];
#pragma unroll
  for (int kk = 0; kk < KLD; ++kk) {
    const int it = tid + kk * NT;
    const int c = it >> LGM, n = it & (M - 1);
    v[kk] = mkc<T>(T(0), T(0));
    if ((NLD % NT == 0 || it < NLD) && c < nrows) {
      const long long gi = (row0 + c) * (long long)(2 * M) + 2 * n;
      v[kk] = *reinterpret_cast<const V *>(a + gi);
      if (PRO == PRO_DIFF) {
        const V w = *reinterpret_cast<const V *>(b + gi);
        v[kk].x -= w.x;
        v[kk].y -= w.y;
      }
    }
  }
#pragma unroll
  for (int kk = 0; kk < KLD; ++kk) {
    const int it = tid + kk * NT;
    const int c = it >> LGM, n = it & (M - 1);
    if (NLD % NT == 0 || it < NLD) {
      if (PRO == PRO_CLAMP && c < nrows) {
        const long long gi = (row0 + c) * (long long)(2 * M) + 2 * n;
        v[kk].x = spatial_clamp(v[kk].x, eps, sedits, gi);
        v[kk].y = spatial_clamp(v[kk].y, eps, sedits, gi + 1);
      }
      buf[n * P + c] = v[kk];
    }
  }
  __syncthreads();
  sfft<T, -1, M, LGTW, NT>(buf, p, tid);
  constexpr int HZ = M + 1;
  constexpr int NST = HZ * TW, KST = (NST + NT - 1) / NT;
#pragma unroll
  for (int kk = 0; kk < KST; ++kk) {
    const int it = tid + kk * NT;
    if (it >= NST) break;
    const int c = it / HZ;
    const int k = it - c * HZ;
    if (c >= nrows) continue;
    const int k1 = (k == M) ? 0 : k;
    const int k2 = (k == 0) ? 0 : M - k;
    const V A = buf[k1 * P + c];
    const V B = cconj(buf[k2 * P + c]);
    const V w = post[k];
    const V s = cadd(A, B);
    const V d = csub(A, B);
    const V t = cmul(mkc<T>(-w.y, w.x), d);
    V X;
    X.x = T(0.5) * (s.x - t.x);
    X.y = T(0.5) * (s.y - t.y);
    spec[(row0 + c) * (long long)z.Hzp + k] = X;
  }
}

// C2R along z (even Nz = 2M) for TW rows + 1/N + violation; see k_zinv.
template <typename T, int M, int LGTW, int NT>
__global__ void __launch_bounds__(NT) ks_zinv(const c2<T> *__restrict__ spec, T *__restrict__ e, T eps, T factor,
                                             LoopCtl *ctl, ZArgs z, AxisPlan p, const c2<T> *__restrict__ post) {
  using V = c2<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  constexpr int TW = 1 << LGTW, P = TW + 1, LGM = ilog2(M), HZ = M + 1;
  const int tid = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * TW;
  const int nrows = (int)min((long long)TW, z.rows - row0);
  {
    constexpr int NLD = HZ * TW, KLD = (NLD + NT - 1) / NT;
    V v[KLD];
#pragma unroll
    for (int kk = 0; kk < KLD; ++kk) {
      const int it = tid + kk * NT;
      const int c = it / HZ;
      const int k = it - c * HZ;
      v[kk] = mkc<T>(T(0), T(0));
      if (it < NLD && c < nrows) v[kk] = spec[(row0 + c) * (long long)z.Hzp + k];
    }
#pragma unroll
    for (int kk = 0; kk < KLD; ++kk) {
      const int it = tid + kk * NT;
      const int c = it / HZ;
      const int k = it - c * HZ;
      if (it < NLD) buf[k * P + c] = v[kk];
    }
  }
  __syncthreads();
  {
    constexpr int HALF = M / 2;
    constexpr int NPR = (HALF + 1) * TW, KPR = (NPR + NT - 1) / NT;
#pragma unroll
    for (int kk = 0; kk < KPR; ++kk) {
      const int it = tid + kk * NT;
      if (it >= NPR) break;
      const int c = it / (HALF + 1);
      const int k = it - c * (HALF + 1);
      if (k == 0) {
        const T x0 = buf[c].x, xm = buf[M * P + c].x;
        buf[c] = mkc<T>(x0 + xm, x0 - xm);
      } else {
        const int km = M - k;
        const V Xk = buf[k * P + c];
        const V Xm = buf[km * P + c];
        const V w = post[k];
        const V s1 = cadd(Xk, cconj(Xm));
        const V d1 = csub(Xk, cconj(Xm));
        const V t1 = cmul(mkc<T>(w.y, w.x), d1);
        buf[k * P + c] = cadd(s1, t1);
        if (km != k) {
          const V s2 = cadd(Xm, cconj(Xk));
          const V d2 = csub(Xm, cconj(Xk));
          const V t2 = cmul(mkc<T>(-w.y, w.x), d2);
          buf[km * P + c] = csub(s2, t2);
        }
      }
    }
  }
  __syncthreads();
  sfft<T, +1, M, LGTW, NT>(buf, p, tid);
  T vmax = T(0);
  constexpr int NST = M * TW, KST = (NST + NT - 1) / NT;
#pragma unroll
  for (int kk = 0; kk < KST; ++kk) {
    const int it = tid + kk * NT;
    const int c = it >> LGM, n = it & (M - 1);
    if ((NST % NT == 0 || it < NST) && c < nrows) {
      const V v = buf[n * P + c];
      V o;
      o.x = v.x * factor;
      o.y = v.y * factor;
      *reinterpret_cast<V *>(e + (row0 + c) * (long long)(2 * M) + 2 * n) = o;
      const T a0 = fabs(o.x), a1 = fabs(o.y);
      if (a0 > eps) vmax = max(vmax, a0 - eps);
      if (a1 > eps) vmax = max(vmax, a1 - eps);
    }
  }
  block_max_to_ctl<T>(vmax, ctl);
}

// C2C along a strided axis of length L for TW columns; see k_strided.
template <typename T, int MODE, int L, int LGTW, int NT>
__global__ void __launch_bounds__(NT) ks_strided(c2<T> *__restrict__ spec, SArgs s, AxisPlan p, T delta,
                                                T *__restrict__ fedits, long long H) {
  using V = c2<T>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V *buf = reinterpret_cast<V *>(smem_raw);
  constexpr int TW = 1 << LGTW, P = TW + 1, N = L * TW, K = (N + NT - 1) / NT;
  const int tid = threadIdx.x;
  const long long tile = blockIdx.x;
  const long long per_b = (long long)s.Q * s.tpq;
  const long long bb = tile / per_b;
  const int rem = (int)(tile - bb * per_b);
  const int q = rem / s.tpq;
  const int kb = rem - q * s.tpq;
  const int kz0 = kb * TW;
  const int ncol = min(TW, s.Hz - kz0);
  const long long base = bb * (long long)L * s.Wtot + (long long)q * s.Hzp + kz0;
  {
    V v[K];
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int it = tid + kk * NT;
      const int l = it >> LGTW, c = it & (TW - 1);
      v[kk] = mkc<T>(T(0), T(0));
      if ((N % NT == 0 || it < N) && c < ncol) v[kk] = spec[base + (long long)l * s.Wtot + c];
    }
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int it = tid + kk * NT;
      if (N % NT == 0 || it < N) buf[(it >> LGTW) * P + (it & (TW - 1))] = v[kk];
    }
  }
  __syncthreads();
  if (MODE == MODE_INV) sfft<T, +1, L, LGTW, NT>(buf, p, tid);
  else sfft<T, -1, L, LGTW, NT>(buf, p, tid);
  if (MODE == MODE_FCI) {
#pragma unroll
    for (int kk = 0; kk < K; ++kk) {
      const int it = tid + kk * NT;
      const int l = it >> LGTW, c = it & (TW - 1);
      if ((N % NT == 0 || it < N) && c < ncol) {
        const long long k = ((bb * L + l) * (long long)s.Q + q) * s.Hz + kz0 + c;
        buf[l * P + c] = freq_clamp<T>(buf[l * P + c], delta, fedits, k, H);
      }
    }
    __syncthreads();
    sfft<T, +1, L, LGTW, NT>(buf, p, tid);
  }
#pragma unroll
  for (int kk = 0; kk < K; ++kk) {
    const int it = tid + kk * NT;
    const int l = it >> LGTW, c = it & (TW - 1);
    if ((N % NT == 0 || it < N) && c < ncol) spec[base + (long long)l * s.Wtot + c] = buf[l * P + c];
  }
}

}  // namespace ffcz
