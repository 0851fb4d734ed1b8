// Kernels of one alternating-projection iteration (FP32 / FP64).
//
// Spectrum layout in HBM: rows (ix,iy) of the half spectrum, row pitch Hzp
// (Hz = Nz/2+1 rounded up to 128 bytes) so that every tile of TW columns
// starts on a 128-byte line.  The frequency edit accumulator keeps the
// reference's planar, unpadded layout and flat index
// k = (ix*Ny + iy)*Hz + kz (projection_algorithm.cu:148-188).
//
// Passes of a 3D iteration (x, y, z axes non-trivial):
//   k_zfwd    : [prologue] + R2C along z            R N*s   W 2H*s
//   k_strided : C2C forward along y                 R 2H*s  W 2H*s
//   k_strided : C2C fwd along x + clamp + C2C inv   R 2H*s  W 2H*s (+ sparse edits)
//   k_strided : C2C inverse along y                 R 2H*s  W 2H*s
//   k_zinv    : C2R along z + 1/N + violation max   R 2H*s  W N*s
// The prologue of k_zfwd is either nothing, e0 = x' - x, or the spatial
// clamp of the previous iteration (projection_algorithm.cu:336-361), which
// is applied to the values as they are loaded: the clamped e is only ever
// consumed by this transform, so it is not written back.
#pragma once

#include "common.cuh"
#include "fft_engine.cuh"

namespace ffcz {

enum { PRO_PLAIN = 0, PRO_DIFF = 1, PRO_CLAMP = 2 };
// MODE_FCI: fused forward / all-abs clamp / inverse; MODE_FCIX: the same
// with the other constraint modes (a kernel of its own, so that the all-abs
// kernel keeps the code and registers of a plain clamp).  MODE_FC: forward
// with the all-abs clamp in its epilogue, stored to HBM (the plain form's
// last forward pass; the inverse is a MODE_INV pass of its own).
enum { MODE_FWD = 0, MODE_INV = 1, MODE_FCI = 2, MODE_FCIX = 3, MODE_FC = 4 };
constexpr int kStridedModes = 5;

struct ZArgs {
  long long rows;  // Nx*Ny
  int Nz, M, even, Hz, Hzp;
  int TW, log2TW, P;
};

struct SArgs {
  int L;           // axis length
  int Q;           // rows (q) of Hzp columns between consecutive l
  int Hz, Hzp;
  long long Wtot;  // Q*Hzp: element stride between consecutive l
  int TW, log2TW, P;
  int tpq;         // tiles per q row = ceil(Hz/TW)
};

// Spatial box (projection_algorithm.cu:347-360) on one value.
template <typename T>
__device__ __forceinline__ T spatial_clamp(T v, T eps, T *__restrict__ sedits, long long i) {
  if (v > eps) {
    sedits[i] += eps - v;
    v = eps;
  } else if (v < -eps) {
    sedits[i] += -eps - v;
    v = -eps;
  }
  return v;
}

// Frequency box (projection_algorithm.cu:160-187) on one coefficient.  A
// clamp also sets `hit`; the caller publishes it once per warp with
// mark_dirty (the accumulator is no longer all zeros, so its compaction has
// to read it).
template <typename T>
__device__ __forceinline__ c2<T> freq_clamp(c2<T> v, T delta, T *__restrict__ fedits, long long k,
                                            long long H, bool &hit) {
  T re = v.x;
  if (re > delta) {
    fedits[k] += delta - re;
    v.x = delta;
    hit = true;
  } else if (re < -delta) {
    fedits[k] += -delta - re;
    v.x = -delta;
    hit = true;
  }
  T im = v.y;
  if (im > delta) {
    fedits[k + H] += delta - im;
    v.y = delta;
    hit = true;
  } else if (im < -delta) {
    fedits[k + H] += -delta - im;
    v.y = -delta;
    hit = true;
  }
  return v;
}

// One store per warp at most (the first lane that clamped, and only while
// the flag still reads 0): many clamps must not serialise on one address.
__device__ __forceinline__ void mark_dirty(unsigned *dirty, bool hit) {
  const unsigned m = __ballot_sync(__activemask(), hit);
  if (hit && dirty && (int)(threadIdx.x & 31) == __ffs(m) - 1 && *dirty == 0u) *dirty = 1u;
}

// Publishes the active lanes' max(|Re|, |Im|) once per warp: the FP32 bits
// of a non-negative value order like the value, so one warp reduction and
// one atomicMax of the first active lane.  m is rounded up to FP32.
__device__ __forceinline__ void record_fmax(unsigned *dst, float m) {
  const unsigned act = __activemask();
  const unsigned b = __reduce_max_sync(act, __float_as_uint(m));
  if (dst && (int)(threadIdx.x & 31) == __ffs(act) - 1) atomicMax(dst, b);
}
__device__ __forceinline__ void record_fmax(unsigned *dst, double m) { record_fmax(dst, __double2float_ru(m)); }

// Frequency projection of every constraint mode, applied where the forward
// transform's last pass holds coefficient k (flat index) at padded offset p:
//   CLAMP_ABS    all coefficients, +-delta (projection_algorithm.cu:148-188)
//   CLAMP_DIRECT +-bound[k], +inf where unconstrained (:93-145)
//   CLAMP_PTW    pointwise power-spectrum box against the spectrum of x
//                (:191-333): coefficient 0 by the DC rule, the others (mask
//                null = all) clamped to +-cd when |orig+err|^2/|orig|^2
//                leaves [sqrt(1-d), sqrt(1+d)].
enum { CLAMP_ABS = 0, CLAMP_DIRECT = 1, CLAMP_PTW = 2 };

template <typename T>
struct ClampArgs {
  int mode = CLAMP_ABS;
  int dc = 0;                          // PTW: apply the DC rule at k = 0
  T delta = T(0);                      // ABS
  const T *bound = nullptr;            // DIRECT: H bounds
  const c2<T> *orig = nullptr;         // PTW: spectrum of x, padded layout
  const unsigned char *mask = nullptr; // PTW: constrained coefficients
  T sp = T(0), sm = T(0), lo = T(0), hi = T(0), cd = T(0);  // PTW constants
  unsigned *fdirty = nullptr;          // set when a frequency edit is written
  // all-abs clamp: receives max(|Re|, |Im|) of the clamped coefficients
  // (FP32 bits of the value rounded up, atomicMax); null: not recorded
  unsigned *fmax = nullptr;
};

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__device__ __forceinline__ c2<T> freq_project(c2<T> v, const ClampArgs<T> &ca, T *__restrict__ fedits, long long k,
                                              long long p, long long H, bool &hit) {
  if (ca.mode == CLAMP_ABS) return freq_clamp<T>(v, ca.delta, fedits, k, H, hit);
  if (ca.mode == CLAMP_DIRECT) return freq_clamp<T>(v, ca.bound[k], fedits, k, H, hit);
  if (k == 0) {
    if (ca.dc) {
      const T o = ca.orig[0].x;
      const T lower = mul_rn(o, ca.lo), upper = mul_rn(o, ca.hi);
      if (v.x > upper || v.x < lower) {
        fedits[0] += -v.x;
        v.x = T(0);
        hit = true;
      }
    }
    return v;
  }
  if (ca.mask && !ca.mask[k]) return v;
  const c2<T> o = ca.orig[p];
  const T om = add_rn(mul_rn(o.x, o.x), mul_rn(o.y, o.y));
  const T cx = add_rn(o.x, v.x), cy = add_rn(o.y, v.y);
  const T cm = add_rn(mul_rn(cx, cx), mul_rn(cy, cy));
  const T ratio = cm / om;
  if (ratio <= ca.sp && ratio >= ca.sm) return v;
  return freq_clamp<T>(v, ca.cd, fedits, k, H, hit);
}

// ---------------------------------------------------------------------------
// R2C along z for TW consecutive rows.  Even Nz: the row is read as M = Nz/2
// complex values z[n] = x[2n] + i x[2n+1], transformed with length M, and
// split: X[k] = (Z[k] + conj Z[M-k])/2 - i W^k (Z[k] - conj Z[M-k])/2,
// W = exp(-2 pi i/Nz), k = 0..M.  Odd Nz: full-length complex transform of
// the real row.
template <typename T, int PRO, int EPT>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_zfwd(const T *__restrict__ a, const T *__restrict__ b,
                                              T *__restrict__ sedits, T eps,
                                              c2<T> *__restrict__ spec, ZArgs z, AxisPlan p,
                                              const c2<T> *__restrict__ post) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  c2<T> *buf = reinterpret_cast<c2<T> *>(smem_raw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long long row0 = (long long)blockIdx.x * z.TW;
  const int nrows = (int)min((long long)z.TW, z.rows - row0);
  const int P = z.P;
  if (z.even) {
    const int M = z.M;
    const int total = M * z.TW;
    for (int it = tid; it < total; it += nthr) {
      const int c = it / M;
      const int n = it - c * M;
      c2<T> v = mkc<T>(T(0), T(0));
      if (c < nrows) {
        const long long gi = (row0 + c) * (long long)z.Nz + 2 * n;
        v = *reinterpret_cast<const c2<T> *>(a + gi);
        if (PRO == PRO_DIFF) {
          const c2<T> w = *reinterpret_cast<const c2<T> *>(b + gi);
          v.x -= w.x;
          v.y -= w.y;
        } else if (PRO == PRO_CLAMP) {
          v.x = spatial_clamp(v.x, eps, sedits, gi);
          v.y = spatial_clamp(v.y, eps, sedits, gi + 1);
        }
      }
      buf[n * P + c] = v;
    }
  } else {
    const int L = z.Nz;
    const int total = L * z.TW;
    for (int it = tid; it < total; it += nthr) {
      const int c = it / L;
      const int n = it - c * L;
      T v = T(0);
      if (c < nrows) {
        const long long gi = (row0 + c) * (long long)z.Nz + n;
        v = a[gi];
        if (PRO == PRO_DIFF) v -= b[gi];
        else if (PRO == PRO_CLAMP) v = spatial_clamp(v, eps, sedits, gi);
      }
      buf[n * P + c] = mkc<T>(v, T(0));
    }
  }
  __syncthreads();
  fft_tile<T, -1, EPT>(buf, p, P, z.log2TW, tid, nthr);
  const int Hz = z.Hz;
  const int total = Hz * z.TW;
  if (z.even) {
    const int M = z.M;
    for (int it = tid; it < total; it += nthr) {
      const int c = it / Hz;
      const int k = it - c * Hz;
      if (c >= nrows) continue;
      const int k1 = (k == M) ? 0 : k;
      const int k2 = (k == 0) ? 0 : M - k;
      const c2<T> A = buf[k1 * P + c];
      const c2<T> B = cconj(buf[k2 * P + c]);
      const c2<T> w = post[k];
      const c2<T> s = cadd(A, B);
      const c2<T> d = csub(A, B);
      const c2<T> iw = mkc<T>(-w.y, w.x);  // i * W^k
      const c2<T> t = cmul(iw, d);
      c2<T> X;
      X.x = T(0.5) * (s.x - t.x);
      X.y = T(0.5) * (s.y - t.y);
      spec[(row0 + c) * (long long)z.Hzp + k] = X;
    }
  } else {
    for (int it = tid; it < total; it += nthr) {
      const int c = it / Hz;
      const int k = it - c * Hz;
      if (c >= nrows) continue;
      spec[(row0 + c) * (long long)z.Hzp + k] = buf[k * P + c];
    }
  }
}

// ---------------------------------------------------------------------------
// Statistics of the e that a z-inverse pass writes, for the strict finish
// after a loop that converged (its last pass wrote the final e): per block
// its sum of squares and its max |e| (zpart[2 block + 0, 1]; no atomics on
// one address).  The sum runs in T over at most ZS_TERMS values per thread,
// then over the warp's five-level tree (or in FP64 past ZS_TERMS values),
// then in FP64.
constexpr int ZS_TERMS = 64;

// One output value of a z-inverse pass: |v| into the running max and its
// square into the running sum (one max with an |.| operand and one FMA).
template <typename T>
__device__ __forceinline__ void zs_note(T v, T &amax, T &ssq) {
  amax = fmax(amax, fabs(v));
  ssq = fma(v, v, ssq);
}

// Block-wide reductions of a z-inverse pass: the violation max(|e|-eps, 0)
// to ctl->viol_bits (atomicMax of the bits, only by blocks that have one;
// the violation of the largest |e| is the largest violation, rounding being
// monotonic), the block's sum of squares and max |e| to zpart.  The sum
// runs in Q (T: the warps' five-level trees in T, then FP64 over the warps
// in a fixed order, so that FP32 data keeps the FP64 pipe to a few
// operations per block).  HAS_V: the caller also passes a violation of its
// own (vmax), folded in with the one of amax.
template <typename T, bool HAS_V = false, typename Q>
__device__ __forceinline__ void block_stats_to_ctl(T amax, Q qt, T eps, LoopCtl *ctl, double *zpart,
                                                   T vmax = T(0)) {
  __shared__ T ra[32], rv[HAS_V ? 32 : 1];
  __shared__ double rq[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(0xffffffffu, amax, o);
    amax = w > amax ? w : amax;
    qt += __shfl_xor_sync(0xffffffffu, qt, o);
    if constexpr (HAS_V) {
      const T u = __shfl_xor_sync(0xffffffffu, vmax, o);
      vmax = u > vmax ? u : vmax;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    ra[warp] = amax;
    rq[warp] = (double)qt;
    if constexpr (HAS_V) rv[warp] = vmax;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    amax = lane < nw ? ra[lane] : T(0);
    double q = lane < nw ? rq[lane] : 0.0;
    if constexpr (HAS_V) vmax = lane < nw ? rv[lane] : T(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T w = __shfl_xor_sync(0xffffffffu, amax, o);
      amax = w > amax ? w : amax;
      q += __shfl_xor_sync(0xffffffffu, q, o);
      if constexpr (HAS_V) {
        const T u = __shfl_xor_sync(0xffffffffu, vmax, o);
        vmax = u > vmax ? u : vmax;
      }
    }
    if (lane == 0) {
      if (amax > eps) vmax = max(vmax, amax - eps);
      if (vmax > T(0)) atomicMax(&ctl->viol_bits, to_bits<T>(vmax));
      zpart[2 * blockIdx.x] = q;
      zpart[2 * blockIdx.x + 1] = (double)amax;
    }
  }
}

// C2R along z for TW rows, times the normalisation factor
// (projection_algorithm_impl.cuh:241-247), and the violation
// max(|e|-eps, 0) (projection_algorithm.cu:586-594).  Even Nz: from X[k],
// k = 0..M (imaginary parts of X[0] and X[M] ignored, as a C2R of a
// Hermitian spectrum does), Z[k] = (X[k] + conj X[M-k])
// + i W^-k (X[k] - conj X[M-k]); z = IFFT_M(Z); e[2n] = Re z[n], e[2n+1] =
// Im z[n].  Odd Nz: Hermitian extension to length Nz, inverse transform,
// real part.
template <typename T, int EPT>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_zinv(const c2<T> *__restrict__ spec, T *__restrict__ e,
                                              T eps, T factor, LoopCtl *ctl, double *zpart, ZArgs z,
                                              AxisPlan p, const c2<T> *__restrict__ post) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  c2<T> *buf = reinterpret_cast<c2<T> *>(smem_raw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long long row0 = (long long)blockIdx.x * z.TW;
  const int nrows = (int)min((long long)z.TW, z.rows - row0);
  const int P = z.P;
  const int Hz = z.Hz;
  {
    const int total = Hz * z.TW;
    for (int it = tid; it < total; it += nthr) {
      const int c = it / Hz;
      const int k = it - c * Hz;
      c2<T> v = mkc<T>(T(0), T(0));
      if (c < nrows) v = spec[(row0 + c) * (long long)z.Hzp + k];
      buf[k * P + c] = v;
    }
  }
  __syncthreads();
  if (z.even) {
    const int M = z.M;
    const int half = M / 2;  // pairs (k, M-k), k = 0..half
    const int total = (half + 1) * z.TW;
    for (int it = tid; it < total; it += nthr) {
      const int c = it / (half + 1);
      const int k = it - c * (half + 1);
      if (k == 0) {
        const T x0 = buf[c].x, xm = buf[M * P + c].x;
        buf[c] = mkc<T>(x0 + xm, x0 - xm);
      } else {
        const int km = M - k;
        const c2<T> Xk = buf[k * P + c];
        const c2<T> Xm = buf[km * P + c];
        const c2<T> w = post[k];  // W^k
        // Z[k]   = (Xk + conj Xm) + i W^-k (Xk - conj Xm)
        const c2<T> s1 = cadd(Xk, cconj(Xm));
        const c2<T> d1 = csub(Xk, cconj(Xm));
        const c2<T> t1 = cmul(mkc<T>(w.y, w.x), d1);  // i*conj(W^k) = (wy, wx)
        buf[k * P + c] = cadd(s1, t1);
        if (km != k) {
          // Z[M-k] = (Xm + conj Xk) - i W^k (Xm - conj Xk)
          const c2<T> s2 = cadd(Xm, cconj(Xk));
          const c2<T> d2 = csub(Xm, cconj(Xk));
          const c2<T> t2 = cmul(mkc<T>(-w.y, w.x), d2);  // i*W^k
          buf[km * P + c] = csub(s2, t2);
        }
      }
    }
    __syncthreads();
    fft_tile<T, +1, EPT>(buf, p, P, z.log2TW, tid, nthr);
    T amax = T(0), ssq = T(0);
    double dsq = 0.0;
    int terms = 0;
    const int tot2 = M * z.TW;
    for (int it = tid; it < tot2; it += nthr) {
      const int c = it / M;
      const int n = it - c * M;
      if (c >= nrows) continue;
      const c2<T> v = buf[n * P + c];
      c2<T> o;
      o.x = v.x * factor;
      o.y = v.y * factor;
      const long long i = (row0 + c) * (long long)z.Nz + 2 * n;
      *reinterpret_cast<c2<T> *>(e + i) = o;
      zs_note<T>(o.x, amax, ssq);
      zs_note<T>(o.y, amax, ssq);
      if ((terms += 2) == ZS_TERMS) {
        dsq += (double)ssq;
        ssq = T(0);
        terms = 0;
      }
    }
    block_stats_to_ctl<T>(amax, dsq + (double)ssq, eps, ctl, zpart);
  } else {
    const int L = z.Nz;
    // Hermitian extension: rows Hz..L-1 from conj of rows L-Hz+1..1.
    const int ext = L - Hz;
    for (int it = tid; it < ext * z.TW; it += nthr) {
      const int c = it / ext;
      const int k = Hz + (it - c * ext);
      buf[k * P + c] = cconj(buf[(L - k) * P + c]);
    }
    __syncthreads();
    for (int c = tid; c < z.TW; c += nthr) buf[c].y = T(0);
    __syncthreads();
    fft_tile<T, +1, EPT>(buf, p, P, z.log2TW, tid, nthr);
    T amax = T(0), ssq = T(0);
    double dsq = 0.0;
    int terms = 0;
    for (int it = tid; it < L * z.TW; it += nthr) {
      const int c = it / L;
      const int n = it - c * L;
      if (c >= nrows) continue;
      const T o = buf[n * P + c].x * factor;
      const long long i = (row0 + c) * (long long)z.Nz + n;
      e[i] = o;
      zs_note<T>(o, amax, ssq);
      if (++terms == ZS_TERMS) {
        dsq += (double)ssq;
        ssq = T(0);
        terms = 0;
      }
    }
    block_stats_to_ctl<T>(amax, dsq + (double)ssq, eps, ctl, zpart);
  }
}

// ---------------------------------------------------------------------------
// C2C transform along one strided axis for a tile of TW columns.  Element
// (b, l, q, kz) lives at spec[b*L*Wtot + l*Wtot + q*Hzp + kz].
// MODE_FCI: forward, frequency clamp with edit accumulation, inverse.
template <typename T, int MODE, int EPT>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 512 : 256) k_strided(c2<T> *__restrict__ spec, SArgs s, AxisPlan p,
                                                 ClampArgs<T> ca, T *__restrict__ fedits, long long H) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  c2<T> *buf = reinterpret_cast<c2<T> *>(smem_raw);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const long long tile = blockIdx.x;
  const long long per_b = (long long)s.Q * s.tpq;
  const long long bb = tile / per_b;
  const int rem = (int)(tile - bb * per_b);
  const int q = rem / s.tpq;
  const int kb = rem - q * s.tpq;
  const int kz0 = kb * s.TW;
  const int ncol = min(s.TW, s.Hz - kz0);
  const long long base = bb * (long long)s.L * s.Wtot + (long long)q * s.Hzp + kz0;
  const int TW = s.TW, P = s.P, lg = s.log2TW;
  const int total = s.L << lg;
  for (int it = tid; it < total; it += nthr) {
    const int l = it >> lg;
    const int c = it & (TW - 1);
    c2<T> v = mkc<T>(T(0), T(0));
    if (c < ncol) v = spec[base + (long long)l * s.Wtot + c];
    buf[l * P + c] = v;
  }
  __syncthreads();
  if (MODE == MODE_INV) {
    fft_tile<T, +1, EPT>(buf, p, P, lg, tid, nthr);
  } else {
    fft_tile<T, -1, EPT>(buf, p, P, lg, tid, nthr);
  }
  if (MODE == MODE_FCI || MODE == MODE_FCIX || MODE == MODE_FC) {
    bool hit = false;
    double fm = 0.0;
    for (int it = tid; it < total; it += nthr) {
      const int l = it >> lg;
      const int c = it & (TW - 1);
      if (c < ncol) {
        const long long k = ((bb * s.L + l) * (long long)s.Q + q) * s.Hz + kz0 + c;
        if (MODE == MODE_FCI || MODE == MODE_FC) {
          const c2<T> w = freq_clamp<T>(buf[l * P + c], ca.delta, fedits, k, H, hit);
          buf[l * P + c] = w;
          fm = fmax(fm, (double)fmax(fabs(w.x), fabs(w.y)));
        } else {
          buf[l * P + c] =
              freq_project<T>(buf[l * P + c], ca, fedits, k, base + (long long)l * s.Wtot + c, H, hit);
        }
      }
    }
    mark_dirty(ca.fdirty, hit);
    if (MODE != MODE_FCIX) record_fmax(ca.fmax, fm);
    __syncthreads();
    if (MODE != MODE_FC) fft_tile<T, +1, EPT>(buf, p, P, lg, tid, nthr);
  }
  for (int it = tid; it < total; it += nthr) {
    const int l = it >> lg;
    const int c = it & (TW - 1);
    if (c < ncol) spec[base + (long long)l * s.Wtot + c] = buf[l * P + c];
  }
}

// Frequency box over the whole half spectrum when no strided axis exists
// (Nx = Ny = 1).
template <typename T>
__global__ void k_clamp_freq(c2<T> *__restrict__ spec, long long rows, int Hz, int Hzp, ClampArgs<T> ca,
                             T *__restrict__ fedits, long long H) {
  const long long total = rows * Hz;
  bool hit = false;
  double fm = 0.0;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total;
       it += (long long)gridDim.x * blockDim.x) {
    const long long r = it / Hz;
    const int kz = (int)(it - r * Hz);
    c2<T> *ptr = spec + r * Hzp + kz;
    const c2<T> w = freq_project<T>(*ptr, ca, fedits, it, r * Hzp + kz, H, hit);
    *ptr = w;
    fm = fmax(fm, (double)fmax(fabs(w.x), fabs(w.y)));
  }
  mark_dirty(ca.fdirty, hit);
  if (ca.mode == CLAMP_ABS) record_fmax(ca.fmax, fm);
}

// ---------------------------------------------------------------------------
static __global__ void k_init_ctl(LoopCtl *ctl) {
  ctl->fmax_cur = 0u;
  ctl->fmax_last = 0u;
  ctl->viol_bits = 0ull;
  ctl->last_viol = 0.0;
  ctl->iterations = 0;
  ctl->converged = 0;
  ctl->cont = 1;
  ctl->err = 0;
}

// End of one iteration (projection_algorithm_impl.cuh:841-848): records the
// metric, counts the iteration, decides whether the loop goes on and, inside
// a graph, sets the WHILE condition.
template <typename T>
__global__ void k_check(LoopCtl *ctl, T tol, int max_iter, cudaGraphConditionalHandle h,
                        int use_graph, unsigned *sdirty) {
  const T v = from_bits<T>(ctl->viol_bits);
  ctl->viol_bits = 0ull;
  ctl->fmax_last = ctl->fmax_cur;
  ctl->fmax_cur = 0u;
  ctl->last_viol = (double)v;
  const int it = ctl->iterations + 1;
  ctl->iterations = it;
  const int conv = (v < tol) ? 1 : 0;
  ctl->converged = conv;
  const int cont = (!conv && it < max_iter) ? 1 : 0;
  ctl->cont = cont;
  // the next iteration's prologue clamps every |e| > eps: spatial edits
  if (cont && v > T(0)) *sdirty = 1u;
  if (use_graph) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// Iteration count of a solve made of several loop runs (strict re-runs).
static __global__ void k_set_iterations(LoopCtl *ctl, int n) { ctl->iterations = n; }

// Spatial projection after the last iteration when the loop stopped without
// converging (projection_algorithm_impl.cuh:851 on the final pass); with ctl
// NULL, on every element (the strict-bounds clamp).
template <typename T>
__global__ void k_final_clamp(T *__restrict__ e, T *__restrict__ sedits, T eps, long long n,
                              const LoopCtl *ctl, unsigned *sdirty) {
  if (ctl && (ctl->converged || ctl->iterations == 0)) return;  // ctl NULL: always
  if (blockIdx.x == 0 && threadIdx.x == 0 && (!ctl || ctl->last_viol > 0.0)) *sdirty = 1u;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const T v = e[i];
    if (v > eps || v < -eps) e[i] = spatial_clamp(v, eps, sedits, i);
  }
}

// e = a (- b): materialises e0 when no iteration runs.
template <typename T>
__global__ void k_set_e(T *__restrict__ e, const T *__restrict__ a, const T *__restrict__ b,
                        long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    e[i] = b ? a[i] - b[i] : a[i];
}

}  // namespace ffcz
