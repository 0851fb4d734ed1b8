// Strided C2C passes with TMA-staged tiles (FP32): a persistent variant of
// ks_strided whose tiles arrive in shared memory by tensor-map copies that
// are issued several tiles ahead, so that HBM reads of the next tiles run
// while the current tile is transformed.
//
// ks_strided loads its tile straight into registers: while a block computes,
// it has nothing in flight, and the passes that carry the most arithmetic
// per byte (the fused forward + clamp + inverse pass) stall on memory
// latency at the occupancy their registers allow.  Here each block owns
// NBUF tile slots.  Thread 0 issues the copies of tile i + NBUF into the
// slot tile i used, as soon as every thread is done with that slot; the
// other slots' copies are in flight meanwhile.  A tile is one box per 256
// (or fewer) positions of a rank-4 tensor map over the padded spectrum
//   (kz: Hz columns, q: Q rows, position: L, batch: B),
// TW columns wide; columns past Hz are zero-filled by the copy (the register
// kernel zeroes them too).  The staged tile is dense (position * TW + c);
// the first stage reads its inputs from it, the stage exchanges reuse the
// slot in the padded layout of ks_strided, the last stage stores straight
// to HBM.  Stage lists, twiddles, butterflies, clamps and the order of
// every operation are those of ks_strided, so both give identical bits.
//
// A wait for a tile that does not arrive within about two seconds sets
// *err and ends the block (every thread of the block decides together).
#pragma once

#include "passes_static.cuh"
#include "tma.cuh"

namespace ffcz {

// Boxes per tile: the fewest that split the L positions evenly into boxes
// of at most 256 positions (a box dimension's limit) whose TW-column rows
// fill whole 128-byte lines, so that every box lands on a 128-byte
// boundary of shared memory, as tensor copies require; 0 if none does.
__host__ __device__ constexpr int pipe_nbox(int L, int TW, int k = 1) {
  return k > L ? 0 : (L % k == 0 && L / k <= 256 && (L / k) * TW % 16 == 0) ? k : pipe_nbox(L, TW, k + 1);
}
// Bytes of one tile slot: the larger of the exchange layout and the dense
// staged tile, rounded up to 128 bytes.
__host__ __device__ constexpr size_t pipe_slot_bytes(int L, int TW, int cap) {
  return ((size_t)(sl_size(L, TW, 4, cap) > L * TW ? sl_size(L, TW, 4, cap) : L * TW) * 8 + 127) / 128 * 128;
}
// Dynamic shared memory: the slots, their barriers, alignment slack.
__host__ __device__ constexpr size_t pipe_smem_bytes(int L, int TW, int cap, int NBUF) {
  return NBUF * pipe_slot_bytes(L, TW, cap) + 64 + 128;
}
// Slots per block: three where MINB blocks of three fit an SM's 228 KB
// (1 KB of it reserved per block), else two; 0 when two do not fit.
__host__ __device__ constexpr int pipe_nbuf(int L, int TW, int cap, int MINB) {
  return pipe_smem_bytes(L, TW, cap, 3) + 1024 <= (size_t)228 * 1024 / MINB ? 3
       : pipe_smem_bytes(L, TW, cap, 2) + 1024 <= (size_t)228 * 1024 / MINB ? 2
       : pipe_smem_bytes(L, TW, cap, 2) <= (size_t)227 * 1024 ? 2 : 0;
}

template <int MODE, int L, int LGTW, int CAP, int NBUF, int MINB>
__global__ void __launch_bounds__((L / rp_elems(L, CAP)) << LGTW, MINB)
    ks_strided_pipe(const __grid_constant__ CUtensorMap tm, c2<float> *__restrict__ spec, SArgs s, AxisPlan p,
                    ClampArgs<float> ca, float *__restrict__ fedits, long long H, long long ntiles, int *err) {
  using T = float;
  using V = c2<float>;
  constexpr int E = rp_elems(L, CAP), TW = 1 << LGTW;
  constexpr int NBOX = pipe_nbox(L, TW), BOX = NBOX ? L / NBOX : 1;
  constexpr unsigned TILE_BYTES = (unsigned)L * TW * sizeof(V);
  constexpr size_t SLOT = pipe_slot_bytes(L, TW, CAP);
  static_assert(NBUF >= 2, "at least two tile slots");
  static_assert(LGTW >= 1, "a box row must be a multiple of 16 bytes");
  static_assert(NBOX > 0 && SLOT % 128 == 0 && (BOX * TW * sizeof(V)) % 128 == 0,
                "every box must start on a 128-byte boundary of shared memory");
  using LY = ColLayout<sl_p(L, TW, 4, CAP), sl_b(L, TW, 4, CAP), TW>;
  extern __shared__ __align__(128) unsigned char pipe_smem[];
  unsigned char *base = pipe_smem + ((128u - (smem_u32(pipe_smem) & 127u)) & 127u);
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + NBUF * SLOT);
  const int tid = threadIdx.x;
  const int c = tid & (TW - 1);
  const int t = tid >> LGTW;
  // tile -> (batch, row, first column): the order of ks_strided's blocks,
  // in 32-bit arithmetic (a pass has fewer than 2^31 tiles)
  const unsigned per_b = (unsigned)s.Q * (unsigned)s.tpq;
  const unsigned nt32 = (unsigned)ntiles;
  auto coords = [&](unsigned tile, long long &bb, int &q, int &kz0) {
    const unsigned b = tile / per_b;
    const unsigned rem = tile - b * per_b;
    bb = b;
    q = (int)(rem / (unsigned)s.tpq);
    kz0 = ((int)rem - q * s.tpq) * TW;
  };
  auto issue = [&](unsigned tile, int slot) {
    long long bb;
    int q, kz0;
    coords(tile, bb, q, kz0);
    const uint32_t dst = smem_u32(base + slot * SLOT), mb = smem_u32(bar + slot);
    mbar_expect_tx(mb, TILE_BYTES);
#pragma unroll
    for (int k = 0; k < NBOX; ++k)
      tma_load_4d(dst + (uint32_t)(k * BOX * TW * sizeof(V)), &tm, kz0, q, k * BOX, (int)bb, mb);
  };
  if (tid == 0) {
    prefetch_tmap(&tm);
#pragma unroll
    for (int b = 0; b < NBUF; ++b) mbar_init(smem_u32(bar + b), 1);
    fence_mbar_init();
#pragma unroll
    for (int b = 0; b < NBUF; ++b) {
      const unsigned tile = blockIdx.x + (unsigned)b * gridDim.x;
      if (tile < nt32) issue(tile, b);
    }
  }
  __syncthreads();
  constexpr int D0 = (MODE == MODE_INV) ? +1 : -1;
  constexpr int DL = (MODE == MODE_FWD || MODE == MODE_FC) ? -1 : +1;
  for (unsigned i = 0;; ++i) {
    const unsigned tile = blockIdx.x + i * gridDim.x;
    if (tile >= nt32) break;
    const int slot = (int)(i % NBUF);
    const unsigned parity = (i / NBUF) & 1u;
    V *buf = reinterpret_cast<V *>(base + slot * SLOT);
    long long bb;
    int q, kz0;
    coords(tile, bb, q, kz0);
    const bool live = c < s.Hz - kz0;
    const bool ok = mbar_wait_bounded(smem_u32(bar + slot), parity);
    V v[E];
    if (ok) {
#pragma unroll
      for (int j = 0; j < E; ++j) v[j] = buf[first_pos<L, D0, CAP>(t, j) * TW + c];
    }
    // every thread has read the staged tile before the exchanges overwrite it
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(err, 1);
        // let the copies still in flight land (again with a limit) before
        // the block's shared memory is released
        for (int k = 0; k < NBUF; ++k) {
          const unsigned ii = i + k;
          if (blockIdx.x + ii * gridDim.x < nt32) mbar_wait_bounded(smem_u32(bar + (int)(ii % NBUF)), (ii / NBUF) & 1u);
        }
      }
      return;
    }
    RRun<T, D0, L, LY, 0, CAP, T>::run(v, buf, t, c, p);
    if (MODE == MODE_FCI || MODE == MODE_FCIX || MODE == MODE_FC) {
      tile_clamp<T, MODE, L, CAP, false>(v, t, c, bb, q, kz0, live, s, ca, fedits, H);
      if constexpr (MODE != MODE_FC) {
        __syncthreads();
        RRun<T, +1, L, LY, 0, CAP, T>::run(v, buf, t, c, p);
      }
    }
    // The slot is free once every thread is past its last access; the
    // proxy fence orders those accesses before the next copy into it.
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      const unsigned nt = tile + (unsigned)NBUF * gridDim.x;
      if (nt < nt32) issue(nt, slot);
    }
    V *dst = spec + bb * (long long)L * s.Wtot + (long long)q * s.Hzp + kz0 + c;
    if (live) {
#pragma unroll
      for (int j = 0; j < E; ++j) dst[(long long)last_pos<L, DL, CAP>(t, j) * s.Wtot] = v[j];
    }
  }
}

}  // namespace ffcz
