// Allocation-free variant of the edit compaction (the work ffcz_extract does
// for one accumulator): flags, whole-array min/max, scan, scatter, uint16
// quantisation and flag pack, for callers that cannot allocate device memory.
//
// Who cannot allocate: applications that reserve the GPU's memory up front
// in their own pool and forbid further device allocations (a cudaMalloc
// there fails or fragments the pool), and latency-bound pipelines in which
// the implicit device-wide synchronisation of cudaMalloc/cudaFree would
// stall work on other streams.  This entry point therefore takes all its
// inputs and outputs from the caller and keeps its scratch (per-block
// counts, minima, maxima and the result words) in the fixed array below,
// which every GPU that loads the library holds until the process exits.
//
// Set-up: every call resolves the array's device address on the current
// device with cudaGetSymbolAddress (host code cannot use the array's name as
// a device address).  Resolving it per call, rather than caching it per
// device index, keeps the address right when the caller destroys and
// re-creates the device's primary context (cudaDeviceReset reloads the
// module, which moves the array); the lookup is negligible next to the
// stream synchronisation every call ends with.  The first call on a device
// may load the library's device code, so make it before any stream capture
// starts.
//
// Sharing: all calls on a device use the same array and it keeps the last
// call's contents.  Every scratch word a call reads is written earlier in
// the same call, so nothing needs clearing, but calls whose work overlaps
// on the GPU (different streams or host threads without ordering) race on
// the array and give wrong results.
#include "extract.cuh"

namespace ffcz {

constexpr size_t kNoallocMaxBlocks = FFCZ_NOALLOC_MAX_ELEMS / EX_CHUNK;  // 16384
constexpr size_t kScratchCnt = 0;                                          // u32[blocks]
constexpr size_t kScratchMn = kScratchCnt + kNoallocMaxBlocks * 4;          // f64[blocks]
constexpr size_t kScratchMx = kScratchMn + kNoallocMaxBlocks * 8;           // f64[blocks]
constexpr size_t kScratchMnMx = kScratchMx + kNoallocMaxBlocks * 8;         // f64[2]
constexpr size_t kScratchCtl = kScratchMnMx + 256;                          // LoopCtl
constexpr size_t kScratchBytes = kScratchCtl + ((sizeof(LoopCtl) + 255) / 256) * 256;
static_assert(kScratchBytes == FFCZ_NOALLOC_SCRATCH_BYTES, "scratch size in ffcz.h is stale");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Device address of the scratch array on the current device and context.
int scratch_for_current_device(unsigned char **out) {
  void *p = nullptr;
  FFCZ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  *out = (unsigned char *)p;
  return FFCZ_OK;
}

template <typename T>
int run(const T *a, size_t n, T *compact, uint16_t *quant, uint8_t *pack, int pack_mode, cudaStream_t st,
        unsigned char *scr, size_t *count, double *mn, double *mx) {
  const size_t nblk = ceil_div(n, (size_t)EX_CHUNK);
  unsigned *blk_cnt = (unsigned *)(scr + kScratchCnt);
  T *blk_mn = (T *)(scr + kScratchMn);
  T *blk_mx = (T *)(scr + kScratchMx);
  T *mnmx = (T *)(scr + kScratchMnMx);
  LoopCtl *ctl = (LoopCtl *)(scr + kScratchCtl);
  const T thr = T(1e-7);
  const size_t pack_bytes = ceil_div(n, (size_t)32) * 4;
  k_ex_stats<T><<<(unsigned)nblk, EX_THREADS, 0, st>>>(a, (long long)n, thr, blk_cnt, blk_mn, blk_mx);
  k_ex_scan<T><<<1, 1024, 0, st>>>(blk_cnt, (long long)nblk, blk_mn, blk_mx, mnmx, ctl, 0);
  k_ex_compact<T><<<(unsigned)nblk, EX_THREADS, 0, st>>>(a, (long long)n, thr, blk_cnt, mnmx, compact, quant,
                                                         (unsigned *)pack, pack_mode == FFCZ_PACK_CORRECT);
  FFCZ_CUDA(cudaGetLastError());
  unsigned long long h_count = 0;
  double h_mm[2] = {0, 0};
  FFCZ_CUDA(cudaMemcpyAsync(&h_count, &ctl->count[0], sizeof(h_count), cudaMemcpyDeviceToHost, st));
  FFCZ_CUDA(cudaMemcpyAsync(&h_mm[0], &ctl->mn[0], sizeof(double), cudaMemcpyDeviceToHost, st));
  FFCZ_CUDA(cudaMemcpyAsync(&h_mm[1], &ctl->mx[0], sizeof(double), cudaMemcpyDeviceToHost, st));
  FFCZ_CUDA(cudaStreamSynchronize(st));
  if (pack_mode == FFCZ_PACK_REFERENCE) {
    // The reference packs only a non-empty stream (impl:429-449).
    if (h_count) {
      const unsigned g = (unsigned)std::min<size_t>(ceil_div(pack_bytes, 256), 152 * 16);
      k_pack_reference<T><<<g, 256, 0, st>>>(a, (long long)n, thr, pack, (long long)pack_bytes);
    } else {
      FFCZ_CUDA(cudaMemsetAsync(pack, 0, pack_bytes, st));
    }
    FFCZ_CUDA(cudaGetLastError());
    FFCZ_CUDA(cudaStreamSynchronize(st));
  }
  *count = (size_t)h_count;
  if (mn) *mn = h_mm[0];
  if (mx) *mx = h_mm[1];
  return FFCZ_OK;
}

}  // namespace
}  // namespace ffcz

using namespace ffcz;

extern "C" int ffcz_compact_quantize_noalloc(const void *d_edits, size_t n, int dtype, void *d_compact,
                                             uint16_t *d_quant, uint8_t *d_pack, int pack_mode, void *stream,
                                             size_t *count, double *min_edit, double *max_edit) {
  if (!d_edits || !d_compact || !d_quant || !d_pack || !count)
    return fail(FFCZ_ERR_INVALID, "NULL argument");
  if (dtype != FFCZ_F32 && dtype != FFCZ_F64) return fail(FFCZ_ERR_INVALID, "dtype must be FFCZ_F32 or FFCZ_F64");
  if (pack_mode != FFCZ_PACK_CORRECT && pack_mode != FFCZ_PACK_REFERENCE)
    return fail(FFCZ_ERR_INVALID, "unknown pack mode");
  if (n == 0) return fail(FFCZ_ERR_EMPTY, "empty edit array");
  if (n > (size_t)FFCZ_NOALLOC_MAX_ELEMS)
    return fail(FFCZ_ERR_CAPACITY, "ffcz_compact_quantize_noalloc: n = " + std::to_string(n) +
                                       " exceeds the fixed scratch limit of " +
                                       std::to_string((size_t)FFCZ_NOALLOC_MAX_ELEMS) + " elements");
  // The kernels read d_edits with 16-byte vector loads, write the flag pack
  // as 32-bit words and the compact values and codes as whole elements; a
  // misaligned pointer is rejected here instead of faulting on the device.
  if (((uintptr_t)d_edits) & 15) return fail(FFCZ_ERR_INVALID, "d_edits must be 16-byte aligned");
  if (((uintptr_t)d_compact) & (dtype == FFCZ_F32 ? 3 : 7))
    return fail(FFCZ_ERR_INVALID, "d_compact must be aligned to its element size");
  if (((uintptr_t)d_quant) & 1) return fail(FFCZ_ERR_INVALID, "d_quant must be 2-byte aligned");
  if (((uintptr_t)d_pack) & 3) return fail(FFCZ_ERR_INVALID, "d_pack must be 4-byte aligned");
  unsigned char *scr = nullptr;
  FFCZ_TRY(scratch_for_current_device(&scr));
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == FFCZ_F32)
    return run<float>((const float *)d_edits, n, (float *)d_compact, d_quant, d_pack, pack_mode, st, scr, count,
                      min_edit, max_edit);
  return run<double>((const double *)d_edits, n, (double *)d_compact, d_quant, d_pack, pack_mode, st, scr, count,
                     min_edit, max_edit);
}
