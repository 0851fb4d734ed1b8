// Launches every kernel projection_algorithm.cuh declares (and the host
// compact_and_quantize_active_elements) on seeded inputs, for float and
// double, and writes each output array to a record file.  The same source
// is compiled twice: against the reference's own header and
// projection_algorithm.cu (the fixture tests/golden/ref_legacy_kernels.npz
// comes from that build run on a GPU), and against this repository's
// include/ with libffcz.so (tests/test_gpu_legacy_kernels.py compares the
// two outputs bit for bit).
//
//   legacy_kernels_driver <out.bin>
//
// Record: u32 name length, name, u32 element bytes, u64 byte count, bytes.
// Inputs avoid the reference's races: constraint indices are distinct, so
// every atomicAdd lands on its own accumulator entry.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "projection_algorithm.cuh"

namespace {

FILE *g_out = nullptr;

#define DCHECK(call)                                                                       \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_));           \
      exit(2);                                                                             \
    }                                                                                      \
  } while (0)

struct Rng {  // xorshift64*: the same inputs on every machine
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 1) {}
  double uniform() {  // [-1, 1)
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    const uint64_t r = s * 0x2545F4914F6CDD1Dull;
    return (double)(r >> 11) * (1.0 / 4503599627370496.0) - 1.0;
  }
};

void record(const std::string &name, const void *host, size_t bytes, uint32_t elem) {
  const uint32_t n = (uint32_t)name.size();
  const uint64_t b = bytes;
  fwrite(&n, 4, 1, g_out);
  fwrite(name.data(), 1, n, g_out);
  fwrite(&elem, 4, 1, g_out);
  fwrite(&b, 8, 1, g_out);
  fwrite(host, 1, bytes, g_out);
}

template <typename V>
void record_dev(const std::string &name, const V *dev, size_t count) {
  std::vector<V> h(count);
  DCHECK(cudaMemcpy(h.data(), dev, count * sizeof(V), cudaMemcpyDeviceToHost));
  record(name, h.data(), count * sizeof(V), (uint32_t)sizeof(V));
}

template <typename V>
V *upload(const std::vector<V> &h) {
  V *d = nullptr;
  DCHECK(cudaMalloc(&d, h.size() * sizeof(V) + 16));
  DCHECK(cudaMemcpy(d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice));
  return d;
}

template <typename T>
std::vector<T> randv(Rng &r, size_t n, double scale) {
  std::vector<T> v(n);
  for (auto &x : v) x = (T)(scale * r.uniform());
  return v;
}

template <typename T>
void run(const char *tn, uint64_t seed) {
  using C = typename CufftTraits<T>::ComplexType;
  const std::string p = std::string(tn) + ".";
  const size_t Nx = 4, Ny = 6, Nz = 10, H = Nx * Ny * (Nz / 2 + 1), N = Nx * Ny * Nz;
  const unsigned B = 256;
  auto grid = [&](size_t n) { return (unsigned)((n + B - 1) / B); };
  Rng r(seed);

  // normalize_kernel (projection_algorithm.cu:85-91)
  {
    T *d = upload(randv<T>(r, N, 3.0));
    normalize_kernel<T><<<grid(N), B>>>(d, T(1) / static_cast<T>(N), N);
    DCHECK(cudaGetLastError());
    record_dev(p + "normalize", d, N);
    cudaFree(d);
  }
  // frequency clamps: spectrum, bound and pre-filled accumulators
  std::vector<T> spec_h = randv<T>(r, 2 * H, 3.0);
  std::vector<T> orig_h = randv<T>(r, 2 * H, 3.0);
  std::vector<T> edits_h = randv<T>(r, 2 * H, 0.01);
  // project_frequency_constraints_all_abs (:148-188)
  {
    C *f = (C *)upload(spec_h);
    T *e = upload(edits_h);
    project_frequency_constraints_all_abs<T><<<grid(2 * H), B>>>(f, T(1), e, Nx, Ny, Nz, H);
    DCHECK(cudaGetLastError());
    record_dev(p + "all_abs.spec", (T *)f, 2 * H);
    record_dev(p + "all_abs.edits", e, 2 * H);
    cudaFree(f);
    cudaFree(e);
  }
  // project_frequency_constraints_direct (:93-145): distinct indices
  {
    std::vector<size_t> idx;
    for (size_t k = 1; k < H; k += 3) idx.push_back(k);
    std::vector<T> dk(idx.size());
    for (auto &x : dk) x = (T)(0.5 + 0.75 * (r.uniform() + 1.0));
    C *f = (C *)upload(spec_h);
    T *e = upload(edits_h);
    size_t *di = upload(idx);
    T *dd = upload(dk);
    const size_t nc = idx.size();
    project_frequency_constraints_direct<T><<<grid(2 * nc), B>>>(f, di, dd, e, Nx, Ny, Nz, H, nc);
    DCHECK(cudaGetLastError());
    record_dev(p + "direct.spec", (T *)f, 2 * H);
    record_dev(p + "direct.edits", e, 2 * H);
    cudaFree(f);
    cudaFree(e);
    cudaFree(di);
    cudaFree(dd);
  }
  // project_frequency_constraints_all_ptw (:191-259): small errors around
  // the original spectrum so that both the DC rule and the ratio test take
  // either branch
  std::vector<T> perr_h = randv<T>(r, 2 * H, 0.15);
  perr_h[0] = (T)(orig_h[0] * 0.01);
  {
    C *f = (C *)upload(perr_h);
    C *o = (C *)upload(orig_h);
    T *e = upload(edits_h);
    project_frequency_constraints_all_ptw<T><<<grid(H), B>>>(f, o, T(0.05), e, Nx, Ny, Nz, H);
    DCHECK(cudaGetLastError());
    record_dev(p + "all_ptw.spec", (T *)f, 2 * H);
    record_dev(p + "all_ptw.edits", e, 2 * H);
    cudaFree(f);
    cudaFree(o);
    cudaFree(e);
  }
  // project_frequency_constraints_partial_ptw (:262-333): constraint 0 is
  // the DC rule whatever index it lists
  {
    std::vector<T> pe = perr_h;
    pe[0] = (T)(orig_h[0] * 0.5);
    std::vector<size_t> idx = {7};
    for (size_t k = 2; k < H; k += 5) idx.push_back(k);
    C *f = (C *)upload(pe);
    C *o = (C *)upload(orig_h);
    T *e = upload(edits_h);
    size_t *di = upload(idx);
    project_frequency_constraints_partial_ptw<T><<<grid(idx.size()), B>>>(f, o, di, T(0.05), e, Nx, Ny, Nz, H,
                                                                         idx.size());
    DCHECK(cudaGetLastError());
    record_dev(p + "partial_ptw.spec", (T *)f, 2 * H);
    record_dev(p + "partial_ptw.edits", e, 2 * H);
    cudaFree(f);
    cudaFree(o);
    cudaFree(e);
    cudaFree(di);
  }
  // project_spatial_constraints_direct (:336-361)
  {
    T *d = upload(randv<T>(r, N, 2.0));
    T *s = upload(randv<T>(r, N, 0.01));
    project_spatial_constraints_direct<T><<<grid(N), B>>>(d, T(1), s, N);
    DCHECK(cudaGetLastError());
    record_dev(p + "spatial.e", d, N);
    record_dev(p + "spatial.edits", s, N);
    cudaFree(d);
    cudaFree(s);
  }
  // edit array with inactive and sub-threshold entries
  std::vector<T> ed = randv<T>(r, 2 * H, 0.01);
  for (size_t i = 0; i < ed.size(); ++i) {
    if (i % 3 == 0) ed[i] = T(0);
    if (i % 7 == 0) ed[i] = (T)(5e-8 * r.uniform());
  }
  const size_t n = ed.size();
  // extract_active_flags (:365-379), pack_bools (:382-405)
  std::vector<int> iflag_h(n);
  std::vector<char> flag_h(n);
  {
    T *a = upload(ed);
    bool *fl = nullptr;
    int *ifl = nullptr;
    DCHECK(cudaMalloc(&fl, n));
    DCHECK(cudaMalloc(&ifl, n * sizeof(int)));
    extract_active_flags<T><<<grid(n), B>>>(a, fl, ifl, n, T(1e-7));
    DCHECK(cudaGetLastError());
    record_dev(p + "flags.bool", (const uint8_t *)fl, n);
    record_dev(p + "flags.int", ifl, n);
    DCHECK(cudaMemcpy(iflag_h.data(), ifl, n * sizeof(int), cudaMemcpyDeviceToHost));
    DCHECK(cudaMemcpy(flag_h.data(), fl, n, cudaMemcpyDeviceToHost));
    const size_t nbytes = (n + 7) / 8;
    uint8_t *pk = nullptr;
    DCHECK(cudaMalloc(&pk, nbytes));
    DCHECK(cudaMemset(pk, 0xAB, nbytes));  // bytes the kernel leaves alone stay visible
    pack_bools<<<grid(n), B>>>(fl, pk, nbytes);
    DCHECK(cudaGetLastError());
    record_dev(p + "pack_bools", pk, nbytes);
    // compact_with_prefix_positions (:408-425) and
    // compact_and_quantize_with_prefix_positions (:427-457)
    std::vector<int> pre(n);
    int run = 0;
    for (size_t i = 0; i < n; ++i) {
      pre[i] = run;
      run += iflag_h[i];
    }
    int *dp = upload(pre);
    T *comp = nullptr;
    uint16_t *q = nullptr;
    DCHECK(cudaMalloc(&comp, n * sizeof(T)));
    DCHECK(cudaMalloc(&q, n * sizeof(uint16_t)));
    compact_with_prefix_positions<T><<<grid(n), B>>>(a, fl, dp, comp, n);
    DCHECK(cudaGetLastError());
    record_dev(p + "compact", comp, (size_t)run);
    T mn = ed[0], mx = ed[0];
    for (T v : ed) {
      mn = v < mn ? v : mn;
      mx = v > mx ? v : mx;
    }
    T *dmn = upload(std::vector<T>{mn});
    T *dmx = upload(std::vector<T>{mx});
    DCHECK(cudaMemset(comp, 0, n * sizeof(T)));
    compact_and_quantize_with_prefix_positions<T><<<grid(n), B>>>(a, fl, dp, comp, dmn, dmx, q, n);
    DCHECK(cudaGetLastError());
    record_dev(p + "cq.compact", comp, (size_t)run);
    record_dev(p + "cq.quant", q, (size_t)run);
    // compact_and_quantize_active_elements (:459-550), the host driver
    T hmn = 0, hmx = 0;
    size_t cnt = 0;
    DCHECK(cudaMemset(comp, 0, n * sizeof(T)));
    DCHECK(cudaMemset(q, 0, n * sizeof(uint16_t)));
    compact_and_quantize_active_elements<T>(a, fl, ifl, comp, q, &hmn, &hmx, n, &cnt);
    DCHECK(cudaDeviceSynchronize());
    const T mm[2] = {hmn, hmx};
    record(p + "cqa.minmax", mm, sizeof(mm), sizeof(T));
    const uint64_t c64 = cnt;
    record(p + "cqa.count", &c64, 8, 8);
    record_dev(p + "cqa.compact", comp, cnt);
    record_dev(p + "cqa.quant", q, cnt);
    // quantize_and_dequantize (:616-644)
    T *dq = nullptr;
    DCHECK(cudaMalloc(&dq, n * sizeof(T)));
    quantize_and_dequantize<T><<<grid(n), B>>>(a, dq, mn, mx, n, T(1e-7));
    DCHECK(cudaGetLastError());
    record_dev(p + "dequant", dq, n);
    cudaFree(dq);
    cudaFree(a);
    cudaFree(fl);
    cudaFree(ifl);
    cudaFree(pk);
    cudaFree(dp);
    cudaFree(comp);
    cudaFree(q);
    cudaFree(dmn);
    cudaFree(dmx);
  }
  // reset_accumulators (:553-572), on a grid smaller than the arrays
  {
    T *f = upload(randv<T>(r, 2 * H, 1.0));
    T *s = upload(randv<T>(r, N, 1.0));
    reset_accumulators<T><<<1, 64>>>(f, s, H, N);
    DCHECK(cudaGetLastError());
    record_dev(p + "reset.freq", f, 2 * H);
    record_dev(p + "reset.spatial", s, N);
    cudaFree(f);
    cudaFree(s);
  }
  // compute_convergence_metric (:575-613): per-block maxima, 256 threads
  {
    const size_t ne = 1000;
    T *d = upload(randv<T>(r, ne, 2.0));
    T *res = nullptr;
    DCHECK(cudaMalloc(&res, grid(ne) * sizeof(T)));
    compute_convergence_metric<T><<<grid(ne), B>>>(d, T(1), res, ne);
    DCHECK(cudaGetLastError());
    record_dev(p + "convergence", res, grid(ne));
    cudaFree(d);
    cudaFree(res);
  }
  // frequency_float_to_complex (:647-659), add_two_arrays (:662-673)
  {
    T *sp = upload(randv<T>(r, 2 * H, 1.0));
    C *cx = nullptr;
    DCHECK(cudaMalloc(&cx, H * sizeof(C)));
    frequency_float_to_complex<T><<<grid(H), B>>>(sp, cx, H);
    DCHECK(cudaGetLastError());
    record_dev(p + "float_to_complex", (T *)cx, 2 * H);
    T *a1 = upload(randv<T>(r, N, 1.0));
    T *a2 = upload(randv<T>(r, N, 1.0));
    add_two_arrays<T><<<grid(N), B>>>(a1, a2, N);
    DCHECK(cudaGetLastError());
    record_dev(p + "add", a2, N);
    cudaFree(sp);
    cudaFree(cx);
    cudaFree(a1);
    cudaFree(a2);
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <out.bin>\n", argv[0]);
    return 1;
  }
  g_out = fopen(argv[1], "wb");
  if (!g_out) return 1;
  run<float>("f32", 11);
  run<double>("f64", 12);
  DCHECK(cudaDeviceSynchronize());
  fclose(g_out);
  return 0;
}
