#include "huffman_host.h"

#include <dlfcn.h>

#include <algorithm>
#include <functional>
#include <mutex>
#include <queue>
#include <thread>
#include <utility>

#include "../../include/ffcz.h"

namespace ffcz {

int fail(int code, const std::string &msg);

void build_codebook(const uint32_t *hist, size_t nbins, Codebook &cb) {
  cb.sym.clear();
  cb.freq.clear();
  for (size_t s = 0; s < nbins; ++s) {
    if (hist[s]) {
      cb.sym.push_back((uint32_t)s);
      cb.freq.push_back(hist[s]);
    }
  }
  const int n = (int)cb.sym.size();
  cb.code.assign(n, 0u);
  cb.len.assign(n, 0);
  cb.max_len = 0;
  if (n == 0) return;
  if (n == 1) {
    cb.code[0] = 0u;
    cb.len[0] = 1;
    cb.max_len = 1;
    return;
  }
  std::vector<int> left, right;
  std::vector<uint64_t> wt;
  build_tree(cb.freq.data(), n, left, right, wt);
  // Codes from the root down, as the reference's recursive walk gives them
  // (0 to the left child, 1 to the right, MSB-first in a uint32 that keeps
  // its low 32 bits): every child has a smaller index than its parent
  // (internal nodes are created in increasing order from smaller ones), so
  // one sweep from the root (2n-2) downwards reaches each node after its
  // parent.
  const int nodes = 2 * n - 1;
  std::vector<uint32_t> code(nodes);
  std::vector<int32_t> len(nodes);
  code[nodes - 1] = 0u;
  len[nodes - 1] = 0;
  for (int k = nodes - 1; k >= n; --k) {
    const int a = left[k], b = right[k];
    code[a] = code[k] << 1;
    len[a] = len[k] + 1;
    code[b] = (code[k] << 1) | 1u;
    len[b] = len[k] + 1;
  }
  for (int i = 0; i < n; ++i) {
    cb.code[i] = code[i];
    cb.len[i] = len[i];
    cb.max_len = std::max(cb.max_len, len[i]);
  }
}

void build_tree(const uint32_t *freq, int n, std::vector<int> &left, std::vector<int> &right,
                std::vector<uint64_t> &wt) {
  // Nodes: leaves 0..n-1, internal n..2n-2.  The reference pops the two
  // smallest (freq, node index) keys of a min-heap.  The same sequence comes
  // from two queues: the leaves sorted by (freq, index), and the internal
  // nodes in creation order, whose keys are already sorted (merged weights
  // never decrease and indices grow); the smaller head is the heap's top.
  left.assign(std::max(2 * n - 1, 1), -1);
  right.assign(std::max(2 * n - 1, 1), -1);
  wt.assign(std::max(2 * n - 1, 1), 0);
  if (n <= 1) {
    if (n == 1) wt[0] = freq[0];
    return;
  }
  // Leaves in (freq, index) order: they start in index order, so a stable
  // LSD counting sort on freq alone (16-bit digits, only the digits in use,
  // count arrays sized to the largest digit) orders ties by index.
  uint32_t maxf = 0;
  for (int i = 0; i < n; ++i) {
    wt[i] = freq[i];
    maxf = std::max(maxf, freq[i]);
  }
  std::vector<int> leaves(n), tmp(n);
  for (int i = 0; i < n; ++i) leaves[i] = i;
  std::vector<uint32_t> count;
  for (int shift = 0; shift < 32 && (maxf >> shift); shift += 16) {
    const uint32_t top = std::min<uint32_t>(maxf >> shift, 0xffffu);
    count.assign((size_t)top + 1, 0u);
    for (int i = 0; i < n; ++i) ++count[(freq[leaves[i]] >> shift) & 0xffffu];
    uint32_t run = 0;
    for (uint32_t &c : count) {
      const uint32_t t = c;
      c = run;
      run += t;
    }
    for (int i = 0; i < n; ++i) tmp[count[(freq[leaves[i]] >> shift) & 0xffffu]++] = leaves[i];
    leaves.swap(tmp);
  }
  int qa = 0, qb = n;  // heads: sorted leaves, internal nodes
  int next = n;
  auto take = [&]() {
    if (qa < n && (qb >= next || wt[leaves[qa]] < wt[qb] || (wt[leaves[qa]] == wt[qb] && leaves[qa] < qb)))
      return leaves[qa++];
    return qb++;
  };
  while (next < 2 * n - 1) {
    const int a = take();
    const int b = take();
    left[next] = a;
    right[next] = b;
    wt[next] = wt[a] + wt[b];
    ++next;
  }
}

std::vector<uint32_t> huffman_decode(const uint8_t *bits, size_t nbytes, const uint32_t *symbols,
                                     const uint32_t *codes, const int32_t *lengths, size_t nsym,
                                     size_t num_elements) {
  // Binary trie of the codes of length 1..32 (longer codes are never
  // matched by the reference decoder).  node 0 = root; child[2*i + bit].
  std::vector<int> child(2, -1), leaf(1, -1);
  for (size_t s = 0; s < nsym; ++s) {
    const int L = lengths[s];
    // the reference keys on (length, code): a stored code of 2^L or more
    // never matches the L bits read
    if (L < 1 || L > 32 || (L < 32 && (codes[s] >> L) != 0)) continue;
    int node = 0;
    for (int d = L - 1; d >= 0; --d) {
      const int bit = (codes[s] >> d) & 1u;
      int &c = child[2 * node + bit];
      if (c < 0) {
        c = (int)leaf.size();
        leaf.push_back(-1);
        child.push_back(-1);
        child.push_back(-1);
      }
      node = child[2 * node + bit];
    }
    if (leaf[node] < 0) leaf[node] = (int)s;
  }
  std::vector<uint32_t> out;
  out.reserve(num_elements);
  const size_t total = nbytes * 8;
  size_t pos = 0;
  while (out.size() < num_elements && pos < total) {
    int node = 0;
    size_t p = pos;
    int sym = -1;
    int depth = 0;
    while (p < total && depth < 32) {
      const int bit = (bits[p >> 3] >> (7 - (p & 7))) & 1;
      node = child[2 * node + bit];
      ++p;
      ++depth;
      if (node < 0) break;
      if (leaf[node] >= 0) {
        sym = leaf[node];
        break;
      }
    }
    if (sym >= 0) {
      out.push_back(symbols[sym]);
      pos = p;
    } else {
      ++pos;  // no code matches here: skip one bit (HuffmanZSTDCoder.cuh:442-446)
    }
  }
  return out;
}

// ------------------------------------------------------------------ ZSTD --
namespace {
struct Zstd {
  size_t (*compressBound)(size_t) = nullptr;
  size_t (*compress)(void *, size_t, const void *, size_t, int) = nullptr;
  size_t (*decompress)(void *, size_t, const void *, size_t) = nullptr;
  unsigned (*isError)(size_t) = nullptr;
  const char *(*getErrorName)(size_t) = nullptr;
  // optional: a context kept per thread keeps level-20 match tables (tens of
  // MB) mapped between calls; ZSTD_compressCCtx writes ZSTD_compress's bytes
  void *(*createCCtx)() = nullptr;
  size_t (*freeCCtx)(void *) = nullptr;
  size_t (*compressCCtx)(void *, void *, size_t, const void *, size_t, int) = nullptr;
  bool ok = false;
  std::string why;
};
Zstd &zstd() {
  static Zstd z;
  static std::once_flag once;
  std::call_once(once, [] {
    void *h = dlopen("libzstd.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libzstd.so", RTLD_NOW | RTLD_LOCAL);
    if (!h) {
      z.why = "libzstd.so.1 not found";
      return;
    }
    z.compressBound = (size_t(*)(size_t))dlsym(h, "ZSTD_compressBound");
    z.compress = (size_t(*)(void *, size_t, const void *, size_t, int))dlsym(h, "ZSTD_compress");
    z.decompress = (size_t(*)(void *, size_t, const void *, size_t))dlsym(h, "ZSTD_decompress");
    z.isError = (unsigned (*)(size_t))dlsym(h, "ZSTD_isError");
    z.getErrorName = (const char *(*)(size_t))dlsym(h, "ZSTD_getErrorName");
    z.createCCtx = (void *(*)())dlsym(h, "ZSTD_createCCtx");
    z.freeCCtx = (size_t(*)(void *))dlsym(h, "ZSTD_freeCCtx");
    z.compressCCtx = (size_t(*)(void *, void *, size_t, const void *, size_t, int))dlsym(h, "ZSTD_compressCCtx");
    if (!z.createCCtx || !z.freeCCtx || !z.compressCCtx) z.createCCtx = nullptr;
    z.ok = z.compressBound && z.compress && z.decompress && z.isError && z.getErrorName;
    if (!z.ok) z.why = "libzstd.so.1 lacks a required symbol";
  });
  return z;
}
}  // namespace

bool zstd_available(std::string *why) {
  Zstd &z = zstd();
  if (!z.ok && why) *why = z.why;
  return z.ok;
}

namespace {
struct ThreadCCtx {
  void *ctx = nullptr;
  ~ThreadCCtx() {
    if (ctx) zstd().freeCCtx(ctx);
  }
};
}  // namespace

static int compress_one(const uint8_t *src, size_t n, int level, std::vector<uint8_t> &out) {
  Zstd &z = zstd();
  const size_t bound = z.compressBound(n);
  out.resize(bound);
  thread_local ThreadCCtx tc;
  if (z.createCCtx && !tc.ctx) tc.ctx = z.createCCtx();
  const size_t r = tc.ctx ? z.compressCCtx(tc.ctx, out.data(), bound, src, n, level)
                          : z.compress(out.data(), bound, src, n, level);
  if (z.isError(r)) return fail(FFCZ_ERR_ZSTD, std::string("ZSTD compression failed: ") + z.getErrorName(r));
  out.resize(r);
  return FFCZ_OK;
}

static size_t chunk_size(size_t n) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  return std::max<size_t>((n + hw - 1) / hw, 128u << 10);
}

size_t zstd_bound(size_t n) {
  if (!zstd_available(nullptr)) return 0;
  Zstd &z = zstd();
  const size_t chunk = chunk_size(n);
  const size_t nch = (n + chunk - 1) / chunk;
  return std::max(z.compressBound(n), nch * z.compressBound(std::min(chunk, n)));
}

int zstd_compress(const uint8_t *src, size_t n, int level, bool chunked, std::vector<uint8_t> &out) {
  std::string why;
  if (!zstd_available(&why)) return fail(FFCZ_ERR_ZSTD, why);
  if (!chunked || n < (256u << 10)) return compress_one(src, n, level, out);
  const size_t chunk = chunk_size(n);
  const size_t nch = (n + chunk - 1) / chunk;
  std::vector<std::vector<uint8_t>> parts(nch);
  std::vector<int> rc(nch, FFCZ_OK);
  std::vector<std::thread> th;
  for (size_t c = 0; c < nch; ++c) {
    th.emplace_back([&, c] {
      const size_t off = c * chunk;
      rc[c] = compress_one(src + off, std::min(chunk, n - off), level, parts[c]);
    });
  }
  for (auto &t : th) t.join();
  out.clear();
  for (size_t c = 0; c < nch; ++c) {
    if (rc[c] != FFCZ_OK) return rc[c];
    out.insert(out.end(), parts[c].begin(), parts[c].end());
  }
  return FFCZ_OK;
}

int zstd_decompress(const uint8_t *src, size_t n, size_t expect, std::vector<uint8_t> &out) {
  std::string why;
  if (!zstd_available(&why)) return fail(FFCZ_ERR_ZSTD, why);
  Zstd &z = zstd();
  out.resize(expect);
  const size_t r = z.decompress(out.data(), expect, src, n);
  if (z.isError(r))
    return fail(FFCZ_ERR_ZSTD, std::string("ZSTD decompression failed: ") + z.getErrorName(r));
  out.resize(r);
  return FFCZ_OK;
}

}  // namespace ffcz
