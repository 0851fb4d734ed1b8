/*
 * ffcz_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference FFCz integer/byte stages, used by the
 * tests, __graft_entry__.smoke() and bench.py's CPU baseline as the checker.
 * Nothing in the product links or calls this file.
 *
 *   orc_flags_minmax / orc_compact_quantize : projection_algorithm_impl.cuh:384-424,
 *       projection_algorithm.cu:365-379 (flags |v| > thr), :480-490 (whole-array
 *       min/max, zeros included), :499-523 (exclusive scan / count),
 *       :427-457 (scatter + uint16 quantiser).
 *   orc_pack_flags : correct LSB-first packing, and the reference's
 *       pack_bools (projection_algorithm.cu:382-405) as launched by
 *       projection_algorithm_impl.cuh:429-449.
 *   orc_huff_codebook : HuffmanZSTDCoder.cuh:48-83 (sorted histogram),
 *       :85-152 (min-heap on (freq, node index), first pop = left = bit 0),
 *       :154-178 (uint32 codes from the root, single symbol -> (0, 1)).
 *   orc_huff_pack : HuffmanZSTDCoder.cuh:307-357 (exclusive scan of lengths,
 *       MSB-first placement in 64-bit words, big-endian word split,
 *       truncated to ceil(bits/8) bytes).
 *   orc_huff_decode : HuffmanZSTDCoder.cuh:394-449 (lengths 1..32 tried in
 *       order against a (length, code) table, one bit skipped on a miss).
 *
 * Compile with -ffp-contract=off so float arithmetic is rounded per
 * operation, as the CUDA kernels do for these expressions.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ flags */
#define DEF_FLAGS(T, SUF)                                                             \
  void orc_flags_minmax_##SUF(const T *a, size_t n, T thr, uint8_t *flags, T *mn,     \
                              T *mx, size_t *count) {                                 \
    size_t c = 0;                                                                     \
    T lo = a[0], hi = a[0];                                                           \
    for (size_t i = 0; i < n; ++i) {                                                  \
      const T v = a[i];                                                               \
      const int f = fabs((double)v) > (double)thr;                                    \
      if (flags) flags[i] = (uint8_t)f;                                               \
      c += (size_t)f;                                                                 \
      if (v < lo) lo = v;                                                             \
      if (v > hi) hi = v;                                                             \
    }                                                                                 \
    *mn = lo;                                                                         \
    *mx = hi;                                                                         \
    *count = c;                                                                       \
  }

DEF_FLAGS(float, f32)
DEF_FLAGS(double, f64)

/* n = (v - mn)/(mx - mn); q = n > 0.5 ? ceil(n*65535) : floor(n*65535). */
static uint16_t quant_f32(float v, float mn, float mx) {
  volatile float num = v - mn;
  volatile float den = mx - mn;
  volatile float nrm = num / den;
  volatile float s = nrm * 65535.0f;
  float q = ((double)nrm > 0.5) ? ceilf(s) : floorf(s);
  if (q != q) return 0;
  return (uint16_t)(unsigned)q;
}

static uint16_t quant_f64(double v, double mn, double mx) {
  volatile double num = v - mn;
  volatile double den = mx - mn;
  volatile double nrm = num / den;
  volatile double s = nrm * 65535.0;
  double q = (nrm > 0.5) ? ceil(s) : floor(s);
  if (q != q) return 0;
  return (uint16_t)(unsigned)q;
}

#define DEF_COMPACT(T, SUF)                                                              \
  size_t orc_compact_quantize_##SUF(const T *a, size_t n, T thr, T mn, T mx, T *compact, \
                                    uint16_t *quant) {                                   \
    size_t pos = 0;                                                                      \
    for (size_t i = 0; i < n; ++i) {                                                     \
      const T v = a[i];                                                                  \
      if (fabs((double)v) > (double)thr) {                                               \
        if (compact) compact[pos] = v;                                                   \
        if (quant) quant[pos] = quant_##SUF(v, mn, mx);                                  \
        ++pos;                                                                           \
      }                                                                                  \
    }                                                                                    \
    return pos;                                                                          \
  }

DEF_COMPACT(float, f32)
DEF_COMPACT(double, f64)

uint16_t orc_quantize_f32(float v, float mn, float mx) { return quant_f32(v, mn, mx); }
uint16_t orc_quantize_f64(double v, double mn, double mx) { return quant_f64(v, mn, mx); }

/* pack: ref_compat = 0 -> every flag, LSB first; ref_compat = 1 -> bytes
 * b < ceil(nbytes/8) hold flags [8b, 8b+8) below nbytes = ceil(n/8), all
 * later bytes zero.  `pack` has ceil(n/8) bytes. */
void orc_pack_flags(const uint8_t *flags, size_t n, uint8_t *pack, int ref_compat) {
  const size_t nbytes = (n + 7) / 8;
  memset(pack, 0, nbytes);
  if (!ref_compat) {
    for (size_t i = 0; i < n; ++i)
      if (flags[i]) pack[i >> 3] |= (uint8_t)(1u << (i & 7));
    return;
  }
  const size_t written = (nbytes + 7) / 8;
  for (size_t b = 0; b < written; ++b) {
    unsigned v = 0;
    for (int i = 0; i < 8; ++i) {
      const size_t idx = 8 * b + (size_t)i;
      if (idx < nbytes && flags[idx]) v |= 1u << i;
    }
    pack[b] = (uint8_t)v;
  }
}

/* ---------------------------------------------------------------- Huffman */
typedef struct { uint32_t freq; int idx; } Key;

static int key_less(Key a, Key b) { return a.freq < b.freq || (a.freq == b.freq && a.idx < b.idx); }

static void heap_push(Key *h, int *n, Key k) {
  int i = (*n)++;
  h[i] = k;
  while (i > 0) {
    int p = (i - 1) / 2;
    if (!key_less(h[i], h[p])) break;
    Key t = h[i]; h[i] = h[p]; h[p] = t;
    i = p;
  }
}

static Key heap_pop(Key *h, int *n) {
  Key top = h[0];
  h[0] = h[--(*n)];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < *n && key_less(h[l], h[m])) m = l;
    if (r < *n && key_less(h[r], h[m])) m = r;
    if (m == i) break;
    Key t = h[i]; h[i] = h[m]; h[m] = t;
    i = m;
  }
  return top;
}

/* Histogram of `data` (symbol values < nbins), then codebook.  Outputs,
 * in ascending symbol order: sym, freq, code, len; returns the number of
 * distinct symbols. */
size_t orc_huff_codebook(const uint32_t *data, size_t n, size_t nbins, uint32_t *sym, uint32_t *freq,
                         uint32_t *code, int32_t *len) {
  uint32_t *hist = (uint32_t *)calloc(nbins, sizeof(uint32_t));
  for (size_t i = 0; i < n; ++i) hist[data[i]]++;
  size_t ns = 0;
  for (size_t s = 0; s < nbins; ++s)
    if (hist[s]) {
      sym[ns] = (uint32_t)s;
      freq[ns] = hist[s];
      ++ns;
    }
  free(hist);
  if (ns == 0) return 0;
  if (ns == 1) {
    code[0] = 0;
    len[0] = 1;
    return 1;
  }
  const int nn = (int)ns;
  int *left = (int *)malloc(sizeof(int) * (2 * nn - 1));
  int *right = (int *)malloc(sizeof(int) * (2 * nn - 1));
  Key *heap = (Key *)malloc(sizeof(Key) * (2 * nn));
  int hn = 0;
  for (int i = 0; i < 2 * nn - 1; ++i) left[i] = right[i] = -1;
  for (int i = 0; i < nn; ++i) {
    Key k = {freq[i], i};
    heap_push(heap, &hn, k);
  }
  int next = nn;
  while (hn > 1) {
    Key a = heap_pop(heap, &hn);
    Key b = heap_pop(heap, &hn);
    left[next] = a.idx;
    right[next] = b.idx;
    Key k = {a.freq + b.freq, next};
    heap_push(heap, &hn, k);
    ++next;
  }
  const int root = heap[0].idx;
  /* explicit-stack depth-first walk */
  int *st_node = (int *)malloc(sizeof(int) * (2 * nn));
  uint32_t *st_code = (uint32_t *)malloc(sizeof(uint32_t) * (2 * nn));
  int *st_len = (int *)malloc(sizeof(int) * (2 * nn));
  int sp = 0;
  st_node[sp] = root; st_code[sp] = 0; st_len[sp] = 0; ++sp;
  while (sp > 0) {
    --sp;
    const int nd = st_node[sp];
    const uint32_t c = st_code[sp];
    const int l = st_len[sp];
    if (left[nd] < 0 && right[nd] < 0) {
      code[nd] = c;
      len[nd] = l ? l : 1;
      continue;
    }
    st_node[sp] = right[nd]; st_code[sp] = (c << 1) | 1u; st_len[sp] = l + 1; ++sp;
    st_node[sp] = left[nd]; st_code[sp] = c << 1; st_len[sp] = l + 1; ++sp;
  }
  free(left); free(right); free(heap); free(st_node); free(st_code); free(st_len);
  return ns;
}

/* Bit packing with the reference's 64-bit word placement.  lut_code /
 * lut_len are indexed by symbol value.  Returns the byte count
 * ceil(total_bits/8) written to out (which must hold that many bytes),
 * or (size_t)-1 when a code is longer than 64 bits. */
size_t orc_huff_pack(const uint32_t *data, size_t n, const uint32_t *lut_code, const int32_t *lut_len,
                     uint8_t *out, uint64_t *total_bits_out) {
  uint64_t total = 0;
  for (size_t i = 0; i < n; ++i) {
    if (lut_len[data[i]] > 64) return (size_t)-1;
    total += (uint64_t)lut_len[data[i]];
  }
  const size_t nwords = (size_t)((total + 63) / 64);
  uint64_t *w = (uint64_t *)calloc(nwords ? nwords : 1, sizeof(uint64_t));
  uint64_t pos = 0;
  for (size_t i = 0; i < n; ++i) {
    const uint32_t c = lut_code[data[i]];
    const int L = lut_len[data[i]];
    const size_t wi = (size_t)(pos / 64);
    const int off = (int)(pos % 64);
    if (off + L <= 64) {
      w[wi] |= (uint64_t)c << (64 - off - L);
    } else {
      const int first = 64 - off, second = L - first;
      w[wi] |= (uint64_t)(c >> second);
      if (second > 0) w[wi + 1] |= ((uint64_t)(c & ((1ull << second) - 1))) << (64 - second);
    }
    pos += (uint64_t)L;
  }
  const size_t nbytes = (size_t)((total + 7) / 8);
  for (size_t b = 0; b < nbytes; ++b) out[b] = (uint8_t)(w[b / 8] >> (8 * (7 - (b % 8))));
  free(w);
  if (total_bits_out) *total_bits_out = total;
  return nbytes;
}

/* Reference decoder.  The (length, code) -> symbol table of
 * HuffmanZSTDCoder.cuh:395-402 is held as one (code, table index)-sorted
 * array per length and searched by bisection.  A code matches only the
 * L-bit value it holds (stored codes of 2^L or more never match, as in the
 * reference's (length << 32 | code) key).  Where two entries share a
 * (length, code) key -- which the reference resolves by its hash map's
 * iteration order -- the first table entry is taken.  Returns the number
 * of decoded symbols (<= num_elements). */
typedef struct { uint32_t code; uint32_t sym; size_t idx; } CodeSym;

static int cs_cmp(const void *a, const void *b) {
  const CodeSym *p = (const CodeSym *)a, *q = (const CodeSym *)b;
  if (p->code != q->code) return p->code < q->code ? -1 : 1;
  return p->idx < q->idx ? -1 : p->idx > q->idx;
}

/* first entry with this code (lower bound), or NULL */
static const CodeSym *cs_find(const CodeSym *t, size_t n, uint32_t code) {
  size_t lo = 0, hi = n;
  while (lo < hi) {
    const size_t mid = lo + (hi - lo) / 2;
    if (t[mid].code < code) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && t[lo].code == code) ? &t[lo] : NULL;
}

size_t orc_huff_decode(const uint8_t *bits, size_t nbytes, const uint32_t *sym, const uint32_t *code,
                       const int32_t *len, size_t nsym, size_t num_elements, uint32_t *out) {
  CodeSym *tab[33] = {0};
  size_t cnt[33] = {0};
  for (size_t s = 0; s < nsym; ++s)
    if (len[s] >= 1 && len[s] <= 32) cnt[len[s]]++;
  for (int L = 1; L <= 32; ++L) {
    tab[L] = (CodeSym *)malloc(sizeof(CodeSym) * (cnt[L] ? cnt[L] : 1));
    cnt[L] = 0;
  }
  for (size_t s = 0; s < nsym; ++s)
    if (len[s] >= 1 && len[s] <= 32) {
      CodeSym e = {code[s], sym[s], s};
      tab[len[s]][cnt[len[s]]++] = e;
    }
  for (int L = 1; L <= 32; ++L) qsort(tab[L], cnt[L], sizeof(CodeSym), cs_cmp);
  const uint64_t total = (uint64_t)nbytes * 8;
  uint64_t pos = 0;
  size_t got = 0;
  while (got < num_elements && pos < total) {
    int found = 0;
    uint32_t c = 0;
    for (int L = 1; L <= 32 && pos + (uint64_t)L <= total && !found; ++L) {
      const uint64_t p = pos + (uint64_t)(L - 1);
      c = (c << 1) | ((bits[p >> 3] >> (7 - (p & 7))) & 1u);
      if (!cnt[L]) continue;
      const CodeSym *hit = cs_find(tab[L], cnt[L], c);
      if (hit) {
        out[got++] = hit->sym;
        pos += (uint64_t)L;
        found = 1;
      }
    }
    if (!found) ++pos;
  }
  for (int L = 1; L <= 32; ++L) free(tab[L]);
  return got;
}
