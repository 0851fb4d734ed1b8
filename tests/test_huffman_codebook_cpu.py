"""The library's host codebook builder (ffcz_huff_codebook: the tree of
buildHuffmanTree and the codes of generateCodesRecursive,
HuffmanZSTDCoder.cuh:85-178) against the oracle's min-heap restatement, on
histograms with many ties, skewed and flat counts, counts above 2^16 (two
sort digits), one and two symbols, and a nearly full 16-bit alphabet.  No
GPU: the builder runs on the host."""
import ctypes as C

import numpy as np
import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O


def lib_codebook(hist):
    hist = np.ascontiguousarray(hist, np.uint32)
    nz = int(np.count_nonzero(hist))
    sym = np.zeros(max(nz, 1), np.uint32)
    code = np.zeros(max(nz, 1), np.uint32)
    ln = np.zeros(max(nz, 1), np.int32)
    n = C.c_size_t()
    rc = F.lib().ffcz_huff_codebook(hist.ctypes.data, hist.size, sym.ctypes.data, code.ctypes.data, ln.ctypes.data,
                                    sym.size, C.byref(n))
    assert rc == F.FFCZ_OK
    assert n.value == nz
    return sym[:nz], code[:nz], ln[:nz]


def data_of(hist):
    return np.repeat(np.arange(hist.size, dtype=np.uint32), hist.astype(np.int64))


def cases():
    rng = np.random.default_rng(7)
    yield "ties", np.tile(np.array([3, 3, 3, 1, 1, 2, 2, 2, 0, 5], np.uint32), 20)
    yield "one", np.array([0, 0, 9, 0], np.uint32)
    yield "two", np.array([4, 0, 4], np.uint32)
    yield "geometric", np.bincount(rng.geometric(0.05, 20000), minlength=256).astype(np.uint32)[:256]
    yield "flat", np.full(300, 7, np.uint32)
    yield "fibonacci", np.array([1, 1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233, 377, 610, 987, 1597, 2584, 4181,
                                 6765, 10946, 17711], np.uint32)
    wide = rng.integers(0, 4, 65536).astype(np.uint32)
    wide[rng.integers(0, 65536, 50)] = rng.integers(1, 200, 50)
    yield "wide_16bit", wide
    big = np.zeros(1000, np.uint32)
    big[::7] = rng.integers(1, 300, big[::7].size)
    big[3] = 70000  # a count above 2^16: the sort's second digit
    yield "count_above_2^16", big
    normal = np.clip(rng.normal(32768, 3000, 200000), 0, 65535).astype(np.int64)
    yield "peaked_quantised", np.bincount(normal, minlength=65536).astype(np.uint32)


@pytest.mark.parametrize("name,hist", list(cases()), ids=[c[0] for c in cases()])
def test_codebook_equals_oracle(name, hist):
    sym, code, ln = lib_codebook(hist)
    book = O.huffman_codebook(data_of(hist), nbins=hist.size)
    assert np.array_equal(sym, book["symbols"])
    assert np.array_equal(ln, book["lengths"])
    assert np.array_equal(code, book["codes"])


def test_codebook_empty_and_capacity():
    n = C.c_size_t()
    assert F.lib().ffcz_huff_codebook(np.zeros(4, np.uint32).ctypes.data, 4, None, None, None, 0, C.byref(n)) == 0
    assert n.value == 0
    h = np.array([1, 1, 1], np.uint32)
    out = np.zeros(2, np.uint32)
    rc = F.lib().ffcz_huff_codebook(h.ctypes.data, 3, out.ctypes.data, out.ctypes.data, out.ctypes.data, 2,
                                    C.byref(n))
    assert rc == F.FFCZ_ERR_CAPACITY and n.value == 3
