"""Decoder side on the GPU: the segmented Huffman decode equals the
sequential decoder (HuffmanZSTDCoder.cuh:394-449 rules) symbol for symbol,
the flag/code unpacking equals the oracle's dequantisation bit for bit, and
the reconstruction x^ = x' + C2R(F)/N + S matches the FP64 oracle."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu


def gpu_decode(cuda, bits: bytes, book: dict, n: int, dtype):
    d_bits = cuda.from_numpy(np.frombuffer(bits, np.uint8).copy() if bits else np.zeros(1, np.uint8)).cuda()
    out = cuda.zeros(max(n, 1), dtype=cuda.int16 if dtype == np.uint16 else cuda.uint8, device="cuda")
    k = F.huff_decode_device(d_bits, len(bits), (book["symbols"], book["codes"], book["lengths"]), n, dtype, out)
    return out.cpu().numpy().view(dtype)[:k]


def test_golden_streams(cuda, golden_huffman):
    for name, g in golden_huffman.items():
        book = {"symbols": g["ref_sym"], "codes": g["ref_code"], "lengths": g["ref_len"]}
        sym = g["symbols"]
        bits, _ = O.huffman_bitstream(sym, book)
        got = gpu_decode(cuda, bits, book, sym.size, sym.dtype)
        assert np.array_equal(got, sym), name
        # fewer symbols asked than the stream holds, and more
        assert np.array_equal(gpu_decode(cuda, bits, book, sym.size // 2, sym.dtype), sym[: sym.size // 2]), name
        seq = O.huffman_decode(bits, book, sym.size + 50)
        assert np.array_equal(gpu_decode(cuda, bits, book, sym.size + 50, sym.dtype), seq.astype(sym.dtype)), name


@pytest.mark.parametrize("n,p", [(300_000, 0.3), (200_000, 0.02), (70_000, 0.6)])
def test_long_skewed_streams(cuda, n, p):
    """Many 1024-bit segments, codes from 1 to 20+ bits (table + trie path)."""
    sym = np.minimum(np.random.default_rng(n).geometric(p, n) - 1, 65535).astype(np.uint16)
    book = O.huffman_codebook(sym)
    bits, _ = O.huffman_bitstream(sym, book)
    assert np.array_equal(gpu_decode(cuda, bits, book, n, np.uint16), sym)


def test_garbage_bits_follow_the_sequential_rules(cuda):
    """Random bytes under tables with missing branches: misses skip one bit
    and the segments resynchronise on the sequential path."""
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 256, 40_000, dtype=np.uint8).tobytes()
    tables = [
        {"symbols": np.array([7], np.uint32), "codes": np.array([0], np.uint32), "lengths": np.array([1], np.int32)},
        {"symbols": np.array([1, 2, 3], np.uint32), "codes": np.array([0b0, 0b10, 0b1101], np.uint32),
         "lengths": np.array([1, 2, 4], np.int32)},
        {"symbols": np.arange(5, dtype=np.uint32), "codes": np.array([0, 2, 6, 0x3FFFFFFF, 0xFFFFFFFE], np.uint32),
         "lengths": np.array([1, 2, 3, 30, 32], np.int32)},
        O.huffman_codebook(rng.geometric(0.1, 5000).astype(np.uint16)),
        # not prefix-free: a code with a shorter code as prefix is never
        # reached, duplicates resolve to the first, long codes share prefixes
        {"symbols": np.arange(5, dtype=np.uint32), "codes": np.array([1, 2, 0, 0, 0], np.uint32),
         "lengths": np.array([1, 2, 1, 1, 20], np.int32)},
        {"symbols": np.arange(7, dtype=np.uint32),
         "codes": np.array([0xFFFF, 0xFFFF, 0x3FFFF, 0x0001, 0b01, 0xFFFFFFFF, 0x7FFE], np.uint32),
         "lengths": np.array([16, 16, 18, 16, 2, 32, 15], np.int32)},
    ]
    for book in tables:
        for n in (10, 100_000, 1_000_000):
            seq = O.huffman_decode(bits, book, n)
            got = gpu_decode(cuda, bits, book, n, np.uint16)
            assert np.array_equal(got, seq.astype(np.uint16)), (book["lengths"][:5], n)


def test_zstd_decompress_to_device(cuda):
    sym = np.random.default_rng(2).geometric(0.05, 100_000).astype(np.uint16)
    res = F.cuda_huffman_zstd_compress(sym, 5)
    out = cuda.zeros(sym.size, dtype=cuda.int16, device="cuda")
    k = F.huff_zstd_decompress_device(res.compressed_data, res.arrays(), res.num_elements,
                                      res.original_bitstream_size, np.uint16, out)
    assert k == sym.size and np.array_equal(out.cpu().numpy().view(np.uint16), sym)


@pytest.mark.parametrize("shape,dtype,c", [((16, 24, 10), np.float32, 1.0), ((64, 64, 64), np.float32, 1.5),
                                           ((3, 250, 500), np.float32, 1.0), ((1, 90, 100), np.float32, 1.0),
                                           ((1, 1, 4096), np.float32, 1.0), ((12, 10, 16), np.float64, 1.0),
                                           ((5, 7, 9), np.float32, 2.0)])
def test_encode_decode_reconstruct(cuda, shape, dtype, c):
    fld = synth.make_field(shape, 11 / 3, 21, 1e-3, 1e-3, dtype, noise=0.3)
    delta = synth.stress_delta(fld, c)
    dx = cuda.from_numpy(fld.x.reshape(-1).copy()).cuda()
    dxp = cuda.from_numpy(fld.xp.reshape(-1).copy()).cuda()
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs_device(dx, fld.eps, delta)
        s.solve_all_abs_pair_device(dx, dxp, 100, 1e-7)
        streams = s.encode(3)
        mm = s.minmax()
        fq, sq = s.get_active_freq_quant_edit_distances(), s.get_active_spatial_quant_edit_distances()
        fp, sp = s.get_freq_flags_pack(), s.get_spatial_flags_pack()
        xhat = fld.x.astype(np.float64).reshape(-1) + s.get_results().astype(np.float64).reshape(-1)
        fe_acc = s.get_freq_edits_full()
        nf, ns = s.active_counts()
    assert nf + ns > 0
    N = int(np.prod(shape))
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)
    fe = O.unpack_edits(fq, fp.tobytes(), 2 * H, mm[0], mm[1], dtype)
    se = O.unpack_edits(sq, sp.tobytes(), N, mm[2], mm[3], dtype)
    ref = O.reconstruct(fld.xp, shape, fe, se).reshape(-1)
    with F.ProjectionSolver(*shape, dtype=dtype) as d:
        out = cuda.empty_like(dxp)
        d.decode_device(dxp, streams, mm, out)
        got = out.cpu().numpy().astype(np.float64)
        assert np.array_equal(d.get_spatial_edits_full(), se)  # dequantisation bit-exact
    tol = (2e-6 if dtype == np.float32 else 1e-13) * max(1.0, float(np.abs(ref).max()))
    assert np.abs(got - ref).max() <= tol
    # against the corrector's own x^: the difference is the edit quantisation
    fq_err = (mm[1] - mm[0]) / 65535 if nf else 0.0
    sq_err = (mm[3] - mm[2]) / 65535 if ns else 0.0
    bound = sq_err + 2 * nf * fq_err / N + 1e-5 * max(1.0, float(np.abs(xhat).max()))
    assert np.abs(got - xhat).max() <= bound
    # unquantised frequency edits give the corrector's x^ (the frequency
    # projections sum to C2R(F)/N)
    exact = O.reconstruct(fld.xp, shape, fe_acc, se).reshape(-1)
    assert np.abs(exact - xhat).max() <= sq_err + 1e-4 * fld.eps * max(1, N ** 0.5) + 1e-5


def test_decode_rejects_bad_streams(cuda):
    shape = (8, 8, 8)
    fld = synth.make_field(shape, 11 / 3, 4, 1e-3, 1e-3, np.float32, noise=0.3)
    dx = cuda.from_numpy(fld.x.reshape(-1).copy()).cuda()
    dxp = cuda.from_numpy(fld.xp.reshape(-1).copy()).cuda()
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs_device(dx, fld.eps, synth.stress_delta(fld, 1.0))
        s.solve_all_abs_pair_device(dx, dxp, 100, 1e-7)
        streams = s.encode(3)
        mm = s.minmax()
        out = cuda.empty_like(dxp)
        present = [i for i in (0, 2) if streams[i] is not None]
        assert present
        bad = list(streams)
        bad[present[0] + 1] = None  # a code stream without its flag pack
        with pytest.raises(F.FFCzError):
            s.decode_device(dxp, bad, mm, out)
        # no streams at all: x^ = x'
        s.decode_device(dxp, [None] * 4, mm, out)
        assert np.array_equal(out.cpu().numpy(), fld.xp.reshape(-1))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_base_quantizer_matches_generator(cuda, dtype):
    """The GPU base compressor gives the synthetic generator's x' (no noise)
    bit for bit, and its indices."""
    fld = synth.make_field((16, 24, 40), 11 / 3, 23, 1e-3, 1e-3, dtype)
    dx = cuda.from_numpy(fld.x.reshape(-1).copy()).cuda()
    out = cuda.empty_like(dx)
    idx = cuda.empty(dx.numel(), dtype=cuda.int32, device="cuda")
    eps = 1e-3 * float(fld.x.astype(np.float64).max() - fld.x.astype(np.float64).min())
    F.base_quantize_device(dx, eps, out, idx)
    x64 = fld.x.astype(np.float64).reshape(-1)
    ref = (2 * eps * np.round(x64 / (2 * eps))).astype(dtype)
    assert np.array_equal(out.cpu().numpy(), ref)
    assert np.array_equal(idx.cpu().numpy(), np.round(x64 / (2 * eps)).astype(np.int32))
    assert np.abs(out.cpu().numpy().astype(np.float64) - x64).max() <= eps * (1 + 1e-6)
