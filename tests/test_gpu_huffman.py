"""GPU Huffman encoder: bit-exact with the reference's codebook (golden
fixtures made by the reference's own functions) and with the oracle's
bitstream; ZSTD bytes equal libzstd's ZSTD_compress of that bitstream;
decode round trips."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu


def _table_arrays(res):
    syms, codes, lens = res.arrays()
    return syms, codes, lens


@pytest.mark.parametrize("level", [3, 20])
def test_golden_codebooks_and_bitstreams(cuda, golden_huffman, level):
    for name, g in golden_huffman.items():
        sym = g["symbols"]
        res = F.cuda_huffman_zstd_compress(sym, level)
        syms, codes, lens = _table_arrays(res)
        assert np.array_equal(syms, g["ref_sym"]), name
        assert np.array_equal(codes, g["ref_code"]), name
        assert np.array_equal(lens, g["ref_len"]), name
        book = O.huffman_codebook(sym)
        bits, nbits = O.huffman_bitstream(sym, book)
        assert nbits == int(g["nbits"]), name
        assert res.bitstream == bits, name
        assert res.original_bitstream_size == len(bits)
        assert res.num_elements == sym.size
        assert res.compressed_data == O.zstd_compress(bits, level), name
        dec = F.cuda_huffman_zstd_decompress(res.compressed_data, res.code_table, res.num_elements,
                                             res.original_bitstream_size, sym.dtype)
        assert np.array_equal(dec, sym), name


@pytest.mark.parametrize("n,kind", [(1, "u16"), (7, "u8"), (2047, "u16"), (2048, "u16"), (2049, "u8"),
                                    (32769, "u16"), (1_000_003, "u16"), (3_000_001, "u8")])
def test_sizes_and_tails(cuda, n, kind):
    rng = np.random.default_rng(n)
    if kind == "u16":
        sym = np.clip(np.round(rng.normal(30000, 3000, n)), 0, 65535).astype(np.uint16)
    else:
        sym = (rng.random(n) < 0.2).astype(np.uint8) * rng.integers(0, 256, n).astype(np.uint8)
    res = F.cuda_huffman_zstd_compress(sym, 3)
    book = O.huffman_codebook(sym)
    bits, _ = O.huffman_bitstream(sym, book)
    assert res.bitstream == bits
    dec = F.cuda_huffman_zstd_decompress(res.compressed_data, res.code_table, res.num_elements,
                                         res.original_bitstream_size, sym.dtype)
    assert np.array_equal(dec, sym)


def test_device_entry_and_chunked_zstd(cuda):
    torch = cuda
    rng = np.random.default_rng(5)
    sym = np.clip(np.round(rng.normal(20000, 500, 2_000_000)), 0, 65535).astype(np.uint16)
    d = torch.from_numpy(sym.view(np.int16)).cuda()
    r1 = F.cuda_huffman_zstd_compress_device(d, sym.size, 2, 20, F.FFCZ_ZSTD_SINGLE)
    r2 = F.cuda_huffman_zstd_compress_device(d, sym.size, 2, 20, F.FFCZ_ZSTD_CHUNKED)
    assert r1.bitstream == r2.bitstream
    assert r1.compressed_data == O.zstd_compress(r1.bitstream, 20)
    # independent frames decode with the same ZSTD_decompress call
    for r in (r1, r2):
        dec = F.cuda_huffman_zstd_decompress(r.compressed_data, r.code_table, r.num_elements,
                                             r.original_bitstream_size, np.uint16)
        assert np.array_equal(dec, sym)


def test_empty_and_too_long(cuda):
    with pytest.raises(F.FFCzError) as ei:
        F.cuda_huffman_zstd_compress(np.zeros(0, np.uint16), 3)
    assert ei.value.code == -8 and "Empty data" in str(ei.value)
    # Fibonacci counts F(1)..F(34): the deepest code has 33 bits
    fib = [1, 1]
    while len(fib) < 34:
        fib.append(fib[-1] + fib[-2])
    sym = np.repeat(np.arange(34, dtype=np.uint16), fib)
    assert max(O.huffman_codebook(sym)["lengths"]) > 32
    with pytest.raises(F.FFCzError) as ei:
        F.cuda_huffman_zstd_compress(sym, 3)
    assert ei.value.code == -7


def test_solver_encode_matches_cli_pipeline(cuda):
    """The four streams of projection_example.cu:230-246."""
    shape = (32, 32, 32)
    fld = synth.make_field(shape, 11 / 3, 12, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs((fld.xp - fld.x).astype(np.float32), 100, 1e-7)
        nf, ns = s.active_counts()
        assert nf > 0 and ns > 0
        streams = s.encode(zstd_level=20)
        datas = [s.get_active_freq_quant_edit_distances(), s.get_freq_flags_pack(),
                 s.get_active_spatial_quant_edit_distances(), s.get_spatial_flags_pack()]
        for res, data in zip(streams, datas):
            ref = O.huffman_zstd_compress(data, 20)
            assert res.bitstream == ref["bitstream"]
            assert res.compressed_data == ref["compressed"]
            assert res.num_elements == data.size
