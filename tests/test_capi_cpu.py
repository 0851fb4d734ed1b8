"""C ABI checks that need no GPU: the library loads, exports every entry
point include/ffcz.h declares, and its host-only entry points (file
formats, Huffman+ZSTD decode) agree with the reference / oracle."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O

HEADER = Path(__file__).resolve().parents[1] / "include" / "ffcz.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ffcz_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = F.lib()
    names = declared_functions()
    assert len(names) >= 45
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(F.SIGNATURES), set(names) ^ set(F.SIGNATURES)


def test_version_and_errors():
    assert "sm_103a" in F.version()
    with pytest.raises(F.FFCzError):
        F.read_raw_array_binary("/nonexistent/file.bin", 4, np.float32)


def test_raw_roundtrip_and_size_check(tmp_path):
    a = np.arange(37, dtype=np.float32) * 0.5
    p = tmp_path / "a.bin"
    F.write_raw_array_binary(a, p)
    assert p.read_bytes() == a.tobytes()  # headerless little-endian
    assert np.array_equal(F.read_raw_array_binary(p, 37, np.float32), a)
    with pytest.raises(F.FFCzError) as ei:
        F.read_raw_array_binary(p, 36, np.float32)
    assert "File size does not match array size" in str(ei.value)


def test_map_bytes_equal_reference_writeMap(golden_huffman, tmp_path):
    g = golden_huffman["geometric"]
    m = {int(s): (int(c), int(l)) for s, c, l in zip(g["ref_sym"], g["ref_code"], g["ref_len"])}
    p = tmp_path / "t.map"
    F.write_map(m, p)
    assert p.read_bytes() == g["ref_map_bytes"].tobytes()
    assert F.read_map(p) == m


def test_decompress_golden_through_cabi(golden_huffman):
    """ffcz_huff_decompress_* (host side of the coder) on the reference's code
    tables and the oracle's bitstreams, ZSTD-framed by libzstd."""
    for name, g in golden_huffman.items():
        sym = g["symbols"]
        book = O.huffman_codebook(sym)
        bits, _ = O.huffman_bitstream(sym, book)
        comp = O.zstd_compress(bits, 19)
        table = {int(s): (int(c), int(l)) for s, c, l in zip(g["ref_sym"], g["ref_code"], g["ref_len"])}
        dec = F.cuda_huffman_zstd_decompress(comp, table, sym.size, len(bits), sym.dtype)
        assert np.array_equal(dec, sym), name


def test_decompress_skip_rule_and_truncation():
    table = {9: (0, 1)}
    comp = O.zstd_compress(bytes([0b10100000]), 3)
    dec = F.cuda_huffman_zstd_decompress(comp, table, 3, 1, np.uint16)
    assert list(dec) == [9, 9, 9]
    # fewer bits than elements: decoding stops at the end of the stream
    dec = F.cuda_huffman_zstd_decompress(O.zstd_compress(bytes([0xFF]), 3), {1: (1, 1)}, 20, 1, np.uint8)
    assert list(dec) == [1] * 8


def test_zstd_error_reported():
    with pytest.raises(F.FFCzError) as ei:
        F.cuda_huffman_zstd_decompress(b"not a zstd frame", {1: (0, 1)}, 4, 4, np.uint8)
    assert ei.value.code == -5


def test_solver_create_without_gpu_fails_cleanly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(F.FFCzError) as ei:
        F.ProjectionSolver(8, 8, 8)
    assert ei.value.code == -2


def test_zstd_stage_bytes_equal_zstd_compress():
    """The native ZSTD stage reuses one compression context per thread; its
    bytes must stay ZSTD_compress's for every size and level, in any order,
    from any thread (HuffmanZSTDCoder.cuh:359-365)."""
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.default_rng(7)
    cases = []
    for n, level in ((0, 3), (1, 20), (1000, 1), (70_000, 20), (300_000, 3), (5_000, 19), (300_000, 20)):
        # skewed bytes, like a Huffman bitstream of a peaked histogram
        cases.append((rng.geometric(0.2, n).astype(np.uint8).tobytes(), level))
    expect = [O.zstd_compress(d, lv) for d, lv in cases]
    assert [F.zstd_compress(d, lv) for d, lv in cases] == expect
    assert [F.zstd_compress(d, lv) for d, lv in reversed(cases)] == expect[::-1]
    with ThreadPoolExecutor(3) as pool:
        got = list(pool.map(lambda c: F.zstd_compress(*c), cases * 2))
    assert got == expect * 2


def test_container_round_trip(tmp_path):
    """Header fields, code tables, ZSTD frames and the restored bitstreams of
    a .ffcz container survive write + read (host only)."""
    rng = np.random.default_rng(3)
    streams = []
    for i, (n, dt) in enumerate(((500, np.uint16), (100, np.uint8), None, None)[:2]):
        sym = rng.geometric(0.2, n).astype(dt)
        book = O.huffman_codebook(sym)
        bits, _ = O.huffman_bitstream(sym, book)
        comp = O.zstd_compress(bits, 3)
        streams.append(F.CompressionResult(comp, book["symbols"], book["codes"], book["lengths"], len(bits), n, b""))
    streams += [None, None]
    h = F.ContainerHeader(dtype=F.FFCZ_F32, pack_mode=0, nx=2, ny=3, nz=40, eps=1e-3, delta=2.5, freq_min=-1.0,
                          freq_max=1.5, spatial_min=-0.1, spatial_max=0.2, iterations=7)
    path = tmp_path / "c.ffcz"
    F.write_container(path, h, streams)
    h2, got = F.read_container(path)
    for f, _ in F.ContainerHeader._fields_:
        assert getattr(h2, f) == getattr(h, f), f
    assert got[2] is None and got[3] is None
    for a, b in zip(streams[:2], got[:2]):
        assert b.compressed_data == a.compressed_data and b.num_elements == a.num_elements
        assert np.array_equal(b.symbols, a.symbols) and np.array_equal(b.codes, a.codes)
        assert np.array_equal(b.lengths, a.lengths)
        assert b.bitstream == O.zstd_decompress(a.compressed_data, a.original_bitstream_size)
    path.write_bytes(path.read_bytes()[:50])
    with pytest.raises(F.FFCzError):
        F.read_container(path)
