"""The drop-in headers' device-side surface, compiled the way a user of the
reference headers compiles it (nvcc against include/, linked to libffcz.so):

* every kernel projection_algorithm.cuh declares, plus the host
  compact_and_quantize_active_elements, launched by
  tests/legacy_kernels_driver.cu on seeded inputs, bit-exact with the
  reference's own kernels (projection_algorithm.cu:85-673) run by the same
  driver on a GPU (tests/golden/ref_legacy_kernels.npz);
* the coder's helper templates (HuffmanZSTDCoder.cuh:32-233:
  HuffmanNodeGPU, cudaFrequencyCount, buildHuffmanTree,
  generateCodesRecursive, packBitsKernel) composed by
  tests/coder_helpers_driver.cu as the reference's compress() composes
  them: code tables equal to the reference's on the golden streams, packed
  bytes equal to the encoder's bitstream, and the drop-in class round-trips
  8/16-bit signed and unsigned symbols.
"""
import shutil
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import ref_cases as RC  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
GOLDEN = ROOT / "tests" / "golden"


def build(src: str, out: Path, extra=()) -> Path:
    lib = F.LIB_PATH.parent
    cmd = [NVCC, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           f"-I{ROOT / 'include'}", str(ROOT / "tests" / src),
           f"-L{lib}", "-lffcz", "-Xlinker", f"-rpath,{lib}", "-o", str(out), *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.fixture(scope="module")
def legacy_driver(cuda, tmp_path_factory):
    return build("legacy_kernels_driver.cu", tmp_path_factory.mktemp("drv") / "legacy_kernels_driver")


@pytest.fixture(scope="module")
def coder_driver(cuda, tmp_path_factory):
    return build("coder_helpers_driver.cu", tmp_path_factory.mktemp("drv") / "coder_helpers_driver")


def test_declared_kernels_match_reference_kernels(legacy_driver, tmp_path):
    fx = GOLDEN / "ref_legacy_kernels.npz"
    if not fx.exists():
        pytest.skip("ref_legacy_kernels.npz not generated")
    out = tmp_path / "ours.bin"
    r = subprocess.run([str(legacy_driver), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ours = RC.read_records(out)
    ref = np.load(fx)
    names = sorted(ref.files)
    assert sorted(ours) == names
    # every kernel of the header appears, for both element types
    kernels = {"normalize", "all_abs", "direct", "all_ptw", "partial_ptw", "spatial", "flags", "pack_bools",
               "compact", "cq", "cqa", "reset", "convergence", "dequant", "float_to_complex", "add"}
    for t in ("f32", "f64"):
        assert {n.split(".")[1] for n in names if n.startswith(t + ".")} == kernels
    bad = [n for n in names if not np.array_equal(ours[n], ref[n])]
    assert not bad, bad


def run_coder(driver, tmp_path, kind, symbols):
    src = tmp_path / f"{kind}.bin"
    out = tmp_path / f"{kind}.out"
    np.ascontiguousarray(symbols).tofile(src)
    r = subprocess.run([str(driver), kind, str(src), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    b = out.read_bytes()
    (ne,) = struct.unpack_from("<Q", b, 0)
    tab = np.frombuffer(b, np.dtype([("sym", "<i8"), ("code", "<u4"), ("len", "<i4")]), count=ne, offset=8)
    i = 8 + 16 * ne
    root, nb = struct.unpack_from("<QQ", b, i)
    i += 16
    packed = b[i:i + nb]
    ok = b[i + nb]
    return tab, int(root), packed, bool(ok)


def test_coder_helpers_reproduce_reference_tables(coder_driver, tmp_path, golden_huffman):
    for name, g in golden_huffman.items():
        sym = g["symbols"]
        kind = "u16" if sym.dtype == np.uint16 else "u8"
        tab, root, packed, ok = run_coder(coder_driver, tmp_path, kind, sym)
        assert np.array_equal(tab["sym"], g["ref_sym"].astype(np.int64)), name
        assert np.array_equal(tab["code"], g["ref_code"]), name
        assert np.array_equal(tab["len"], g["ref_len"]), name
        assert root == max(0, 2 * tab.size - 2), name
        bits, _ = O.huffman_bitstream(sym, O.huffman_codebook(sym))
        assert packed == bits, name
        assert ok, name


@pytest.mark.parametrize("kind,dtype", [("i16", np.int16), ("i8", np.int8), ("u16", np.uint16)])
def test_coder_helpers_signed_symbols(coder_driver, tmp_path, kind, dtype):
    """Signed symbols sort by value (the reference's thrust::sort): the
    codebook equals the unsigned one of the order-preserving map v ^ sign."""
    rng = np.random.default_rng(4)
    info = np.iinfo(dtype)
    sym = np.clip(np.round(rng.normal(0, info.max / 8, 50_000)), info.min, info.max).astype(dtype)
    tab, root, packed, ok = run_coder(coder_driver, tmp_path, kind, sym)
    udt = np.uint16 if np.dtype(dtype).itemsize == 2 else np.uint8
    flip = udt(1 << (8 * np.dtype(dtype).itemsize - 1)) if np.issubdtype(dtype, np.signedinteger) else udt(0)
    mapped = sym.view(udt) ^ flip
    book = O.huffman_codebook(mapped)
    bits, _ = O.huffman_bitstream(mapped, book)
    assert packed == bits
    assert np.all(np.diff(tab["sym"]) > 0)
    assert ok
