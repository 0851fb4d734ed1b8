"""Generates the golden fixtures in tests/golden/ from the reference itself.

Needs the reference sources (FFCZ_REF: the directory holding them) and nvcc:
oracle/build_ref.sh compiles the reference's Huffman host code
(HuffmanZSTDCoder.cuh:48-178, 378-450, thrust on its CPP backend) and
fileIO.cpp into oracle/_ref/ref_harness.  For each symbol stream below the
fixture stores the stream, the reference's code table, and whether the
reference decoder (SimpleCudaHuffmanZstdCompressor<T>::decompress) decodes
the oracle's bitstream back to the stream; plus one code-table file written
by the reference's writeMap.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import ffcz_oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"
TAB = np.dtype([("sym", "<u4"), ("code", "<u4"), ("len", "<i4")])


def cases() -> dict:
    rng = np.random.default_rng(20261203)
    fib = [1, 1]
    while len(fib) < 25:
        fib.append(fib[-1] + fib[-2])
    sparse_bytes = ((rng.random(40000) < 0.1) * rng.integers(0, 256, 40000)).astype(np.uint8)
    bitmap = np.packbits(rng.random(200000) < 0.075, bitorder="little")
    return {
        # the reference's own (commented-out) round-trip example, HuffmanZSTDCoder.cuh:475
        "ref_example": np.array([1, 2, 3, 1, 2, 1, 4, 5, 1, 2, 3, 3, 3], np.uint16),
        "single_symbol": np.full(50, 7, np.uint16),
        "two_symbols": np.array([3, 3, 3, 9], np.uint16),
        "equal_counts": np.repeat(np.arange(16, dtype=np.uint16), 5),
        "geometric": np.minimum(rng.geometric(0.05, 60000), 65535).astype(np.uint16),
        "near_uniform16": rng.integers(0, 65536, 60000).astype(np.uint16),
        "fibonacci_24bit": np.repeat(np.arange(25, dtype=np.uint16), fib[:25]),
        "clustered16": np.clip(np.round(rng.normal(32768, 900, 50000)), 0, 65535).astype(np.uint16),
        "sparse_bytes": sparse_bytes,
        "flag_bitmap": bitmap,
        "all_byte_values": np.arange(256, dtype=np.uint8).repeat(3),
    }


def main() -> None:
    subprocess.run([str(ROOT / "oracle" / "build_ref.sh")], check=True)
    data = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for name, sym in cases().items():
            t = "u8" if sym.dtype == np.uint8 else "u16"
            sym.tofile(td / "sym.bin")
            subprocess.run([str(HARNESS), "book", t, str(td / "sym.bin"), str(td / "tab.bin")], check=True)
            tab = np.fromfile(td / "tab.bin", dtype=TAB)
            book = O.huffman_codebook(sym)
            bits, nbits = O.huffman_bitstream(sym, book)
            (td / "bits.bin").write_bytes(bits)
            subprocess.run([str(HARNESS), "decode", t, str(td / "bits.bin"), str(td / "tab.bin"), str(sym.size),
                            str(td / "dec.bin")], check=True)
            dec = np.fromfile(td / "dec.bin", dtype=sym.dtype)
            data[f"{name}__symbols"] = sym
            data[f"{name}__ref_sym"] = tab["sym"]
            data[f"{name}__ref_code"] = tab["code"]
            data[f"{name}__ref_len"] = tab["len"]
            data[f"{name}__ref_decodes_oracle_bits"] = np.array(np.array_equal(dec, sym))
            data[f"{name}__nbits"] = np.array(nbits)
        # writeMap of the geometric table, as the reference writes it
        tab_g = np.stack([data["geometric__ref_sym"], data["geometric__ref_code"],
                          data["geometric__ref_len"].view(np.uint32)], axis=1).astype(np.uint32)
        tab_g.tofile(td / "tab.bin")
        subprocess.run([str(HARNESS), "map", str(td / "tab.bin"), str(td / "ref.map")], check=True)
        data["geometric__ref_map_bytes"] = np.frombuffer((td / "ref.map").read_bytes(), np.uint8)
    np.savez_compressed(OUT / "huffman_reference.npz", **data)
    print(OUT / "huffman_reference.npz", sum(v.nbytes for v in data.values()), "bytes")


if __name__ == "__main__":
    main()
