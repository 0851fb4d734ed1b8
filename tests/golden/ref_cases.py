"""Cases of the reference-build fixtures (tests/golden/ref_*.npz), shared by
the script that generates them (make_ref_goldens.py, which runs the
reference's own cuFFT build on a GPU) and the parity tests that read them.

Solve cases are fields of the seeded generator in ffcz_gb300.synth run
through the reference's projection_example.cu sequence; extract cases are
seeded synthetic edit accumulators fed to the reference's
extract_compact_representation and coder.  Everything here is
deterministic: fields come from numpy's PCG64 generators, the synthetic
edits from PCG64's raw 64-bit output, which numpy keeps stable across
versions.
"""
from __future__ import annotations

import hashlib
import struct

import numpy as np

from ffcz_gb300 import synth

# name -> (field builder arguments, delta rule, max_iter, keep the full e)
#   field: (shape, alpha, seed, f_eps, f_delta, dtype, noise)
#   delta: None (the field's own Delta) or c (Delta = c E sqrt(N/6))
SOLVE_CASES = {
    # the plain small workload exactly (64^3, alpha 11/3, seed 0, f_E = f_D = 1e-3)
    "small64": (("workload", "small64"), None, 100, True),
    # the plain FP32 workload at scale exactly (256^3, seed 1, f_E 1e-4, f_D 5e-4, +0.3E noise)
    "plain256": (("workload", "plain256"), None, 100, False),
    # stress variants of the small field: Delta near the noise level, so both boxes bind
    "stress64_c1": ((((64, 64, 64), 11 / 3, 0, 1e-3, 1e-3, "float32", 0.0)), 1.0, 100, False),
    "stress64_c2": ((((64, 64, 64), 11 / 3, 0, 1e-3, 1e-3, "float32", 0.0)), 2.0, 100, False),
    "stress64_c3": ((((64, 64, 64), 11 / 3, 0, 1e-3, 1e-3, "float32", 0.0)), 3.0, 100, False),
    # mixed-radix axes (48 = 2^4 3, 40 = 2^3 5, 36 = 2^2 3^2)
    "mixed48x40x36_c2": ((((48, 40, 36), 11 / 3, 5, 1e-3, 1e-3, "float32", 0.3)), 2.0, 100, True),
    # a 2D field (the CLI's -2 ny nz: cufftPlan3d with Nx = 1)
    "plane90x180_c1p5": ((((90, 180), 2.0, 10, 1e-3, 1e-3, "float32", 0.0)), 1.5, 100, True),
    # FP64 data (D2Z / Z2D plans)
    "f64_32x24x20_c2": ((((32, 24, 20), 11 / 3, 4, 1e-3, 1e-3, "float64", 0.3)), 2.0, 100, True),
}

# name -> (shape, dtype, (freq density, freq scale), (spatial density, spatial scale), seed)
EXTRACT_CASES = {
    # the size and density of the 256^3 workload's spatial edits (7.5%)
    "extract256": ((256, 256, 256), "float32", (0.002, 5e-2), (0.075, 3e-5), 101),
    "extract_f64": ((24, 20, 18), "float64", (0.05, 1e-2), (0.2, 1e-3), 102),
    # a frequency accumulator with sub-threshold entries only: count 0, min/max != 0
    "extract_subthreshold": ((16, 16, 16), "float32", (0.0, 1e-2), (0.1, 1e-3), 103),
}

ZSTD_LEVEL = 20  # projection_example.cu:235-244
TOL = 1e-7       # projection_example.cu:200


def field(case: str):
    """(synth.Field, Delta, max_iter) of a solve case."""
    spec, c, max_iter, _ = SOLVE_CASES[case]
    if spec[0] == "workload":
        fld, mi = synth.workload(spec[1])
        max_iter = mi
    else:
        shape, alpha, seed, fe, fd, dtype, noise = spec
        fld = synth.make_field(shape, alpha, seed, fe, fd, np.dtype(dtype), noise=noise)
    delta = fld.delta if c is None else synth.stress_delta(fld, c)
    return fld, delta, max_iter


def _uniform(bg: np.random.PCG64, n: int) -> np.ndarray:
    """n doubles in [0, 1) from the top 53 bits of PCG64's raw output."""
    return (bg.random_raw(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def synthetic_edits(n: int, density: float, scale: float, seed: int, dtype) -> np.ndarray:
    """A sparse edit accumulator: a `density` fraction of entries with values
    scale * (2u - 1)^3 (concentrated near zero, so the uint16 codes are
    skewed), plus 0.1% of entries below the 1e-7 activity threshold."""
    bg = np.random.PCG64(seed)
    u_pos = _uniform(bg, n)
    u_val = _uniform(bg, n)
    v = 2.0 * u_val - 1.0
    out = np.zeros(n, np.float64)
    act = u_pos < density
    out[act] = scale * v[act] ** 3
    tiny = (u_pos >= density) & (u_pos < density + 1e-3)
    out[tiny] = 0.9e-7 * v[tiny]
    return out.astype(np.dtype(dtype))


def extract_inputs(case: str):
    shape, dtype, (fd, fs), (sd, ss), seed = EXTRACT_CASES[case]
    nx, ny, nz = synth.solver_shape(shape)
    n, h = nx * ny * nz, nx * ny * (nz // 2 + 1)
    fe = synthetic_edits(2 * h, fd, fs, seed, dtype)
    se = synthetic_edits(n, sd, ss, seed + 5000, dtype)
    return (nx, ny, nz), np.dtype(dtype), fe, se


def sample_indices(n: int, k: int = 65536, seed: int = 7) -> np.ndarray:
    """k distinct sorted indices below n (all of them when n <= k)."""
    if n <= k:
        return np.arange(n, dtype=np.int64)
    u = _uniform(np.random.PCG64(seed), 4 * k)
    idx = np.unique((u * n).astype(np.int64))
    return np.sort(idx[:k]) if idx.size >= k else idx


def digest(a) -> str:
    b = a if isinstance(a, (bytes, bytearray)) else np.ascontiguousarray(a).tobytes()
    return hashlib.sha256(b).hexdigest()


def checksums(a: np.ndarray) -> np.ndarray:
    """(sum, sum |a|, sum a^2, max |a|, count of nonzeros) in FP64."""
    a = a.astype(np.float64).reshape(-1)
    return np.array([a.sum(), np.abs(a).sum(), (a * a).sum(), np.abs(a).max() if a.size else 0.0,
                     float(np.count_nonzero(a))])


def read_records(path) -> dict:
    """Records of tests/legacy_kernels_driver.cu: u32 name length, name, u32
    element bytes, u64 byte count, bytes -> {name: uint8 array}."""
    with open(path, "rb") as f:
        b = f.read()
    out, i = {}, 0
    while i < len(b):
        (n,) = struct.unpack_from("<I", b, i)
        i += 4
        name = b[i:i + n].decode()
        i += n
        _, nbytes = struct.unpack_from("<IQ", b, i)
        i += 12
        out[name] = np.frombuffer(b[i:i + nbytes], np.uint8).copy()
        i += nbytes
    return out
