"""The fftz CLI end to end on files: the reference's flags and output lines,
with counts equal to the library's."""
import re
import subprocess

import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth

pytestmark = pytest.mark.gpu


def test_fftz_matches_library(cuda, tmp_path):
    shape = (24, 20, 16)
    fld = synth.make_field(shape, 11 / 3, 31, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    F.write_raw_array_binary(fld.x, tmp_path / "x.bin")
    F.write_raw_array_binary(fld.xp, tmp_path / "xp.bin")
    exe = F.LIB_PATH.parent / "fftz"
    r = subprocess.run([str(exe), "-i", str(tmp_path / "x.bin"), "-e", str(tmp_path / "xp.bin"), "-3",
                        *map(str, shape), "-f", "-M", "ABS", repr(fld.eps), "-F", "ABS", repr(delta)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    it = int(re.search(r"Total number of iterations: (\d+)", r.stdout).group(1))
    nf = int(re.search(r"# Active frequency edits: (\d+)", r.stdout).group(1))
    ns = int(re.search(r"# Active spatial edits: (\d+)", r.stdout).group(1))
    assert re.search(r"Compression time: \d+ ms", r.stdout) and re.search(r"Decompression time: \d+ ms", r.stdout)
    with F.ProjectionSolver(*shape) as s:
        # the CLI parses eps and delta with stof and subtracts on the host in float
        s.initialize_all_abs(fld.x, float(np.float32(fld.eps)), float(np.float32(delta)))
        it2 = s.solve_all_abs((fld.xp - fld.x).astype(np.float32), 100, float(np.float32(1e-7)))
        assert (it, nf, ns) == (it2, *s.active_counts())


@pytest.mark.parametrize("dims,dt,flag", [(("-3", 24, 20, 16), np.float32, "-f"), (("-2", 30, 50), np.float64, "-d")])
def test_fftz_container_and_decompression(cuda, tmp_path, dims, dt, flag):
    """-z writes the .ffcz container, -o the decoder's x^; decompression
    from the container (no -i) gives the same x^ bit for bit, which matches
    the FP64 reconstruction of the container's streams."""
    from oracle import ffcz_oracle as O

    shape = synth.solver_shape(dims[1:])
    fld = synth.make_field(dims[1:], 11 / 3, 33, 1e-3, 1e-3, dt, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    F.write_raw_array_binary(fld.x, tmp_path / "x.bin")
    F.write_raw_array_binary(fld.xp, tmp_path / "xp.bin")
    exe = str(F.LIB_PATH.parent / "fftz")
    z, o1, o2 = tmp_path / "c.ffcz", tmp_path / "o1.bin", tmp_path / "o2.bin"
    r = subprocess.run([exe, "-i", str(tmp_path / "x.bin"), "-e", str(tmp_path / "xp.bin"), "-z", str(z), "-o",
                        str(o1), *map(str, dims), flag, "-M", "ABS", repr(fld.eps), "-F", "ABS", repr(delta)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    r2 = subprocess.run([exe, "-e", str(tmp_path / "xp.bin"), "-z", str(z), "-o", str(o2)], capture_output=True,
                        text=True, timeout=300)
    assert r2.returncode == 0, r2.stdout + r2.stderr
    assert re.search(r"Decompression time: \d+ ms", r2.stdout)
    a = np.fromfile(o1, dt)
    b = np.fromfile(o2, dt)
    assert np.array_equal(a, b)
    h, streams = F.read_container(z)
    assert h.shape == shape and h.dtype == (F.FFCZ_F32 if dt == np.float32 else F.FFCZ_F64)
    assert abs(h.eps - float(np.float32(fld.eps))) <= 1e-12 * max(1.0, h.eps)
    N = int(np.prod(shape))
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)

    def symbols(r):  # the oracle's sequential decode of one container stream
        book = dict(zip(("symbols", "codes", "lengths"), r.arrays()))
        return O.huffman_decode(r.bitstream, book, r.num_elements)

    assert streams[0] is not None or streams[2] is not None
    fe = (O.unpack_edits(symbols(streams[0]), symbols(streams[1]).astype(np.uint8).tobytes(), 2 * H, h.freq_min,
                         h.freq_max, dt) if streams[0] else np.zeros(2 * H, dt))
    se = (O.unpack_edits(symbols(streams[2]), symbols(streams[3]).astype(np.uint8).tobytes(), N, h.spatial_min,
                         h.spatial_max, dt) if streams[2] else np.zeros(N, dt))
    ref = O.reconstruct(np.fromfile(tmp_path / "xp.bin", dt), shape, fe, se).reshape(-1)
    tol = (2e-6 if dt == np.float32 else 1e-13) * max(1.0, float(np.abs(ref).max()))
    assert np.abs(a.astype(np.float64) - ref).max() <= tol
