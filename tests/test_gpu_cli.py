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
