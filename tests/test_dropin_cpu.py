"""Source compatibility of the drop-in headers: the reference's own CLI
(projection_example.cu, compiled from a temporary copy so that its quoted
includes resolve to include/) builds against include/ and links libffcz.so
with no change.  Needs nvcc and the reference sources; skipped without
them.  Also: argument errors of our fftz CLI print the reference's usage."""
import shutil
import subprocess
from pathlib import Path

import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O

ROOT = Path(__file__).resolve().parents[1]
REF = O.reference_sources() or Path("/nonexistent")
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.mark.skipif(not (REF / "projection_example.cu").exists() or not Path(NVCC).exists(),
                    reason="reference sources (FFCZ_REF or baseline/_ref) or nvcc not available")
def test_reference_cli_builds_against_dropin_headers(tmp_path):
    src = tmp_path / "projection_example.cu"
    shutil.copy(REF / "projection_example.cu", src)
    lib = F.LIB_PATH.parent
    exe = tmp_path / "fftz_from_reference_source"
    r = subprocess.run([NVCC, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{ROOT / 'include'}",
                        str(src), f"-L{lib}", "-lffcz", "-Xlinker", f"-rpath,{lib}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    # parsing happens before any CUDA call: a missing file is reported the
    # reference's way (readRawArrayBinary throws "Error opening file")
    r = subprocess.run([str(exe), "-i", str(tmp_path / "missing.bin"), "-e", str(tmp_path / "missing.bin"), "-3", "4",
                        "4", "4", "-f", "-M", "ABS", "0.1", "-F", "ABS", "0.1"], capture_output=True, text=True)
    assert r.returncode != 0 and "Error opening file" in r.stderr


def test_our_cli_usage():
    exe = F.LIB_PATH.parent / "fftz"
    if not exe.exists():
        pytest.skip("fftz not built")
    r = subprocess.run([str(exe), "-q"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "Unknown argument" in r.stdout and "-M ABS <xi>" in r.stdout
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 1 and "are mandatory" in r.stdout
