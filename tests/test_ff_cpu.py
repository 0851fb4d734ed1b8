"""Float-float arithmetic of the split-precision FP64 kernels (ff in
ffcz_gb300/csrc/common.cuh), compiled for the host from the same header and
checked against FP64 on a million random operand pairs spanning 12 decades:
conversion, sum and product each within 2^-45 relative (the sum relative to
|a| + |b|), and exact round trips of values that fit in 48 bits."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"

SRC = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "common.cuh"
using namespace ffcz;
int main() {
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1, 1);
  double wc = 0, wa = 0, wm = 0;
  for (int i = 0; i < 1000000; ++i) {
    const double a = u(g) * std::pow(10.0, (int)(u(g) * 6)), b = u(g) * std::pow(10.0, (int)(u(g) * 6));
    const ff A(a), B(b);
    wc = std::fmax(wc, std::fabs(ff_to_double(A) - a) / std::fabs(a));
    wa = std::fmax(wa, std::fabs(ff_to_double(A + B) - (a + b)) / (std::fabs(a) + std::fabs(b)));
    wm = std::fmax(wm, std::fabs(ff_to_double(A * B) - a * b) / std::fabs(a * b));
    int ex = 0;
    const double m = std::frexp(a, &ex);
    const double c = std::ldexp(std::round(std::ldexp(m, 48)), ex - 48);  // 48 significant bits
    if (ff_to_double(ff(c)) != c) { std::printf("roundtrip %.17g\n", c); return 2; }
  }
  std::printf("%.6e %.6e %.6e\n", wc, wa, wm);
  return 0;
}
"""


@pytest.mark.skipif(not Path(NVCC).exists(), reason="nvcc not available")
def test_float_float_arithmetic(tmp_path):
    src = tmp_path / "ff_check.cu"
    src.write_text(SRC)
    exe = tmp_path / "ff_check"
    r = subprocess.run([NVCC, "-std=c++17", "-O2", str(src), "-o", str(exe), f"-I{ROOT / 'include'}",
                        f"-I{ROOT / 'ffcz_gb300' / 'csrc'}"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    conv, add, mul = map(float, r.stdout.split())
    bound = 2.0 ** -45
    assert conv <= bound and add <= bound and mul <= bound, (conv, add, mul)
