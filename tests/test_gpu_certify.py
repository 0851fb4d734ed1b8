"""The strict finish's certificate: the solver's own transforms plus an
a-posteriori bound on their rounding error decide both bounds without an
FP64 transform when no coefficient is near Delta -- either from the maximum
the last clamp pass recorded (after a converged loop) or from a forward
transform of e.

The bound, B = 16 u L sqrt(N sum e_i^2) (L = sum of ceil(log2 n) over the
axes + 2), is checked against the measured rounding of the solver's own
forward passes (their spectrum of a field, read back through the pointwise
mode's spectrum of x, against numpy's FP64 rfftn): the measured error must
stay below B / MARGIN on smooth, noisy, spiky and single-frequency inputs,
power-of-two and mixed-radix, 1D/2D/3D, FP32 and FP64."""
import math

import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

MARGIN = 4.0


def bound(shape, e, u):
    """16 u L sqrt(N sum e^2), the sum widened as the library widens its
    per-thread partial sums (k terms each in the field's precision)."""
    L = sum(math.ceil(math.log2(n)) if n > 1 else 0 for n in shape) + 2
    n = e.size
    g = min(-(-n // 256), 152 * 16)
    k = math.ceil(n / (g * 256.0))
    widen = (1.0 + (k + 2.0) * u) * 1.001
    return 16.0 * u * L * math.sqrt(n * float(np.sum(e.astype(np.float64) ** 2)) * widen)


def inputs(shape, dtype):
    n = int(np.prod(shape))
    rng = np.random.default_rng(3)
    out = {"gauss": rng.standard_normal(n), "uniform": rng.uniform(-1, 1, n)}
    spike = np.zeros(n)
    spike[n // 3] = 1.0
    out["spike"] = spike
    idx = np.indices(shape).reshape(len(shape), -1).astype(np.float64)
    k = [max(1, s // 5) for s in shape]
    out["tone"] = np.cos(2 * np.pi * sum(k[a] * idx[a] / shape[a] for a in range(len(shape))))
    out["grf"] = synth.grf(shape, 11 / 3, 9, np.float64).reshape(-1) if min(shape) > 1 else rng.standard_normal(n)
    return {name: v.astype(dtype) for name, v in out.items()}


SHAPES = [((64, 64, 64), np.float32), ((3, 250, 500), np.float32), ((1, 96, 1800), np.float32),
          ((1, 1, 4096), np.float32), ((20, 35, 49), np.float32), ((32, 24, 20), np.float64),
          ((1, 100, 250), np.float64)]


@pytest.mark.parametrize("shape,dtype", SHAPES)
def test_bound_covers_the_measured_rounding(cuda, shape, dtype):
    u = 2.0 ** -24 if dtype == np.float32 else 2.0 ** -53
    worst = 0.0
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        for name, e in inputs(shape, dtype).items():
            s.initialize_all_ptw(e, 1.0, 0.05)  # its spectrum of x: the solver's forward passes
            spec = s.get_orig_spectrum().reshape(-1)
            ref = np.fft.rfftn(e.reshape(shape).astype(np.float64)).reshape(-1)
            err = max(np.abs(spec.real - ref.real).max(), np.abs(spec.imag - ref.imag).max())
            B = bound(shape, e, u)
            assert err * MARGIN <= B, (name, err, B)
            worst = max(worst, err / B)
            # the certificate's own numbers on the same e (max_iter 0: e = e0)
            s.initialize_all_abs(np.zeros_like(e), 1e30, 1e30)
            s.solve_all_abs(e, 0, 1e-7)
            c = s.certify_bounds()
            assert c["freq_max"] == max(np.abs(spec.real).max(), np.abs(spec.imag).max())
            assert c["bound"] == pytest.approx(B, rel=1e-5)  # the device sums in the field's precision
            assert c["spatial_max"] == float(np.abs(e).max())
    print(f"{shape} {np.dtype(dtype).name}: worst measured error / bound = {worst:.3g}")


def test_certificate_decides_when_delta_is_far(cuda):
    """The plain small workload (no frequency clamp binds): the strict
    finish is decided by the certificate, and numpy's FP64 check agrees."""
    fld, max_iter = synth.workload("small64")
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*fld.shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, fld.delta)
        s.solve_all_abs(e0, max_iter, 1e-7)
        st = s.strict_finish(max_iter, 1e-7, 4)
        assert st["met"] and st["certified"] and st["rounds"] == 0
        # the loop converged on a frequency projection: the clamp pass's
        # recorded maximum decides without another transform
        assert st["certified_by"] == "recorded clamp maximum"
        chk = O.check_bounds(np.zeros(1), s.get_results(), fld.eps, fld.delta)
        assert chk["spatial_max"] <= fld.eps and chk["freq_max"] <= fld.delta
        assert chk["freq_max"] <= st["freq_max"]  # the certified value bounds the FP64 one
        assert st["spatial_max"] == chk["spatial_max"]


def test_certificate_defers_to_fp64_near_delta(cuda):
    """A stress field whose clamped coefficients sit on Delta: the
    certificate cannot decide, the FP64 check does."""
    fld = synth.make_field((32, 32, 32), 11 / 3, 5, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*fld.shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        st = s.strict_finish(100, 1e-7, 4)
        assert st["met"] and not st["certified"]
        chk = O.check_bounds(np.zeros(1), s.get_results(), fld.eps, float(np.float32(delta)))
        assert chk["freq_max"] <= float(np.float32(delta)) and chk["spatial_max"] <= fld.eps
