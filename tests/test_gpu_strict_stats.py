"""The strict finish after a converged loop clamps e from the per-block
statistics its last z-inverse pass recorded (each block's sum of squares
and max |e|): only the rows of the blocks whose maximum exceeds the limit
are read, instead of a pass over e.  e and the spatial accumulator must
equal numpy's clamp of the values before the finish to the largest value
<= E, with few values above the limit and with more than the accumulator's
index list holds, the reported spatial maximum must be exact, and the
recorded certificate must bound the FP64 spectrum of the clamped e."""
import numpy as np
import pytest

import ffcz_gb300 as F

pytestmark = pytest.mark.gpu


def strict_lim(eps, dtype):
    t = dtype(eps)
    if float(t) > eps:
        t = np.nextafter(t, dtype(0))
    return t


def run(shape, dtype, seed, spread):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    eps = 1e-2
    # |e0| <= spread * E converges in one iteration for tol = 0.5 E when
    # spread < 1.5 (the frequency box is inactive)
    e0 = (rng.uniform(-spread, spread, n) * eps).astype(dtype)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs(np.zeros(n, dtype), eps, 1e30)
        s.reset_edit_accumulators()
        assert s.solve_all_abs(e0, 100, 0.5 * eps) == 1
        e_before = s.get_results().reshape(-1).copy()
        se_before = s.get_spatial_edits_full().copy()
        st = s.strict_finish(100, 0.5 * eps, 4)
        e_after = s.get_results().reshape(-1)
        se_after = s.get_spatial_edits_full()
    lim = strict_lim(eps, dtype)
    over = np.abs(e_before) > lim
    want = np.clip(e_before, -lim, lim)
    want_se = se_before.copy()
    want_se[over] = (se_before[over] + (want[over] - e_before[over])).astype(dtype)
    assert np.array_equal(e_after, want)
    assert np.array_equal(se_after, want_se)
    assert st["met"] and st["rounds"] == 0
    assert st["spatial_max"] == float(np.abs(want).max())
    assert st["certified"]
    spec = np.fft.rfftn(want.astype(np.float64).reshape(shape))
    fm = max(np.abs(spec.real).max(), np.abs(spec.imag).max())
    assert fm <= st["cert_freq_max"] + st["cert_bound"]
    return int(over.sum())


# z lengths 16 and 30 run the runtime-planned z inverse, 64 the
# compile-time one
@pytest.mark.parametrize("shape", [(16, 16, 16), (12, 10, 64)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_strict_clamp_from_zinv_statistics(cuda, dtype, shape):
    # about a fifth of the values above E, every block holds some
    assert 0 < run(shape, dtype, 21, 1.3) <= 4096


@pytest.mark.parametrize("shape", [(40, 36, 30), (24, 24, 64)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_strict_clamp_many_values(cuda, dtype, shape):
    # about a fifth above E: more than the accumulator's list holds
    assert run(shape, dtype, 22, 1.3) > 4096


def test_strict_clamp_nothing_above_limit(cuda):
    assert run((24, 20, 18), np.float32, 23, 0.9) == 0


def test_strict_clamp_odd_z(cuda):
    assert run((10, 12, 15), np.float32, 24, 1.3) > 0
