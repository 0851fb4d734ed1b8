"""The plain form (six HBM passes per 3D iteration: the x forward pass
stores the clamped spectrum and the x inverse is a pass of its own; in 2D
the same on y) against the fused form and the oracle.  Both compute the
reference's iteration (projection_algorithm_impl.cuh:201-249, 816-858); the
plain passes use other stage lists than the fused pass, so the two agree to
FP32 rounding, with the same iteration counts."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

TOL = 2e-5

CASES = [((64, 64, 64), 1.0), ((32, 48, 20), 2.0), ((1, 90, 100), 1.5), ((4, 100, 200), 2.0),
         ((2, 384, 768), 1.0), ((20, 35, 49), 2.0), ((1, 1, 4096), 1.0), ((512, 8, 6), 1.5)]


def solve(fld, delta, form, dtype=np.float32):
    e0 = (fld.xp - fld.x).astype(dtype)
    s = F.ProjectionSolver(*fld.shape, dtype=dtype)
    s.set_form(form)
    s.initialize_all_abs(fld.x, fld.eps, delta)
    it = s.solve_all_abs(e0, 100, 1e-7)
    out = (it, s.get_results().reshape(-1), s.get_freq_edits_full(), s.get_spatial_edits_full(), s.active_counts())
    s.close()
    return e0, out


@pytest.mark.parametrize("shape,c", CASES)
def test_plain_form_matches_fused_and_oracle(cuda, shape, c):
    fld = synth.make_field(shape, 11 / 3, 7, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, c)
    e0, (itp, ep, fep, sep, cp) = solve(fld, delta, F.FFCZ_FORM_PLAIN)
    _, (itf, ef, fef, sef, cf) = solve(fld, delta, F.FFCZ_FORM_FUSED)
    ref = O.solve_all_abs(e0, fld.shape, fld.eps, delta, 100, 1e-7, np.float32)
    assert itp == itf == ref["iterations"]
    escale = float(np.abs(e0).max())
    fscale = float(np.abs(np.fft.rfftn(e0.reshape(fld.shape).astype(np.float64))).max())
    k = max(1, itp)
    for e in (ep, ef):
        assert np.abs(e - ref["e"].reshape(-1)).max() <= TOL * escale * k
    assert np.abs(fep - ref["freq_edits"]).max() <= TOL * fscale * k
    assert np.abs(sep - ref["spatial_edits"]).max() <= TOL * escale * k
    assert np.abs(ep - ef).max() <= 2 * TOL * escale * k


def test_plain_form_pass_count(cuda):
    """Six timed passes per 3D iteration in the plain form, five fused."""
    fld = synth.make_field((32, 32, 32), 11 / 3, 1, 1e-3, 1e-3, np.float32)
    e0 = (fld.xp - fld.x).astype(np.float32)
    for form, npass in ((F.FFCZ_FORM_PLAIN, 6), (F.FFCZ_FORM_FUSED, 5)):
        with F.ProjectionSolver(*fld.shape) as s:
            s.set_form(form)
            s.set_profiling(True)
            s.initialize_all_abs(fld.x, fld.eps, fld.delta)
            s.solve_all_abs(e0, 100, 1e-7)
            assert len(s.pass_times()) == npass


def test_form_rejects_unknown_value(cuda):
    with F.ProjectionSolver(8, 8, 8) as s:
        with pytest.raises(F.FFCzError):
            s.set_form(7)
