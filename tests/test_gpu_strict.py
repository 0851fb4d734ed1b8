"""Strict bounds, an addition to the reference schedule (which stops once
the spatial violation is below tol, projection_algorithm_impl.cuh:845-848):
after ffcz_strict_finish both bounds hold in FP64 with no tolerance,
|e_i| <= E and |Re/Im rfftn(e)_k| <= Delta, as the oracle's FP64 checker
computes them; the edit arrays still rebuild e the way the decoder does, and
the compaction describes the final edits."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu


def setup(shape, dtype, seed, c):
    fld = synth.make_field(shape, 11 / 3, seed, 1e-3, 1e-3, dtype, noise=0.3)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)
    return fld, e0, synth.stress_delta(fld, c)


CASES = [((24, 20, 16), np.float32, 1.5), ((64, 64, 64), np.float32, 1.0), ((3, 250, 500), np.float32, 1.0),
         ((1, 90, 100), np.float64, 1.0), ((12, 10, 16), np.float64, 2.0), ((32, 32, 32), np.float32, 1e3)]


@pytest.mark.parametrize("shape,dtype,c", CASES)
def test_strict_finish_meets_both_bounds_in_fp64(cuda, shape, dtype, c):
    fld, e0, delta = setup(shape, dtype, 5, c)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        before = O.check_bounds(np.zeros(1), s.get_results(), float(dtype(fld.eps)), float(dtype(delta)))
        st = s.strict_finish(100, 1e-7, 4)
        e = s.get_results().astype(np.float64)
        # the bounds as the solver holds them (rounded to its type, like the
        # reference CLI's stof)
        E, D = float(dtype(fld.eps)), float(dtype(delta))
        chk = O.check_bounds(np.zeros(1), e, E, D)
        assert st["met"], (st, chk)
        assert chk["spatial_max"] <= E and chk["freq_max"] <= D
        assert st["spatial_max"] == chk["spatial_max"]
        if st["certified"]:  # the certificate's value bounds the FP64 one
            assert chk["freq_max"] <= st["freq_max"] <= D
        else:
            assert abs(st["freq_max"] - chk["freq_max"]) <= 1e-12 * D
        if before["spatial_excess"] <= 0 and before["freq_excess"] <= 0:
            assert st["rounds"] == 0
        if before["freq_excess"] > 0:
            assert st["rounds"] >= 1
        assert s.iterations >= it
        # e = e0 + C2R(freq edits)/N + spatial edits
        fe, se = s.get_freq_edits_full(), s.get_spatial_edits_full()
        rec = O.reconstruct(e0, s.shape, fe, se).reshape(-1)
        t = (2e-5 if dtype == np.float32 else 1e-12) * max(1, s.iterations) * float(np.abs(e0).max())
        assert np.abs(rec - e.reshape(-1)).max() <= t
        # the compaction was redone on the final edits
        assert s.active_counts() == (O.extract(fe)["count"], O.extract(se)["count"])


def test_strict_case_is_not_vacuous(cuda):
    """The FP32 stress case exceeds a bound in FP64 under the reference
    schedule (frequency clamps land on Delta up to the transform's rounding)."""
    fld, e0, delta = setup((24, 20, 16), np.float32, 5, 1.5)
    with F.ProjectionSolver(24, 20, 16) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        assert s.active_counts()[0] > 0
        b = O.check_bounds(np.zeros(1), s.get_results(), float(np.float32(fld.eps)), float(np.float32(delta)))
        assert b["spatial_excess"] > 0 or b["freq_excess"] > 0


def test_strict_zero_rounds_clamps_only(cuda):
    """max_rounds 0: the clamp and the check only; the spatial bound holds."""
    fld, e0, delta = setup((24, 20, 16), np.float32, 6, 1.5)
    with F.ProjectionSolver(24, 20, 16) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        st = s.strict_finish(100, 1e-7, 0)
        assert st["rounds"] == 0 and s.iterations == it
        assert float(np.abs(s.get_results().astype(np.float64)).max()) <= float(np.float32(fld.eps))
        assert st["met"] == (st["freq_max"] <= float(np.float32(delta)))


def test_strict_needs_an_all_abs_solve(cuda):
    fld, e0, delta = setup((12, 10, 16), np.float32, 7, 1.0)
    with F.ProjectionSolver(12, 10, 16) as s:
        with pytest.raises(F.FFCzError) as ei:
            s.strict_finish()
        assert ei.value.code == -4  # not initialised
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.initialize_all_ptw(fld.x, fld.eps, 0.5)
        s.solve_all_ptw(e0, 10, 1e-7)
        with pytest.raises(F.FFCzError) as ei:
            s.strict_finish()
        assert ei.value.code == -1  # the pointwise box is not the all-abs box


@pytest.mark.parametrize("c", [1e3, 1.0])
def test_split_precision_strict_finish(cuda, c):
    """FP64 fields on the float-float passes: the fused pass records an upper
    bound of the clamped spectrum's |Re|, |Im| (|hi| + |lo| rounded up), so
    after a loop that converged well inside the frequency box the strict
    finish certifies both bounds from it without an FP64 transform (c = 1e3:
    no coefficient reaches the box); with clamps at the bound (c = 1) it
    decides otherwise.  Either way both
    bounds hold under the oracle's numpy FP64 check."""
    shape = (8, 128, 256)
    fld, e0, delta = setup(shape, np.float64, 23, c)
    with F.ProjectionSolver(*shape, dtype=np.float64) as s:
        s.set_precision(F.FFCZ_PRECISION_SPLIT)
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        st = s.strict_finish(100, 1e-7, 4)
        e = s.get_results()
    chk = O.check_bounds(np.zeros(1), e, fld.eps, delta)
    assert st["met"] and chk["spatial_max"] <= fld.eps and chk["freq_max"] <= delta, (st, chk)
    if c > 10:
        assert st["certified_by"] == "recorded clamp maximum", st
        # the recorded maximum plus the rounding bound covers the final spectrum
        assert st["cert_freq_max"] + st["cert_bound"] >= chk["freq_max"]
