"""The reference's other constraint modes on the fused passes -- per-index
bounds (direct, projection_algorithm.cu:93-145) and the pointwise
power-spectrum box over all or listed coefficients (:191-333) -- against
the oracle's restatement.  FP64 cases are compared tightly; FP32 cases are
kept small, since a clamp decision taken at the roundoff level of the
transform (a ratio within ~1e-7 of its bound) can differ between two
correct FP32 implementations."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu


def setup(shape, dtype, seed, c=1.0):
    fld = synth.make_field(shape, 11 / 3, seed, 1e-3, 1e-3, dtype, noise=0.3)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)
    return fld, e0, synth.stress_delta(fld, c)


def H_of(shape):
    return shape[0] * shape[1] * (shape[2] // 2 + 1)


def tol_of(dtype):
    return 2e-5 if dtype == np.float32 else 1e-12


def compare(s, ref, e0, it, dtype):
    assert it == ref["iterations"]
    t = tol_of(dtype) * max(1, it)
    es = float(np.abs(e0).max())
    assert np.abs(s.get_results().reshape(-1) - ref["e"].reshape(-1)).max() <= t * es
    fs = float(np.abs(np.fft.rfftn(e0.astype(np.float64))).max())
    assert np.abs(s.get_freq_edits_full() - ref["freq_edits"]).max() <= t * fs
    assert np.abs(s.get_spatial_edits_full() - ref["spatial_edits"]).max() <= t * es


@pytest.mark.parametrize("shape,dtype", [((16, 24, 10), np.float32), ((64, 64, 64), np.float32),
                                         ((3, 250, 500), np.float32), ((1, 90, 100), np.float64),
                                         ((12, 10, 16), np.float64)])
def test_direct_with_every_index_equals_all_abs(cuda, shape, dtype):
    """One bound Delta on every coefficient is the all-abs mode: same kernels,
    same arithmetic, so the outputs are identical bit for bit."""
    fld, e0, delta = setup(shape, dtype, 3)
    H = H_of(shape)
    out = []
    for direct in (False, True):
        with F.ProjectionSolver(*shape, dtype=dtype) as s:
            if direct:
                s.initialize(fld.x, np.arange(H), np.full(H, delta, dtype), fld.eps)
                it = s.solve(e0, 100, 1e-7)
            else:
                s.initialize_all_abs(fld.x, fld.eps, delta)
                it = s.solve_all_abs(e0, 100, 1e-7)
            out.append((it, s.get_results(), s.get_freq_edits_full(), s.get_spatial_edits_full(),
                        s.get_active_spatial_quant_edit_distances()))
    assert out[0][0] == out[1][0] and out[0][0] > 1
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("shape,dtype", [((16, 24, 10), np.float32), ((8, 12, 10), np.float32),
                                         ((64, 64, 64), np.float64), ((1, 90, 100), np.float64),
                                         ((3, 250, 500), np.float64)])
def test_direct_vs_oracle(cuda, shape, dtype):
    fld, e0, delta = setup(shape, dtype, 5)
    H = H_of(shape)
    rng = np.random.default_rng(9)
    idx = rng.choice(H, H // 3, replace=True)  # with repeats: the smaller bound holds
    dk = (delta * rng.uniform(0.2, 2.0, idx.size)).astype(dtype)
    bounds = O.direct_bounds(shape, idx, dk, dtype)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize(fld.x, idx, dk, fld.eps)
        it = s.solve(e0, 100, 1e-7)
        ref = O.solve_direct(e0, shape, fld.eps, bounds, 100, 1e-7, dtype)
        compare(s, ref, e0, it, dtype)
        assert np.all(s.get_freq_edits_full()[:H][np.isinf(bounds)] == 0)


@pytest.mark.parametrize("shape,dtype,dptw", [((16, 24, 10), np.float32, 0.1), ((64, 64, 64), np.float64, 0.05),
                                              ((1, 90, 100), np.float64, 0.2), ((3, 250, 500), np.float64, 0.1),
                                              ((12, 10, 14), np.float64, 0.02)])
@pytest.mark.parametrize("partial", [False, True])
def test_pointwise_vs_oracle(cuda, shape, dtype, dptw, partial):
    fld, e0, _ = setup(shape, dtype, 7)
    H = H_of(shape)
    rng = np.random.default_rng(11)
    idx = rng.choice(H, max(1, H // 4), replace=False)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        if partial:
            s.initialize_partial_ptw(fld.x, idx, dptw, fld.eps)
        else:
            s.initialize_all_ptw(fld.x, fld.eps, dptw)
        # the spectrum of x the kernels compare against, from the device
        orig = s.get_orig_spectrum()
        ref64 = np.fft.rfftn(fld.x.astype(np.float64)).reshape(-1)
        assert np.abs(orig - ref64).max() <= (2e-6 if dtype == np.float32 else 1e-12) * np.abs(ref64).max()
        mask = None
        if partial:
            mask = np.zeros(H, bool)
            mask[idx[1:]] = True
        it = s.solve(e0, 3, -1.0) if partial else s.solve_all_ptw(e0, 3, -1.0)
        ref = O.solve_ptw(e0, shape, fld.eps, dptw, orig, mask=mask, dc=True, max_iter=3, tol=-1.0, dtype=dtype)
        assert it == 3
        compare(s, ref, e0, it, dtype)
        assert np.any(s.get_freq_edits_full())


def test_mode_errors(cuda):
    shape = (8, 8, 8)
    fld, e0, delta = setup(shape, np.float32, 2)
    with F.ProjectionSolver(*shape) as s:
        with pytest.raises(F.FFCzError):
            s.solve(e0)  # no direct or partial initialiser
        s.initialize_all_abs(fld.x, fld.eps, delta)
        with pytest.raises(F.FFCzError):
            s.solve_all_ptw(e0)
        with pytest.raises(F.FFCzError):
            s.initialize(fld.x, [H_of(shape)], [1.0], fld.eps)  # index past the half spectrum
        s.initialize(fld.x, [0, 5], [1.0, 2.0], fld.eps)
        assert s.solve(e0, 5, 1e-7) >= 1
        # both modes stay available: all-abs still runs with its own bound
        assert s.solve_all_abs(e0, 5, 1e-7) >= 1
