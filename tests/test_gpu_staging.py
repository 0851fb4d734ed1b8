"""TMA-staged strided passes: the persistent kernels fed by tensor-map
copies compute what the register-staged kernels compute, in the same
order, so every output is bit-identical -- for every constraint mode, both
forms, power-of-two and mixed-radix lengths, partial last tiles (Nz/2 + 1
not a multiple of the tile width), 2D fields (fused y pass) and both tile
variants.  The register path itself is checked against the oracle and the
reference's own cuFFT build elsewhere."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth

pytestmark = pytest.mark.gpu

# (shape, what it covers)
SHAPES = [
    ((64, 64, 64), "64-point x and y"),
    ((128, 96, 30), "x 128, Hz 16 (full tiles)"),
    ((256, 40, 34), "x 256, Hz 18 (partial last tile, zero-filled columns)"),
    ((512, 24, 20), "x 512 fused [8,8,8], Hz 11"),
    ((24, 512, 18), "y 512 plain [16,16,2]"),
    ((16, 1024, 32), "y 1024"),
    ((100, 40, 26), "x 100 mixed radix"),
    ((12, 500, 40), "y 500 mixed radix"),
    ((1, 1800, 24), "2D, fused y pass of 1800"),
    ((1, 256, 64), "2D, fused y pass of 256"),
]


def solve(shape, staging, form=F.FFCZ_FORM_FUSED, mode="abs", c=1.5, seed=31):
    fld = synth.make_field(shape, 11 / 3, seed, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, c)
    e0 = (fld.xp - fld.x).astype(np.float32)
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)
    with F.ProjectionSolver(*shape) as s:
        s.set_form(form)
        if mode == "abs":
            s.initialize_all_abs(fld.x, fld.eps, delta)
        elif mode == "direct":
            bound = np.full(H, delta, np.float32)
            bound[::3] = delta / 2
            s.initialize(fld.x, np.arange(H), bound, fld.eps)
        else:
            s.initialize_all_ptw(fld.x, fld.eps, 0.05)
        s.set_staging(staging)
        if staging == F.FFCZ_STAGING_TMA:
            ch = s.tuning()["choice"]
            assert ch["y"][1] or ch["x"][1], ch
        if mode == "abs":
            it = s.solve_all_abs(e0, 100, 1e-7)
        elif mode == "direct":
            it = s.solve(e0, 100, 1e-7)
        else:
            it = s.solve_all_ptw(e0, 3, -1.0)
        return (it, s.get_results(), s.get_freq_edits_full(), s.get_spatial_edits_full(),
                s.active_counts(), s.get_active_freq_quant_edit_distances(),
                s.get_active_spatial_quant_edit_distances())


def same(a, b):
    assert a[0] == b[0], (a[0], b[0])
    for x, y in zip(a[1:], b[1:]):
        if isinstance(x, np.ndarray):
            assert x.shape == y.shape and np.array_equal(x.view(np.uint8), y.view(np.uint8))
        else:
            assert x == y


@pytest.mark.parametrize("shape,what", SHAPES, ids=[w for _, w in SHAPES])
def test_tma_staging_bit_identical(cuda, shape, what):
    reg = solve(shape, F.FFCZ_STAGING_REGISTERS)
    tma = solve(shape, F.FFCZ_STAGING_TMA)
    assert reg[4][0] > 0, "frequency clamps must fire for the test to mean something"
    same(reg, tma)


@pytest.mark.parametrize("shape", [(512, 24, 20), (24, 512, 18), (64, 64, 64), (100, 40, 26)])
def test_tma_staging_plain_form(cuda, shape):
    """The six-pass form: forward-with-clamp and inverse passes staged."""
    same(solve(shape, F.FFCZ_STAGING_REGISTERS, F.FFCZ_FORM_PLAIN), solve(shape, F.FFCZ_STAGING_TMA, F.FFCZ_FORM_PLAIN))


@pytest.mark.parametrize("mode", ["direct", "ptw"])
@pytest.mark.parametrize("shape", [(64, 64, 64), (1, 256, 64)])
def test_tma_staging_other_constraint_modes(cuda, shape, mode):
    same(solve(shape, F.FFCZ_STAGING_REGISTERS, mode=mode), solve(shape, F.FFCZ_STAGING_TMA, mode=mode))


def test_autotune_with_staging_keeps_results(cuda):
    """The autotuner chooses among register and staged kernels of both tile
    widths; whatever it keeps gives the same bits."""
    shape = (256, 40, 34)
    fld = synth.make_field(shape, 11 / 3, 5, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = (fld.xp - fld.x).astype(np.float32)
    out = []
    for tune in (False, True):
        with F.ProjectionSolver(*shape) as s:
            s.initialize_all_abs(fld.x, fld.eps, delta)
            if tune:
                ms = s.autotune(3)
                assert ms["x_tma"][0] > 0, ms  # (y = 40 has no compile-time kernel)
            it = s.solve_all_abs(e0, 100, 1e-7)
            out.append((it, s.get_results(), s.get_freq_edits_full(), s.get_spatial_edits_full()))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)


def test_staging_rejected_where_unavailable(cuda):
    with F.ProjectionSolver(8, 8, 8, dtype=np.float64) as s:
        with pytest.raises(F.FFCzError):
            s.set_staging(F.FFCZ_STAGING_TMA)
        s.set_staging(F.FFCZ_STAGING_REGISTERS)
    with F.ProjectionSolver(7, 11, 16) as s:  # no compile-time strided kernels
        with pytest.raises(F.FFCzError):
            s.set_staging(F.FFCZ_STAGING_TMA)
        with pytest.raises(F.FFCzError):
            s.set_staging(7)
