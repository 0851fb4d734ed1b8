"""Tensor-core DFT stages (FFCZ_DFT_TENSOR): the radix-16 stages of the FP32
strided passes of length 256 and 512 as 16-point DFT matrix products on the
tensor cores (mma.sync, operands split into two TF32 terms, three products,
FP32 accumulation), against the FP64 oracle (the reference loop,
projection_algorithm_impl.cuh:816-858) and against the FP32 (SIMT) passes.

Tolerances: the products keep ~21 bits (against FP32's 24), so e and the
edit accumulators are held to TOL_TC = 1e-4 of the field's scale per
iteration (the SIMT passes' tests use 2e-5); iteration counts within one of
the FP64 loop's (its stop rule compares an absolute violation with 1e-7).
Measured on a GB300: max |e - e_fp64| within 1.6e-5 of max|e0| on these
cases, round trips within 2.3e-6."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

TOL_TC = 1e-4

CASES = [((256, 256, 16), 1.0, F.FFCZ_FORM_FUSED), ((512, 256, 8), 2.0, F.FFCZ_FORM_FUSED),
         ((256, 512, 10), 1.5, F.FFCZ_FORM_PLAIN), ((1, 512, 96), 1.5, F.FFCZ_FORM_FUSED),
         ((1, 256, 40), 1.0, F.FFCZ_FORM_PLAIN), ((256, 6, 20), 2.0, F.FFCZ_FORM_FUSED)]


@pytest.mark.parametrize("shape,c,form", CASES)
def test_tensor_stages_against_fp64_oracle(cuda, shape, c, form):
    fld = synth.make_field(shape, 11 / 3, 12, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, c)
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*fld.shape) as s:
        s.set_form(form)
        s.set_dft_stages(F.FFCZ_DFT_TENSOR)
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        ref = O.solve_all_abs(e0, fld.shape, fld.eps, delta, 100, 1e-7, np.float64)
        # the loop stops on an absolute violation below 1e-7; the ~21-bit
        # products may move a field that sits at that threshold by one
        # iteration against the FP64 loop
        assert abs(it - ref["iterations"]) <= 1, (it, ref["iterations"])
        k = max(1, it, ref["iterations"])
        escale = float(np.abs(e0).max())
        fscale = float(np.abs(np.fft.rfftn(e0.reshape(fld.shape).astype(np.float64))).max())
        e = s.get_results().reshape(-1).astype(np.float64)
        err = float(np.abs(e - ref["e"].reshape(-1)).max())
        assert err <= TOL_TC * escale * k, (err, escale)
        assert np.abs(s.get_freq_edits_full() - ref["freq_edits"]).max() <= TOL_TC * fscale * k
        assert np.abs(s.get_spatial_edits_full() - ref["spatial_edits"]).max() <= TOL_TC * escale * k
        print(f"{shape} form {form}: iterations {it}, max |e - e_fp64| = {err:.3e} ({err / escale:.2e} of max|e0|)")


@pytest.mark.parametrize("shape", [(256, 256, 8), (512, 512, 4), (1, 512, 256)])
def test_tensor_stages_round_trip(cuda, shape):
    """Huge bounds: one forward + inverse returns e0 to the products'
    rounding."""
    e0 = np.random.default_rng(3).standard_normal(int(np.prod(shape))).astype(np.float32)
    with F.ProjectionSolver(*shape) as s:
        s.set_dft_stages(F.FFCZ_DFT_TENSOR)
        s.initialize_all_abs(np.zeros_like(e0), 1e30, 1e30)
        assert s.solve_all_abs(e0, 5, 1e-7) == 1
        e = s.get_results().reshape(-1)
        err = float(np.abs(e - e0).max())
        assert err <= 2e-5 * float(np.abs(e0).max()), err
        print(f"{shape}: round-trip max error {err:.3e}")


def test_tensor_stages_agree_with_simt(cuda):
    fld = synth.make_field((512, 256, 16), 3.0, 2, 1e-4, 1e-4, np.float32)
    e0 = (fld.xp - fld.x).astype(np.float32)
    out = []
    for stages in (F.FFCZ_DFT_SIMT, F.FFCZ_DFT_TENSOR):
        with F.ProjectionSolver(*fld.shape) as s:
            s.set_dft_stages(stages)
            s.initialize_all_abs(fld.x, fld.eps, fld.delta)
            it = s.solve_all_abs(e0, 100, 1e-7)
            out.append((it, s.get_results().reshape(-1)))
    assert out[0][0] == out[1][0]
    assert np.abs(out[0][1] - out[1][1]).max() <= 2e-5 * float(np.abs(e0).max())


def test_tensor_stages_need_fp32_and_a_tensor_axis(cuda):
    with F.ProjectionSolver(256, 256, 8, dtype=np.float64) as s:
        with pytest.raises(F.FFCzError):
            s.set_dft_stages(F.FFCZ_DFT_TENSOR)
    with F.ProjectionSolver(100, 100, 8) as s:
        with pytest.raises(F.FFCzError):
            s.set_dft_stages(F.FFCZ_DFT_TENSOR)
        s.set_dft_stages(F.FFCZ_DFT_SIMT)
