"""On-demand extraction: a solve that leaves its compaction pending gives,
call for call, what the eager (reference) mode gives -- after a plain
solve, after the strict finish (which changes the edit arrays), across a
reset that clears the arrays the pending compaction describes, and
through the encoder."""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPE = (40, 36, 30)


def field(c=1.5):
    fld = synth.make_field(SHAPE, 11 / 3, 23, 1e-3, 1e-3, np.float32, noise=0.3)
    return fld, synth.stress_delta(fld, c), (fld.xp - fld.x).astype(np.float32)


def snapshot(s):
    return (s.active_counts(), s.minmax(), s.get_active_freq_quant_edit_distances(),
            s.get_active_spatial_quant_edit_distances(), s.get_freq_flags_pack(), s.get_spatial_flags_pack())


def same(a, b):
    for x, y in zip(a, b):
        if isinstance(x, np.ndarray):
            assert x.dtype == y.dtype and np.array_equal(x, y)
        else:
            assert x == y


@pytest.mark.parametrize("strict", [False, True])
def test_on_demand_equals_eager(cuda, strict):
    fld, delta, e0 = field()
    out = []
    for mode in (F.FFCZ_EXTRACT_EAGER, F.FFCZ_EXTRACT_ON_DEMAND):
        with F.ProjectionSolver(*SHAPE) as s:
            s.set_extraction(mode)
            s.initialize_all_abs(fld.x, fld.eps, delta)
            it = s.solve_all_abs(e0, 100, 1e-7)
            st = s.strict_finish(100, 1e-7, 4) if strict else None
            snap = snapshot(s)
            streams = s.encode(zstd_level=3)
            out.append((it, st, snap, [None if r is None else (r.bitstream, r.compressed_data) for r in streams]))
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]
    same(out[0][2], out[1][2])
    assert out[0][3] == out[1][3]
    assert out[0][2][0][0] > 0 and out[0][2][0][1] > 0  # both accumulators hold edits


def test_pending_compaction_runs_before_reset(cuda):
    """Reset clears the arrays a pending compaction describes: it runs
    first, so the getters afterwards return the solve's results, as in the
    eager mode."""
    fld, delta, e0 = field()
    snaps = []
    for mode in (F.FFCZ_EXTRACT_EAGER, F.FFCZ_EXTRACT_ON_DEMAND):
        with F.ProjectionSolver(*SHAPE) as s:
            s.set_extraction(mode)
            s.initialize_all_abs(fld.x, fld.eps, delta)
            s.solve_all_abs(e0, 100, 1e-7)
            s.reset_edit_accumulators()
            snaps.append(snapshot(s))
            assert not s.get_freq_edits_full().any()
    same(*snaps)


def test_set_extraction_rejects_unknown_mode(cuda):
    with F.ProjectionSolver(*SHAPE) as s:
        with pytest.raises(F.FFCzError):
            s.set_extraction(5)
