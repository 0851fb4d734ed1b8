"""Compaction of untouched accumulators without a pass: while an
accumulator's dirty flag reads 0 and its records and flag words still hold
the all-zero array's results, a compaction only writes count 0 and min =
max = 0; a listed fold's flag bits are cleared by the next compaction.
Sequences of steps whose accumulators go from untouched to listed (with
other indices each step), written throughout, untouched again, through a
pack-mode switch and a decode, must give the oracle's compaction of the
arrays after every step."""
import numpy as np
import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

SHAPE = (16, 16, 16)
EPS = 1e-2


def check(s, mode=0):
    fe, se = s.get_freq_edits_full(), s.get_spatial_edits_full()
    nf, ns = s.active_counts()
    mm = s.minmax()
    for edits, count, (mn, mx), quant, pack in (
            (fe, nf, mm[:2], s.get_active_freq_quant_edit_distances(), s.get_freq_flags_pack()),
            (se, ns, mm[2:], s.get_active_spatial_quant_edit_distances(), s.get_spatial_flags_pack())):
        ref = O.extract(edits, mode)
        assert count == ref["count"]
        assert (mn, mx) == (ref["min"], ref["max"])
        assert np.array_equal(quant[:count], ref["quant"])
        assert np.array_equal(pack, ref["pack"])
    return nf, ns


def step(s, e0, delta=1e30, strict=True):
    s.reset_edit_accumulators()
    s.initialize_all_abs(np.zeros(e0.size, e0.dtype), EPS, delta)
    s.solve_all_abs(e0, 100, 0.5 * EPS)
    if strict:
        s.strict_finish(100, 0.5 * EPS, 4)


def e0_of(seed, spread, dtype):
    rng = np.random.default_rng(seed)
    return (rng.uniform(-spread, spread, int(np.prod(SHAPE))) * EPS).astype(dtype)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_untouched_listed_written_sequence(cuda, dtype):
    with F.ProjectionSolver(*SHAPE, dtype=dtype) as s:
        quiet = e0_of(1, 0.9, dtype)
        step(s, quiet)
        assert check(s) == (0, 0)
        step(s, quiet)  # the outputs are known clean: no pass
        assert check(s) == (0, 0)
        step(s, e0_of(2, 1.3, dtype))  # listed, active spatial edits
        assert check(s)[1] > 0
        step(s, e0_of(3, 1.3, dtype))  # listed at other indices: the old bits go
        assert check(s)[1] > 0
        step(s, quiet)  # no list: every old bit goes
        assert check(s) == (0, 0)
        # frequency clamps and spatial projections: both written throughout
        step(s, e0_of(4, 1.3, dtype), delta=0.05, strict=False)
        nf, ns = check(s)
        assert nf > 0
        step(s, quiet)
        assert check(s) == (0, 0)
        step(s, quiet)
        assert check(s) == (0, 0)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_listed_values_below_threshold(cuda, dtype):
    # the strict clamp moves a few values by less than the 1e-7 threshold:
    # listed but inactive (count 0, min and max from the small edits)
    rng = np.random.default_rng(10)
    e0 = e0_of(11, 0.9, dtype)
    idx = rng.choice(e0.size, 50, replace=False)
    e0[idx] = (np.where(rng.random(50) < 0.5, -1.0, 1.0) * (EPS + 5e-8)).astype(dtype)
    with F.ProjectionSolver(*SHAPE, dtype=dtype) as s:
        step(s, e0)
        se = s.get_spatial_edits_full()
        assert 0 < np.count_nonzero(se) <= 50 and np.abs(se).max() <= 1e-7
        assert check(s)[1] == 0
        mm = s.minmax()
        assert mm[2] < 0.0 < mm[3]
        step(s, e0_of(12, 1.3, dtype))  # then active listed values
        assert check(s)[1] > 0
        step(s, e0)
        assert check(s)[1] == 0


def test_pack_mode_switch_and_decode(cuda):
    dtype = np.float32
    with F.ProjectionSolver(*SHAPE, dtype=dtype) as s:
        quiet = e0_of(5, 0.9, dtype)
        step(s, e0_of(6, 1.3, dtype))
        assert check(s)[1] > 0
        s.set_pack_mode(F.FFCZ_PACK_REFERENCE)
        step(s, e0_of(7, 1.3, dtype))
        assert check(s, 1)[1] > 0
        step(s, quiet)
        assert check(s, 1) == (0, 0)
        s.set_pack_mode(F.FFCZ_PACK_CORRECT)
        step(s, e0_of(8, 1.3, dtype))
        assert check(s)[1] > 0
        step(s, quiet)
        assert check(s) == (0, 0)
        # a decode writes the flag words; the next compaction of untouched
        # accumulators must not take them for its own
        step(s, e0_of(9, 1.3, dtype))
        streams = s.encode(zstd_level=1)
        mm = s.minmax()
        import torch

        dxp = torch.zeros(int(np.prod(SHAPE)), dtype=torch.float32, device="cuda")
        out = torch.empty_like(dxp)
        s.decode_device(dxp, streams, mm, out)
        step(s, quiet)
        assert check(s) == (0, 0)
