"""Listed spatial accumulators: after a solve that converged without
writing the spatial accumulator, the strict finish's clamp records the
entries it writes in a short list instead of marking the whole array; the
compaction then folds the listed values in without reading the array, and
the reset zeroes only them.  The results must equal the oracle's
compaction of the final arrays, the reset must leave zeros, and a second
step must repeat the first bit for bit -- including when every entry is
listed (no implicit zeros in the min and max)."""
import numpy as np
import pytest

import ffcz_gb300 as F
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu


def one_step(s, e0, eps):
    s.reset_edit_accumulators()
    it = s.solve_all_abs(e0, 100, 0.5 * eps)  # converges in one iteration: |e| <= 1.3 E < E + tol
    st = s.strict_finish(100, 0.5 * eps, 4)
    se = s.get_spatial_edits_full()
    out = (it, st["met"], s.active_counts(), s.minmax(), s.get_active_spatial_quant_edit_distances(),
           s.get_spatial_flags_pack(), s.get_active_spatial_edit_distances())
    return out, se


def check(shape, dtype, e0, eps):
    n = int(np.prod(shape))
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs(np.zeros(n, dtype), eps, 1e30)
        first, se = one_step(s, e0, eps)
        assert first[0] == 1 and first[1]
        nz = int(np.count_nonzero(se))
        assert 0 < nz <= 4096, nz  # the list cannot overflow: the listed path ran
        ref = O.extract(se)
        assert first[2][1] == ref["count"] > 0
        assert first[3][2:] == (ref["min"], ref["max"])
        assert np.array_equal(first[4], ref["quant"])
        assert np.array_equal(first[5], ref["pack"])
        assert np.array_equal(first[6], ref["compact"])
        s.reset_edit_accumulators()
        assert not s.get_spatial_edits_full().any()
        second, se2 = one_step(s, e0, eps)
        assert np.array_equal(se, se2)
        for a, b in zip(first, second):
            if isinstance(a, np.ndarray):
                assert np.array_equal(a, b)
            else:
                assert a == b


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_listed_accumulator_some_entries(cuda, dtype):
    rng = np.random.default_rng(12)
    eps = 1e-2
    e0 = (rng.uniform(-1.3, 1.3, 16 ** 3) * eps).astype(dtype)
    check((16, 16, 16), dtype, e0, eps)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_listed_accumulator_every_entry(cuda, dtype):
    rng = np.random.default_rng(13)
    eps = 1e-2
    shape = (3, 5, 7)
    e0 = (np.where(rng.random(105) < 0.5, -1.0, 1.0) * rng.uniform(1.1, 1.2, 105) * eps).astype(dtype)
    check(shape, dtype, e0, eps)
