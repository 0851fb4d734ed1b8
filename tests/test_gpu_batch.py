"""Batched form: fields of uneven shapes corrected in one graph launch, each
field in a device-side loop of its own that retires when it converges.

Every field's outputs (iterations, e, both edit accumulators, the compacted
streams, flag packs and min/max) must equal, bit for bit, a single-field
solve of the same field on a handle of its own; the single-field path is in
turn checked against the oracle (test_gpu_solver.py), and the iteration
counts here are checked against the oracle directly.
"""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

# shape, stress factor c (delta = c * E * sqrt(N/6)), dtype
FIELDS = [((1, 36, 60), 1.0, np.float32), ((10, 20, 24), 2.0, np.float32), ((16, 16, 16), 1.0, np.float32),
          ((16, 16, 16), 3.0, np.float32), ((8, 12, 10), 1.5, np.float32), ((12, 10, 16), 1.0, np.float64),
          ((1, 1, 64), 1.0, np.float32), ((20, 9, 14), 1e6, np.float32)]


def make_fields(cuda, fields=FIELDS, seed0=40):
    out = []
    for i, (shape, c, dt) in enumerate(fields):
        fld = synth.make_field(shape, 11 / 3, seed0 + i, 1e-3, 1e-3, dt, noise=0.3)
        delta = synth.stress_delta(fld, c)
        dx = cuda.from_numpy(np.ascontiguousarray(fld.x.reshape(-1))).cuda()
        dxp = cuda.from_numpy(np.ascontiguousarray(fld.xp.reshape(-1))).cuda()
        out.append((fld, delta, dx, dxp))
    return out


def outputs(s):
    return {"e": s.get_results(), "fe": s.get_freq_edits_full(), "se": s.get_spatial_edits_full(),
            "counts": s.active_counts(), "minmax": s.minmax(),
            "fq": s.get_active_freq_quant_edit_distances(), "sq": s.get_active_spatial_quant_edit_distances(),
            "fc": s.get_active_freq_edit_distances(), "sc": s.get_active_spatial_edit_distances(),
            "fp": s.get_freq_flags_pack(), "sp": s.get_spatial_flags_pack()}


def assert_same(a, b, what):
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert a[k].dtype == b[k].dtype and np.array_equal(a[k], b[k]), (what, k)
        else:
            assert a[k] == b[k], (what, k)


def solvers_for(fields):
    out = []
    for fld, delta, _, _ in fields:
        s = F.ProjectionSolver(*fld.shape, dtype=fld.x.dtype)
        s.initialize_all_abs(fld.x, fld.eps, delta)
        out.append(s)
    return out


def test_batch_equals_single_field_solves(cuda):
    fields = make_fields(cuda)
    batch_solvers = solvers_for(fields)
    with F.Batch(batch_solvers) as b:
        its = b.solve_pair_device([f[2] for f in fields], [f[3] for f in fields], 100, 1e-7)
        got = [outputs(s) for s in batch_solvers]
        # a second launch of the cached graph gives the same outputs
        b.reset_edit_accumulators()
        assert b.solve_pair_device([f[2] for f in fields], [f[3] for f in fields], 100, 1e-7) == its
        for s, g in zip(batch_solvers, got):
            assert_same(g, outputs(s), "relaunch")
    assert len(set(its)) > 1, its  # fields retire at different iterations
    for i, ((fld, delta, dx, dxp), g) in enumerate(zip(fields, got)):
        with F.ProjectionSolver(*fld.shape, dtype=fld.x.dtype) as s:
            s.initialize_all_abs(fld.x, fld.eps, delta)
            assert s.solve_all_abs_pair_device(dx, dxp, 100, 1e-7) == its[i]
            assert_same(outputs(s), g, f"field {i} {fld.shape}")
        e0 = (fld.xp - fld.x).astype(fld.x.dtype)
        ref = O.solve_all_abs(e0, fld.shape, fld.eps, delta, 100, 1e-7, fld.x.dtype)
        assert its[i] == ref["iterations"], (i, fld.shape)
        escale = float(np.abs(e0).max())
        assert np.abs(g["e"].reshape(-1) - ref["e"].reshape(-1)).max() <= 2e-5 * escale * max(1, its[i])
    for s in batch_solvers:
        s.close()


def test_batch_rebuilds_on_new_bounds_and_encodes(cuda):
    fields = make_fields(cuda, FIELDS[:4], seed0=70)
    ss = solvers_for(fields)
    b = F.Batch(ss)
    xs, xps = [f[2] for f in fields], [f[3] for f in fields]
    b.solve_pair_device(xs, xps, 100, 1e-7)
    # new bounds for field 1: the graph is rebuilt
    fld, delta, dx, dxp = fields[1]
    ss[1].initialize_all_abs(fld.x, fld.eps, 2 * delta)
    for s in ss:
        s.reset_edit_accumulators()
    its = b.solve_pair_device(xs, xps, 100, 1e-7)
    with F.ProjectionSolver(*fld.shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, 2 * delta)
        assert s.solve_all_abs_pair_device(dx, dxp, 100, 1e-7) == its[1]
        assert_same(outputs(s), outputs(ss[1]), "rebuilt")
        enc_single = s.encode(3)
    enc_batch = ss[1].encode(3)
    assert [r and r.compressed_data for r in enc_single] == [r and r.compressed_data for r in enc_batch]
    # max_iter 1: fields stopped by max_iter get the final spatial clamp
    for s in ss:
        s.reset_edit_accumulators()
    assert b.solve_pair_device(xs, xps, 1, 1e-7) == [1] * 4
    for (fld, delta, dx, dxp), s in zip(fields, ss):
        e = s.get_results().reshape(-1)
        assert float(np.abs(e).max()) <= float(np.float32(fld.eps)) + 1e-7
    fld, delta, dx, dxp = fields[0]
    with F.ProjectionSolver(*fld.shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        assert s.solve_all_abs_pair_device(dx, dxp, 1, 1e-7) == 1
        assert_same(outputs(s), outputs(ss[0]), "max_iter 1")
    b.close()
    for s in ss:
        s.close()


def test_batch_errors(cuda):
    fields = make_fields(cuda, FIELDS[:2], seed0=90)
    ss = solvers_for(fields)
    with pytest.raises(F.FFCzError):
        F.Batch([])
    with pytest.raises(F.FFCzError):
        F.Batch([ss[0], ss[0]])
    fresh = F.ProjectionSolver(4, 4, 4)
    with F.Batch([ss[0], fresh]) as b:
        with pytest.raises(F.FFCzError) as ei:
            b.solve_pair_device([fields[0][2], fields[0][2]], [fields[0][3], fields[0][3]], 10, 1e-7)
        assert ei.value.code == -4  # FFCZ_ERR_NOT_INITIALIZED
    with F.Batch(ss) as b:
        with pytest.raises(ValueError):
            b.solve_pair_device([fields[0][2]], [fields[0][3]], 10, 1e-7)
        # max_iter 0: e = x' - x per field, no loop
        assert b.solve_pair_device([f[2] for f in fields], [f[3] for f in fields], 0, 1e-7) == [0, 0]
        for (fld, _, _, _), s in zip(fields, ss):
            assert np.array_equal(s.get_results().reshape(-1), (fld.xp - fld.x).reshape(-1).astype(fld.x.dtype))
    fresh.close()
    for s in ss:
        s.close()


def test_batch_alternating_input_sets(cuda):
    """Inputs alternating between buffer sets (the next step's fields copied
    in while this step runs): each set's cached graph reads its own buffers,
    and a third set evicts the older entry without disturbing the results."""
    fields = make_fields(cuda, FIELDS[:5], seed0=90)
    ss = solvers_for(fields)
    sets = [([f[2] for f in fields], [f[3] for f in fields])]
    for _ in range(2):
        sets.append(([d.clone() for d in sets[0][0]], [d.clone() for d in sets[0][1]]))
    with F.Batch(ss) as b:
        ref_its = b.solve_pair_device(*sets[0], 100, 1e-7)
        ref = [outputs(s) for s in ss]
        for k in (1, 0, 1, 2, 0, 2):
            b.reset_edit_accumulators()
            assert b.solve_pair_device(*sets[k], 100, 1e-7) == ref_its, k
            for s, g in zip(ss, ref):
                assert_same(g, outputs(s), f"set {k}")
        # a set whose buffers now hold other data gives that data's results
        other = make_fields(cuda, FIELDS[:5], seed0=95)
        for d, f in zip(sets[1][0] + sets[1][1], [f[2] for f in other] + [f[3] for f in other]):
            d.copy_(f)
        b.reset_edit_accumulators()
        its = b.solve_pair_device(*sets[1], 100, 1e-7)
        for i, (fld, delta, dx, dxp) in enumerate(other):
            with F.ProjectionSolver(*fld.shape, dtype=fld.x.dtype) as s:
                s.initialize_all_abs(fields[i][0].x, fields[i][0].eps, fields[i][1])
                assert s.solve_all_abs_pair_device(dx, dxp, 100, 1e-7) == its[i]
                assert_same(outputs(s), outputs(ss[i]), f"refilled field {i}")
    for s in ss:
        s.close()
