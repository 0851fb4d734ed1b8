"""GPU parity of the projection loop and the compaction against the oracle.

Tolerances (FP32 transforms vs the oracle's FP64 transforms rounded to
FP32): the corrected error e agrees to TOL_E * max|e|, the edit
accumulators to TOL_EDIT * max|F(e0)| (frequency) and TOL_E * max|e0|
(spatial).  Compaction, quantisation and flag packs of the GPU's own edit
arrays are compared bit for bit with the C restatement.
"""
import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth
from oracle import ffcz_oracle as O

pytestmark = pytest.mark.gpu

TOL_E = 2e-5
TOL_EDIT = 2e-5

SHAPES = [(16, 24, 10), (8, 8, 8), (1, 1, 17), (1, 1, 64), (1, 30, 50), (5, 7, 9), (12, 10, 14), (3, 1, 40),
          (2, 3, 1), (20, 35, 49), (64, 64, 64), (4, 6, 250), (11, 13, 34), (1, 1, 1), (1, 2, 2),
          (2, 96, 192), (500, 2, 6), (1, 900, 1800), (100, 3, 200)]
# axes with a compile-time mixed-radix stage list (100, 250, 500, 900, 1800, 96, 384, ...)
MIXED = [(4, 100, 200), (3, 250, 500), (2, 96, 192), (2, 384, 768), (2, 400, 1000), (1, 900, 1800),
         (100, 3, 10), (500, 2, 6), (1800, 2, 4), (3, 1000, 2000), (2, 200, 400), (2, 192, 384)]


def rand_e0(shape, seed, scale=1.0, dtype=np.float32):
    return (np.random.default_rng(seed).standard_normal(int(np.prod(shape))) * scale).astype(dtype)


@pytest.mark.parametrize("shape", SHAPES)
def test_roundtrip_no_clamp(cuda, shape):
    """Huge bounds: one R2C + C2R/N pass returns e0 (FFT round trip)."""
    e0 = rand_e0(shape, 1)
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(np.zeros_like(e0), 1e30, 1e30)
        it = s.solve_all_abs(e0, 5, 1e-7)
        assert it == 1
        e = s.get_results().reshape(-1)
        assert np.abs(e - e0).max() <= 2e-6 * max(1.0, np.abs(e0).max())
        assert s.active_counts() == (0, 0)
        assert not s.get_freq_edits_full().any() and not s.get_spatial_edits_full().any()


@pytest.mark.parametrize("shape", SHAPES)
def test_frequency_clamp_one_pass(cuda, shape):
    """Only the frequency box binds: edits equal the oracle's clamp deltas."""
    e0 = rand_e0(shape, 2)
    Fm = np.abs(np.fft.rfftn(e0.reshape(shape).astype(np.float64)))
    delta = float(np.float32(0.3 * Fm.max()))
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(np.zeros_like(e0), 1e30, delta)
        it = s.solve_all_abs(e0, 1, 1e-7)
        ref = O.solve_all_abs(e0, shape, 1e30, delta, 1, 1e-7, np.float32)
        assert it == ref["iterations"] == 1
        fe = s.get_freq_edits_full()
        scale = float(Fm.max())
        assert np.abs(fe - ref["freq_edits"]).max() <= TOL_EDIT * scale
        e = s.get_results().reshape(-1)
        assert np.abs(e - ref["e"].reshape(-1)).max() <= TOL_E * float(np.abs(ref["e"]).max())


@pytest.mark.parametrize("shape,c", [((64, 64, 64), 1.0), ((64, 64, 64), 3.0), ((32, 48, 20), 2.0),
                                     ((1, 90, 100), 1.5), ((1, 1, 4096), 1.0), ((25, 20, 16), 2.0),
                                     ((4, 100, 200), 2.0), ((3, 250, 500), 1.5), ((2, 384, 768), 1.0),
                                     ((100, 6, 10), 2.0), ((1, 1800, 3600), 1.0)])
def test_loop_parity(cuda, shape, c):
    """Stress bounds (several iterations): iterations, e and both edit
    accumulators agree with the FP32-rounded oracle."""
    fld = synth.make_field(shape, 11 / 3, 7, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, c)
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*fld.shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        ref = O.solve_all_abs(e0, fld.shape, fld.eps, delta, 100, 1e-7, np.float32)
        assert it == ref["iterations"]
        e = s.get_results().reshape(-1)
        escale = float(np.abs(e0).max())
        assert np.abs(e - ref["e"].reshape(-1)).max() <= TOL_E * escale * max(1, it)
        fscale = float(np.abs(np.fft.rfftn(e0.reshape(fld.shape).astype(np.float64))).max())
        assert np.abs(s.get_freq_edits_full() - ref["freq_edits"]).max() <= TOL_EDIT * fscale * max(1, it)
        assert np.abs(s.get_spatial_edits_full() - ref["spatial_edits"]).max() <= TOL_E * escale * max(1, it)
        # FP64 check of the bounds the reference schedule guarantees: |e| <= E
        # + tol; x^ = x + e stored in float32 adds up to half an ulp of |x^|
        b = O.check_bounds(fld.x, fld.x + e.reshape(fld.shape), fld.eps, delta)
        half_ulp = 0.5 * float(np.spacing(np.float32(np.abs(fld.x).max() + fld.eps)))
        if ref["converged"]:
            assert b["spatial_excess"] <= 1e-7 + half_ulp + 1e-6 * fld.eps


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("pack_mode", [F.FFCZ_PACK_CORRECT, F.FFCZ_PACK_REFERENCE])
def test_extract_bitexact(cuda, dtype, pack_mode):
    shape = (24, 20, 18)
    fld = synth.make_field(shape, 11 / 3, 3, 1e-3, 1e-3, dtype, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)
    with F.ProjectionSolver(*fld.shape, dtype=dtype) as s:
        s.set_pack_mode(pack_mode)
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        nf, ns = s.active_counts()
        assert nf > 0 and ns > 0
        for edits, which in ((s.get_freq_edits_full(), "freq"), (s.get_spatial_edits_full(), "spatial")):
            ex = O.extract(edits, pack_mode)
            q = getattr(s, f"get_active_{which}_quant_edit_distances")()
            comp = getattr(s, f"get_active_{which}_edit_distances")()
            pk = getattr(s, f"get_{which}_flags_pack")()
            assert q.size == ex["count"]
            assert np.array_equal(q, ex["quant"])
            assert np.array_equal(comp, ex["compact"])
            assert np.array_equal(pk, ex["pack"])
            fl = getattr(s, f"get_{which}_flags")()
            assert np.array_equal(fl, ex["flags"])
        mm = s.minmax()
        exf, exs = O.extract(s.get_freq_edits_full()), O.extract(s.get_spatial_edits_full())
        assert mm == (exf["min"], exf["max"], exs["min"], exs["max"])


def test_graph_and_host_loop_identical(cuda):
    shape = (32, 32, 32)
    fld = synth.make_field(shape, 11 / 3, 5, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    e0 = (fld.xp - fld.x).astype(np.float32)
    out = []
    for drv in (F.FFCZ_LOOP_GRAPH, F.FFCZ_LOOP_HOST):
        with F.ProjectionSolver(*shape) as s:
            s.set_loop_driver(drv)
            s.initialize_all_abs(fld.x, fld.eps, delta)
            it = s.solve_all_abs(e0, 100, 1e-7)
            out.append((it, s.get_results(), s.get_freq_edits_full(), s.get_spatial_edits_full()))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)


def test_repeat_solve_same_result(cuda):
    """The cached graph is replayed; accumulators are reset between solves."""
    shape = (16, 16, 16)
    fld = synth.make_field(shape, 11 / 3, 6, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        a = (s.get_results(), s.get_freq_edits_full())
        s.reset_edit_accumulators()
        s.solve_all_abs(e0, 100, 1e-7)
        b = (s.get_results(), s.get_freq_edits_full())
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_pair_device_matches_host(cuda):
    torch = cuda
    shape = (20, 18, 16)
    fld = synth.make_field(shape, 11 / 3, 8, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.2)
    e0 = (fld.xp - fld.x).astype(np.float32)
    with F.ProjectionSolver(*shape) as s1, F.ProjectionSolver(*shape) as s2:
        s1.initialize_all_abs(fld.x, fld.eps, delta)
        s1.solve_all_abs(e0, 100, 1e-7)
        dx = torch.from_numpy(fld.x.reshape(-1)).cuda()
        dxp = torch.from_numpy(fld.xp.reshape(-1)).cuda()
        s2.initialize_all_abs_device(dx, fld.eps, delta)
        s2.solve_all_abs_pair_device(dx, dxp, 100, 1e-7)
        torch.cuda.synchronize()
        assert s1.iterations == s2.iterations
        assert np.array_equal(s1.get_results(), s2.get_results())
        assert np.array_equal(s1.get_spatial_edits_full(), s2.get_spatial_edits_full())


def test_fp64_loop_parity(cuda):
    shape = (24, 16, 20)
    fld = synth.make_field(shape, 11 / 3, 9, 1e-3, 1e-3, np.float64, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = fld.xp - fld.x
    with F.ProjectionSolver(*shape, dtype=np.float64) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        ref = O.solve_all_abs(e0, shape, fld.eps, delta, 100, 1e-7, np.float64)
        assert it == ref["iterations"]
        e = s.get_results().reshape(-1)
        assert np.abs(e - ref["e"].reshape(-1)).max() <= 1e-12 * float(np.abs(e0).max()) * it


def test_max_iter_zero_returns_e0(cuda):
    shape = (8, 8, 8)
    e0 = rand_e0(shape, 4)
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(np.zeros_like(e0), 0.1, 0.1)
        assert s.solve_all_abs(e0, 0, 1e-7) == 0
        assert np.array_equal(s.get_results().reshape(-1), e0)


def test_not_converged_ends_with_spatial_clamp(cuda):
    """max_iter reached: the last step is the spatial projection (impl:851)."""
    shape = (16, 16, 16)
    fld = synth.make_field(shape, 11 / 3, 10, 1e-3, 1e-3, np.float32, noise=0.3)
    e0 = (fld.xp - fld.x).astype(np.float32)
    # a loose frequency box leaves spatial violations after each pass
    for c in (1.0, 1.5, 2.0, 3.0, 4.0, 6.0, 8.0):
        delta = synth.stress_delta(fld, c)
        ref = O.solve_all_abs(e0, shape, fld.eps, delta, 2, 1e-7, np.float32)
        if not ref["converged"]:
            break
    assert ref["iterations"] == 2 and not ref["converged"]
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 2, 1e-7)
        assert it == 2
        e = s.get_results()
        assert np.abs(e).max() <= np.float32(fld.eps)
        assert np.abs(e.reshape(-1) - ref["e"].reshape(-1)).max() <= TOL_E * float(np.abs(e0).max()) * 2


def test_errors(cuda):
    with F.ProjectionSolver(8, 8, 8) as s:
        with pytest.raises(F.FFCzError) as ei:
            s.solve_all_abs(np.zeros(512, np.float32), 10, 1e-7)
        assert ei.value.code == -4 and "not initialized" in str(ei.value)
    with pytest.raises(F.FFCzError) as ei:
        F.ProjectionSolver(0, 8, 8)
    assert ei.value.code == -1
    with pytest.raises(F.FFCzError) as ei:
        F.ProjectionSolver(8, 8, 2 * 4099)  # prime factor above the largest generic radix
    assert ei.value.code == -3


def test_launch_count_reported(cuda):
    shape = (16, 16, 16)
    fld = synth.make_field(shape, 11 / 3, 11, 1e-3, 1e-3, np.float32, noise=0.3)
    with F.ProjectionSolver(*shape) as s:
        s.initialize_all_abs(fld.x, fld.eps, synth.stress_delta(fld, 1.0))
        s.project_all_abs_device(cuda.from_numpy((fld.xp - fld.x).reshape(-1)).cuda(), 100, 1e-7)
        it = s.iterations
        assert s.launch_count() == 2 + 6 * it


@pytest.mark.parametrize("shape", [(64, 64, 64), (32, 48, 20), (16, 1024, 32), (8, 16, 2048), (40, 512, 256)]
                         + MIXED)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_static_kernels_match_generic(cuda, shape, dtype, monkeypatch):
    """Compile-time-sized pass kernels (power-of-two and mixed-radix axes)
    against the runtime-planned engine on the same input."""
    fld = synth.make_field(shape, 11 / 3, 13, 1e-3, 1e-3, dtype, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)
    out = []
    if dtype == np.float64 and max(shape) > 2048:
        pytest.skip("FP64 axis length above the runtime-planned engine's 2048")
    for generic in ("0", "1"):
        monkeypatch.setenv("FFCZ_GENERIC_KERNELS", generic)
        with F.ProjectionSolver(*shape, dtype=dtype) as s:
            s.initialize_all_abs(fld.x, fld.eps, delta)
            # tol < 0: exactly 3 iterations on both paths (a convergence
            # decision at the roundoff level cannot split them)
            it = s.solve_all_abs(e0, 3, -1.0)
            out.append((it, s.get_results().reshape(-1), s.get_freq_edits_full()))
    assert out[0][0] == out[1][0] == 3
    tol = 1e-6 if dtype == np.float32 else 1e-14
    assert np.abs(out[0][1] - out[1][1]).max() <= tol * np.abs(e0).max() * out[0][0]
    fs = float(np.abs(out[1][2]).max()) or 1.0
    assert np.abs(out[0][2] - out[1][2]).max() <= tol * max(fs, float(delta))


@pytest.mark.parametrize("shape,dtype", [((16, 24, 10), np.float32), ((64, 64, 64), np.float32),
                                         ((1, 90, 100), np.float32), ((3, 250, 500), np.float32),
                                         ((1, 1, 4096), np.float32), ((12, 10, 16), np.float64),
                                         ((5, 7, 9), np.float32)])
def test_verify_bounds_on_device_matches_fp64_host(cuda, shape, dtype):
    """ffcz_verify_bounds: max |e| exactly, and the FP64 half-spectrum maximum
    of e within FP64 transform roundoff of numpy's."""
    fld = synth.make_field(shape, 11 / 3, 17, 1e-3, 1e-3, dtype, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs((fld.xp - fld.x).astype(dtype), 100, 1e-7)
        sm, fm = s.verify_bounds()
        e = s.get_results().astype(np.float64)
    assert sm == float(np.abs(e).max())
    Fe = np.fft.rfftn(e.reshape(shape))
    ref = float(max(np.abs(Fe.real).max(), np.abs(Fe.imag).max()))
    assert abs(fm - ref) <= 1e-12 * max(ref, float(np.abs(e).sum()))
    assert sm <= fld.eps + 1e-7 and fm <= delta * (1 + 1e-6)


def test_allocation_failure_is_reported_and_cleaned_up(cuda, monkeypatch):
    """Host-side fault injection (FFCZ_FAIL_ALLOC=k fails the k-th device
    allocation of a solver without calling the allocator): each failure is a
    CUDA-class status naming the injected call, and nothing is left behind."""
    F.ProjectionSolver(96, 96, 96).close()  # first creation's one-time costs
    cuda.cuda.synchronize()
    free0 = cuda.cuda.mem_get_info()[0]
    k = 0
    while k < 64:  # fail allocation 1, 2, ... until k is past the last one
        k += 1
        monkeypatch.setenv("FFCZ_FAIL_ALLOC", str(k))
        try:
            F.ProjectionSolver(96, 96, 96).close()
        except F.FFCzError as e:
            assert e.code == -2 and "injected" in str(e), k
            continue
        break
    assert 10 < k < 64, k
    monkeypatch.delenv("FFCZ_FAIL_ALLOC")
    with F.ProjectionSolver(96, 96, 96) as s:
        s.initialize_all_abs(np.zeros(96 ** 3, np.float32), 1e30, 1e30)
        assert s.solve_all_abs(np.ones(96 ** 3, np.float32), 3, 1e-7) == 1
    cuda.cuda.synchronize()
    assert free0 - cuda.cuda.mem_get_info()[0] < 16 << 20


@pytest.mark.parametrize("shape", [(1, 900, 1800), (3, 1250, 16), (2, 6, 3000), (1, 1, 4096)])
def test_fp64_long_axes(cuda, shape):
    """FP64 axes beyond the 4-values-per-thread tile (1024): runtime-planned
    tiles at 8 values per thread, or the compile-time kernels, against the
    FP64 oracle."""
    fld = synth.make_field(shape, 11 / 3, 19, 1e-3, 1e-3, np.float64, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    e0 = fld.xp - fld.x
    with F.ProjectionSolver(*shape, dtype=np.float64) as s:
        s.initialize_all_abs(fld.x, fld.eps, delta)
        it = s.solve_all_abs(e0, 100, 1e-7)
        ref = O.solve_all_abs(e0, shape, fld.eps, delta, 100, 1e-7, np.float64)
        assert it == ref["iterations"]
        es = float(np.abs(e0).max())
        assert np.abs(s.get_results().reshape(-1) - ref["e"].reshape(-1)).max() <= 1e-12 * es * max(1, it)
        fs = float(np.abs(np.fft.rfftn(e0.reshape(shape))).max())
        assert np.abs(s.get_freq_edits_full() - ref["freq_edits"]).max() <= 1e-12 * fs * max(1, it)


@pytest.mark.parametrize("shape", [(40, 512, 256), (8, 16, 2048), (4, 100, 200), (16, 1024, 32), (3, 250, 500)])
def test_autotune_keeps_results(cuda, shape):
    """The autotuner swaps tile widths only: results stay bit-identical."""
    fld = synth.make_field(shape, 11 / 3, 29, 1e-3, 1e-3, np.float32, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = (fld.xp - fld.x).astype(np.float32)
    out = []
    for tune in (False, True):
        with F.ProjectionSolver(*shape) as s:
            s.initialize_all_abs(fld.x, fld.eps, delta)
            if tune:
                rep = s.autotune(3)
                assert all(v[0] >= 0 and v[1] >= 0 for v in rep.values())
            it = s.solve_all_abs(e0, 100, 1e-7)
            out.append((it, s.get_results(), s.get_freq_edits_full(), s.get_spatial_edits_full()))
    assert out[0][0] == out[1][0]
    for a, b in zip(out[0][1:], out[1][1:]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_untouched_frequency_accumulator_compacts_without_reading(cuda, dtype):
    """While no frequency clamp has fired since the accumulator was cleared,
    its compaction writes zero flags and zero min/max without reading it;
    the results equal the oracle's compaction of the (all-zero) array, and
    a clamp makes the next compaction read it again."""
    shape = (24, 20, 16)
    fld = synth.make_field(shape, 11 / 3, 41, 1e-3, 1e-3, dtype, noise=0.3)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)

    def check(s):
        fe = s.get_freq_edits_full()
        ref = O.extract(fe)
        nf = s.active_counts()[0]
        assert nf == ref["count"]
        assert s.minmax()[:2] == (ref["min"], ref["max"])
        assert np.array_equal(s.get_freq_flags_pack(), ref["pack"])
        assert np.array_equal(s.get_active_freq_quant_edit_distances(), ref["quant"])
        return nf

    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.initialize_all_abs(fld.x, fld.eps, 1e30)  # no frequency clamp
        s.solve_all_abs(e0, 100, 1e-7)
        assert check(s) == 0 and not s.get_freq_edits_full().any()
        s.initialize_all_abs(fld.x, fld.eps, synth.stress_delta(fld, 1.5))  # clamps fire
        s.solve_all_abs(e0, 100, 1e-7)
        assert check(s) > 0
        s.initialize_all_abs(fld.x, fld.eps, 1e30)  # edits kept: still read
        s.solve_all_abs(e0, 100, 1e-7)
        assert check(s) > 0
        s.reset_edit_accumulators()  # cleared: skipped again
        s.solve_all_abs(e0, 100, 1e-7)
        assert check(s) == 0


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_untouched_spatial_accumulator_compacts_without_reading(cuda, loop):
    """The spatial accumulator is written only by the clamping prologue of
    an iteration after a violation and by the final clamp; while neither
    ran since the accumulator was cleared, its compaction skips reading it.
    Both cases match the oracle's compaction of the accumulator."""
    shape = (20, 18, 16)
    fld = synth.make_field(shape, 11 / 3, 43, 1e-3, 1e-3, np.float32, noise=0.3)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(np.float32)

    def check(s):
        se = s.get_spatial_edits_full()
        ref = O.extract(se)
        ns = s.active_counts()[1]
        assert ns == ref["count"]
        assert s.minmax()[2:] == (ref["min"], ref["max"])
        assert np.array_equal(s.get_spatial_flags_pack(), ref["pack"])
        assert np.array_equal(s.get_active_spatial_quant_edit_distances(), ref["quant"])
        return ns

    with F.ProjectionSolver(*shape) as s:
        s.set_loop_driver(F.FFCZ_LOOP_GRAPH if loop == "graph" else F.FFCZ_LOOP_HOST)
        s.initialize_all_abs(fld.x, 1e30, 1e30)  # converges at once: no clamp
        assert s.solve_all_abs(e0, 100, 1e-7) == 1
        assert check(s) == 0 and not s.get_spatial_edits_full().any()
        s.initialize_all_abs(fld.x, fld.eps, 1e30)  # x' - x exceeds E: clamps
        assert s.solve_all_abs(e0, 100, 1e-7) > 1
        assert check(s) > 0
        s.reset_edit_accumulators()
        s.initialize_all_abs(fld.x, fld.eps, 1e30)
        assert s.solve_all_abs(e0, 1, 1e-7) == 1  # stopped by max_iter: final clamp
        assert check(s) > 0
        s.reset_edit_accumulators()
        s.initialize_all_abs(fld.x, 1e30, 1e30)
        s.solve_all_abs(e0, 100, 1e-7)
        assert check(s) == 0


@pytest.mark.parametrize("shape", [(8, 128, 256), (4, 256, 512), (2, 512, 128)])
def test_fp64_split_precision_against_fp64_oracle(cuda, shape):
    """FP64 fields with the float-float pass kernels (FP64 storage, boxes and
    violation in FP64): the corrected error and the edits stay within 1e-11
    (relative to the field's scale, per iteration) of the FP64 oracle and of
    the native FP64 solver; the FP64 device check of the bounds still
    holds."""
    fld = synth.make_field(shape, 11 / 3, 23, 1e-3, 1e-3, np.float64, noise=0.3)
    delta = synth.stress_delta(fld, 1.0)
    e0 = fld.xp - fld.x
    ref = O.solve_all_abs(e0, shape, fld.eps, delta, 100, 1e-7, np.float64)
    out = {}
    for prec in (F.FFCZ_PRECISION_NATIVE, F.FFCZ_PRECISION_SPLIT):
        with F.ProjectionSolver(*shape, dtype=np.float64) as s:
            s.set_precision(prec)
            s.initialize_all_abs(fld.x, fld.eps, delta)
            it = s.solve_all_abs(e0, 100, 1e-7)
            out[prec] = (it, s.get_results().reshape(-1), s.get_freq_edits_full(), s.get_spatial_edits_full(),
                         s.verify_bounds())
    it, e, fe, se, (sm, fm) = out[F.FFCZ_PRECISION_SPLIT]
    assert it == ref["iterations"] == out[F.FFCZ_PRECISION_NATIVE][0]
    es = float(np.abs(e0).max())
    fs = float(np.abs(np.fft.rfftn(e0)).max())
    t = 1e-11 * max(1, it)
    assert np.abs(e - ref["e"].reshape(-1)).max() <= t * es
    assert np.abs(fe - ref["freq_edits"]).max() <= t * fs
    assert np.abs(se - ref["spatial_edits"]).max() <= t * es
    assert np.abs(e - out[F.FFCZ_PRECISION_NATIVE][1]).max() <= t * es
    assert sm <= fld.eps + 1e-7 and fm <= delta * (1 + 1e-9)


def test_precision_setting_rules(cuda):
    with F.ProjectionSolver(8, 8, 8) as s:  # FP32: native only
        s.set_precision(F.FFCZ_PRECISION_NATIVE)
        with pytest.raises(F.FFCzError) as ei:
            s.set_precision(F.FFCZ_PRECISION_SPLIT)
        assert ei.value.code == -3
        with pytest.raises(F.FFCzError):
            s.set_precision(7)
