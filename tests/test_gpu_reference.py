"""GPU parity against the reference's own cuFFT build.

The fixtures tests/golden/ref_*.npz come from the unmodified reference run on
a GB300 (tests/golden/make_ref_goldens.py driving oracle/ref_solver.cu):
projection_example.cu's sequence on seeded fields (the plain small and
plain 256^3 workloads exactly, stress variants of the small field, a
mixed-radix, a 2D and an FP64 field), and the reference's
extract_compact_representation + cudaHuffmanZstdCompress on seeded
synthetic accumulators up to the 256^3 workload's size and density.

What is compared, and how closely:
  * iteration counts: equal;
  * the corrected error e and both edit accumulators (cuFFT against this
    library's transforms, both FP32 or both FP64): within TOL (FP32) or
    TOL64 (FP64) of the field's scale per iteration -- e and the spatial
    edits against max|e0|, the frequency edits against max|F(e0)|;
  * active counts: equal up to a few entries that sit on the 1e-7 activity
    threshold or a clamp boundary (COUNT_SLACK);
  * compaction (count, whole-array min/max, compact values, uint16 codes),
    flag packs in the reference's pack mode, Huffman code tables,
    bitstreams and ZSTD frames: bit-exact when this library is fed the
    reference's own edit arrays (or the same synthetic ones).
"""
import json
import sys
from pathlib import Path

import numpy as np
import pytest

import ffcz_gb300 as F

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import ref_cases as RC  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 2e-5      # FP32 transforms: relative to the field's scale, per iteration
TOL64 = 1e-12   # FP64 transforms
COUNT_SLACK = 1e-3
STREAMS = ("freq_quant", "freq_pack", "spatial_quant", "spatial_pack")


def load(case):
    path = GOLDEN / f"ref_{case}.npz"
    if not path.exists():
        pytest.skip(f"{path.name} not generated")
    d = np.load(path)
    return json.loads(str(d["meta"])), {k: d[k] for k in d.files if k != "meta"}


def dense(arrs, name, n, dtype):
    a = np.zeros(n, dtype)
    a[arrs[name + "__idx"]] = arrs[name + "__val"]
    return a


def check_array(meta, arrs, name, got):
    """Bit-exact: the stored array when present, its digest otherwise."""
    got = np.ascontiguousarray(got)
    want = meta["digests"][name]
    if name in arrs:
        assert np.array_equal(got, arrs[name]), name
    assert RC.digest(got) == want["sha256"], name


def run_solver(fld, delta, max_iter, pack_mode=F.FFCZ_PACK_REFERENCE):
    s = F.ProjectionSolver(*fld.shape, dtype=fld.x.dtype)
    s.set_pack_mode(pack_mode)
    s.initialize_all_abs(fld.x, fld.eps, delta)
    # the reference computes e0 = x' - x in T on the host (projection_example.cu:173-176)
    e0 = (fld.xp - fld.x).astype(fld.x.dtype)
    it = s.solve_all_abs(e0, max_iter, RC.TOL)
    return s, e0, it


def compare_compaction_and_coder(meta, arrs, s, dtype):
    """The solver's compaction of its current accumulators and its encode,
    bit for bit against the reference's outputs."""
    nf, ns = s.active_counts()
    assert (nf, ns) == (meta["num_active_freq"], meta["num_active_spatial"])
    fmin, fmax, smin, smax = s.minmax()
    assert (fmin, fmax, smin, smax) == (meta["min_freq"], meta["max_freq"], meta["min_spatial"], meta["max_spatial"])
    check_array(meta, arrs, "freq_quant", s.get_active_freq_quant_edit_distances())
    check_array(meta, arrs, "spatial_quant", s.get_active_spatial_quant_edit_distances())
    check_array(meta, arrs, "freq_compact", s.get_active_freq_edit_distances())
    check_array(meta, arrs, "spatial_compact", s.get_active_spatial_edit_distances())
    check_array(meta, arrs, "freq_pack", s.get_freq_flags_pack())
    check_array(meta, arrs, "spatial_pack", s.get_spatial_flags_pack())
    res = s.encode(meta["zstd_level"], F.FFCZ_ZSTD_SINGLE)
    for name, r in zip(STREAMS, res):
        assert (r is None) == (name not in meta), name
        if r is None:
            continue
        assert r.num_elements == meta[name]["num_elements"]
        assert r.original_bitstream_size == meta[name]["bitstream_bytes"]
        table = np.stack([r.symbols.astype(np.uint32), r.codes.astype(np.uint32),
                          r.lengths.astype(np.uint32)], axis=1)
        check_array(meta, arrs, name + "__table", table)
        check_array(meta, arrs, name + "__bits", np.frombuffer(r.bitstream, np.uint8))
        check_array(meta, arrs, name + "__zst", np.frombuffer(r.compressed_data, np.uint8))


@pytest.mark.parametrize("case", list(RC.SOLVE_CASES))
def test_loop_against_reference(cuda, case):
    """This library's projection loop on the reference's inputs: iterations,
    e and both accumulators against the reference's cuFFT run."""
    meta, arrs = load(case)
    fld, delta, max_iter = RC.field(case)
    assert meta["shape"] == list(fld.shape) and meta["delta"] == delta and meta["eps"] == fld.eps
    dt = fld.x.dtype
    tol = TOL64 if dt == np.float64 else TOL
    s, e0, it = run_solver(fld, delta, max_iter)
    with s:
        assert it == meta["iterations"], (it, meta["iterations"])
        n, h = fld.x.size, s.H
        escale = float(np.abs(e0).max())
        fscale = float(np.abs(np.fft.rfftn(e0.reshape(fld.shape).astype(np.float64))).max())
        k = max(1, it)
        e = s.get_results().reshape(-1)
        if "e" in arrs:
            ref_e = arrs["e"]
        else:
            idx = RC.sample_indices(n)
            assert RC.digest(idx) == meta["digests"]["e"]["sample_idx_sha256"]
            e, ref_e = e[idx], arrs["e__sample"]
        err_e = float(np.abs(e.astype(np.float64) - ref_e).max())
        assert err_e <= tol * escale * k, (err_e, escale)
        # accumulators
        fe, se = s.get_freq_edits_full(), s.get_spatial_edits_full()
        for name, ours, size, scale in (("freq_edits", fe, 2 * h, fscale), ("spatial_edits", se, n, escale)):
            if name + "__idx" in arrs:
                ref = dense(arrs, name, size, dt)
                got = ours
            else:
                idx = RC.sample_indices(size)
                ref, got = arrs[name + "__sample"], ours[idx]
            err = float(np.abs(got.astype(np.float64) - ref).max())
            assert err <= tol * scale * k, (name, err, scale)
            # whole-array checksums: sum |a| and the nonzero count
            cs = RC.checksums(ours)
            ref_cs = arrs[name + "__checksums"]
            assert abs(cs[1] - ref_cs[1]) <= tol * scale * k * max(1.0, ref_cs[4]), (name, cs, ref_cs)
        nf, ns = s.active_counts()
        for got, want in ((nf, meta["num_active_freq"]), (ns, meta["num_active_spatial"])):
            assert abs(got - want) <= max(2, COUNT_SLACK * want), (got, want)


@pytest.mark.parametrize("case", [c for c in RC.SOLVE_CASES if c != "plain256"])
def test_compaction_and_coder_on_reference_edits(cuda, case):
    """The reference's own edit accumulators fed to this library's
    compaction and coder: every output bit-exact with the reference's."""
    meta, arrs = load(case)
    fld, delta, max_iter = RC.field(case)
    dt = fld.x.dtype
    with F.ProjectionSolver(*fld.shape, dtype=dt) as s:
        s.set_pack_mode(F.FFCZ_PACK_REFERENCE)
        s.set_edit_accumulators(dense(arrs, "freq_edits", 2 * s.H, dt), dense(arrs, "spatial_edits", s.N, dt))
        s.extract_compact_representation()
        compare_compaction_and_coder(meta, arrs, s, dt)


@pytest.mark.parametrize("case", list(RC.EXTRACT_CASES))
def test_extract_against_reference(cuda, case):
    """Seeded synthetic accumulators (up to the 256^3 workload's size and
    7.5% density): compaction, packs, code tables, bitstreams and ZSTD
    frames bit-exact with the reference's."""
    meta, arrs = load(case)
    shape, dt, fe, se = RC.extract_inputs(case)
    assert meta["inputs"] == {"freq_edits": RC.digest(fe), "spatial_edits": RC.digest(se)}
    with F.ProjectionSolver(*shape, dtype=dt) as s:
        s.set_pack_mode(F.FFCZ_PACK_REFERENCE)
        s.set_edit_accumulators(fe, se)
        s.extract_compact_representation()
        compare_compaction_and_coder(meta, arrs, s, dt)


def test_plain256_own_compaction_bitexact_with_oracle(cuda):
    """The plain 256^3 workload run by this library: its 1.26 M spatial
    edits compacted, packed and Huffman-coded bit-exactly as the C
    restatement of the reference does it, and the same counts and
    code-length profile as the reference's run."""
    from oracle import ffcz_oracle as O

    meta, arrs = load("plain256")
    fld, delta, max_iter = RC.field("plain256")
    s, e0, it = run_solver(fld, delta, max_iter)
    with s:
        assert it == meta["iterations"]
        se = s.get_spatial_edits_full()
        ex = O.extract(se, F.FFCZ_PACK_REFERENCE)
        q = s.get_active_spatial_quant_edit_distances()
        assert q.size == ex["count"]
        assert np.array_equal(q, ex["quant"])
        assert np.array_equal(s.get_active_spatial_edit_distances(), ex["compact"])
        assert np.array_equal(s.get_spatial_flags_pack(), ex["pack"])
        res = s.encode(3, F.FFCZ_ZSTD_NONE)
        for r, data in ((res[2], q), (res[3], ex["pack"])):
            book = O.huffman_codebook(data)
            bits, _ = O.huffman_bitstream(data, book)
            assert r.bitstream == bits
        assert res[2].symbols.size == pytest.approx(meta["spatial_quant"]["symbols"], rel=0.02)
        assert int(res[2].lengths.max()) == pytest.approx(meta["spatial_quant"]["max_code_length"], abs=1)
