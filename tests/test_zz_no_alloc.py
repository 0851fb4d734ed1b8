"""The allocation-free compaction entry point (ffcz_compact_quantize_noalloc)
against the solver's own compaction (ffcz_extract).

Some callers cannot allocate device memory: applications that reserve the
GPU's memory in their own pool up front and forbid further allocations, and
latency-bound pipelines that cannot take the device synchronisation of
cudaMalloc/cudaFree.  For them the entry point takes every input and output
from the caller and keeps its scratch in a fixed array inside the library.
Its outputs are integer codes, flag bytes and copies of input values, so the
comparison with ffcz_extract is exact.  Two calls in a row on arrays of
different sizes check that scratch left by one call does not leak into the
next."""
import ctypes as C

import numpy as np
import pytest

import ffcz_gb300 as F
from ffcz_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_ELEMS = 67108864


def _noalloc(torch, d_edits, n, dtype, pack_mode, stream):
    elt = torch.float32 if dtype == np.float32 else torch.float64
    compact = torch.empty(n, dtype=elt, device="cuda")
    quant = torch.empty(n, dtype=torch.int16, device="cuda")
    pack = torch.full((4 * ((n + 31) // 32),), 0x5A, dtype=torch.uint8, device="cuda")
    count, mn, mx = C.c_size_t(), C.c_double(), C.c_double()
    rc = F.lib().ffcz_compact_quantize_noalloc(
        C.c_void_p(d_edits), n, F.FFCZ_F32 if dtype == np.float32 else F.FFCZ_F64, C.c_void_p(compact.data_ptr()),
        C.c_void_p(quant.data_ptr()), C.c_void_p(pack.data_ptr()), pack_mode, C.c_void_p(stream),
        C.byref(count), C.byref(mn), C.byref(mx))
    assert rc == 0, F.lib().ffcz_last_error().decode()
    k = count.value
    return {"count": k, "min": mn.value, "max": mx.value,
            "compact": compact[:k].cpu().numpy(),
            "quant": quant[:k].cpu().numpy().view(np.uint16),
            "pack": pack[: (n + 7) // 8].cpu().numpy()}


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("pack_mode", [F.FFCZ_PACK_CORRECT, F.FFCZ_PACK_REFERENCE])
def test_noalloc_matches_extract(cuda, dtype, pack_mode):
    torch = cuda
    shape = (40, 36, 30)
    fld = synth.make_field(shape, 11 / 3, 21, 1e-3, 1e-3, dtype, noise=0.3)
    delta = synth.stress_delta(fld, 1.5)
    e0 = (fld.xp.astype(np.float64) - fld.x.astype(np.float64)).astype(dtype)
    with F.ProjectionSolver(*shape, dtype=dtype) as s:
        s.set_pack_mode(pack_mode)
        s.initialize_all_abs(fld.x, fld.eps, delta)
        s.solve_all_abs(e0, 100, 1e-7)
        nf, ns = s.active_counts()
        assert nf > 0 and ns > 0
        fmin, fmax, smin, smax = s.minmax()
        expected = {
            "freq": (nf, fmin, fmax, s.get_active_freq_edit_distances(), s.get_active_freq_quant_edit_distances(),
                     s.get_freq_flags_pack()),
            "spatial": (ns, smin, smax, s.get_active_spatial_edit_distances(),
                        s.get_active_spatial_quant_edit_distances(), s.get_spatial_flags_pack()),
        }
        stream = torch.cuda.current_stream().cuda_stream
        # two calls in a row (different sizes), then the first again
        for which, idx in (("freq", 1), ("spatial", 2), ("freq", 1)):
            d_edits, nbytes = s.device_array(idx)
            n = nbytes // np.dtype(dtype).itemsize
            got = _noalloc(torch, d_edits, n, dtype, pack_mode, stream)
            cnt, mn, mx, comp, quant, pack = expected[which]
            assert got["count"] == cnt
            assert got["min"] == mn and got["max"] == mx
            assert np.array_equal(got["compact"], comp)
            assert np.array_equal(got["quant"], quant)
            assert np.array_equal(got["pack"], pack)


def test_noalloc_rejects_oversized_input(cuda):
    torch = cuda
    buf = torch.zeros(64, dtype=torch.float32, device="cuda")
    count = C.c_size_t()
    ptr = C.c_void_p(buf.data_ptr())
    rc = F.lib().ffcz_compact_quantize_noalloc(ptr, MAX_ELEMS + 1, F.FFCZ_F32, ptr, ptr, ptr, F.FFCZ_PACK_CORRECT,
                                               None, C.byref(count), None, None)
    assert rc == -6
    assert "exceeds the fixed scratch limit" in F.lib().ffcz_last_error().decode()


def test_noalloc_rejects_misaligned_edits(cuda):
    """An edit pointer off a 16-byte boundary (an offset sub-array) is
    rejected on the host: the kernels read it with 16-byte vector loads."""
    torch = cuda
    buf = torch.zeros(256, dtype=torch.float32, device="cuda")
    out = torch.empty(256, dtype=torch.float32, device="cuda")
    quant = torch.empty(256, dtype=torch.int16, device="cuda")
    pack = torch.empty(64, dtype=torch.uint8, device="cuda")
    count = C.c_size_t(12345)
    rc = F.lib().ffcz_compact_quantize_noalloc(
        C.c_void_p(buf.data_ptr() + 4), 200, F.FFCZ_F32, C.c_void_p(out.data_ptr()), C.c_void_p(quant.data_ptr()),
        C.c_void_p(pack.data_ptr()), F.FFCZ_PACK_CORRECT, None, C.byref(count), None, None)
    assert rc == F.FFCZ_ERR_INVALID
    assert "16-byte aligned" in F.lib().ffcz_last_error().decode()
    assert count.value == 12345  # nothing ran


@pytest.mark.parametrize("pack_mode", [F.FFCZ_PACK_CORRECT, F.FFCZ_PACK_REFERENCE])
def test_noalloc_large_sparse_against_oracle(cuda, pack_mode):
    """More than 1024 chunks of 4096 values, so the one-block scan carries
    its running offset across rounds; compared with the C restatement of
    the reference's compaction (projection_algorithm.cu:365-550)."""
    from oracle import ffcz_oracle as O

    torch = cuda
    n = 6_000_001
    rng = np.random.default_rng(77)
    a = np.zeros(n, np.float32)
    idx = rng.choice(n, 450_000, replace=False)
    a[idx] = (rng.standard_normal(idx.size) * 1e-3).astype(np.float32)
    a[rng.choice(n, 5_000, replace=False)] = np.float32(5e-8)  # below the activity threshold
    d = torch.from_numpy(a).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    got = _noalloc(torch, d.data_ptr(), n, np.float32, pack_mode, stream)
    ex = O.extract(a, pack_mode)
    assert got["count"] == ex["count"]
    assert got["min"] == ex["min"] and got["max"] == ex["max"]
    assert np.array_equal(got["compact"], ex["compact"])
    assert np.array_equal(got["quant"], ex["quant"])
    assert np.array_equal(got["pack"], ex["pack"])


def test_noalloc_all_below_threshold_reference_pack(cuda):
    """No active value: count 0, min/max still over the whole array, and the
    reference pack mode leaves the pack zero (pack_bools is not launched
    for an empty stream, projection_algorithm_impl.cuh:429-449)."""
    torch = cuda
    n = 50_000
    a = np.zeros(n, np.float64)
    a[::7] = 9e-8
    a[3::11] = -4e-8
    d = torch.from_numpy(a).cuda()
    got = _noalloc(torch, d.data_ptr(), n, np.float64, F.FFCZ_PACK_REFERENCE, torch.cuda.current_stream().cuda_stream)
    assert got["count"] == 0
    assert got["min"] == -4e-8 and got["max"] == 9e-8
    assert not got["pack"].any()
