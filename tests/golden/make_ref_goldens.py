"""Generates tests/golden/ref_<case>.npz from the reference's own cuFFT build.

Needs a CUDA GPU and oracle/_ref/ref_solver, which oracle/build_ref_solver.sh
builds from the unmodified reference sources (FFCZ_REF).  For every case of
ref_cases.py it writes the case's inputs to a scratch directory, runs

  * solve cases: `ref_solver solve` -- projection_example.cu's Run<T>
    sequence (e0 = x' - x, initialize_all_abs, solve_all_abs, the getters,
    cudaHuffmanZstdCompress of the four streams at ZSTD level 20);
  * extract cases: `ref_solver extract` -- extract_compact_representation
    and the same four coder calls on the case's synthetic accumulators;
  * the reference's kernels: `legacy_kernels_ref` (tests/legacy_kernels_driver.cu
    built against the reference's header and projection_algorithm.cu) ->
    ref_legacy_kernels.npz;

and stores what the parity tests compare: the iteration count, the active
counts and min/max, the corrected error e (whole, or a fixed sample plus
checksums for the 256^3 field), the edit accumulators (their nonzero
entries, or a sample plus checksums), the compact values, uint16 codes and
flag packs, and per coded stream its code table, Huffman bitstream and ZSTD
frame.  Arrays above LIMIT bytes, and the ZSTD frames, are stored as SHA-256
digests.

    python tests/golden/make_ref_goldens.py [outdir]      (default tests/golden)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))
import ref_cases as RC  # noqa: E402

HARNESS = ROOT / "oracle" / "_ref" / "ref_solver"
LIMIT = 300_000
SPARSE_LIMIT = 200_000
STREAMS = ("freq_quant", "freq_pack", "spatial_quant", "spatial_pack")


def _read(d: Path, name: str, dtype) -> np.ndarray:
    p = d / name
    return np.fromfile(p, dtype=dtype) if p.exists() else np.zeros(0, dtype)


class Store:
    def __init__(self):
        self.arrays, self.digests = {}, {}

    def put(self, name, a, force_full=False, digest_only=False):
        a = np.ascontiguousarray(a)
        self.digests[name] = {"sha256": RC.digest(a), "nbytes": int(a.nbytes), "dtype": str(a.dtype)}
        if force_full or (a.nbytes <= LIMIT and not digest_only):
            self.arrays[name] = a

    def put_sparse(self, name, a):
        nz = np.flatnonzero(a)
        self.digests[name] = {"sha256": RC.digest(a), "nbytes": int(a.nbytes), "nnz": int(nz.size)}
        self.arrays[name + "__checksums"] = RC.checksums(a)
        if nz.size <= SPARSE_LIMIT:
            self.arrays[name + "__idx"] = nz.astype(np.int64)
            self.arrays[name + "__val"] = a[nz]
        else:
            idx = RC.sample_indices(a.size)
            self.digests[name]["sample_idx_sha256"] = RC.digest(idx)
            self.arrays[name + "__sample"] = a[idx]


def store_outputs(st: Store, d: Path, dt, meta: dict):
    st.put("freq_quant", _read(d, "freq_quant.bin", np.uint16))
    st.put("spatial_quant", _read(d, "spatial_quant.bin", np.uint16))
    st.put("freq_pack", _read(d, "freq_pack.bin", np.uint8))
    st.put("spatial_pack", _read(d, "spatial_pack.bin", np.uint8))
    st.put("freq_compact", _read(d, "freq_compact.bin", dt))
    st.put("spatial_compact", _read(d, "spatial_compact.bin", dt))
    for name in STREAMS:
        if name not in meta:
            continue
        tab = _read(d, name + ".tab", np.uint32).reshape(-1, 3)
        st.put(name + "__table", tab)
        st.put(name + "__bits", _read(d, name + ".bits", np.uint8))
        st.put(name + "__zst", _read(d, name + ".zst", np.uint8), digest_only=True)
        lens = tab[:, 2].astype(np.int64)
        meta[name]["max_code_length"] = int(lens.max()) if lens.size else 0


def run(cmd):
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[:2]} failed ({r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    return r.stdout


def solve_case(name: str, out: Path, tmp: Path):
    fld, delta, max_iter = RC.field(name)
    keep_e = RC.SOLVE_CASES[name][3]
    dt = fld.x.dtype
    nx, ny, nz = fld.shape
    d = tmp / name
    d.mkdir()
    fld.x.tofile(d / "x.bin")
    fld.xp.tofile(d / "xp.bin")
    t0 = time.time()
    stdout = run([HARNESS, "solve", "f64" if dt == np.float64 else "f32", nx, ny, nz, d / "x.bin", d / "xp.bin",
                  repr(float(fld.eps)), repr(float(delta)), max_iter, repr(RC.TOL), RC.ZSTD_LEVEL, d])
    wall = time.time() - t0
    meta = json.loads((d / "meta.json").read_text())
    meta.pop("done", None)
    printed = [ln for ln in stdout.splitlines() if ln.startswith("Total number of iterations")]
    meta.update({"case": name, "mode": "solve", "shape": list(fld.shape), "dtype": str(dt), "eps": fld.eps,
                 "delta": delta, "max_iter": max_iter, "tol": RC.TOL, "zstd_level": RC.ZSTD_LEVEL,
                 "printed": printed, "harness_wall_s": round(wall, 3)})
    st = Store()
    e = _read(d, "e.bin", dt)
    if keep_e:
        st.put("e", e, force_full=True)
    else:
        idx = RC.sample_indices(e.size)
        st.arrays["e__sample"] = e[idx]
        st.put("e", e)
        st.digests["e"]["sample_idx_sha256"] = RC.digest(idx)
    st.arrays["e__checksums"] = RC.checksums(e)
    st.put_sparse("freq_edits", _read(d, "freq_edits.bin", dt))
    st.put_sparse("spatial_edits", _read(d, "spatial_edits.bin", dt))
    store_outputs(st, d, dt, meta)
    finish(out, name, meta, st)


def extract_case(name: str, out: Path, tmp: Path):
    (nx, ny, nz), dt, fe, se = RC.extract_inputs(name)
    d = tmp / name
    d.mkdir()
    fe.tofile(d / "fe.bin")
    se.tofile(d / "se.bin")
    run([HARNESS, "extract", "f64" if dt == np.float64 else "f32", nx, ny, nz, d / "fe.bin", d / "se.bin",
         RC.ZSTD_LEVEL, d])
    meta = json.loads((d / "meta.json").read_text())
    meta.pop("done", None)
    meta.update({"case": name, "mode": "extract", "shape": [nx, ny, nz], "dtype": str(dt),
                 "zstd_level": RC.ZSTD_LEVEL, "inputs": {"freq_edits": RC.digest(fe), "spatial_edits": RC.digest(se)}})
    st = Store()
    store_outputs(st, d, dt, meta)
    finish(out, name, meta, st)


def finish(out: Path, name: str, meta: dict, st: Store):
    meta["digests"] = st.digests
    np.savez_compressed(out / f"ref_{name}.npz", meta=np.array(json.dumps(meta, sort_keys=True)), **st.arrays)
    print(f"{name}: iterations={meta.get('iterations')} active=({meta['num_active_freq']}, "
          f"{meta['num_active_spatial']}) -> {out / f'ref_{name}.npz'}", flush=True)


def legacy_kernels(out: Path, tmp: Path):
    """The reference's own kernels (projection_algorithm.cu:85-673) and host
    compaction (:459-550) run by tests/legacy_kernels_driver.cu."""
    exe = ROOT / "oracle" / "_ref" / "legacy_kernels_ref"
    if not exe.exists():
        raise SystemExit(f"{exe} is missing: run oracle/build_ref_solver.sh")
    run([exe, tmp / "legacy.bin"])
    rec = RC.read_records(tmp / "legacy.bin")
    np.savez_compressed(out / "ref_legacy_kernels.npz", **rec)
    print(f"legacy kernels: {len(rec)} outputs -> {out / 'ref_legacy_kernels.npz'}", flush=True)


def main():
    out = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent
    out.mkdir(parents=True, exist_ok=True)
    if not HARNESS.exists():
        raise SystemExit(f"{HARNESS} is missing: run oracle/build_ref_solver.sh (FFCZ_REF=<reference sources>)")
    only = set(os.environ.get("FFCZ_REF_CASES", "").split(",")) - {""}
    with tempfile.TemporaryDirectory() as t:
        tmp = Path(t)
        for name in RC.SOLVE_CASES:
            if not only or name in only:
                solve_case(name, out, tmp)
        for name in RC.EXTRACT_CASES:
            if not only or name in only:
                extract_case(name, out, tmp)
        if not only or "legacy_kernels" in only:
            legacy_kernels(out, tmp)


if __name__ == "__main__":
    main()
