"""Python binding of the GB300 FFCz corrector and edit encoder (libffcz.so).

Thin ctypes layer over the C ABI declared in include/ffcz.h, mirroring the
reference's C++ interface:

* ``ProjectionSolver`` -- ProjectionSolver<T> (projection_algorithm.cuh:238-333)
* ``cuda_huffman_zstd_compress`` / ``cuda_huffman_zstd_decompress`` --
  cudaHuffmanZstdCompress / cudaHuffmanZstdDecompress (HuffmanZSTDCoder.cuh:454-470)
* ``read_raw_array_binary`` / ``write_raw_array_binary`` / ``write_map`` /
  ``read_map`` -- fileIO.h:17-55

All compute runs in the native library; this module only moves arguments.
Importing it does not need a GPU; calling into the solver does.  If the
library has not been built the import fails loudly (there is no fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libffcz.so"

FFCZ_OK = 0
FFCZ_F32, FFCZ_F64 = 0, 1
FFCZ_PACK_CORRECT, FFCZ_PACK_REFERENCE = 0, 1
FFCZ_MODE_ALL_ABS, FFCZ_MODE_DIRECT, FFCZ_MODE_ALL_PTW, FFCZ_MODE_PARTIAL_PTW = 0, 1, 2, 3
FFCZ_LOOP_GRAPH, FFCZ_LOOP_HOST = 0, 1
FFCZ_PRECISION_NATIVE, FFCZ_PRECISION_SPLIT = 0, 1
FFCZ_ZSTD_SINGLE, FFCZ_ZSTD_CHUNKED, FFCZ_ZSTD_NONE = 0, 1, 2
FFCZ_FORM_FUSED, FFCZ_FORM_PLAIN = 0, 1
FFCZ_DFT_SIMT, FFCZ_DFT_TENSOR = 0, 1
FFCZ_STAGING_REGISTERS, FFCZ_STAGING_TMA, FFCZ_STAGING_AUTO = 0, 1, 2
FFCZ_EXTRACT_EAGER, FFCZ_EXTRACT_ON_DEMAND = 0, 1
FFCZ_ERR_INVALID, FFCZ_ERR_CUDA, FFCZ_ERR_UNSUPPORTED, FFCZ_ERR_NOT_INITIALIZED = -1, -2, -3, -4
FFCZ_ERR_ZSTD, FFCZ_ERR_CAPACITY, FFCZ_ERR_CODE_TOO_LONG, FFCZ_ERR_EMPTY, FFCZ_ERR_IO = -5, -6, -7, -8, -9
ERRORS = {-1: "INVALID", -2: "CUDA", -3: "UNSUPPORTED", -4: "NOT_INITIALIZED", -5: "ZSTD",
          -6: "CAPACITY", -7: "CODE_TOO_LONG", -8: "EMPTY", -9: "IO"}


class FFCzError(RuntimeError):
    """A non-zero status from the C ABI; ``code`` is the FFCZ_ERR_* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    """Loads libffcz.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = os.environ.get("FFCZ_LIB", str(LIB_PATH))
        if not Path(path).exists():
            raise ImportError(f"libffcz.so not found at {path}; run `python -m ffcz_gb300.build`")
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


_sz = C.c_size_t
_p = C.c_void_p
_i = C.c_int
_d = C.c_double
_PP = C.POINTER(C.c_void_p)
_SP = C.POINTER(C.c_size_t)
_DP = C.POINTER(C.c_double)

# name -> argtypes (all return int unless listed in _RET)
SIGNATURES = {
    "ffcz_solver_create": [_sz, _sz, _sz, _i, _PP],
    "ffcz_solver_destroy": [_p],
    "ffcz_solver_set_stream": [_p, _p],
    "ffcz_solver_set_loop_driver": [_p, _i],
    "ffcz_solver_set_pack_mode": [_p, _i],
    "ffcz_solver_set_form": [_p, _i],
    "ffcz_solver_set_dft_stages": [_p, _i],
    "ffcz_solver_set_staging": [_p, _i],
    "ffcz_solver_set_extraction": [_p, _i],
    "ffcz_solver_get_tuning": [_p, _p, _p],
    "ffcz_init_all_abs": [_p, _p, _d, _d],
    "ffcz_init_all_abs_device": [_p, _p, _d, _d],
    "ffcz_solve_all_abs": [_p, _p, _i, _d],
    "ffcz_solve_all_abs_device": [_p, _p, _i, _d],
    "ffcz_solve_all_abs_pair_device": [_p, _p, _p, _i, _d],
    "ffcz_project_all_abs_device": [_p, _p, _i, _d],
    "ffcz_extract": [_p],
    "ffcz_reset_edit_accumulators": [_p],
    "ffcz_set_edit_accumulators": [_p, _p, _p],
    "ffcz_huff_histogram_device": [_p, _sz, _i, _p, _p],
    "ffcz_huff_tree": [_p, _sz, _p, _p, _p, _p],
    "ffcz_huff_codebook": [_p, _sz, _p, _p, _p, _sz, _SP],
    "ffcz_solver_synchronize": [_p],
    "ffcz_get_iterations": [_p, C.POINTER(C.c_int)],
    "ffcz_get_convergence": [_p, C.POINTER(C.c_double)],
    "ffcz_get_active_counts": [_p, _SP, _SP],
    "ffcz_get_minmax": [_p] + [C.POINTER(C.c_double)] * 4,
    "ffcz_get_results": [_p, _p],
    "ffcz_get_freq_edits_full": [_p, _p, _sz],
    "ffcz_get_spatial_edits_full": [_p, _p, _sz],
    "ffcz_get_freq_quant": [_p, _p, _sz, _SP],
    "ffcz_get_spatial_quant": [_p, _p, _sz, _SP],
    "ffcz_get_freq_compact": [_p, _p, _sz, _SP],
    "ffcz_get_spatial_compact": [_p, _p, _sz, _SP],
    "ffcz_get_freq_flags_pack": [_p, _p, _sz, _SP],
    "ffcz_get_spatial_flags_pack": [_p, _p, _sz, _SP],
    "ffcz_get_freq_flags": [_p, _p, _sz, _SP],
    "ffcz_get_spatial_flags": [_p, _p, _sz, _SP],
    "ffcz_get_device_array": [_p, _i, _PP, _SP],
    "ffcz_get_sizes": [_p, _SP, _SP],
    "ffcz_get_launch_count": [_p, C.POINTER(C.c_longlong)],
    "ffcz_solver_set_profiling": [_p, _i],
    "ffcz_get_pass_times": [_p, _p, _p, _i, C.POINTER(C.c_int)],
    "ffcz_huff_compress_u16": [_p, _sz, _i, _PP],
    "ffcz_huff_compress_u8": [_p, _sz, _i, _PP],
    "ffcz_huff_compress_device": [_p, _sz, _i, _i, _i, _p, _PP],
    "ffcz_huff_result_free": [_p],
    "ffcz_huff_result_sizes": [_p, _SP, _SP, _SP, _SP],
    "ffcz_huff_result_compressed": [_p, _p, _sz],
    "ffcz_huff_result_bitstream": [_p, _p, _sz],
    "ffcz_huff_result_codes": [_p, _p, _p, _p, _sz],
    "ffcz_huff_result_view": [_p, _i, _PP, _SP],
    "ffcz_huff_decompress_u16": [_p, _sz, _p, _p, _p, _sz, _sz, _sz, _p, _SP],
    "ffcz_huff_decompress_u8": [_p, _sz, _p, _p, _p, _sz, _sz, _sz, _p, _SP],
    "ffcz_solver_encode": [_p, _i, _i, C.POINTER(C.c_void_p * 4)],
    "ffcz_zstd_bound": [_sz],
    "ffcz_zstd_compress": [_p, _sz, _i, _i, _p, _sz, _SP],
    "ffcz_compact_quantize_noalloc": [_p, _sz, _i, _p, _p, _p, _i, _p, _SP, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)],
    "ffcz_read_raw": [C.c_char_p, _p, _sz, _sz],
    "ffcz_write_raw": [C.c_char_p, _p, _sz, _sz],
    "ffcz_batch_create": [_PP, _i, _PP],
    "ffcz_batch_destroy": [_p],
    "ffcz_batch_set_stream": [_p, _p],
    "ffcz_batch_reset_edit_accumulators": [_p],
    "ffcz_batch_solve_pair_device": [_p, _PP, _PP, _i, _d],
    "ffcz_huff_decode_device": [_p, _sz, _p, _p, _p, _sz, _sz, _i, _p, _SP, _p],
    "ffcz_huff_zstd_decompress_device": [_p, _sz, _p, _p, _p, _sz, _sz, _sz, _i, _p, _SP, _p],
    "ffcz_huff_result_create": [_p, _sz, _p, _sz, _p, _p, _p, _sz, _sz, _PP],
    "ffcz_reconstruct_device": [_p, _p, _p, _sz, _p, _d, _d, _p, _sz, _p, _d, _d, _p],
    "ffcz_solver_decode": [_p, _p, _PP, _d, _d, _d, _d, _p],
    "ffcz_solver_container_header": [_p, _p],
    "ffcz_container_write": [C.c_char_p, _p, _PP],
    "ffcz_container_read": [C.c_char_p, _p, _PP],
    "ffcz_init_direct": [_p, _p, _p, _p, _d, _sz],
    "ffcz_get_orig_spectrum": [_p, _p, _sz],
    "ffcz_verify_bounds": [_p, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "ffcz_strict_finish": [_p, _i, _d, _i, _p, _p, _p, _p],
    "ffcz_certify_bounds": [_p, _DP, _DP, _DP, C.POINTER(C.c_int)],
    "ffcz_get_strict_report": [_p, C.POINTER(C.c_int), _DP, _DP],
    "ffcz_solver_autotune": [_p, _i, _p],
    "ffcz_solver_set_precision": [_p, _i],
    "ffcz_init_all_ptw": [_p, _p, _d, _d],
    "ffcz_init_all_ptw_device": [_p, _p, _d, _d],
    "ffcz_init_partial_ptw": [_p, _p, _p, _d, _d, _sz],
    "ffcz_solve": [_p, _p, _i, _d],
    "ffcz_solve_all_ptw": [_p, _p, _i, _d],
    "ffcz_solve_mode_device": [_p, _i, _p, _i, _d],
    "ffcz_base_quantize_device": [_p, _sz, _i, _d, _p, _p, _p],
    "ffcz_write_map": [C.c_char_p, _p, _p, _p, _sz],
    "ffcz_read_map": [C.c_char_p, _p, _p, _p, _sz, _SP],
    "ffcz_last_error": [],
    "ffcz_version": [],
}
_RET = {"ffcz_last_error": C.c_char_p, "ffcz_version": C.c_char_p, "ffcz_huff_result_free": None,
        "ffcz_zstd_bound": C.c_size_t}


def _declare(L: C.CDLL) -> None:
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _RET.get(name, C.c_int)


def _check(rc: int) -> None:
    if rc != FFCZ_OK:
        raise FFCzError(rc, lib().ffcz_last_error().decode())


def version() -> str:
    return lib().ffcz_version().decode()


def _np_ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _dev_ptr(t) -> int:
    """Device address of a torch CUDA tensor (or an int address)."""
    if isinstance(t, int):
        return t
    return t.data_ptr()


class ProjectionSolver:
    """ProjectionSolver<T> (projection_algorithm.cuh:238-333) for T = float32/float64.

    Host methods take numpy arrays (borrowed for the call), ``*_device``
    methods take torch CUDA tensors (or raw device addresses)."""

    def __init__(self, nx: int, ny: int, nz: int, dtype=np.float32):
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.float32, np.float64):
            raise ValueError("dtype must be float32 or float64")
        self.shape = (int(nx), int(ny), int(nz))
        self.N = int(nx) * int(ny) * int(nz)
        self.H = int(nx) * int(ny) * (int(nz) // 2 + 1)
        h = C.c_void_p()
        _check(lib().ffcz_solver_create(nx, ny, nz, FFCZ_F32 if self.dtype == np.float32 else FFCZ_F64,
                                        C.byref(h)))
        self._h = h
        self.iterations = 0

    # -- lifetime ----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().ffcz_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration -------------------------------------------------------
    def set_stream(self, stream) -> None:
        """stream: torch.cuda.Stream, a raw cudaStream_t int, or None."""
        ptr = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
        _check(lib().ffcz_solver_set_stream(self._h, C.c_void_p(ptr)))

    def set_loop_driver(self, driver: int) -> None:
        _check(lib().ffcz_solver_set_loop_driver(self._h, driver))

    def set_precision(self, precision: int) -> None:
        """FFCZ_PRECISION_NATIVE or FFCZ_PRECISION_SPLIT (FP64 solvers:
        float-float pass kernels on the FP32 pipes where a length has them)."""
        _check(lib().ffcz_solver_set_precision(self._h, int(precision)))

    def set_pack_mode(self, mode: int) -> None:
        _check(lib().ffcz_solver_set_pack_mode(self._h, mode))

    def set_form(self, form: int) -> None:
        """FFCZ_FORM_FUSED (five passes per 3D iteration) or FFCZ_FORM_PLAIN
        (six: x forward + clamp and x inverse as separate passes)."""
        _check(lib().ffcz_solver_set_form(self._h, int(form)))

    def set_dft_stages(self, stages: int) -> None:
        """FFCZ_DFT_SIMT or FFCZ_DFT_TENSOR (radix-16 stages of the FP32
        strided passes of length 256/512 as tensor-core DFT matrix products)."""
        _check(lib().ffcz_solver_set_dft_stages(self._h, int(stages)))

    def set_staging(self, staging: int) -> None:
        """FFCZ_STAGING_REGISTERS, FFCZ_STAGING_TMA (persistent strided passes
        fed by tensor-map copies issued ahead; identical results) or
        FFCZ_STAGING_AUTO (the autotuner picks per axis)."""
        _check(lib().ffcz_solver_set_staging(self._h, int(staging)))

    def set_extraction(self, mode: int) -> None:
        """FFCZ_EXTRACT_EAGER (compact at the end of every solve, as the
        reference) or FFCZ_EXTRACT_ON_DEMAND (compact when the results are
        first read or the edit arrays about to change; same results)."""
        _check(lib().ffcz_solver_set_extraction(self._h, int(mode)))

    def tuning(self) -> dict:
        """Current tile choice per pass ({"z"|"y"|"x": (variant, staged)})
        and the autotuner's last timings."""
        ch = np.zeros(3, np.int32)
        ms = np.zeros(10)
        _check(lib().ffcz_solver_get_tuning(self._h, _np_ptr(ch), _np_ptr(ms)))
        return {"choice": {k: (int(ch[i]) & 1, bool(int(ch[i]) & 2)) for i, k in enumerate("zyx")},
                "ms": {"z": (ms[0], ms[1]), "y": (ms[2], ms[3]), "x": (ms[4], ms[5]),
                       "y_tma": (ms[6], ms[7]), "x_tma": (ms[8], ms[9])}}

    # -- reference API -------------------------------------------------------
    def _host(self, a) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=self.dtype).reshape(-1)
        if a.size != self.N:
            raise ValueError(f"expected {self.N} elements, got {a.size}")
        return a

    def initialize_all_abs(self, x, spatial_epsilon: float, delta: float) -> None:
        x = self._host(x)
        _check(lib().ffcz_init_all_abs(self._h, _np_ptr(x), float(spatial_epsilon), float(delta)))

    def initialize_all_abs_device(self, d_x, spatial_epsilon: float, delta: float) -> None:
        _check(lib().ffcz_init_all_abs_device(self._h, _dev_ptr(d_x), float(spatial_epsilon), float(delta)))

    def solve_all_abs(self, e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        e0 = self._host(e0)
        _check(lib().ffcz_solve_all_abs(self._h, _np_ptr(e0), int(max_iterations), float(tol)))
        return self._iters()

    def solve_all_abs_device(self, d_e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        _check(lib().ffcz_solve_all_abs_device(self._h, _dev_ptr(d_e0), int(max_iterations), float(tol)))
        return self._iters()

    def solve_all_abs_pair_device(self, d_x, d_xprime, max_iterations: int = 100, tol: float = 1e-7) -> int:
        _check(lib().ffcz_solve_all_abs_pair_device(self._h, _dev_ptr(d_x), _dev_ptr(d_xprime),
                                                     int(max_iterations), float(tol)))
        return self._iters()

    # -- the other constraint modes (impl:598-738, 772-814, 860-902) --------
    def _indices(self, idx) -> np.ndarray:
        return np.ascontiguousarray(idx, dtype=np.uint64).reshape(-1)

    def initialize(self, x, freq_indices, delta_k, spatial_epsilon: float) -> None:
        """Direct mode: coefficient freq_indices[c] within +-delta_k[c]."""
        x = self._host(x)
        idx = self._indices(freq_indices)
        dk = np.ascontiguousarray(delta_k, dtype=self.dtype).reshape(-1)
        if dk.size != idx.size:
            raise ValueError("one delta_k per index")
        _check(lib().ffcz_init_direct(self._h, _np_ptr(x), _np_ptr(idx) if idx.size else None,
                                      _np_ptr(dk) if dk.size else None, float(spatial_epsilon), idx.size))

    def initialize_all_ptw(self, x, spatial_epsilon: float, delta_ptw: float) -> None:
        x = self._host(x)
        _check(lib().ffcz_init_all_ptw(self._h, _np_ptr(x), float(spatial_epsilon), float(delta_ptw)))

    def initialize_all_ptw_device(self, d_x, spatial_epsilon: float, delta_ptw: float) -> None:
        _check(lib().ffcz_init_all_ptw_device(self._h, _dev_ptr(d_x), float(spatial_epsilon), float(delta_ptw)))

    def initialize_partial_ptw(self, x, freq_indices, delta_ptw: float, spatial_epsilon: float) -> None:
        x = self._host(x)
        idx = self._indices(freq_indices)
        _check(lib().ffcz_init_partial_ptw(self._h, _np_ptr(x), _np_ptr(idx) if idx.size else None,
                                           float(delta_ptw), float(spatial_epsilon), idx.size))

    def autotune(self, reps: int = 5) -> dict:
        """Keeps the fastest of two tile widths per pass, and for the FP32
        strided passes of register or TMA staging (results unchanged);
        returns {pass: (default ms, alternative ms)} with the staged strided
        passes as "y_tma" / "x_tma" (0 = not timed)."""
        ms = np.zeros(6)
        _check(lib().ffcz_solver_autotune(self._h, int(reps), _np_ptr(ms)))
        return self.tuning()["ms"]

    def verify_bounds(self) -> tuple[float, float]:
        """(max |e|, max over the half spectrum of max(|Re|, |Im|) of e's R2C),
        both in FP64 on the device."""
        a, b = C.c_double(), C.c_double()
        _check(lib().ffcz_verify_bounds(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def strict_finish(self, max_iterations: int = 100, tol: float = 1e-7, max_rounds: int = 4) -> dict:
        """Makes the last all-abs result meet both bounds in FP64 (clamp to
        the largest value <= eps, FP64 check, re-runs on a shrunk frequency
        box while a coefficient exceeds delta).  Returns rounds, met and the
        FP64 maxima; iterations() is the total afterwards."""
        r, m = C.c_int(), C.c_int()
        a, b = C.c_double(), C.c_double()
        _check(lib().ffcz_strict_finish(self._h, int(max_iterations), float(tol), int(max_rounds), C.byref(r),
                                        C.byref(m), C.byref(a), C.byref(b)))
        self._iters()
        c, f, bd = C.c_int(), C.c_double(), C.c_double()
        _check(lib().ffcz_get_strict_report(self._h, C.byref(c), C.byref(f), C.byref(bd)))
        return {"rounds": r.value, "met": bool(m.value), "spatial_max": a.value, "freq_max": b.value,
                "certified": bool(c.value),
                "certified_by": {0: None, 1: "transform", 2: "recorded clamp maximum"}[c.value],
                "cert_freq_max": f.value, "cert_bound": bd.value}

    def certify_bounds(self) -> dict:
        """Certificate of both bounds from the solver's own transform of e and
        a bound on its rounding (no FP64 transform); e is not changed."""
        a, f, bd, c = C.c_double(), C.c_double(), C.c_double(), C.c_int()
        _check(lib().ffcz_certify_bounds(self._h, C.byref(a), C.byref(f), C.byref(bd), C.byref(c)))
        return {"spatial_max": a.value, "freq_max": f.value, "bound": bd.value, "certified": bool(c.value)}

    def get_orig_spectrum(self) -> np.ndarray:
        """The spectrum of x the pointwise modes compare against (H complex)."""
        out = np.empty(self.H, np.complex64 if self.dtype == np.float32 else np.complex128)
        _check(lib().ffcz_get_orig_spectrum(self._h, _np_ptr(out), self.H))
        return out

    def solve(self, e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        e0 = self._host(e0)
        _check(lib().ffcz_solve(self._h, _np_ptr(e0), int(max_iterations), float(tol)))
        return self._iters()

    def solve_all_ptw(self, e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        e0 = self._host(e0)
        _check(lib().ffcz_solve_all_ptw(self._h, _np_ptr(e0), int(max_iterations), float(tol)))
        return self._iters()

    def solve_mode_device(self, mode: int, d_e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        _check(lib().ffcz_solve_mode_device(self._h, int(mode), _dev_ptr(d_e0), int(max_iterations), float(tol)))
        return self._iters()

    def project_all_abs_device(self, d_e0, max_iterations: int = 100, tol: float = 1e-7) -> int:
        _check(lib().ffcz_project_all_abs_device(self._h, _dev_ptr(d_e0), int(max_iterations), float(tol)))
        return self._iters()

    def extract_compact_representation(self) -> None:
        _check(lib().ffcz_extract(self._h))

    def reset_edit_accumulators(self) -> None:
        _check(lib().ffcz_reset_edit_accumulators(self._h))

    def set_edit_accumulators(self, freq_edits=None, spatial_edits=None) -> None:
        """Loads edit arrays computed elsewhere (2H planar frequency edits,
        N spatial edits; None keeps an accumulator) for extract / encode."""
        keep = []
        ptrs = []
        for a, n in ((freq_edits, 2 * self.H), (spatial_edits, self.N)):
            if a is None:
                ptrs.append(None)
                continue
            a = np.ascontiguousarray(a, self.dtype).reshape(-1)
            if a.size != n:
                raise ValueError(f"edit array of {a.size} elements, expected {n}")
            keep.append(a)
            ptrs.append(_np_ptr(a))
        _check(lib().ffcz_set_edit_accumulators(self._h, *ptrs))

    def synchronize(self) -> None:
        _check(lib().ffcz_solver_synchronize(self._h))

    def _iters(self) -> int:
        v = C.c_int()
        _check(lib().ffcz_get_iterations(self._h, C.byref(v)))
        self.iterations = v.value
        return v.value

    # -- getters ---------------------------------------------------------------
    @property
    def convergence_metric(self) -> float:
        v = C.c_double()
        _check(lib().ffcz_get_convergence(self._h, C.byref(v)))
        return v.value

    def active_counts(self) -> tuple[int, int]:
        a, b = C.c_size_t(), C.c_size_t()
        _check(lib().ffcz_get_active_counts(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def minmax(self) -> tuple[float, float, float, float]:
        v = [C.c_double() for _ in range(4)]
        _check(lib().ffcz_get_minmax(self._h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def get_min_freq_edit(self): return self.dtype.type(self.minmax()[0])
    def get_max_freq_edit(self): return self.dtype.type(self.minmax()[1])
    def get_min_spatial_edit(self): return self.dtype.type(self.minmax()[2])
    def get_max_spatial_edit(self): return self.dtype.type(self.minmax()[3])

    def get_results(self) -> np.ndarray:
        out = np.empty(self.N, self.dtype)
        _check(lib().ffcz_get_results(self._h, _np_ptr(out)))
        return out.reshape(self.shape)

    def get_freq_edits_full(self) -> np.ndarray:
        out = np.empty(2 * self.H, self.dtype)
        _check(lib().ffcz_get_freq_edits_full(self._h, _np_ptr(out), out.size))
        return out

    def get_spatial_edits_full(self) -> np.ndarray:
        out = np.empty(self.N, self.dtype)
        _check(lib().ffcz_get_spatial_edits_full(self._h, _np_ptr(out), out.size))
        return out

    def _stream(self, fn, count: int, dtype) -> np.ndarray:
        out = np.empty(max(count, 1), dtype)
        n = C.c_size_t()
        _check(getattr(lib(), fn)(self._h, _np_ptr(out), out.size, C.byref(n)))
        return out[: n.value]

    def get_active_freq_quant_edit_distances(self):
        return self._stream("ffcz_get_freq_quant", self.active_counts()[0], np.uint16)

    def get_active_spatial_quant_edit_distances(self):
        return self._stream("ffcz_get_spatial_quant", self.active_counts()[1], np.uint16)

    def get_active_freq_edit_distances(self):
        return self._stream("ffcz_get_freq_compact", self.active_counts()[0], self.dtype)

    def get_active_spatial_edit_distances(self):
        return self._stream("ffcz_get_spatial_compact", self.active_counts()[1], self.dtype)

    def get_freq_flags_pack(self):
        return self._stream("ffcz_get_freq_flags_pack", (2 * self.H + 7) // 8, np.uint8)

    def get_spatial_flags_pack(self):
        return self._stream("ffcz_get_spatial_flags_pack", (self.N + 7) // 8, np.uint8)

    def get_freq_flags(self):
        return self._stream("ffcz_get_freq_flags", 2 * self.H, np.uint8).astype(bool)

    def get_spatial_flags(self):
        return self._stream("ffcz_get_spatial_flags", self.N, np.uint8).astype(bool)

    def device_array(self, which: int) -> tuple[int, int]:
        p, n = C.c_void_p(), C.c_size_t()
        _check(lib().ffcz_get_device_array(self._h, which, C.byref(p), C.byref(n)))
        return p.value or 0, n.value

    def set_profiling(self, on: bool) -> None:
        _check(lib().ffcz_solver_set_profiling(self._h, int(bool(on))))

    def pass_times(self) -> list[tuple[float, float]]:
        """[(ms, algorithmic bytes)] per pass of the last solve's first iteration."""
        ms, by = np.zeros(8), np.zeros(8)
        n = C.c_int()
        _check(lib().ffcz_get_pass_times(self._h, _np_ptr(ms), _np_ptr(by), 8, C.byref(n)))
        return [(float(ms[i]), float(by[i])) for i in range(n.value)]

    def launch_count(self) -> int:
        v = C.c_longlong()
        _check(lib().ffcz_get_launch_count(self._h, C.byref(v)))
        return v.value

    def reconstruct_device(self, d_xprime, d_out, freq=None, spatial=None) -> None:
        """x^ = x' + (C2R(F)/N + S) from decoded streams on the device.
        freq / spatial: (d_quant, count, d_pack, min, max) or None."""
        fq, nf, fp, fmn, fmx = freq if freq else (0, 0, 0, 0.0, 0.0)
        sq, ns, sp, smn, smx = spatial if spatial else (0, 0, 0, 0.0, 0.0)
        _check(lib().ffcz_reconstruct_device(self._h, _dev_ptr(d_xprime), _dev_ptr(fq) or None, nf,
                                             _dev_ptr(fp) or None, fmn, fmx, _dev_ptr(sq) or None, ns,
                                             _dev_ptr(sp) or None, smn, smx, _dev_ptr(d_out)))

    def container_header(self) -> "ContainerHeader":
        h = ContainerHeader()
        _check(lib().ffcz_solver_container_header(self._h, C.byref(h)))
        return h

    def decode_device(self, d_xprime, streams, minmax, d_out) -> None:
        """The decoder: the four CompressionResults of :meth:`encode` (None
        where empty) and :meth:`minmax`'s values -> x^ in d_out (device)."""
        handles = [None if r is None else r.native() for r in streams]
        arr = (C.c_void_p * 4)(*[h.value if h is not None else None for h in handles])
        try:
            _check(lib().ffcz_solver_decode(self._h, _dev_ptr(d_xprime), arr, *[float(v) for v in minmax],
                                            _dev_ptr(d_out)))
        finally:
            for h in handles:
                if h is not None:
                    lib().ffcz_huff_result_free(h)

    def encode(self, zstd_level: int = 20, zstd_mode: int = FFCZ_ZSTD_SINGLE) -> list:
        """The four streams of projection_example.cu:230-246 (None where skipped).
        FFCZ_ZSTD_NONE returns the Huffman bitstreams with empty compressed_data."""
        arr = (C.c_void_p * 4)()
        _check(lib().ffcz_solver_encode(self._h, zstd_level, zstd_mode, C.byref(arr)))
        return [None if not p else _take_result(p) for p in arr]


# ---------------------------------------------------------------------------
class CompressionResult:
    """SimpleCudaHuffmanZstdCompressor<T>::CompressionResult (HuffmanZSTDCoder.cuh:240-246).

    ``compressed_data`` (bytes), ``original_bitstream_size``, ``num_elements``;
    the code table as arrays (``symbols``, ``codes``, ``lengths``, ascending
    symbols) and as the reference's map ``code_table`` (built on first use)."""

    def __init__(self, compressed_data, symbols, codes, lengths, original_bitstream_size, num_elements,
                 bitstream=b""):
        self.compressed_data = compressed_data
        self.symbols, self.codes, self.lengths = symbols, codes, lengths
        self.original_bitstream_size = original_bitstream_size
        self.num_elements = num_elements
        self.bitstream = bitstream
        self._table = None

    @property
    def code_table(self) -> dict:
        if self._table is None:
            self._table = dict(zip(self.symbols.tolist(), zip(self.codes.tolist(), self.lengths.tolist())))
        return self._table

    def arrays(self):
        return self.symbols, self.codes, self.lengths

    def native(self) -> C.c_void_p:
        """A C-ABI result handle of this result (caller frees it with
        ffcz_huff_result_free); the bitstream is recovered from the ZSTD
        frame when this result does not hold it."""
        syms, codes, lens = (np.ascontiguousarray(a, dt) for a, dt in
                             zip((self.symbols, self.codes, self.lengths), (np.uint32, np.uint32, np.int32)))
        comp = np.frombuffer(self.compressed_data, np.uint8) if len(self.compressed_data) else None
        bits = np.frombuffer(self.bitstream, np.uint8) if len(self.bitstream) else None
        h = C.c_void_p()
        _check(lib().ffcz_huff_result_create(None if comp is None else _np_ptr(comp), len(self.compressed_data),
                                             None if bits is None else _np_ptr(bits), self.original_bitstream_size,
                                             _np_ptr(syms) if syms.size else None,
                                             _np_ptr(codes) if codes.size else None,
                                             _np_ptr(lens) if lens.size else None, syms.size, self.num_elements,
                                             C.byref(h)))
        return h

    def __repr__(self):
        return (f"CompressionResult(compressed={len(self.compressed_data)} B, bitstream="
                f"{self.original_bitstream_size} B, elements={self.num_elements}, symbols={self.symbols.size})")


class Batch:
    """Many fields of uneven shapes corrected in one graph launch (no
    counterpart in the reference, whose CLI corrects one field per run).

    ``solvers`` are initialised ProjectionSolver handles, one per field; the
    batch keeps them alive.  After :meth:`solve_pair_device` each field's
    results are read through its own solver, and equal what
    ``solver.solve_all_abs_pair_device`` gives, bit for bit: every field runs
    its own device-side loop and retires when it converges."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        _check(lib().ffcz_batch_create(arr, len(self.solvers), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            lib().ffcz_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream) -> None:
        ptr = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
        _check(lib().ffcz_batch_set_stream(self._h, C.c_void_p(ptr)))

    def reset_edit_accumulators(self) -> None:
        _check(lib().ffcz_batch_reset_edit_accumulators(self._h))

    def solve_pair_device(self, d_xs, d_xprimes, max_iterations: int = 100, tol: float = 1e-7) -> list[int]:
        """Returns each field's iteration count."""
        n = len(self.solvers)
        if len(d_xs) != n or len(d_xprimes) != n:
            raise ValueError(f"expected {n} fields")
        a = (C.c_void_p * n)(*[_dev_ptr(t) for t in d_xs])
        b = (C.c_void_p * n)(*[_dev_ptr(t) for t in d_xprimes])
        _check(lib().ffcz_batch_solve_pair_device(self._h, a, b, int(max_iterations), float(tol)))
        return [s._iters() for s in self.solvers]


def _view(p, which):
    ptr, n = C.c_void_p(), C.c_size_t()
    _check(lib().ffcz_huff_result_view(p, which, C.byref(ptr), C.byref(n)))
    return ptr.value, n.value


def _take_result(p: int) -> CompressionResult:
    """Copies a native result into Python objects and frees it."""
    try:
        cp, cn = _view(p, 0)
        bp, bn = _view(p, 1)
        bits = C.string_at(bp, bn) if bn else b""
        comp = C.string_at(cp, cn) if cn else b""
        arrs = []
        for which, dt in ((2, np.uint32), (3, np.uint32), (4, np.int32)):
            ap, an = _view(p, which)
            arrs.append(np.frombuffer(C.string_at(ap, an * 4), dt) if an else np.zeros(0, dt))
        nel = C.c_size_t()
        _check(lib().ffcz_huff_result_sizes(p, None, None, C.byref(nel), None))
        return CompressionResult(comp, *arrs, bn, nel.value, bits)
    finally:
        lib().ffcz_huff_result_free(p)


class ContainerHeader(C.Structure):
    """ffcz_container_header: what the decoder needs besides x' and the streams."""
    _fields_ = [("dtype", C.c_uint32), ("pack_mode", C.c_uint32), ("nx", C.c_uint64), ("ny", C.c_uint64),
                ("nz", C.c_uint64), ("eps", C.c_double), ("delta", C.c_double), ("freq_min", C.c_double),
                ("freq_max", C.c_double), ("spatial_min", C.c_double), ("spatial_max", C.c_double),
                ("iterations", C.c_uint32)]

    @property
    def shape(self):
        return (self.nx, self.ny, self.nz)

    @property
    def minmax(self):
        return (self.freq_min, self.freq_max, self.spatial_min, self.spatial_max)


def write_container(path, header: ContainerHeader, streams) -> None:
    """Writes the .ffcz container (header + the four coder results)."""
    handles = [None if r is None else r.native() for r in streams]
    arr = (C.c_void_p * 4)(*[h.value if h is not None else None for h in handles])
    try:
        _check(lib().ffcz_container_write(str(path).encode(), C.byref(header), arr))
    finally:
        for h in handles:
            if h is not None:
                lib().ffcz_huff_result_free(h)


def read_container(path):
    """(ContainerHeader, [four CompressionResult or None]) of a .ffcz file."""
    h = ContainerHeader()
    arr = (C.c_void_p * 4)()
    _check(lib().ffcz_container_read(str(path).encode(), C.byref(h), arr))
    return h, [None if not p else _take_result(p) for p in arr]


def cuda_huffman_zstd_compress(data, zstd_level: int = 3) -> CompressionResult:
    """cudaHuffmanZstdCompress<T> for uint8 / uint16 host data."""
    a = np.ascontiguousarray(data)
    if a.dtype not in (np.uint8, np.uint16):
        raise TypeError("symbols must be uint8 or uint16")
    out = C.c_void_p()
    fn = lib().ffcz_huff_compress_u16 if a.dtype == np.uint16 else lib().ffcz_huff_compress_u8
    _check(fn(_np_ptr(a) if a.size else None, a.size, int(zstd_level), C.byref(out)))
    return _take_result(out.value)


def cuda_huffman_zstd_compress_device(d_data, n: int, symbol_bytes: int, zstd_level: int = 3,
                                      zstd_mode: int = FFCZ_ZSTD_SINGLE, stream=None) -> CompressionResult:
    out = C.c_void_p()
    sp = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
    _check(lib().ffcz_huff_compress_device(_dev_ptr(d_data), n, symbol_bytes, zstd_level, zstd_mode,
                                            C.c_void_p(sp), C.byref(out)))
    return _take_result(out.value)


def zstd_compress(data: bytes, level: int, mode: int = FFCZ_ZSTD_SINGLE) -> bytes:
    """The coder's ZSTD stage on host bytes (native; releases the GIL)."""
    src = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
    cap = lib().ffcz_zstd_bound(len(data))
    if cap == 0:
        raise FFCzError(-5, "libzstd.so.1 not available")
    dst = np.empty(cap, np.uint8)
    n = C.c_size_t()
    _check(lib().ffcz_zstd_compress(_np_ptr(src), len(data), int(level), int(mode), _np_ptr(dst), cap, C.byref(n)))
    return bytes(dst[: n.value])


def _table_arrays(code_table):
    if isinstance(code_table, dict):
        syms = np.array(sorted(code_table), dtype=np.uint32)
        codes = np.array([code_table[s][0] for s in syms], dtype=np.uint32)
        lens = np.array([code_table[s][1] for s in syms], dtype=np.int32)
        return syms, codes, lens
    return tuple(np.ascontiguousarray(a, dt) for a, dt in zip(code_table, (np.uint32, np.uint32, np.int32)))


def base_quantize_device(d_x, eps: float, d_xprime, d_index=None, stream=None) -> None:
    """x' = 2eps * rint(x / 2eps) on the device (torch CUDA tensors of float32
    or float64); d_index (int32) optionally receives the quantisation indices."""
    import torch

    dt = FFCZ_F32 if d_x.dtype == torch.float32 else FFCZ_F64
    ptr = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
    _check(lib().ffcz_base_quantize_device(_dev_ptr(d_x), d_x.numel(), dt, float(eps), _dev_ptr(d_xprime),
                                           None if d_index is None else _dev_ptr(d_index), C.c_void_p(ptr)))


def huff_decode_device(d_bits, nbytes: int, code_table, num_elements: int, dtype, d_out, stream=None) -> int:
    """GPU prefix decode of a device-resident Huffman bitstream (the host
    decoder's rules); returns the number of symbols written to d_out."""
    syms, codes, lens = _table_arrays(code_table)
    n = C.c_size_t()
    ptr = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
    _check(lib().ffcz_huff_decode_device(_dev_ptr(d_bits), nbytes, _np_ptr(syms) if syms.size else None,
                                         _np_ptr(codes) if codes.size else None,
                                         _np_ptr(lens) if lens.size else None, syms.size, num_elements,
                                         np.dtype(dtype).itemsize, _dev_ptr(d_out), C.byref(n), C.c_void_p(ptr)))
    return n.value


def huff_zstd_decompress_device(compressed: bytes, code_table, num_elements: int, original_bitstream_size: int,
                                dtype, d_out, stream=None) -> int:
    """ZSTD on the host, then the GPU decode into d_out; returns the count."""
    syms, codes, lens = _table_arrays(code_table)
    comp = np.frombuffer(compressed, np.uint8) if len(compressed) else np.zeros(1, np.uint8)
    n = C.c_size_t()
    ptr = 0 if stream is None else (stream if isinstance(stream, int) else stream.cuda_stream)
    _check(lib().ffcz_huff_zstd_decompress_device(_np_ptr(comp), len(compressed),
                                                  _np_ptr(syms) if syms.size else None,
                                                  _np_ptr(codes) if codes.size else None,
                                                  _np_ptr(lens) if lens.size else None, syms.size, num_elements,
                                                  original_bitstream_size, np.dtype(dtype).itemsize,
                                                  _dev_ptr(d_out), C.byref(n), C.c_void_p(ptr)))
    return n.value


def cuda_huffman_zstd_decompress(compressed: bytes, code_table, num_elements: int,
                                 original_bitstream_size: int, dtype=np.uint16) -> np.ndarray:
    """cudaHuffmanZstdDecompress<T> (HuffmanZSTDCoder.cuh:462-470).  code_table:
    {symbol: (code, length)} or a (symbols, codes, lengths) array triple."""
    dtype = np.dtype(dtype)
    if isinstance(code_table, dict):
        syms = np.array(sorted(code_table), dtype=np.uint32)
        codes = np.array([code_table[s][0] for s in syms], dtype=np.uint32)
        lens = np.array([code_table[s][1] for s in syms], dtype=np.int32)
    else:
        syms, codes, lens = (np.ascontiguousarray(a, dt) for a, dt in
                             zip(code_table, (np.uint32, np.uint32, np.int32)))
    comp = np.frombuffer(compressed, np.uint8) if len(compressed) else np.zeros(1, np.uint8)
    out = np.empty(max(num_elements, 1), dtype)
    n = C.c_size_t()
    fn = lib().ffcz_huff_decompress_u16 if dtype == np.uint16 else lib().ffcz_huff_decompress_u8
    _check(fn(_np_ptr(comp), len(compressed), _np_ptr(syms) if syms.size else None,
              _np_ptr(codes) if codes.size else None, _np_ptr(lens) if lens.size else None, syms.size,
              num_elements, original_bitstream_size, _np_ptr(out), C.byref(n)))
    return out[: n.value]


# ---------------------------------------------------------------------------
def read_raw_array_binary(path, n: int, dtype) -> np.ndarray:
    """readRawArrayBinary (fileIO.cpp:35-76)."""
    dtype = np.dtype(dtype)
    out = np.empty(max(n, 1), dtype)
    _check(lib().ffcz_read_raw(str(path).encode(), _np_ptr(out), n, dtype.itemsize))
    return out[:n]


def write_raw_array_binary(a, path) -> None:
    """writeRawArrayBinary / writeVectorBinary (fileIO.h:23-55)."""
    a = np.ascontiguousarray(a)
    _check(lib().ffcz_write_raw(str(path).encode(), _np_ptr(a), a.size, a.dtype.itemsize))


def write_map(m: dict, path) -> None:
    """writeMap (fileIO.cpp:3-14): {int key: (uint32 code, int len)}."""
    keys = np.array(sorted(m), dtype=np.int32)
    codes = np.array([m[k][0] for k in keys], dtype=np.uint32)
    lens = np.array([m[k][1] for k in keys], dtype=np.int32)
    _check(lib().ffcz_write_map(str(path).encode(), _np_ptr(keys), _np_ptr(codes), _np_ptr(lens), keys.size))


def read_map(path) -> dict:
    """readMap (fileIO.cpp:16-33)."""
    n = C.c_size_t()
    rc = lib().ffcz_read_map(str(path).encode(), None, None, None, 0, C.byref(n))
    if rc not in (FFCZ_OK, -6):
        _check(rc)
    k = max(n.value, 1)
    keys, codes, lens = np.empty(k, np.int32), np.empty(k, np.uint32), np.empty(k, np.int32)
    _check(lib().ffcz_read_map(str(path).encode(), _np_ptr(keys), _np_ptr(codes), _np_ptr(lens), k,
                               C.byref(n)))
    return {int(keys[i]): (int(codes[i]), int(lens[i])) for i in range(n.value)}
