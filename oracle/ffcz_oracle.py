"""FFCz oracle -- TEST INFRASTRUCTURE ONLY.

CPU restatement of the reference algorithm, used by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
The product never imports this module.

* ``solve_all_abs`` restates ProjectionSolver<T>::solve_all_abs
  (projection_algorithm_impl.cuh:816-858) with pocketfft (scipy.fft) in FP64:
  the transforms are computed in double precision and rounded to T; every
  elementwise step (frequency clamp and edit accumulation,
  projection_algorithm.cu:148-188; normalisation by T(1)/T(N),
  projection_algorithm_impl.cuh:241-247; violation max(|e|-E, 0),
  projection_algorithm.cu:586-594 and impl:762-769; termination
  "metric < tol" after the frequency projection, impl:841-848; spatial clamp,
  projection_algorithm.cu:336-361) runs in T.  With T = float64 this is the
  FP64 oracle.
* ``extract`` restates extract_compact_representation (impl:371-456) via the
  C restatement in ffcz_oracle.c.
* ``huffman_*`` restate HuffmanZSTDCoder.cuh:48-449 via ffcz_oracle.c; ZSTD
  is libzstd itself (the reference's dependency, version 1.5.5 here).
* ``check_bounds`` is the FP64 check of both bounds.

Pinning: the Huffman codebook and decoder are checked against the
reference's own functions (tests/golden/huffman_reference.npz, generated by
oracle/ref_harness.cu compiled from the reference sources); the projection
loop, the compaction, the quantiser, the flag packs and the coder are
checked against the reference's own cuFFT build run on a GPU
(tests/golden/ref_*.npz, generated by oracle/ref_solver.cu).  The
reference ships no golden vectors of its own.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

try:
    import scipy.fft as _sfft

    def _rfftn(a):
        return _sfft.rfftn(a, workers=-1)

    def _irfftn(a, s):
        return _sfft.irfftn(a, s=s, workers=-1)
except ImportError:  # pragma: no cover
    def _rfftn(a):
        return np.fft.rfftn(a)

    def _irfftn(a, s):
        return np.fft.irfftn(a, s=s)

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
THRESHOLD = 1e-7  # projection_algorithm_impl.cuh:389, 398


def reference_sources() -> Path | None:
    """The directory holding the reference sources: FFCZ_REF when set, else
    the repository's git-ignored copy baseline/_ref when present, else None."""
    env = os.environ.get("FFCZ_REF")
    if env:
        return Path(env)
    local = HERE.parent / "baseline" / "_ref"
    return local if (local / "projection_algorithm.cuh").exists() else None


def build() -> Path:
    """Compiles ffcz_oracle.c into oracle/_build/liboracle.so (gcc)."""
    LIB.parent.mkdir(exist_ok=True)
    src = HERE / "ffcz_oracle.c"
    if not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", str(src),
                        "-o", str(LIB), "-lm"], check=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        p, sz = C.c_void_p, C.c_size_t
        L.orc_flags_minmax_f32.argtypes = [p, sz, C.c_float, p, p, p, p]
        L.orc_flags_minmax_f64.argtypes = [p, sz, C.c_double, p, p, p, p]
        L.orc_compact_quantize_f32.argtypes = [p, sz, C.c_float, C.c_float, C.c_float, p, p]
        L.orc_compact_quantize_f64.argtypes = [p, sz, C.c_double, C.c_double, C.c_double, p, p]
        L.orc_compact_quantize_f32.restype = sz
        L.orc_compact_quantize_f64.restype = sz
        L.orc_quantize_f32.argtypes = [C.c_float, C.c_float, C.c_float]
        L.orc_quantize_f32.restype = C.c_uint16
        L.orc_quantize_f64.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_quantize_f64.restype = C.c_uint16
        L.orc_pack_flags.argtypes = [p, sz, p, C.c_int]
        L.orc_huff_codebook.argtypes = [p, sz, sz, p, p, p, p]
        L.orc_huff_codebook.restype = sz
        L.orc_huff_pack.argtypes = [p, sz, p, p, p, p]
        L.orc_huff_pack.restype = sz
        L.orc_huff_decode.argtypes = [p, sz, p, p, p, sz, sz, p]
        L.orc_huff_decode.restype = sz
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# --------------------------------------------------------------- projection
def _loop(e0, shape, eps, max_iter, tol, dtype, clamp):
    """The alternating-projection loop shared by every solve of
    projection_algorithm_impl.cuh:772-902: R2C, clamp(re, im, freq_edits)
    (in place on the half spectrum's real and imaginary parts, flat index
    order), C2R * T(1)/T(N), violation, stop when it is below tol, spatial
    clamp."""
    T = np.dtype(dtype).type
    shape = tuple(int(s) for s in shape)
    N = int(np.prod(shape))
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)
    eps, tol = T(eps), T(tol)
    factor = T(1) / T(N)
    e = np.array(e0, dtype=T).reshape(shape)
    fed = np.zeros(2 * H, T)
    sed = np.zeros(N, T)
    it = 0
    viol = T(0)
    converged = False
    cplx = np.complex64 if T is np.float32 else np.complex128
    for _ in range(max_iter):
        F = _rfftn(e.astype(np.float64)).astype(cplx)
        fshape = F.shape
        re = np.ascontiguousarray(F.real).reshape(-1)
        im = np.ascontiguousarray(F.imag).reshape(-1)
        clamp(re, im, fed)
        G = (re.astype(np.float64) + 1j * im.astype(np.float64)).reshape(fshape)
        e = (_irfftn(G, s=shape) * N).astype(T) * factor
        a = np.abs(e)
        viol = T(np.max(np.where(a > eps, a - eps, T(0))))
        it += 1
        if viol < tol:
            converged = True
            break
        flat = e.reshape(-1)
        hi = flat > eps
        lo = flat < -eps
        sed[hi] += eps - flat[hi]
        flat[hi] = eps
        sed[lo] += -eps - flat[lo]
        flat[lo] = -eps
    return {"e": e, "freq_edits": fed, "spatial_edits": sed, "iterations": it, "metric": float(viol),
            "converged": converged}


def _box(part, bound, view):
    """Re or Im clamp of projection_algorithm.cu:160-187 with a per-entry
    bound (scalar or array): above -> bound, below -bound -> -bound, the
    difference accumulated into view."""
    hi = part > bound
    lo = (part < -bound) & ~hi
    b = np.broadcast_to(bound, part.shape)
    view[hi] += b[hi] - part[hi]
    part[hi] = b[hi]
    view[lo] += -b[lo] - part[lo]
    part[lo] = -b[lo]


def solve_all_abs(e0: np.ndarray, shape, eps: float, delta: float, max_iter: int = 100, tol: float = 1e-7,
                  dtype=np.float32) -> dict:
    """Alternating projections of projection_algorithm_impl.cuh:816-858."""
    T = np.dtype(dtype).type
    d = T(delta)

    def clamp(re, im, fed):
        H = re.size
        _box(re, d, fed[:H])
        _box(im, d, fed[H:])

    return _loop(e0, shape, eps, max_iter, tol, dtype, clamp)


def direct_bounds(shape, indices, delta_k, dtype=np.float32) -> np.ndarray:
    """Per-coefficient bounds of the direct mode (initialize, impl:598-637):
    +inf where unconstrained; an index listed twice keeps the smaller bound."""
    T = np.dtype(dtype).type
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)
    b = np.full(H, np.inf, T)
    np.minimum.at(b, np.asarray(indices, np.int64), np.asarray(delta_k, T))
    return b


def solve_direct(e0, shape, eps, bounds, max_iter=100, tol=1e-7, dtype=np.float32) -> dict:
    """solve() with project_frequency_constraints_direct
    (projection_algorithm.cu:93-145): Re and Im of coefficient k clamped to
    +-bounds[k]."""
    b = np.asarray(bounds, np.dtype(dtype))

    def clamp(re, im, fed):
        H = re.size
        _box(re, b, fed[:H])
        _box(im, b, fed[H:])

    return _loop(e0, shape, eps, max_iter, tol, dtype, clamp)


def ptw_constants(delta_ptw, dtype=np.float32) -> dict:
    """The T constants of projection_algorithm.cu:191-333: sqrt(1 +- d), the
    DC factors 1/sqrt(1 +- d) - 1 and the clamp half-width
    min(1 - sqrt(1-d), sqrt(1+d) - 1) / sqrtf(2) (sqrt(2) rounded to float, as
    sqrt_val(2.0f) gives)."""
    T = np.dtype(dtype).type
    d = T(delta_ptw)
    sp, sm = np.sqrt(T(1) + d), np.sqrt(T(1) - d)
    return {"sp": sp, "sm": sm, "lo": T(1) / sp - T(1), "hi": T(1) / sm - T(1),
            "cd": T(min(T(1) - sm, sp - T(1)) / T(np.sqrt(np.float32(2.0))))}


def solve_ptw(e0, shape, eps, delta_ptw, orig, mask=None, dc=True, max_iter=100, tol=1e-7,
              dtype=np.float32) -> dict:
    """solve_all_ptw (mask None) and the partial form (mask: coefficients
    listed after the first constraint) of projection_algorithm.cu:191-333.
    orig: the half spectrum of x (complex, flat index order).  Coefficient 0
    (when dc): Re error outside [orig0.re*(1/sqrt(1+d)-1), orig0.re*(1/sqrt(1-d)-1)]
    is set to 0.  Others: if |orig+err|^2/|orig|^2 lies outside [sqrt(1-d),
    sqrt(1+d)], Re and Im of the error are clamped to +-cd."""
    T = np.dtype(dtype).type
    c = ptw_constants(delta_ptw, dtype)
    o = np.asarray(orig).reshape(-1)
    ore, oim = o.real.astype(T), o.imag.astype(T)
    om = ore * ore + oim * oim
    sel = np.ones(o.size, bool) if mask is None else np.asarray(mask, bool).copy()
    sel[0] = False

    def clamp(re, im, fed):
        H = re.size
        if dc:
            lo, hi = ore[0] * c["lo"], ore[0] * c["hi"]
            if re[0] > hi or re[0] < lo:
                fed[0] += -re[0]
                re[0] = T(0)
        cx, cy = ore + re, oim + im
        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = (cx * cx + cy * cy) / om
        inside = (ratio <= c["sp"]) & (ratio >= c["sm"])
        act = sel & ~inside
        r_act, i_act = re[act], im[act]
        fr, fi = fed[:H][act], fed[H:][act]
        _box(r_act, c["cd"], fr)
        _box(i_act, c["cd"], fi)
        re[act], im[act] = r_act, i_act
        fed[:H][act], fed[H:][act] = fr, fi

    return _loop(e0, shape, eps, max_iter, tol, dtype, clamp)


def check_bounds(x: np.ndarray, xhat: np.ndarray, eps: float, delta: float) -> dict:
    """FP64 check of |xhat - x| <= E and |Re/Im rfftn(xhat - x)| <= Delta."""
    d = np.asarray(xhat, np.float64) - np.asarray(x, np.float64)
    F = _rfftn(d)
    spatial = float(np.abs(d).max())
    freq = float(max(np.abs(F.real).max(), np.abs(F.imag).max()))
    return {"spatial_max": spatial, "freq_max": freq, "spatial_excess": spatial - eps, "freq_excess": freq - delta}


# --------------------------------------------------------------- compaction
def extract(edits: np.ndarray, pack_mode: int = 0) -> dict:
    """Flags, whole-array min/max, compact values, uint16 codes and flag pack."""
    a = np.ascontiguousarray(edits)
    n = a.size
    f32 = a.dtype == np.float32
    L = lib()
    T = C.c_float if f32 else C.c_double
    flags = np.empty(n, np.uint8)
    mn, mx, cnt = T(), T(), C.c_size_t()
    (L.orc_flags_minmax_f32 if f32 else L.orc_flags_minmax_f64)(
        _ptr(a), n, THRESHOLD, _ptr(flags), C.byref(mn), C.byref(mx), C.byref(cnt))
    compact = np.empty(max(cnt.value, 1), a.dtype)
    quant = np.empty(max(cnt.value, 1), np.uint16)
    k = (L.orc_compact_quantize_f32 if f32 else L.orc_compact_quantize_f64)(
        _ptr(a), n, THRESHOLD, mn.value, mx.value, _ptr(compact), _ptr(quant))
    assert k == cnt.value
    pack = np.empty((n + 7) // 8, np.uint8)
    if cnt.value > 0 or pack_mode == 0:
        L.orc_pack_flags(_ptr(flags), n, _ptr(pack), pack_mode)
    else:
        pack[:] = 0
    return {"count": cnt.value, "min": mn.value, "max": mx.value, "flags": flags.astype(bool),
            "compact": compact[:k], "quant": quant[:k], "pack": pack}


def pack_flags(flags: np.ndarray, ref_compat: bool = False) -> np.ndarray:
    f = np.ascontiguousarray(flags, dtype=np.uint8)
    out = np.empty((f.size + 7) // 8, np.uint8)
    lib().orc_pack_flags(_ptr(f), f.size, _ptr(out), int(ref_compat))
    return out


def quantize(v, mn, mx, dtype=np.float32) -> int:
    L = lib()
    return int((L.orc_quantize_f32 if np.dtype(dtype) == np.float32 else L.orc_quantize_f64)(v, mn, mx))


# ------------------------------------------------------------------ Huffman
def huffman_codebook(data: np.ndarray, nbins: int | None = None) -> dict:
    """{symbol: (code, length)} plus the histogram (HuffmanZSTDCoder.cuh:48-178)."""
    d = np.ascontiguousarray(data, dtype=np.uint32)
    if nbins is None:
        nbins = 256 if np.asarray(data).dtype == np.uint8 else 65536
    sym, freq, code = (np.empty(nbins, np.uint32) for _ in range(3))
    ln = np.empty(nbins, np.int32)
    ns = lib().orc_huff_codebook(_ptr(d), d.size, nbins, _ptr(sym), _ptr(freq), _ptr(code), _ptr(ln))
    return {"symbols": sym[:ns].copy(), "freq": freq[:ns].copy(), "codes": code[:ns].copy(),
            "lengths": ln[:ns].copy()}


def huffman_bitstream(data: np.ndarray, book: dict) -> tuple[bytes, int]:
    """MSB-first bitstream and its bit count (HuffmanZSTDCoder.cuh:307-357)."""
    d = np.ascontiguousarray(data, dtype=np.uint32)
    nb = int(max(d.max(initial=0) + 1, int(book["symbols"].max(initial=0)) + 1))
    lut_c = np.zeros(nb, np.uint32)
    lut_l = np.zeros(nb, np.int32)
    lut_c[book["symbols"]] = book["codes"]
    lut_l[book["symbols"]] = book["lengths"]
    total_bits = int((lut_l[d].astype(np.int64)).sum())
    out = np.empty(max((total_bits + 7) // 8, 1), np.uint8)
    tb = C.c_uint64()
    n = lib().orc_huff_pack(_ptr(d), d.size, _ptr(lut_c), _ptr(lut_l), _ptr(out), C.byref(tb))
    if n == C.c_size_t(-1).value:
        raise ValueError("code longer than 64 bits")
    return bytes(out[:n]), int(tb.value)


def huffman_decode(bits: bytes, book: dict, num_elements: int) -> np.ndarray:
    b = np.frombuffer(bits, np.uint8) if len(bits) else np.zeros(1, np.uint8)
    out = np.empty(max(num_elements, 1), np.uint32)
    s = np.ascontiguousarray(book["symbols"], np.uint32)
    c = np.ascontiguousarray(book["codes"], np.uint32)
    ln = np.ascontiguousarray(book["lengths"], np.int32)
    k = lib().orc_huff_decode(_ptr(b), len(bits), _ptr(s), _ptr(c), _ptr(ln), s.size, num_elements, _ptr(out))
    return out[:k]


# ---------------------------------------------------------------- decoder
def dequantize(quant: np.ndarray, mn: float, mx: float, dtype=np.float32) -> np.ndarray:
    """Inverse of the quantiser in the order of projection_algorithm.cu:638:
    q / 65535 * (max - min) + min, every operation rounded to T."""
    T = np.dtype(dtype).type
    q = np.asarray(quant).astype(T)
    return (q / T(65535)) * (T(mx) - T(mn)) + T(mn)


def unpack_edits(quant: np.ndarray, pack: bytes, n: int, mn: float, mx: float, dtype=np.float32) -> np.ndarray:
    """Dense edit array of n values: the r-th set flag of the LSB-first pack
    (ascending index) receives dequantize(quant[r]); zero elsewhere."""
    flags = np.unpackbits(np.frombuffer(pack, np.uint8), bitorder="little")[:n].astype(bool)
    out = np.zeros(n, dtype)
    idx = np.flatnonzero(flags)
    k = min(idx.size, len(quant))
    out[idx[:k]] = dequantize(np.asarray(quant)[:k], mn, mx, dtype)
    return out


def reconstruct(xprime: np.ndarray, shape, freq_edits: np.ndarray, spatial_edits: np.ndarray) -> np.ndarray:
    """x^ = x' + C2R(F)/N + S in FP64: F the planar half-spectrum edits
    (Re | Im), C2R the unnormalised inverse real transform (imaginary parts of
    the self-conjugate bins of the last axis ignored)."""
    shape = tuple(int(v) for v in shape)
    H = shape[0] * shape[1] * (shape[2] // 2 + 1)
    fe = np.asarray(freq_edits, np.float64)
    F = (fe[:H] + 1j * fe[H:]).reshape(shape[0], shape[1], shape[2] // 2 + 1)
    e = _irfftn(F, s=shape)
    return np.asarray(xprime, np.float64).reshape(shape) + e + np.asarray(spatial_edits, np.float64).reshape(shape)


# --------------------------------------------------------------------- ZSTD
_z = None


def zstd():
    global _z
    if _z is None:
        z = C.CDLL("libzstd.so.1")
        z.ZSTD_compressBound.restype = C.c_size_t
        z.ZSTD_compressBound.argtypes = [C.c_size_t]
        z.ZSTD_compress.restype = C.c_size_t
        z.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
        z.ZSTD_decompress.restype = C.c_size_t
        z.ZSTD_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
        z.ZSTD_isError.restype = C.c_uint
        z.ZSTD_isError.argtypes = [C.c_size_t]
        _z = z
    return _z


def zstd_compress(data: bytes, level: int) -> bytes:
    z = zstd()
    src = np.frombuffer(data, np.uint8) if len(data) else np.zeros(1, np.uint8)
    bound = z.ZSTD_compressBound(len(data))
    out = np.empty(bound, np.uint8)
    n = z.ZSTD_compress(_ptr(out), bound, _ptr(src), len(data), level)
    if z.ZSTD_isError(n):
        raise RuntimeError("ZSTD compression failed")
    return bytes(out[:n])


def zstd_decompress(data: bytes, size: int) -> bytes:
    z = zstd()
    src = np.frombuffer(data, np.uint8)
    out = np.empty(max(size, 1), np.uint8)
    n = z.ZSTD_decompress(_ptr(out), size, _ptr(src), len(data))
    if z.ZSTD_isError(n):
        raise RuntimeError("ZSTD decompression failed")
    return bytes(out[:n])


def huffman_zstd_compress(data: np.ndarray, level: int) -> dict:
    """cudaHuffmanZstdCompress restated: codebook, bitstream, ZSTD_compress."""
    book = huffman_codebook(data)
    bits, nbits = huffman_bitstream(data, book)
    return {"book": book, "bitstream": bits, "bits": nbits, "compressed": zstd_compress(bits, level),
            "num_elements": int(np.asarray(data).size)}
