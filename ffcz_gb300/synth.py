"""Seeded synthetic scientific fields and corrector parameters.

Gaussian random fields with an isotropic power spectrum P(k) ~ |k|^-alpha
stand in for the cosmology / climate fields the corrector targets (no
dataset is used).  Recipe (FP64, deterministic):

1. w = default_rng(seed).standard_normal(shape)
2. W = rfftn(w), scaled by |k|^(-alpha/2) with integer wavenumbers
   (fftfreq(n)*n on leading axes, rfftfreq(n)*n on the last), W[0] = 0
3. x = irfftn(W), divided by its standard deviation, cast to the dtype.

Parameters: range = max(x) - min(x); E = f_E * range;
Delta = f_D * max_k |rfftn64(x)_k|; decompressed field
x' = 2E * round(x / 2E), optionally plus U(-aE, aE) noise drawn from
default_rng(seed + 1000); optional spikes replace 1% of the voxels
(default_rng(seed + 1).permutation(N)[:N//100]) by Laplace(0, 10) draws
before E is computed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

try:  # scipy's pocketfft takes a worker count; numpy's does not
    import scipy.fft as _fft

    def _rfftn(a):
        return _fft.rfftn(a, workers=-1)

    def _irfftn(a, s):
        return _fft.irfftn(a, s=s, workers=-1)
except ImportError:  # pragma: no cover
    def _rfftn(a):
        return np.fft.rfftn(a)

    def _irfftn(a, s):
        return np.fft.irfftn(a, s=s)


def grf(shape, alpha: float, seed: int, dtype=np.float32) -> np.ndarray:
    shape = tuple(int(s) for s in shape)
    w = np.random.default_rng(seed).standard_normal(shape)
    W = _rfftn(w)
    del w
    k2 = np.zeros(W.shape)
    for ax, n in enumerate(shape):
        if ax == len(shape) - 1:
            f = np.fft.rfftfreq(n) * n
        else:
            f = np.fft.fftfreq(n) * n
        sh = [1] * len(shape)
        sh[ax] = f.size
        k2 = k2 + (f.reshape(sh) ** 2)
    with np.errstate(divide="ignore"):
        amp = np.where(k2 > 0, k2 ** (-alpha / 4.0), 0.0)
    W *= amp
    x = _irfftn(W, s=shape)
    x /= x.std()
    return x.astype(dtype)


@dataclass
class Field:
    x: np.ndarray          # original field
    xp: np.ndarray         # decompressed field x'
    eps: float             # spatial bound E (rounded to the field dtype)
    delta: float           # frequency bound Delta (rounded to the field dtype)
    shape: tuple           # (Nx, Ny, Nz) as the solver sees it


def solver_shape(shape) -> tuple:
    """CLI convention: -1 n -> (1,1,n); -2 ny nz -> (1,ny,nz); -3 -> as is."""
    shape = tuple(int(s) for s in shape)
    return (1,) * (3 - len(shape)) + shape


def make_field(shape, alpha: float, seed: int, f_eps: float, f_delta: float, dtype=np.float32,
               noise: float = 0.0, spikes: bool = False) -> Field:
    dtype = np.dtype(dtype)
    x = grf(shape, alpha, seed, np.float64)
    if spikes:
        n = x.size
        idx = np.random.default_rng(seed + 1).permutation(n)[: n // 100]
        flat = x.reshape(-1)
        flat[idx] = np.random.default_rng(seed + 1).laplace(0.0, 10.0, idx.size)
    x = x.astype(dtype)
    x64 = x.astype(np.float64)
    rng_ = float(x64.max() - x64.min())
    eps = f_eps * rng_
    delta = f_delta * float(np.abs(_rfftn(x64)).max())
    xp = 2 * eps * np.round(x64 / (2 * eps))
    if noise:
        xp = xp + np.random.default_rng(seed + 1000).uniform(-noise * eps, noise * eps, x.shape)
    eps_t = float(dtype.type(eps))
    delta_t = float(dtype.type(delta))
    return Field(x, xp.astype(dtype), eps_t, delta_t, solver_shape(shape))


# Named workloads (shape, alpha, seed, f_eps, f_delta, noise, spikes, dtype, max_iter).
WORKLOADS = {
    "small64": ((64, 64, 64), 11 / 3, 0, 1e-3, 1e-3, 0.0, False, np.float32, 100),
    "plain256": ((256, 256, 256), 11 / 3, 1, 1e-4, 5e-4, 0.3, False, np.float32, 100),
    "precision512": ((512, 512, 512), 3.0, 2, 1e-4, 1e-4, 0.0, False, np.float32, 100),
    "large1024x1024x512": ((1024, 1024, 512), 11 / 3, 3, 5e-5, 2e-4, 0.0, True, np.float32, 500),
    "fp64_512": ((512, 512, 512), 11 / 3, 4, 5e-5, 2e-4, 0.0, True, np.float64, 500),
    # the FP64 variant at 256^3: a case small enough for full kernel profiles
    "fp64_256": ((256, 256, 256), 11 / 3, 4, 5e-5, 2e-4, 0.0, True, np.float64, 500),
    # the precision field's spectrum kernels at a profiling size: the same
    # 512-point x and y passes on a quarter of the z extent (2 GB resident)
    "precision_slab": ((512, 512, 128), 3.0, 2, 1e-4, 1e-4, 0.0, False, np.float32, 100),
    # and its 512-point z passes (rows of 257 complex values) on a quarter of
    # the x and y extents (a 142 MB spectrum, larger than L2)
    "precision_rows": ((256, 256, 512), 3.0, 2, 1e-4, 1e-4, 0.0, False, np.float32, 100),
}


def workload(name: str) -> tuple[Field, int]:
    shape, alpha, seed, fe, fd, noise, spikes, dtype, max_iter = WORKLOADS[name]
    return make_field(shape, alpha, seed, fe, fd, dtype, noise, spikes), max_iter


# Batched form: groups of (count, shape, alpha, first seed); every field has
# f_Delta = 1e-3 and a log-uniform spatial bound E_i = range_i * 10^(-5 + 2 u_i),
# u_i = default_rng(seed_i + 2000).random(); x' = 2E round(x / 2E).
BATCHES = {
    "batch48": [(16, (1800, 3600), 2.0, 10), (16, (100, 500, 500), 11 / 3, 30), (16, (128, 128, 128), 5 / 3, 50)],
    # the same three shape families at a size the oracle finishes in seconds
    "batch6_small": [(2, (90, 180), 2.0, 10), (2, (10, 50, 50), 11 / 3, 30), (2, (32, 32, 32), 5 / 3, 50)],
}


def batch_field(shape, alpha: float, seed: int) -> Field:
    u = float(np.random.default_rng(seed + 2000).random())
    return make_field(shape, alpha, seed, 10.0 ** (-5.0 + 2.0 * u), 1e-3, np.float32)


def batch_specs(name: str) -> list[tuple]:
    return [(shape, alpha, seed0 + i) for count, shape, alpha, seed0 in BATCHES[name] for i in range(count)]


def batch_workload(name: str, workers: int = 0) -> tuple[list[Field], int]:
    """The fields of a named batch (max_iter 100).  With workers > 1 they are
    generated in spawned processes (safe next to a CUDA context)."""
    specs = batch_specs(name)
    if workers > 1:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor

        with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as pool:
            fields = list(pool.map(_batch_field_star, specs))
    else:
        fields = [batch_field(*sp) for sp in specs]
    return fields, 100


def _batch_field_star(spec):
    return batch_field(*spec)


def stress_delta(field: Field, c: float) -> float:
    """Delta = c * E * sqrt(N/6): a frequency bound near the noise level of
    the quantisation error, which makes the projections iterate."""
    n = field.x.size
    return float(field.x.dtype.type(c * field.eps * np.sqrt(n / 6.0)))
