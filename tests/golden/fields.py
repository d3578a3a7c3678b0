"""Deterministic test fields on the one-rank grid (no random generator, so the
values are the same with any numpy): smooth waves plus an integer-hash ripple."""
import numpy as np


def field(nfields: int, dims) -> np.ndarray:
    gx, gy, gz = dims
    i = np.arange(gx, dtype=np.float64)[:, None, None]
    j = np.arange(gy, dtype=np.float64)[None, :, None]
    k = np.arange(gz, dtype=np.float64)[None, None, :]
    ii = np.arange(gx, dtype=np.int64)[:, None, None]
    jj = np.arange(gy, dtype=np.int64)[None, :, None]
    kk = np.arange(gz, dtype=np.int64)[None, None, :]
    out = np.empty((nfields, gx, gy, gz))
    for f in range(nfields):
        ripple = ((ii * 7919 + jj * 104729 + kk * 1299709 + f * 15485863) % 1000).astype(np.float64) / 1000.0
        out[f] = np.sin(0.37 * i + 0.11 * f) * np.cos(0.23 * j - 0.05 * f) + 0.5 * np.sin(0.19 * k) + 0.01 * ripple
    return out


def gradient_field(nfields: int, dims) -> np.ndarray:
    """A stand-in gradient array (3 values per node), independent of field()."""
    base = field(3 * nfields, dims)
    return np.ascontiguousarray(np.moveaxis(base.reshape((nfields, 3) + tuple(dims)), 1, -1))
