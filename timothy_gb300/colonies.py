"""Seeded synthetic colonies for the cell-mechanics hot path.

The reference ships no benchmark inputs, so every workload is generated here
from a named seed (numpy PCG64).  A colony is a set of cells in the reference's
cell layout (celldata_t fields used by the hot path, global.h:100-120):
positions x, y, z (FP64), radius ``size`` (FP64), ``young`` (FP32),
``ctype`` (int32) and cell-cycle ``phase`` (int32, 0..5).

Generators
  * ``uniform``    centres uniform in a ball of radius R.
  * ``clustered``  radial Gaussian density rho(r) ~ exp(-r^2 / 2 sigma^2) on
                   r <= R with rho(R) = rho(0)/4, i.e. sigma = R / sqrt(2 ln 4);
                   the core is four times denser than the rim.
Radii are U[0.8, 1.0] * r0, young = 2100 + U(-100, 100), phases uniform in
{0..5}.  ``calibrate_radius`` bisects R so that the mean number of neighbours
within h is the requested value (40 for every configuration of this path).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

H_DEFAULT = 2.5
R0_DEFAULT = 1.0
MEAN_NEIGHBOURS = 40.0
# Radii of the configured colonies that give a mean of 40 neighbours within
# h = 2.5, bisected with full-size neighbour counts: (kind, cells, seed) -> R.
CALIBRATED_RADIUS = {
    ("uniform", 10_000, 1): 15.256856463570728,
    ("clustered", 1_000_000, 2): 76.3271427172167,
    ("clustered", 16_000_000, 3): 192.68257233787858,
}


@dataclass
class CellTypes:
    """Per-type constants of celltype_t (global.h:315-335) used by the path.

    ``h2``, ``h3`` and ``h4`` are passed as given: the reference never derives
    them from ``h`` at run time (initialisation.c:79-82 computes them from the
    default h before cells.inp sets h).  ``consistent`` builds the usual
    h2 = h*h, h3 = h2*h, h4 = h3*h.
    """

    h: np.ndarray
    h2: np.ndarray
    h3: np.ndarray
    h4: np.ndarray
    size: np.ndarray
    randommove: np.ndarray

    @staticmethod
    def consistent(h=(H_DEFAULT,), size=(R0_DEFAULT,), randommove=None) -> "CellTypes":
        h = np.asarray(h, dtype=np.float64)
        h2 = h * h
        h3 = h2 * h
        h4 = h3 * h
        size = np.asarray(size, dtype=np.float64)
        rm = np.zeros(len(h), np.float32) if randommove is None else np.asarray(randommove, np.float32)
        return CellTypes(h, h2, h3, h4, size, rm)

    @property
    def ntypes(self) -> int:
        return int(len(self.h))


@dataclass
class Colony:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    size: np.ndarray
    young: np.ndarray
    ctype: np.ndarray
    phase: np.ndarray
    types: CellTypes = field(default_factory=CellTypes.consistent)
    dim: int = 3
    kind: str = "uniform"
    seed: int = 0
    radius: float = 0.0

    @property
    def n(self) -> int:
        return int(len(self.x))

    def copy(self) -> "Colony":
        return Colony(self.x.copy(), self.y.copy(), self.z.copy(), self.size.copy(), self.young.copy(),
                      self.ctype.copy(), self.phase.copy(), self.types, self.dim, self.kind, self.seed,
                      self.radius)


def sigma_for(radius: float) -> float:
    return radius / math.sqrt(2.0 * math.log(4.0))


def _points(kind: str, n: int, radius: float, rng: np.random.Generator, dim: int) -> np.ndarray:
    out = np.empty((n, 3), np.float64)
    got = 0
    while got < n:
        m = max(1024, int(1.3 * (n - got)) + 64)
        if kind == "uniform":
            p = rng.uniform(-radius, radius, size=(m, 3))
        elif kind == "clustered":
            p = rng.normal(0.0, sigma_for(radius), size=(m, 3))
        else:
            raise ValueError(f"unknown colony kind {kind!r}")
        if dim == 2:
            p[:, 2] = 0.0
        r2 = np.einsum("ij,ij->i", p, p)
        p = p[r2 <= radius * radius]
        take = min(len(p), n - got)
        out[got:got + take] = p[:take]
        got += take
    return out


def make_colony(kind: str, n: int, seed: int, radius: float, *, dim: int = 3,
                types: CellTypes | None = None, type_fractions=None, r0: float = R0_DEFAULT) -> Colony:
    """Draw ``n`` cells of the given kind inside radius ``radius``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pts = _points(kind, n, radius, rng, dim)
    size = rng.uniform(0.8, 1.0, size=n) * r0
    young = (2100.0 + rng.uniform(-100.0, 100.0, size=n)).astype(np.float32)
    phase = rng.integers(0, 6, size=n).astype(np.int32)
    types = types or CellTypes.consistent()
    if types.ntypes > 1:
        frac = np.full(types.ntypes, 1.0 / types.ntypes) if type_fractions is None else np.asarray(type_fractions)
        ctype = rng.choice(types.ntypes, size=n, p=frac).astype(np.int32)
    else:
        ctype = np.zeros(n, np.int32)
    return Colony(np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1]),
                  np.ascontiguousarray(pts[:, 2]), size, young, ctype, phase, types, dim, kind, seed, radius)


def initial_radius(kind: str, n: int, h: float = H_DEFAULT, mean: float = MEAN_NEIGHBOURS, dim: int = 3) -> float:
    """Radius that gives ``mean`` neighbours in the bulk (surface deficit ignored)."""
    if dim == 2:
        rho = mean / (math.pi * h * h)
        r = math.sqrt(n / (math.pi * rho))
    else:
        rho = mean / (4.0 / 3.0 * math.pi * h ** 3)
        r = (3.0 * n / (4.0 * math.pi * rho)) ** (1.0 / 3.0)
    if kind == "clustered":
        r *= 1.35
    return r


def configured_radius(kind: str, n: int, seed: int) -> float:
    """The calibrated radius of a configured colony, else the calibrated one of
    the same generator scaled by n^(1/3)."""
    r = CALIBRATED_RADIUS.get((kind, n, seed))
    if r is None:
        base = {"uniform": (10_000, CALIBRATED_RADIUS[("uniform", 10_000, 1)]),
                "clustered": (1_000_000, CALIBRATED_RADIUS[("clustered", 1_000_000, 2)])}[kind]
        r = base[1] * (n / base[0]) ** (1 / 3)
    return r


def count_neighbours_cpu(col: Colony) -> np.ndarray:
    """Neighbours within h (excluding self) per cell, via a k-d tree."""
    from scipy.spatial import cKDTree

    pts = np.stack([col.x, col.y, col.z], axis=1)
    tree = cKDTree(pts)
    h = col.types.h[col.ctype]
    if np.all(h == h[0]):
        cnt = tree.query_ball_point(pts, r=float(h[0]), return_length=True, workers=-1)
    else:
        cnt = np.array([len(tree.query_ball_point(p, r=float(hh))) for p, hh in zip(pts, h)])
    return np.asarray(cnt, np.int64) - 1


def calibrate_radius(kind: str, n: int, seed: int, *, mean: float = MEAN_NEIGHBOURS, tol: float = 0.5,
                     dim: int = 3, types: CellTypes | None = None, count_fn=None, max_iter: int = 40) -> float:
    """Bisect the colony radius until the mean neighbour count is mean +- tol.

    ``count_fn(colony) -> per-cell counts`` defaults to the k-d tree counter;
    the GPU session offers a device counter for large colonies.
    """
    count_fn = count_fn or count_neighbours_cpu
    types = types or CellTypes.consistent()
    h = float(types.h[0])
    r_mid = initial_radius(kind, n, h, mean, dim)

    def mean_at(r):
        return float(np.mean(count_fn(make_colony(kind, n, seed, r, dim=dim, types=types))))

    lo, hi = 0.5 * r_mid, 1.5 * r_mid
    m_lo, m_hi = mean_at(lo), mean_at(hi)
    while m_lo < mean:
        lo *= 0.7
        m_lo = mean_at(lo)
    while m_hi > mean:
        hi *= 1.4
        m_hi = mean_at(hi)
    r = r_mid
    for _ in range(max_iter):
        r = 0.5 * (lo + hi)
        m = mean_at(r)
        if abs(m - mean) <= tol:
            return r
        if m > mean:
            lo = r
        else:
            hi = r
    return r


def batch_sizes(count: int, seed: int, lo: int = 1000, hi: int = 200_000) -> np.ndarray:
    """Colony sizes log-uniform in [lo, hi] for the batched form."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))).astype(np.int64)
