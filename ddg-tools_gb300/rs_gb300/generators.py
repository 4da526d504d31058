"""Seeded synthetic meshes of the benchmark configurations.

The icosphere and torus recipes follow ``crates/ddg-core/src/generators.rs`` (icosphere
108-175: vertex numbering by first use of each edge midpoint; torus 188-229 with
``quad_grid_faces`` 362-380), and ``SplitMix64`` its lines 58-90. The noise models are this
project's own definitions of the configurations (Box-Muller normals from SplitMix64 draws):

* c1: icosphere(3), every vertex scaled by ``1 + 0.02 z_v`` (seed 1);
* c2: icosphere(6), radius ``1 + 0.05 sum_k c_k Y_k / sum_k |c_k|`` over 8 real spherical
  harmonics of degree 1..8 drawn uniformly, ``c_k ~ U(-1, 1)`` (seed 2);
* c3: torus(320, 320, 1, 0.3) plus ``N(0, 0.01)`` per coordinate (seed 3);
* c5: two interlinked torus(400, 400, 1, 0.25), the second rotated 90 degrees about x and
  moved by +1 along x, plus ``N(0, 0.01)`` per coordinate (seed 5).
"""
from __future__ import annotations

import math

import numpy as np

MASK = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (ddg-core generators.rs:58-90)."""

    def __init__(self, seed: int):
        self.state = seed & MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def next_f64(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.next_f64()

    def draws(self, n: int) -> np.ndarray:
        """The next n outputs of next_u64, vectorised (same sequence)."""
        k = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(self.state) + k * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.state = (self.state + n * 0x9E3779B97F4A7C15) & MASK
        return z

    def normals(self, n: int) -> np.ndarray:
        """n standard normals by Box-Muller, one pair of draws per value."""
        u = (self.draws(2 * n) >> np.uint64(11)).astype(np.float64)
        u *= 1.0 / (1 << 53)
        u1, u2 = u[0::2], u[1::2]
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


def _normalize_rows(p: np.ndarray) -> np.ndarray:
    ln = np.sqrt(p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1] + p[:, 2] * p[:, 2])
    return p / ln[:, None]


def icosphere(level: int):
    """Unit icosphere: ``10 4^level + 2`` vertices, ``20 4^level`` faces."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    P = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 dtype=np.float64)
    P = _normalize_rows(P)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        nv = len(P)
        a, b, c = F[:, 0], F[:, 1], F[:, 2]
        # edges in the order the reference creates midpoints: (a,b), (b,c), (c,a) per face
        e0 = np.stack([a, b, b, c, c, a], axis=1).reshape(-1, 2)
        lo, hi = np.minimum(e0[:, 0], e0[:, 1]), np.maximum(e0[:, 0], e0[:, 1])
        key = lo * nv + hi
        uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
        rank = np.empty(len(uniq), dtype=np.int64)
        rank[np.argsort(first, kind="stable")] = np.arange(len(uniq))
        mid_id = nv + rank[inv]
        ulo, uhi = uniq // nv, uniq % nv
        newp = np.empty((len(uniq), 3))
        newp[rank] = _normalize_rows(P[ulo] + P[uhi])
        P = np.vstack([P, newp])
        m = mid_id.reshape(-1, 3)  # ab, bc, ca
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        F = np.stack([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                      np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3)
    return P, F.astype(np.uint32)


def torus(n_major: int, n_minor: int, major_radius: float, minor_radius: float):
    """Torus around z: ``n_major n_minor`` vertices, twice as many faces."""
    i = np.arange(n_major, dtype=np.float64)
    j = np.arange(n_minor, dtype=np.float64)
    theta = 2.0 * np.pi * i / n_major
    phi = 2.0 * np.pi * j / n_minor
    ring = major_radius + minor_radius * np.cos(phi)
    P = np.empty((n_major, n_minor, 3))
    P[:, :, 0] = ring[None, :] * np.cos(theta)[:, None]
    P[:, :, 1] = ring[None, :] * np.sin(theta)[:, None]
    P[:, :, 2] = (minor_radius * np.sin(phi))[None, :]
    ii, jj = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    idx = lambda a, b: (a % n_major) * n_minor + (b % n_minor)  # noqa: E731
    A, B, C, D = idx(ii, jj), idx(ii + 1, jj), idx(ii + 1, jj + 1), idx(ii, jj + 1)
    F = np.stack([np.stack([A, B, C], -1), np.stack([A, C, D], -1)], 2).reshape(-1, 3)
    return P.reshape(-1, 3), F.astype(np.uint32)


def _real_sh(l: int, m: int, theta: np.ndarray, phi: np.ndarray) -> np.ndarray:
    """Orthonormal real spherical harmonic of degree l, order m (Legendre recurrence)."""
    am = abs(m)
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.ones_like(x)
    for k in range(1, am + 1):
        pmm = -pmm * (2 * k - 1) * s
    if l == am:
        plm = pmm
    else:
        p1 = x * (2 * am + 1) * pmm
        if l == am + 1:
            plm = p1
        else:
            p0 = pmm
            for ll in range(am + 2, l + 1):
                p0, p1 = p1, ((2 * ll - 1) * x * p1 - (ll + am - 1) * p0) / (ll - am)
            plm = p1
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    if m > 0:
        return math.sqrt(2) * norm * plm * np.cos(am * phi)
    if m < 0:
        return math.sqrt(2) * norm * plm * np.sin(am * phi)
    return norm * plm


def config_c1():
    P, F = icosphere(3)
    z = SplitMix64(1).normals(len(P))
    return P * (1.0 + 0.02 * z)[:, None], F


def config_c2(level: int = 6):
    P, F = icosphere(level)
    rng = SplitMix64(2)
    modes = []
    for _ in range(8):
        l = 1 + rng.next_u64() % 8
        m = -l + rng.next_u64() % (2 * l + 1)
        modes.append((int(l), int(m), rng.uniform(-1.0, 1.0)))
    theta = np.arccos(np.clip(P[:, 2], -1.0, 1.0))
    phi = np.arctan2(P[:, 1], P[:, 0])
    acc = np.zeros(len(P))
    for l, m, c in modes:
        acc += c * _real_sh(l, m, theta, phi)
    r = 1.0 + 0.05 * acc / sum(abs(c) for _, _, c in modes)
    return P * r[:, None], F


def noisy_torus(n_major, n_minor, R, r, sigma, seed):
    P, F = torus(n_major, n_minor, R, r)
    z = SplitMix64(seed).normals(P.size).reshape(P.shape)
    return P + sigma * z, F


def config_c3(n: int = 320, sigma: float = 0.01):
    """Torus 320x320 (R = 1, r = 0.3, 204,800 faces), N(0, sigma) per coordinate, seed 3.
    sigma = 0.01 is the configuration as specified; it exceeds the minor-circle edge (0.0059)
    and crumples the surface. config_c3s is the same torus at sigma = 0.001."""
    return noisy_torus(n, n, 1.0, 0.3, sigma, 3)


def config_c3s(n: int = 320):
    return config_c3(n, 0.001)


def config_c5(n: int = 400, sigma: float = 0.01):
    """Two interlinked tori (R = 1, r = 0.25, n x n grids; 640,000 faces at n = 400): the
    second rotated 90 degrees about x and moved +1 along x (a Hopf link), N(0, sigma) per
    coordinate, seed 5. sigma = 0.01 is the configuration as specified (2.5 minor-circle edges
    at n = 400: a crumpled surface)."""
    P, F = torus(n, n, 1.0, 0.25)
    Q = np.stack([P[:, 0] + 1.0, -P[:, 2], P[:, 1]], axis=1)
    PP = np.vstack([P, Q])
    FF = np.vstack([F, F + len(P)]).astype(np.uint32)
    z = SplitMix64(5).normals(PP.size).reshape(PP.shape)
    return PP + sigma * z, FF


CONFIGS = {"c1": config_c1, "c2": config_c2, "c3": config_c3, "c3s": config_c3s, "c5": config_c5}
