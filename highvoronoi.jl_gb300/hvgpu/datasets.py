"""Seeded synthetic point clouds for the mesh workloads.

HighVoronoi.jl draws its benchmark points with Julia's global RNG
(``rand(d, N)`` in src/statistics.jl:98-183), which cannot be reproduced
outside Julia.  The seeds of the workloads therefore refer to this module's
counter-based SplitMix64 stream (Steele, Lea, Flood 2014): draw ``k`` of stream
``seed`` is ``mix(seed + (k + 1) * GAMMA)``, so every draw is a pure function of
its index and the generators vectorise with numpy.

Points are returned as ``(n, d)`` float64 arrays whose C order is the
reference's ``d x n`` column-major layout (point ``i`` occupies
``pts[i*d:(i+1)*d]``), strictly inside the unit cube.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, start: int, count: int) -> np.ndarray:
    """Draws ``start .. start+count-1`` of the SplitMix64 stream ``seed``."""
    k = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, start: int, count: int) -> np.ndarray:
    """Uniform doubles strictly inside (0, 1): ((z >> 11) + 0.5) * 2^-53."""
    z = splitmix64(seed, start, count)
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)


def uniform_points(d: int, n: int, seed: int) -> np.ndarray:
    """``n`` i.i.d. uniform points in (0,1)^d; coordinate ``k`` of point ``i`` is draw ``i*d+k``."""
    return uniform01(seed, 0, n * d).reshape(n, d)


def clustered_points(d: int, n: int, seed: int, n_clusters: int = 8, sigma: float = 0.05,
                     centre_lo: float = 0.2, centre_hi: float = 0.8) -> np.ndarray:
    """Mixture of ``n_clusters`` isotropic Gaussians, rejected to (0,1)^d.

    Centres are uniform in ``[centre_lo, centre_hi]^d`` (draws ``0 .. C*d-1``).
    Candidate ``m`` uses the ``L = 1 + 2*ceil(d/2)`` draws starting at
    ``C*d + m*L``: one picks the cluster, the rest feed Box-Muller pairs.  The
    first ``n`` accepted candidates, in candidate order, are returned.
    """
    C = n_clusters
    centres = centre_lo + (centre_hi - centre_lo) * uniform01(seed, 0, C * d).reshape(C, d)
    pairs = (d + 1) // 2
    L = 1 + 2 * pairs
    out = []
    have = 0
    m0 = 0
    block = max(1024, 2 * n)
    while have < n:
        u = uniform01(seed, C * d + m0 * L, block * L).reshape(block, L)
        cl = np.minimum((u[:, 0] * C).astype(np.int64), C - 1)
        u1 = u[:, 1::2][:, :pairs]
        u2 = u[:, 2::2][:, :pairs]
        r = np.sqrt(-2.0 * np.log(u1))
        g = np.empty((block, 2 * pairs))
        g[:, 0::2] = r * np.cos(2.0 * np.pi * u2)
        g[:, 1::2] = r * np.sin(2.0 * np.pi * u2)
        x = centres[cl] + sigma * g[:, :d]
        ok = np.all((x > 0.0) & (x < 1.0), axis=1)
        acc = x[ok]
        out.append(acc)
        have += acc.shape[0]
        m0 += block
    return np.ascontiguousarray(np.concatenate(out, axis=0)[:n])


def served_stream(count: int, seed: int = 2000):
    """The served stream of mesh requests: request r has d uniform in
    {2,3,4,5}, N log-uniform in [200, 20000] and its points uniform in the unit
    cube drawn with seed r (uniform_points(d, N, r)).  Returns the list of
    (d, N, r) and the arrival gaps in units of the mean gap (exponential)."""
    u = uniform01(seed, 0, 3 * count).reshape(count, 3)
    reqs = []
    for r in range(count):
        d = 2 + min(int(u[r, 0] * 4), 3)
        n = int(round(np.exp(np.log(200) + u[r, 1] * (np.log(20000) - np.log(200)))))
        reqs.append((d, n, r))
    gaps = -np.log(u[:, 2])
    return reqs, gaps


# The five workloads of the hot path (point cloud, boundary and integrator).
WORKLOADS = {
    "2d_uniform_1k": dict(d=2, n=1000, seed=0, kind="uniform", integrator="polygon"),
    "4d_uniform_20k": dict(d=4, n=20000, seed=1, kind="uniform", integrator=None),
    "5d_clustered_50k": dict(d=5, n=50000, seed=2, kind="clustered", integrator="polygon"),
    "6d_uniform_10k_mc": dict(d=6, n=10000, seed=3, kind="uniform", integrator="heuristic_mc", ndir=1000),
    # larger cases for throughput sweeps
    "3d_uniform_100k": dict(d=3, n=100000, seed=4, kind="uniform", integrator="polygon"),
    "5d_uniform_20k": dict(d=5, n=20000, seed=5, kind="uniform", integrator="polygon"),
}


def workload_points(name: str) -> np.ndarray:
    w = WORKLOADS[name]
    if w["kind"] == "uniform":
        return uniform_points(w["d"], w["n"], w["seed"])
    return clustered_points(w["d"], w["n"], w["seed"])
