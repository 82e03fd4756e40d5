"""Convex test domains given as boundary planes (base points and outer normals,
the reference's Plane(base, normal, BC), src/boundary.jl:22-29)."""
import math

import numpy as np


def orthogonal(d, seed):
    """A seeded random orthogonal matrix (QR of a Gaussian matrix, signs fixed)."""
    g = np.random.default_rng(seed).standard_normal((d, d))
    q, r = np.linalg.qr(g)
    return q * np.sign(np.diag(r))


def rotated_cube(d, seed):
    """The unit cube turned by Q about its centre: plane 2k is the image of the
    upper face of axis k and 2k+1 of the lower face (the cuboid order)."""
    Q = orthogonal(d, seed)
    c = np.full(d, 0.5)
    base, normal = [], []
    for k in range(d):
        e = Q[:, k]
        base.append(c + 0.5 * e); normal.append(e.copy())
        base.append(c - 0.5 * e); normal.append(-e)
    return Q, np.array(base), np.array(normal)


def rotate_points(Q, X):
    c = np.full(X.shape[1], 0.5)
    return (X - c) @ Q.T + c


def simplex(d):
    """{x : x_k > 0, sum x < 1}: d coordinate planes then the slanted face; volume 1/d!."""
    base = [np.zeros(d) for _ in range(d)] + [np.full(d, 1.0 / d)]
    normal = [-np.eye(d)[k] for k in range(d)] + [np.ones(d)]
    return np.array(base), np.array(normal), 1.0 / math.factorial(d)


def simplex_points(d, n, seed):
    """n points uniform in the simplex, kept a little away from its faces."""
    rng = np.random.default_rng(seed)
    x = rng.dirichlet(np.ones(d + 1), n)[:, :d]
    return 0.002 + x * (1.0 - 0.002 * (d + 1))


def regular_polygon(m, r=1.0):
    """2D regular m-gon of circumradius r about the origin; area m r^2 sin(2 pi/m) / 2."""
    base, normal = [], []
    for j in range(m):
        a = 2 * math.pi * (j + 0.5) / m
        nrm = np.array([math.cos(a), math.sin(a)])
        base.append(nrm * r * math.cos(math.pi / m)); normal.append(nrm)
    return np.array(base), np.array(normal), 0.5 * m * r * r * math.sin(2 * math.pi / m)


def points_in_planes(base, normal, lo, hi, n, seed, margin=1e-3):
    """n points uniform in the box [lo, hi] that lie inside every plane by margin."""
    rng = np.random.default_rng(seed)
    nn = normal / np.linalg.norm(normal, axis=1, keepdims=True)
    off = np.einsum("pk,pk->p", nn, base)
    out = []
    while sum(len(o) for o in out) < n:
        x = lo + (hi - lo) * rng.random((4 * n, len(lo)))
        out.append(x[np.all(x @ nn.T < off - margin, axis=1)])
    return np.concatenate(out)[:n]
