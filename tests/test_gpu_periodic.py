"""Periodic cuboids (hv_mesh_build_periodic) on the GPU, through the C ABI.

The oracle chooses its own image margin, independently of the GPU's (it
starts at 2.5 mean spacings and doubles until its own certification rule,
oracle.periodic_margin_ok, holds), meshes that extended generator set, and
reduces it to the original cells (oracle.periodic_mesh).  The periodic
tessellation does not depend on the margin once the margin suffices, so a
margin the GPU chose too small shows up as a mismatch.  The GPU's own image
list is checked separately against the oracle's images for the GPU's margin.
Bar: public signatures, neighbour lists and lattice shifts bit-exact;
coordinates within COORD_TOL; VI_POLYGON volumes and areas within POLY_RTOL.
"""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-9
POLY_RTOL = 1e-10


def _mesh(hv, X, per, lo=None, hi=None):
    d = X.shape[1]
    lo = np.zeros(d) if lo is None else lo
    hi = np.ones(d) if hi is None else hi
    return hv.Mesh(hv.default_context(), X, lo, hi, hv.make_params(hv.HV_METHOD_FAST), periodic=per)


def _match_vertices(s, r, ps, pr):
    """The same multiset of signatures, and every vertex within COORD_TOL of an
    oracle vertex with that signature (translates share a signature)."""
    assert s.shape == ps.shape
    groups = {}
    for k in range(len(ps)):
        groups.setdefault(tuple(ps[k]), []).append(pr[k])
    for k in range(len(s)):
        cand = groups.get(tuple(s[k]))
        assert cand, f"vertex {s[k]} not in the oracle's mesh"
        dist = [np.max(np.abs(r[k] - c)) for c in cand]
        j = int(np.argmin(dist))
        assert dist[j] < COORD_TOL
        cand.pop(j)


def _independent_periodic_mesh(X, lo, hi, per):
    """The oracle's periodic mesh with a margin of its own choosing: 2.5 mean
    spacings, doubled until the oracle certifies it (capped at 0.999 L)."""
    n, d = X.shape
    L = hi - lo
    pflag = np.asarray(per, dtype=bool)
    spacing = (np.prod(L) / n) ** (1.0 / d)
    grow = 2.5
    while True:
        dl = np.where(pflag, np.minimum(grow * spacing, 0.999 * L), 0.0)
        img, _, _ = O.periodic_images(X, lo, hi, pflag, dl)
        ext = np.vstack([X, img])
        M = O.OracleMesh(ext, lo=lo - dl, hi=hi + dl)
        es, er = M.vertices()
        if O.periodic_margin_ok(es, er, ext, n, len(ext), lo, hi, pflag, dl):
            return O.periodic_mesh(X, lo, hi, per, delta=dl, integrate=True)
        assert not np.all(dl[pflag] >= 0.999 * L[pflag])
        grow *= 2.0


@pytest.mark.parametrize("d,n,per", [(2, 500, [1, 1]), (3, 400, [1, 1, 1]), (3, 300, [1, 0, 1]),
                                     (4, 300, [1, 1, 1, 1]), (5, 150, [1, 1, 0, 1, 1])])
def test_periodic_matches_oracle(gpu_lib, d, n, per):
    hv = gpu_lib
    X = D.uniform_points(d, n, 50 + d)
    lo, hi = np.full(d, -0.5), np.linspace(1.0, 1.5, d)
    X = lo + (hi - lo) * X
    m = _mesh(hv, X, per, lo, hi)
    delta, ref, sh = m.periodic_images()
    _, iref, ish = O.periodic_images(X, lo, hi, per, delta)
    np.testing.assert_array_equal(ref, iref + 1)
    np.testing.assert_array_equal(sh, ish)
    P = _independent_periodic_mesh(X, lo, hi, per)
    s, r = m.vertices()
    _match_vertices(s, r, P["sig"], P["r"])
    o, nb = m.neighbors()
    np.testing.assert_array_equal(o, P["offs"])
    np.testing.assert_array_equal(nb, P["nbr"])
    np.testing.assert_array_equal(m.periodic_shifts(), P["shift"])
    v, a = m.polygon()
    np.testing.assert_allclose(v, P["vol"], rtol=POLY_RTOL, atol=1e-15)
    np.testing.assert_allclose(a, P["area"], rtol=POLY_RTOL, atol=1e-15 * max(1.0, P["area"].max()))
    assert abs(v.sum() - np.prod(hi - lo)) < 1e-11 * np.prod(hi - lo)


def test_periodic_translation_invariance_and_mc(gpu_lib):
    hv = gpu_lib
    d, n = 4, 2000
    X = D.uniform_points(d, n, 61)
    per = [1, 1, 1, 1]
    a = _mesh(hv, X, per)
    b = _mesh(hv, (X + 0.2718) % 1.0, per)
    va, _ = a.polygon()
    vb, _ = b.polygon()
    np.testing.assert_allclose(va, vb, rtol=1e-9, atol=1e-15)
    assert abs(va.sum() - 1.0) < 1e-11
    mv, ma = a.heuristic_mc(1000, 5)
    assert abs(mv.sum() - 1.0) < 0.02
    assert np.median(np.abs(mv - va) / va) < 0.05


def test_periodic_geometry_api(gpu_lib):
    hv = gpu_lib
    X = D.uniform_points(3, 500, 71)
    geo = hv.VoronoiGeometry(X, hv.cuboid(3), integrator=hv.VI_POLYGON)   # the reference's default: periodic
    vd = hv.VoronoiData(geo)
    assert abs(vd.volume.sum() - 1.0) < 1e-11
    assert vd.offset > 0 and len(vd.references) == vd.offset
    # orientations point at the periodic image: every facet vertex lies on the bisector
    n = len(X)
    for i in range(0, n, 23):
        for k, o in zip(vd.neighbors[i], vd.orientations[i]):
            assert np.linalg.norm(o) < 0.9
        for s, r in vd.vertices[i]:
            assert i + 1 in s


def test_periodic_errors(gpu_lib):
    hv = gpu_lib
    with pytest.raises(hv.HVError):
        _mesh(hv, np.array([[0.5, 0.5], [1.2, 0.5]]), [1, 1])   # a point outside
