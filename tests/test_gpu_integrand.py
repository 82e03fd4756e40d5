"""Integrals of user functions with VI_POLYGON's quadrature on the GPU
(hv_mesh_facet_centers / hv_integrate_polygon_functions) against the oracle's
flag recursion, which follows the reference's Polygon_Integrator with an
integrand (src/polyintegrator.jl:80-123,174-330).  The functions are the
reference's own test integrands (test/basics.jl: x -> [1, x1, x2]) and x1^2.
Bar: interface and cell integrals within RTOL relative; a constant function
reproduces the areas and volumes; the linear one is exact in 2D and 3D."""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def _lin(P):
    return np.stack([np.ones(len(P)), P[:, 0], P[:, 1]], axis=1)


def _sq(P):
    return P[:, :1] ** 2


@pytest.mark.parametrize("d,n,seed", [(2, 400, 1), (3, 300, 2), (4, 150, 3), (5, 60, 4)])
def test_integrands_match_the_oracle(gpu_lib, d, n, seed):
    hv = gpu_lib
    X = D.uniform_points(d, n, seed)
    m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    ref = O.OracleMesh(X, integrate=True)
    s, r = m.vertices()
    rs, rr = ref.vertices()
    np.testing.assert_array_equal(s, rs)
    np.testing.assert_allclose(r, rr, rtol=0, atol=1e-13)
    c = m.facet_centers()
    np.testing.assert_allclose(c, ref.facet_centers(), rtol=0, atol=1e-13)
    vol, area = m.polygon()
    for f in (_lin, _sq):
        gi, gb = m.polygon_functions(f(r), f(c), f(X))
        oi, ob = ref.polygon_functions(f(rr), f(c), f(X))
        scale_i = np.abs(oi).max(axis=0)
        assert np.all(np.abs(gi - oi) <= RTOL * scale_i + 1e-300)
        np.testing.assert_allclose(gb, ob, rtol=RTOL, atol=RTOL * np.abs(ob).max())
    gi, gb = m.polygon_functions(np.ones((len(r), 1)), np.ones((len(c), 1)), np.ones((n, 1)))
    np.testing.assert_allclose(gi[:, 0], area, rtol=1e-11)
    np.testing.assert_allclose(gb[:, 0], vol, rtol=1e-11)
    if d <= 3:  # the reference's rule integrates linear functions exactly in 2D and 3D
        _, gb = m.polygon_functions(_lin(r), _lin(c), _lin(X))
        np.testing.assert_allclose(gb.sum(axis=0), [1.0, 0.5, 0.5], rtol=1e-12)


def test_integrand_through_the_geometry_api(gpu_lib):
    hv = gpu_lib
    X = D.uniform_points(3, 200, 9)
    geo = hv.VoronoiGeometry(X, hv.cuboid(3, periodic=[]), integrator=hv.VI_POLYGON, integrand=_lin)
    vd = hv.VoronoiData(geo)
    assert len(vd.bulk_integral) == 200 and vd.bulk_integral[0].shape == (3,)
    np.testing.assert_allclose(sum(vd.bulk_integral), [1.0, 0.5, 0.5], rtol=1e-12)
    np.testing.assert_allclose([b[0] for b in vd.bulk_integral], vd.volume, rtol=1e-11)
    for i in (0, 17, 101):
        np.testing.assert_allclose(vd.interface_integral[i][:, 0], vd.area[i], rtol=1e-11)


@pytest.mark.parametrize("d,n,seed", [(3, 300, 5), (4, 150, 6), (6, 40, 7)])
def test_heuristic_integrand_matches_the_oracle(gpu_lib, d, n, seed):
    """VI_HEURISTIC_MC with an integrand (src/heuristic.jl:105-166) on the GPU's
    Monte-Carlo areas: GPU and oracle apply the same rule to the same inputs."""
    hv = gpu_lib
    X = D.uniform_points(d, n, seed)
    m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    ref = O.OracleMesh(X, integrate=True)
    _, area = m.heuristic_mc(500, 3)
    s, r = m.vertices()
    c = m.facet_centers()
    for f in (_lin, _sq):
        gi, gb = m.heuristic_functions(area, f(r), f(c), f(X))
        oi, ob = ref.heuristic_functions(area, f(r), f(c), f(X))
        np.testing.assert_allclose(gi, oi, rtol=1e-12, atol=1e-14 * np.abs(oi).max())
        np.testing.assert_allclose(gb, ob, rtol=1e-12, atol=1e-14 * np.abs(ob).max())
    geo = hv.VoronoiGeometry(X, hv.cuboid(d, periodic=[]), integrator=hv.VI_HEURISTIC_MC, integrand=_lin,
                             mc_accurate=(500, 1, 20), mc_seed=3)
    vd = hv.VoronoiData(geo)
    # a constant integrand gives sum_k A_ik h_ik / d per cell (the cone volumes of the MC areas)
    offs, nbr = geo.mesh.neighbors()
    for i in (0, 7, n - 1):
        h = []
        for k in nbr[offs[i]:offs[i + 1]]:
            if k <= n:
                h.append(0.5 * np.linalg.norm(X[k - 1] - X[i]))
            else:
                p = k - n - 1
                h.append(1.0 - X[i, p // 2] if p % 2 == 0 else X[i, p // 2])
        expect = np.sum(vd.area[i] * np.array(h)) / d
        assert abs(vd.bulk_integral[i][0] - expect) < 1e-12 * max(expect, 1e-300)


@pytest.mark.parametrize("d,n,seed", [(3, 300, 21), (4, 150, 22), (5, 80, 23)])
def test_lattice_quadrature_matches_the_flag_walk(gpu_lib, d, n, seed, monkeypatch):
    """HV_QUAD_LATTICE=1: the flag weights as products of centroid heights summed
    over the mesh-wide face lattice (hv_polylat.cu) give the integrals of the
    per-facet flag walk (hv_quad.cu) and the facet areas for a constant."""
    hv = gpu_lib
    X = D.uniform_points(d, n, seed)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("HV_QUAD_LATTICE", mode)
        m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
        s, r = m.vertices()
        c = m.facet_centers()
        res = [m.polygon_functions(f(r), f(c), f(X)) for f in (_lin, _sq)]
        out[mode] = (c, res, m.polygon())
    c0, r0, (v0, a0) = out["0"]
    c1, r1, _ = out["1"]
    np.testing.assert_array_equal(c1, c0)
    for (gi0, gb0), (gi1, gb1) in zip(r0, r1):
        np.testing.assert_allclose(gi1, gi0, rtol=1e-12, atol=1e-15 * np.abs(gi0).max())
        np.testing.assert_allclose(gb1, gb0, rtol=1e-12, atol=1e-15 * np.abs(gb0).max())
    np.testing.assert_allclose(r1[0][0][:, 0], a0, rtol=1e-11)
    np.testing.assert_allclose(r1[0][1][:, 0], v0, rtol=1e-11)


def test_lattice_quadrature_6d_against_the_oracle(gpu_lib):
    """6D: facets beyond the flag walk's vertex cap are no limit for the face
    lattice; the integrals against the oracle's flag recursion."""
    hv = gpu_lib
    d, n = 6, 50
    X = D.uniform_points(d, n, 31)
    m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    ref = O.OracleMesh(X, integrate=True)
    s, r = m.vertices()
    c = m.facet_centers()
    vol, area = m.polygon()
    for f in (_lin, _sq):
        gi, gb = m.polygon_functions(f(r), f(c), f(X))
        oi, ob = ref.polygon_functions(f(r), f(c), f(X))
        assert np.all(np.abs(gi - oi) <= RTOL * np.abs(oi).max(axis=0) + 1e-300)
        np.testing.assert_allclose(gb, ob, rtol=RTOL, atol=RTOL * np.abs(ob).max())
    gi, gb = m.polygon_functions(np.ones((len(r), 1)), np.ones((len(c), 1)), np.ones((n, 1)))
    np.testing.assert_allclose(gi[:, 0], area, rtol=1e-11)
    np.testing.assert_allclose(gb[:, 0], vol, rtol=1e-11)
