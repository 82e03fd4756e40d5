"""GPU integrators against the CPU oracle, through the C ABI.

VI_POLYGON: volumes and interface areas within POLY_RTOL relative (the
hot-path contract asks for 1e-10).  VI_HEURISTIC_MC: both sides use the same
Philox4x32-10 directions at equal sample counts; the GPU samples in FP32 and
accumulates in FP64, so per-cell estimates must agree within 3 sigma of the
oracle's own sampling error (and in practice to ~1e-5 relative).
"""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

POLY_RTOL = 1e-10


def _mesh(hv, pts, **kw):
    d = pts.shape[1]
    return hv.Mesh(hv.default_context(), pts, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST, **kw))


def _poly_compare(hv, pts):
    ref = O.OracleMesh(pts, integrate=True)
    rv, ra = ref.polygon()
    m = _mesh(hv, pts)
    v, a = m.polygon()
    np.testing.assert_allclose(v, rv, rtol=POLY_RTOL, atol=1e-15)
    np.testing.assert_allclose(a, ra, rtol=POLY_RTOL, atol=1e-15 * max(1.0, ra.max()))
    assert abs(v.sum() - 1.0) < 1e-11
    return v, a


@pytest.mark.parametrize("d,n,seed", [(2, 1000, 0), (3, 400, 1), (4, 300, 2), (5, 120, 3)])
def test_polygon_uniform(gpu_lib, d, n, seed):
    _poly_compare(gpu_lib, D.uniform_points(d, n, seed))


def test_polygon_clustered_5d(gpu_lib):
    _poly_compare(gpu_lib, D.clustered_points(5, 600, 2))


@pytest.mark.parametrize("d", [2, 3, 4, 5])
def test_polygon_single_cell(gpu_lib, d):
    v, a = _mesh(gpu_lib, np.full((1, d), 0.41)).polygon()
    assert v[0] == pytest.approx(1.0, rel=1e-13)
    np.testing.assert_allclose(a, 1.0, rtol=1e-13)


def test_polygon_is_deterministic(gpu_lib):
    pts = D.uniform_points(4, 800, 4)
    a = _mesh(gpu_lib, pts).polygon()
    b = _mesh(gpu_lib, pts).polygon()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("d,n,ndir", [(3, 300, 400), (4, 200, 300), (6, 60, 200)])
def test_heuristic_mc_matches_oracle(gpu_lib, d, n, ndir):
    pts = D.uniform_points(d, n, 30 + d)
    ref = O.OracleMesh(pts)
    rv, ra, vvar, avar = ref.heuristic_mc(ndir, 77)
    m = _mesh(gpu_lib, pts)
    v, a = m.heuristic_mc(ndir, 77)
    sig = np.sqrt(np.maximum(vvar, 1e-300))
    assert np.all(np.abs(v - rv) <= 3 * sig + 1e-12)
    np.testing.assert_allclose(v, rv, rtol=1e-4)
    # a direction that lies on a facet boundary within FP32 rounding may be
    # attributed to the other facet: allow that for a handful of interfaces
    close = np.abs(a - ra) <= 1e-4 * np.abs(ra) + 1e-9
    far = ~close
    assert close.mean() > 0.995
    assert np.all(np.abs(a - ra)[far] <= 3 * np.sqrt(avar[far]) + 1e-9)


def test_heuristic_mc_against_exact_volumes(gpu_lib):
    pts = D.uniform_points(3, 200, 8)
    m = _mesh(gpu_lib, pts)
    ev, _ = m.polygon()
    v, _ = m.heuristic_mc(4000, 5)
    assert abs(v.sum() - 1.0) < 0.02
    assert np.median(np.abs(v - ev) / ev) < 0.05


@pytest.mark.parametrize("d,n,seed", [(3, 300, 11), (4, 300, 12), (5, 150, 13), (6, 60, 14)])
def test_polygon_tiers_agree(gpu_lib, d, n, seed, monkeypatch):
    """Tiny vertex caps push facets through the shared-memory and the global-memory
    tier-B kernels; every tier must give the same areas as the default run."""
    pts = D.uniform_points(d, n, seed)
    monkeypatch.setenv("HV_POLY_LATTICE", "0")
    v0, a0 = _mesh(gpu_lib, pts).polygon()
    monkeypatch.setenv("HV_POLY_CAPS", "4,8")
    m = _mesh(gpu_lib, pts)
    v1, a1 = m.polygon()
    st = m.stats()
    assert st["poly_big_facets"] > 0 and st["ms_poly_big"] > 0
    np.testing.assert_allclose(v1, v0, rtol=1e-13, atol=0)
    np.testing.assert_allclose(a1, a0, rtol=1e-12, atol=1e-15 * max(1.0, a0.max()))


def _domain_mesh(hv, kind, d, n, seed):
    if kind == "box":
        return _mesh(hv, D.uniform_points(d, n, seed))
    if kind == "periodic":
        X = D.uniform_points(d, n, seed)
        return hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST),
                       periodic=[1] + [0] * (d - 1))
    E = np.random.default_rng(seed).exponential(size=(n, d + 1))  # uniform in {x > 0, sum x < 1}
    X = np.ascontiguousarray(E[:, :d] / E.sum(axis=1, keepdims=True))
    base = np.array([np.zeros(d) for _ in range(d)] + [np.full(d, 1.0 / d)])
    normal = np.array([-np.eye(d)[q] for q in range(d)] + [np.ones(d)])
    return hv.Mesh(hv.default_context(), X, None, None, hv.make_params(hv.HV_METHOD_FAST), planes=(base, normal, None))


@pytest.mark.parametrize("d,n,seed,kind", [(d, n, s, k) for d, n, s in [(3, 400, 21), (4, 300, 22), (5, 200, 23),
                                                                         (6, 80, 24)]
                                            for k in ("box", "simplex", "periodic") if d < 6 or k != "periodic"])
def test_mesh_face_lattice_matches_the_facet_lattices(gpu_lib, d, n, seed, kind, monkeypatch):
    """HV_POLY_LATTICE=1: every face of the mesh built and integrated once
    (hv_polylat.cu) gives the per-facet face lattices' volumes and areas (the
    same pulling decomposition, summed in another order) on box, plane and
    periodic domains, bitwise the same on a second run."""
    hv = gpu_lib
    m = _domain_mesh(hv, kind, d, n, seed)
    monkeypatch.setenv("HV_POLY_LATTICE", "0")
    v0, a0 = m.polygon()
    assert m.stats()["ms_poly_incidence"] > 0
    monkeypatch.setenv("HV_POLY_LATTICE", "1")
    v1, a1 = m.polygon()
    st = m.stats()
    assert st["ms_poly_big"] == 0 and st["poly_big_facets"] == 0
    assert st["poly_terms"] > 0 and st["poly_term_flops"] > st["poly_terms"] and st["poly_faces"] > 0
    np.testing.assert_allclose(v1, v0, rtol=1e-12, atol=0)
    np.testing.assert_allclose(a1, a0, rtol=1e-11, atol=1e-15 * max(1.0, a0.max()))
    v2, a2 = m.polygon()
    np.testing.assert_array_equal(v2, v1)
    np.testing.assert_array_equal(a2, a1)


@pytest.mark.parametrize("d,n,seed", [(5, 300, 31), (6, 100, 32)])
def test_mesh_face_lattice_against_the_oracle(gpu_lib, d, n, seed):
    """The default VI_POLYGON path from d = 5 on against the oracle's flag
    decomposition (src/polyintegrator.jl:174-468)."""
    _poly_compare(gpu_lib, D.uniform_points(d, n, seed))


def test_fast_polygon_integrator_is_the_polygon_integrator(gpu_lib):
    """VI_FAST_POLYGON (the reference's memoised exact integrator) gives the exact
    volumes and areas of VI_POLYGON."""
    hv = gpu_lib
    pts = D.uniform_points(4, 400, 41)
    a = hv.VoronoiData(hv.VoronoiGeometry(pts, hv.cuboid(4, periodic=[]), integrator=hv.VI_POLYGON))
    b = hv.VoronoiData(hv.VoronoiGeometry(pts, hv.cuboid(4, periodic=[]), integrator=hv.VI_FAST_POLYGON))
    np.testing.assert_array_equal(a.volume, b.volume)
    for x, y in zip(a.area, b.area):
        np.testing.assert_array_equal(x, y)
    ref = O.OracleMesh(pts, integrate=True)
    rv, _ = ref.polygon()
    np.testing.assert_allclose(b.volume, rv, rtol=POLY_RTOL, atol=1e-15)


def test_reference_method_and_integrator_names(gpu_lib):
    """The reference's raycast variants run the GPU search (same tessellation) and
    VI_MONTECARLO gives the volumes and areas VI_HEURISTIC_MC is built from
    (src/heuristic_mc.jl:10)."""
    hv = gpu_lib
    pts = D.uniform_points(3, 300, 44)
    base = hv.VoronoiData(hv.VoronoiGeometry(pts, hv.cuboid(3, periodic=[]), integrator=hv.VI_HEURISTIC_MC))
    for m in (hv.RCOriginal, hv.RCCombined, hv.RCNonGeneralHP, hv.RCStandard):
        g = hv.VoronoiGeometry(pts, hv.cuboid(3, periodic=[]), search_settings=dict(method=m),
                               integrator=hv.VI_MONTECARLO)
        vd = hv.VoronoiData(g)
        np.testing.assert_array_equal(vd.vertex_sigs, base.vertex_sigs)
        np.testing.assert_array_equal(vd.volume, base.volume)


@pytest.mark.parametrize("d,n,seed", [(3, 400, 11), (4, 200, 12), (5, 80, 13)])
def test_vertex_flag_areas_match_the_face_lattice(gpu_lib, d, n, seed, monkeypatch):
    """HV_POLY_FLAGS=1: the areas from every vertex's signed flag terms (the
    reference's flag decomposition with circumcentres of generator subsets as
    reference points) agree with the face-lattice kernels and the oracle."""
    hv = gpu_lib
    X = D.uniform_points(d, n, seed)
    m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    v0, a0 = m.polygon()
    monkeypatch.setenv("HV_POLY_FLAGS", "1")
    v1, a1 = m.polygon()
    np.testing.assert_allclose(v1, v0, rtol=1e-10, atol=0)
    np.testing.assert_allclose(a1, a0, rtol=1e-9, atol=1e-14)
    rv, ra = O.OracleMesh(X, integrate=True).polygon()
    np.testing.assert_allclose(v1, rv, rtol=1e-10, atol=0)
