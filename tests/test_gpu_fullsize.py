"""GPU parity at the full sizes of the hot path's workloads, through the C ABI.

* 5D clustered, N=50,000 (seed 2): vertex set and neighbour CSR bit-exact
  against the oracle, VI_POLYGON volumes and areas within POLY_RTOL on a fixed
  sample of 2,000 cells (each cell integrated by the oracle from its own
  polytope) and the volumes tiling the cube.
* 6D uniform, N=10,000 (seed 3): vertex set bit-exact, VI_HEURISTIC_MC with
  1,000 directions per cell within 3 sigma of the oracle at equal samples.
* The first 20 requests of the served stream at their real sizes, served in
  one mix: vertex sets and neighbours bit-exact, volumes within POLY_RTOL.
* A certificate that does not depend on the oracle's search, on the full 4D
  and 5D GPU meshes: every vertex's circumsphere is empty (kd-tree ball query,
  binary128 near the sphere), every edge has exactly two end points, no
  signature repeats, and the volumes sum to 1.  Since the vertex graph of a
  bounded domain is connected, this proves the vertex set is the Voronoi mesh.
  It generalises the reference's volume test (test/rcmethods.jl:3-13).
"""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-9
POLY_RTOL = 1e-10


def _mesh(hv, pts, **kw):
    d = pts.shape[1]
    return hv.Mesh(hv.default_context(), pts, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST, **kw))


def _assert_certified(pts, s, r):
    c = O.certify_mesh(pts, s, r)
    for key in ("inside", "ties", "invalid", "open_edges", "duplicates"):
        assert c[key] == 0, c
    assert c["max_coord_dev"] < COORD_TOL, c
    return c


def _assert_same_mesh(m, ref):
    s, r = m.vertices()
    rs, rr = ref.vertices()
    assert s.shape == rs.shape, f"{len(s)} vertices, oracle {len(rs)}"
    np.testing.assert_array_equal(s, rs)
    assert np.max(np.abs(r - rr)) < COORD_TOL
    o, nb = m.neighbors()
    ro, rn = ref.neighbors()
    np.testing.assert_array_equal(o, ro)
    np.testing.assert_array_equal(nb, rn)
    return s, r, o, nb


def _assert_polygon_sample(pts, cells, v, a, o, lo=None, hi=None):
    rv, roffs, ritems, ra = O.polygon_cells(pts, cells, lo=lo, hi=hi)
    np.testing.assert_allclose(v[cells], rv, rtol=POLY_RTOL, atol=0)
    for c, i in enumerate(cells):
        ga = a[o[i]:o[i + 1]]
        oa = ra[roffs[c]:roffs[c + 1]]
        assert ga.shape == oa.shape
        np.testing.assert_allclose(ga, oa, rtol=POLY_RTOL, atol=1e-15 * max(1.0, oa.max()))


def test_5d_clustered_50k_full(gpu_lib):
    pts = D.workload_points("5d_clustered_50k")
    assert pts.shape == (50000, 5)
    m = _mesh(gpu_lib, pts)
    ref = O.OracleMesh(pts, nthreads=0)
    s, r, o, nb = _assert_same_mesh(m, ref)
    assert len(s) > 7_000_000
    del ref
    _assert_certified(pts, s, r)
    v, a = m.polygon()
    assert abs(v.sum() - 1.0) < 1e-11
    cells = np.arange(0, len(pts), 25)  # 2,000 cells
    _assert_polygon_sample(pts, cells, v, a, o)


def test_4d_uniform_20k_certificate(gpu_lib):
    pts = D.workload_points("4d_uniform_20k")
    m = _mesh(gpu_lib, pts)
    s, r = m.vertices()
    assert len(s) > 500_000
    _assert_certified(pts, s, r)
    v, _ = m.polygon()
    assert abs(v.sum() - 1.0) < 1e-11


def test_6d_uniform_10k_mc_full(gpu_lib):
    w = D.WORKLOADS["6d_uniform_10k_mc"]
    pts = D.workload_points("6d_uniform_10k_mc")
    m = _mesh(gpu_lib, pts)
    ref = O.OracleMesh(pts, nthreads=0)
    s, r, o, nb = _assert_same_mesh(m, ref)
    assert len(s) > 6_000_000
    _assert_certified(pts, s, r)
    ndir = w["ndir"]
    rv, ra, vvar, avar = ref.heuristic_mc(ndir, 77)
    v, a = m.heuristic_mc(ndir, 77)
    sig = np.sqrt(np.maximum(vvar, 1e-300))
    assert np.all(np.abs(v - rv) <= 3 * sig + 1e-12)
    # a direction on a facet boundary within FP32 rounding may hit the other
    # facet; the two-sided area averaging carries that into both volumes
    assert np.mean(np.abs(v - rv) <= 1e-4 * rv) > 0.995
    close = np.abs(a - ra) <= 1e-4 * np.abs(ra) + 1e-9
    assert close.mean() > 0.995
    far = ~close
    assert np.all(np.abs(a - ra)[far] <= 3 * np.sqrt(avar[far]) + 1e-9)
    assert abs(v.sum() - rv.sum()) < 1e-3 * rv.sum()  # the estimator's own bias in 6D is about 2%


def test_served_stream_first_20_requests(gpu_lib):
    from hvgpu.serve import Server
    reqs, _ = D.served_stream(20)
    with Server(slots=8) as srv:
        tickets = [srv.submit(D.uniform_points(d, n, rid), integrator="polygon") for d, n, rid in reqs]
        results = [srv.result(t) for t in tickets]
    for (d, n, rid), res in zip(reqs, results):
        assert res["status"] == 0, (d, n, rid)
        pts = D.uniform_points(d, n, rid)
        ref = O.OracleMesh(pts, nthreads=0, integrate=d <= 3)
        rs, rr = ref.vertices()
        np.testing.assert_array_equal(res["sig"], rs)
        assert np.max(np.abs(res["r"] - rr)) < COORD_TOL
        ro, rn = ref.neighbors()
        np.testing.assert_array_equal(res["offs"], ro)
        np.testing.assert_array_equal(res["nbr"], rn)
        assert abs(res["vol"].sum() - 1.0) < 1e-11
        if d <= 3:
            rv, ra = ref.polygon()
            np.testing.assert_allclose(res["vol"], rv, rtol=POLY_RTOL, atol=0)
            np.testing.assert_allclose(res["area"], ra, rtol=POLY_RTOL, atol=1e-15 * max(1.0, ra.max()))
        else:
            cells = np.unique(np.linspace(0, n - 1, min(n, 60)).astype(np.int64))
            _assert_polygon_sample(pts, cells, res["vol"], res["area"], res["offs"])
