"""GPU parity of the vertex search against the CPU oracle, through the C ABI.

Bar (from the hot-path contract): the vertex set as sorted 1-based generator
tuples and every neighbour relation are bit-exact; vertex coordinates are FP64
circumcentres and must agree with the oracle's FP64 solve within
COORD_TOL (absolute, unit-box coordinates).
"""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-9


def _build(hv, pts, method, lo=None, hi=None, **kw):
    d = pts.shape[1]
    lo = np.zeros(d) if lo is None else lo
    hi = np.ones(d) if hi is None else hi
    return hv.Mesh(hv.default_context(), pts, lo, hi, hv.make_params(method, **kw))


def _compare(hv, pts, method, lo=None, hi=None, ref=None, **kw):
    ref = ref or O.OracleMesh(pts, lo=lo, hi=hi)
    rs, rr = ref.vertices()
    ro, rn = ref.neighbors()
    m = _build(hv, pts, method, lo, hi, **kw)
    s, r = m.vertices()
    o, nb = m.neighbors()
    assert s.shape == rs.shape, f"{len(s)} vertices, oracle {len(rs)}"
    np.testing.assert_array_equal(s, rs)
    if len(r):
        assert np.max(np.abs(r - rr)) < COORD_TOL
    np.testing.assert_array_equal(o, ro)
    np.testing.assert_array_equal(nb, rn)
    st = m.stats()
    assert st["degenerate"] == 0
    return m, st


METHODS = ["fast", "plain"]


def _code(hv, name):
    return hv.HV_METHOD_FAST if name == "fast" else hv.HV_METHOD_PLAIN


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("d,n,seed", [(2, 300, 0), (3, 300, 1), (4, 300, 2), (5, 150, 3), (6, 60, 4)])
def test_uniform_small(gpu_lib, method, d, n, seed):
    _compare(gpu_lib, D.uniform_points(d, n, seed), _code(gpu_lib, method))


@pytest.mark.parametrize("method", METHODS)
def test_workload_2d_1k(gpu_lib, method):
    """2D, N=1,000 uniform, seed 0: the reference's plain CPU-runnable case."""
    w = D.WORKLOADS["2d_uniform_1k"]
    _compare(gpu_lib, D.workload_points("2d_uniform_1k"), _code(gpu_lib, method))
    assert w["d"] == 2


def test_workload_4d_20k_fast(gpu_lib):
    """4D, N=20,000 uniform, seed 1 at full size: bit-exact vertex set."""
    pts = D.workload_points("4d_uniform_20k")
    m, st = _compare(gpu_lib, pts, gpu_lib.HV_METHOD_FAST, ref=O.OracleMesh(pts, nthreads=0))
    assert st["vertices"] > 500_000


@pytest.mark.parametrize("method", METHODS)
def test_fast_and_plain_agree_4d(gpu_lib, method):
    pts = D.uniform_points(4, 3000, 9)
    a = _build(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)
    b = _build(gpu_lib, pts, _code(gpu_lib, method))
    sa, ra = a.vertices()
    sb, rb = b.vertices()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(ra, rb)  # centres are a pure function of the signature


def test_clustered_5d(gpu_lib):
    _compare(gpu_lib, D.clustered_points(5, 1500, 2), gpu_lib.HV_METHOD_FAST)


@pytest.mark.parametrize("d", [2, 3, 4, 5, 6])
def test_single_generator(gpu_lib, d):
    m, _ = _compare(gpu_lib, np.full((1, d), 0.37), gpu_lib.HV_METHOD_FAST)
    assert m.vertices()[0].shape[0] == 2 ** d


@pytest.mark.parametrize("n", [2, 3, 7])
def test_tiny_point_sets(gpu_lib, n):
    _compare(gpu_lib, D.uniform_points(3, n, 5), gpu_lib.HV_METHOD_FAST)


def test_offset_scaled_box(gpu_lib):
    lo = np.array([-2.0, 1.0, 10.0]); hi = np.array([3.0, 1.5, 12.0])
    pts = lo + (hi - lo) * D.uniform_points(3, 500, 6)
    _compare(gpu_lib, pts, gpu_lib.HV_METHOD_FAST, lo=lo, hi=hi)


def test_points_near_the_boundary(gpu_lib):
    pts = D.uniform_points(3, 400, 8)
    pts[:40, 0] = 1e-9 + pts[:40, 0] * 1e-6
    pts[40:80, 1] = 1.0 - 1e-7 * pts[40:80, 1]
    _compare(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)


def test_small_candidate_lists_fall_back_exactly(gpu_lib):
    """Lists of 8 candidates make most rays insecure: the exact path must take over."""
    pts = D.uniform_points(4, 800, 12)
    m, st = _compare(gpu_lib, pts, gpu_lib.HV_METHOD_FAST, knn=8)
    assert st["fallback_rays"] > 0


def test_capacity_retry(gpu_lib):
    pts = D.uniform_points(3, 500, 13)
    m, st = _compare(gpu_lib, pts, gpu_lib.HV_METHOD_FAST, capacity_factor=0.05)
    assert st["capacity_retries"] >= 1


def test_deterministic_output(gpu_lib):
    pts = D.uniform_points(5, 600, 14)
    a = _build(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)
    b = _build(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)
    for x, y in zip(a.vertices() + a.neighbors(), b.vertices() + b.neighbors()):
        np.testing.assert_array_equal(x, y)


def test_empty_input(gpu_lib):
    m = _build(gpu_lib, np.zeros((0, 3)), gpu_lib.HV_METHOD_FAST)
    s, r = m.vertices()
    o, nb = m.neighbors()
    assert s.shape == (0, 4) and len(nb) == 0 and list(o) == [0]


def test_invalid_inputs_raise(gpu_lib):
    hv = gpu_lib
    bad = D.uniform_points(3, 50, 1)
    bad[3, 1] = 1.5
    with pytest.raises(hv.HVError) as e:
        _build(hv, bad, hv.HV_METHOD_FAST)
    assert e.value.code == -1
    with pytest.raises(hv.HVError):
        _build(hv, D.uniform_points(7, 10, 1), hv.HV_METHOD_FAST)
    nanpts = D.uniform_points(2, 10, 1)
    nanpts[0, 0] = np.nan
    with pytest.raises(hv.HVError):
        _build(hv, nanpts, hv.HV_METHOD_FAST)
    # the context stays usable after an error
    _compare(hv, D.uniform_points(2, 20, 2), hv.HV_METHOD_FAST)


def test_geometry_api(gpu_lib):
    hv = gpu_lib
    pts = D.uniform_points(3, 200, 21)
    geo = hv.VoronoiGeometry(pts, hv.cuboid(3, periodic=[]), search_settings=dict(method=hv.RCGPU))
    data = hv.VoronoiData(geo)
    ref = O.OracleMesh(pts)
    np.testing.assert_array_equal(data.vertex_sigs, ref.vertices()[0])
    ro, rn = ref.neighbors()
    for i in range(len(pts)):
        np.testing.assert_array_equal(data.neighbors[i], rn[ro[i]:ro[i + 1]])


def test_autotune_keeps_the_vertex_set(gpu_lib):
    hv = gpu_lib
    ctx = hv.Context(0)
    best = ctx.autotune(3, 600)
    assert best["knn"] > 0 and best["leaf_size"] in (8, 16) and best["seed_stride"] in (1, 4, 8, 16)
    pts = D.uniform_points(3, 600, 31)
    m = hv.Mesh(ctx, pts, np.zeros(3), np.ones(3), hv.make_params(hv.HV_METHOD_FAST))
    np.testing.assert_array_equal(m.vertices()[0], O.OracleMesh(pts).vertices()[0])
    geo = hv.VoronoiGeometry(pts, hv.cuboid(3, periodic=[]), search_settings=dict(method=hv.RCGPU, autotune=True),
                             context=ctx)
    np.testing.assert_array_equal(geo.mesh.vertices()[0], m.vertices()[0])


def _grid(d, k):
    g = (np.arange(k) + 0.5) / k
    return np.array(np.meshgrid(*([g] * d), indexing="ij")).reshape(d, -1).T.copy()


@pytest.mark.parametrize("d,k", [(2, 6), (3, 4)])
def test_lattice_points_in_box_and_periodic_cuboids(gpu_lib, d, k):
    """Lattice points put more than d+1 generators on one empty sphere: box and
    periodic builds keep all of them (the generic walk; test_gpu_degenerate has
    the oracle comparisons), every cell has volume k^-d, and the context stays
    usable for a general-position build afterwards."""
    hv = gpu_lib
    m = _build(hv, _grid(d, k), hv.HV_METHOD_FAST)
    assert m.max_signature() == 2 ** d
    p = hv.Mesh(hv.default_context(), _grid(d, k), np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST),
                periodic=[1] * d)
    offs, sig, r = p.vertices_csr()
    assert np.all(np.diff(offs) == 2 ** d)
    v, _ = p.polygon()
    np.testing.assert_allclose(v, np.full(k ** d, float(k) ** -d), rtol=1e-12)
    _compare(hv, D.uniform_points(2, 30, 3), hv.HV_METHOD_FAST)


@pytest.mark.parametrize("d,k,eps", [(2, 20, 1e-9), (3, 8, 1e-9), (4, 4, 1e-8), (3, 6, 1e-12)])
def test_near_lattice_points(gpu_lib, d, k, eps):
    """Lattice points moved by tiny amounts: many near-ties per ray, decided
    exactly (double-double over every near-tied candidate); bit-exact against the
    oracle (binary128) and the volumes tile the cube."""
    hv = gpu_lib
    X = _grid(d, k) + eps * np.random.default_rng(d).uniform(-1, 1, (k ** d, d))
    m, st = _compare(hv, X, hv.HV_METHOD_FAST)
    v, _ = m.polygon()
    assert abs(v.sum() - 1.0) < 1e-11


def test_canonical_order_both_sort_paths(gpu_lib):
    """The canonical vertex order comes from one sort of the first d items
    packed in 64 bits when they fit (4D, 2,000 generators: 4 x 11 bits) and
    from d+1 stable passes otherwise (5D, 5,000 generators: 5 x 13 bits); either
    way the vertices come out in lexicographic order of their 1-based generator
    tuples, each once."""
    for d, n, seed in ((4, 2000, 12), (5, 5000, 11)):
        m = _build(gpu_lib, D.uniform_points(d, n, seed), gpu_lib.HV_METHOD_FAST)
        s, _ = m.vertices()
        assert len(s) > 0
        assert np.array_equal(np.lexsort(s.T[::-1]), np.arange(len(s)))
        assert (np.diff(s, axis=0) != 0).any(axis=1).all()


@pytest.mark.parametrize("d,n,seed", [(2, 1000, 0), (3, 3000, 1), (4, 20000, 1), (5, 3000, 3)])
def test_graph_driven_levels_give_the_same_mesh(gpu_lib, d, n, seed, monkeypatch):
    """HV_GRAPH=1 runs all wavefront levels in one CUDA graph launch (a
    conditional WHILE node reads the frontier on the device): the mesh is the
    host-driven one, bit for bit."""
    pts = D.uniform_points(d, n, seed)
    a = _build(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)
    monkeypatch.setenv("HV_GRAPH", "1")
    b = _build(gpu_lib, pts, gpu_lib.HV_METHOD_FAST)
    for x, y in zip(a.vertices() + a.neighbors(), b.vertices() + b.neighbors()):
        np.testing.assert_array_equal(x, y)
    assert b.stats()["levels"] >= a.stats()["levels"] - 1
