"""Convex domains given by boundary planes (hv_mesh_build_planes) on the GPU,
against the CPU oracle and against the box path, through the C ABI.

Bar: signatures and neighbour lists bit-exact against the oracle; coordinates
within COORD_TOL; VI_POLYGON volumes and areas within POLY_RTOL relative.  A
box given as axis planes through the plane entry point runs the same exact
single-coordinate arithmetic as the box entry point, so its mesh is
bit-identical (coordinates included).
"""
import numpy as np
import pytest

import oracle as O
from _domains import points_in_planes, regular_polygon, rotate_points, rotated_cube, simplex, simplex_points
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-9
POLY_RTOL = 1e-10


def _planes_mesh(hv, pts, base, normal, bc=None, method=None, **kw):
    method = hv.HV_METHOD_FAST if method is None else method
    return hv.Mesh(hv.default_context(), pts, None, None, hv.make_params(method, **kw), planes=(base, normal, bc))


def _compare(hv, pts, base, normal, method=None, integrate=False):
    ref = O.OracleMesh(pts, planes=(base, normal), integrate=integrate)
    m = _planes_mesh(hv, pts, base, normal, method=method)
    rs, rr = ref.vertices()
    s, r = m.vertices()
    assert s.shape == rs.shape, f"{len(s)} vertices, oracle {len(rs)}"
    np.testing.assert_array_equal(s, rs)
    assert np.max(np.abs(r - rr)) < COORD_TOL
    ro, rn = ref.neighbors()
    o, nb = m.neighbors()
    np.testing.assert_array_equal(o, ro)
    np.testing.assert_array_equal(nb, rn)
    assert m.stats()["degenerate"] == 0
    if integrate:
        rv, ra = ref.polygon()
        v, a = m.polygon()
        np.testing.assert_allclose(v, rv, rtol=POLY_RTOL, atol=1e-15)
        np.testing.assert_allclose(a, ra, rtol=POLY_RTOL, atol=1e-15 * max(1.0, ra.max()))
    return m


@pytest.mark.parametrize("method", ["fast", "plain"])
@pytest.mark.parametrize("d,n", [(2, 400), (3, 300), (4, 300), (5, 150), (6, 60)])
def test_simplex_domain(gpu_lib, method, d, n):
    hv = gpu_lib
    base, normal, vol = simplex(d)
    X = simplex_points(d, n, 20 + d)
    code = hv.HV_METHOD_FAST if method == "fast" else hv.HV_METHOD_PLAIN
    m = _compare(hv, X, base, normal, method=code, integrate=(method == "fast" and d <= 5))
    if method == "fast":
        v, _ = m.polygon()
        assert abs(v.sum() - vol) < 1e-11 * vol


@pytest.mark.parametrize("d,n", [(2, 500), (3, 400), (4, 300), (5, 150)])
def test_rotated_cube(gpu_lib, d, n):
    """Rotated points in the rotated cube: the oracle's mesh, and the box mesh
    of the unrotated points (same signatures, rotated coordinates, volumes)."""
    hv = gpu_lib
    X = D.uniform_points(d, n, 30 + d)
    Q, base, normal = rotated_cube(d, d)
    Y = rotate_points(Q, X)
    m = _compare(hv, Y, base, normal, integrate=True)
    box = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    sb, rb = box.vertices()
    s, r = m.vertices()
    np.testing.assert_array_equal(s, sb)
    np.testing.assert_allclose(rotate_points(Q, rb), r, atol=1e-11)
    np.testing.assert_allclose(m.polygon()[0], box.polygon()[0], rtol=1e-10, atol=1e-15)


def test_hexagon(gpu_lib):
    base, normal, area = regular_polygon(6)
    X = points_in_planes(base, normal, np.full(2, -1.0), np.full(2, 1.0), 2000, 5)
    m = _compare(gpu_lib, X, base, normal, integrate=True)
    assert abs(m.polygon()[0].sum() - area) < 1e-11


@pytest.mark.parametrize("d,n", [(3, 2000), (4, 2000)])
def test_axis_planes_match_the_box_path_bit_for_bit(gpu_lib, d, n):
    """A box given as axis planes in a shuffled order: same mesh as the box
    entry point up to the renumbering of the planes, identical coordinates."""
    hv = gpu_lib
    lo, hi = np.full(d, -0.5), np.linspace(1.0, 2.0, d)
    X = lo + (hi - lo) * np.random.default_rng(d).random((n, d))
    box = hv.Mesh(hv.default_context(), X, lo, hi, hv.make_params(hv.HV_METHOD_FAST))
    order = np.random.default_rng(99).permutation(2 * d)   # new plane j = box plane order[j]
    base, normal = [], []
    for p in order:
        k = p // 2
        e = np.zeros(d); e[k] = 3.0                          # unnormalised normals are scaled
        if p % 2 == 0:
            b = lo.copy(); b[k] = hi[k]; base.append(b); normal.append(e)
        else:
            base.append(lo.copy()); normal.append(-e)
    m = _planes_mesh(hv, X, np.array(base), np.array(normal), bc=np.zeros(2 * d, dtype=np.int16))
    sb, rb = box.vertices()
    s, r = m.vertices()
    inv = np.empty(2 * d, dtype=np.int64); inv[order] = np.arange(2 * d)
    sb2 = np.where(sb > n, n + 1 + inv[np.clip(sb - n - 1, 0, 2 * d - 1)], sb)
    sb2.sort(axis=1)
    key = np.lexsort(sb2.T[::-1])
    np.testing.assert_array_equal(s, sb2[key])
    np.testing.assert_array_equal(r, rb[key])


def test_integrators_on_a_simplex(gpu_lib):
    hv = gpu_lib
    d = 4
    base, normal, vol = simplex(d)
    X = simplex_points(d, 400, 3)
    m = _planes_mesh(hv, X, base, normal)
    v, a = m.polygon()
    assert abs(v.sum() - vol) < 1e-11 * vol
    ref = O.OracleMesh(X, planes=(base, normal), integrate=True)
    mv, ma = m.heuristic_mc(2000, 7)
    rv, ra, vvar, avar = ref.heuristic_mc(2000, 7)
    assert np.all(np.abs(mv - rv) <= 3 * np.sqrt(np.maximum(vvar, 1e-300)) + 1e-12)
    np.testing.assert_allclose(mv, rv, rtol=1e-4)
    close = np.abs(ma - ra) <= 1e-4 * np.abs(ra) + 1e-9
    assert close.mean() > 0.995
    assert np.all(np.abs(ma - ra)[~close] <= 3 * np.sqrt(avar[~close]) + 1e-9)
    assert abs(mv.sum() - vol) < 0.05 * vol


def test_plane_domain_errors(gpu_lib):
    hv = gpu_lib
    X = np.array([[0.2, 0.2], [0.3, 0.1]])
    base, normal, _ = simplex(2)
    with pytest.raises(hv.HVError):   # one plane: unbounded
        _planes_mesh(hv, X, base[:1], normal[:1])
    with pytest.raises(hv.HVError):   # x < 0.1 and x > 0.5: empty
        _planes_mesh(hv, X, np.array([[0.1, 0], [0.5, 0], [0, 0], [0, 1]]),
                     np.array([[1.0, 0], [-1.0, 0], [0, -1.0], [0, 1.0]]))
    with pytest.raises(hv.HVError):   # periodic plane code
        _planes_mesh(hv, X, base, normal, bc=np.array([0, 0, 2], dtype=np.int16))
    with pytest.raises(hv.HVError):   # a point outside
        _planes_mesh(hv, np.array([[0.2, 0.2], [0.9, 0.9]]), base, normal)
    with pytest.raises(hv.HVError):   # zero normal
        _planes_mesh(hv, X, base, np.array([[0.0, 0.0], [0, -1.0], [1.0, 1.0]]))


def test_geometry_api_with_planes(gpu_lib):
    hv = gpu_lib
    base, normal, area = regular_polygon(5, r=2.0)
    b = hv.Boundary(*[hv.BC_Dirichlet(base[j], normal[j]) for j in range(5)])
    X = points_in_planes(base, normal, np.full(2, -2.0), np.full(2, 2.0), 500, 1)
    g = hv.VoronoiGeometry(X, b, integrator=hv.VI_POLYGON)
    vd = hv.VoronoiData(g)
    assert abs(vd.volume.sum() - area) < 1e-10
    assert all(x in b for x in X[:20])


def test_device_points_with_planes(gpu_lib):
    torch = pytest.importorskip("torch")
    hv = gpu_lib
    base, normal, _ = simplex(3)
    X = simplex_points(3, 500, 9)
    t = torch.from_numpy(X).to("cuda:0")
    torch.cuda.synchronize()
    m = hv.Mesh(hv.default_context(), np.array(X.shape), None, None, hv.make_params(hv.HV_METHOD_FAST),
                device_ptr=t.data_ptr(), planes=(base, normal, None))
    h = _planes_mesh(hv, X, base, normal)
    np.testing.assert_array_equal(m.vertices()[0], h.vertices()[0])
    np.testing.assert_array_equal(m.vertices()[1], h.vertices()[1])


def test_voronoi_data_views_and_device_handoff(gpu_lib):
    """Per-cell vertices, the zero-copy device arrays and the device-output
    integrators agree with the host outputs."""
    torch = pytest.importorskip("torch")
    hv = gpu_lib
    X = D.uniform_points(3, 800, 77)
    geo = hv.VoronoiGeometry(X, hv.cuboid(3, periodic=[]), integrator=hv.VI_POLYGON)
    vd = hv.VoronoiData(geo)
    for i in range(0, len(X), 13):
        assert len(vd.vertices[i]) > 0
        for s, _ in vd.vertices[i]:
            assert i + 1 in s
    # every vertex of the mesh appears in exactly d+1 cells counted over its generators
    cnt = np.bincount(vd.vertex_flat - 1, minlength=len(vd.vertex_sigs))
    np.testing.assert_array_equal(cnt, np.sum(vd.vertex_sigs <= len(X), axis=1))
    m = geo.mesh
    views = m.device_views()
    sig = torch.as_tensor(views["sig"], device="cuda").cpu().numpy()
    np.testing.assert_array_equal(sig + 1, vd.vertex_sigs)
    np.testing.assert_array_equal(torch.as_tensor(views["r"], device="cuda").cpu().numpy(), vd.vertex_coords)
    np.testing.assert_array_equal(torch.as_tensor(views["nbr"], device="cuda").cpu().numpy() + 1, vd.neighbor_flat)
    np.testing.assert_array_equal(torch.as_tensor(views["nbr_off"], device="cuda").cpu().numpy(), vd.neighbor_offsets)
    np.testing.assert_array_equal(torch.as_tensor(views["vtx"], device="cuda").cpu().numpy() + 1, vd.vertex_flat)
    dv = torch.zeros(len(X), dtype=torch.float64, device="cuda")
    da = torch.zeros(len(vd.neighbor_flat), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    m.polygon_device(dv.data_ptr(), da.data_ptr())
    np.testing.assert_array_equal(dv.cpu().numpy(), vd.volume)
    np.testing.assert_array_equal(da.cpu().numpy(), np.concatenate(vd.area))
    mv, ma = m.heuristic_mc(500, 3)
    m.heuristic_mc_device(500, 3, dv.data_ptr(), da.data_ptr())
    np.testing.assert_array_equal(dv.cpu().numpy(), mv)
    np.testing.assert_array_equal(da.cpu().numpy(), ma)


def test_refine_matches_a_fresh_build(gpu_lib):
    """refine!(VG, xs) appends generators: the mesh and volumes equal those of
    one build on all points, for a box, a periodic cuboid and a plane domain."""
    hv = gpu_lib
    X = D.uniform_points(3, 1200, 88)
    base, normal, _ = simplex(3)
    S = simplex_points(3, 1200, 89)
    for b, pts in ((hv.cuboid(3, periodic=[]), X), (hv.cuboid(3), X),
                   (hv.Boundary(*[hv.BC_Dirichlet(base[p], normal[p]) for p in range(4)]), S)):
        g = hv.VoronoiGeometry(pts[:800], b, integrator=hv.VI_POLYGON)
        h = hv.refine(g, pts[800:])
        assert len(g.nodes) == 800
        g.refine(pts[800:])
        f = hv.VoronoiGeometry(pts, b, integrator=hv.VI_POLYGON)
        for x in (g, h):
            np.testing.assert_array_equal(x.mesh.vertices()[0], f.mesh.vertices()[0])
            # a kept vertex's centre comes from the old mesh's solve: equal to rounding
            np.testing.assert_allclose(x.mesh.vertices()[1], f.mesh.vertices()[1], rtol=0, atol=1e-13)
            np.testing.assert_allclose(hv.VoronoiData(x).volume, hv.VoronoiData(f).volume, rtol=1e-12)


@pytest.mark.parametrize("d,n,k,steps", [(4, 20000, 200, 3), (2, 3000, 1, 5), (5, 3000, 60, 2)])
def test_incremental_refine_searches_only_the_new_cells(gpu_lib, d, n, k, steps):
    """hv_mesh_refine: a few new generators at a time; after every step the
    vertex records equal one build of all points, and the refinement walked
    far fewer rays than that build."""
    hv = gpu_lib
    X = D.uniform_points(d, n + k * steps, 123 + d)
    ctx = hv.default_context()
    lo, hi = np.zeros(d), np.ones(d)
    m = hv.Mesh(ctx, X[:n], lo, hi, hv.make_params(hv.HV_METHOD_FAST))
    for st in range(steps):
        m = m.refined(X[n + st * k:n + (st + 1) * k])
        f = hv.Mesh(ctx, X[:n + (st + 1) * k], lo, hi, hv.make_params(hv.HV_METHOD_FAST))
        s, r = m.vertices()
        fs, fr = f.vertices()
        np.testing.assert_array_equal(s, fs)
        np.testing.assert_allclose(r, fr, rtol=0, atol=1e-13)
        o, nb = m.neighbors()
        fo, fnb = f.neighbors()
        np.testing.assert_array_equal(o, fo)
        np.testing.assert_array_equal(nb, fnb)
        assert m.stats()["rays"] < 0.5 * f.stats()["rays"]
    v, _ = m.polygon()
    assert abs(v.sum() - 1.0) < 1e-11


def test_refine_with_a_point_on_an_old_circumsphere(gpu_lib):
    """A new point on an old vertex's circumsphere (within rounding) cannot be
    placed by the kept-vertex test: the whole set is searched, and the result
    is that of one build."""
    hv = gpu_lib
    X = D.uniform_points(2, 400, 5)
    ctx = hv.default_context()
    m = hv.Mesh(ctx, X, np.zeros(2), np.ones(2), hv.make_params(hv.HV_METHOD_FAST))
    s, r = m.vertices()
    v = int(np.argmin(np.sum((r - 0.5) ** 2, axis=1)))       # an interior vertex
    R = np.linalg.norm(X[s[v, 0] - 1] - r[v])
    q = r[v] + R * np.array([0.6, 0.8])
    all_pts = np.vstack([X, q[None, :]])
    try:
        f = hv.Mesh(ctx, all_pts, np.zeros(2), np.ones(2), hv.make_params(hv.HV_METHOD_FAST))
    except hv.HVError as e:  # co-circular within double-double: refused either way
        with pytest.raises(hv.HVError) as e2:
            m.refined(q)
        assert e2.value.code == e.code
        return
    g = m.refined(q)
    np.testing.assert_array_equal(g.vertices()[0], f.vertices()[0])
