"""Pins of the CPU oracle (no GPU needed).

HighVoronoi.jl holds no golden vertex sets, neighbour lists or per-cell
volumes; its own tests only assert the sum of volumes (test/rcmethods.jl:3-13,
test/database.jl:3-12, test/basics.jl:42-46, test/jld.jl:15-20).  The oracle is
pinned here by those property tests, by analytic known-answer meshes, by a
brute-force empty-circumsphere check of every vertex (verify_mesh,
src/abstractmesh.jl:221-254) and by the agreement of its two exploration
orders (per-cell and the reference's lower-cell-first rule).
"""
import math

import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D


@pytest.mark.parametrize("d", [2, 3, 4, 5])
def test_single_generator_is_the_whole_cube(d):
    m = O.OracleMesh(np.full((1, d), 0.3), integrate=True)
    sig, r = m.vertices()
    assert sig.shape == (2 ** d, d + 1)
    # every corner: the generator plus one plane per axis
    assert np.all(sig[:, 0] == 1)
    corners = {tuple(np.round(x).astype(int)) for x in r}
    assert len(corners) == 2 ** d
    vol, area = m.polygon()
    assert vol[0] == pytest.approx(1.0, abs=1e-14)
    offs, nbr = m.neighbors()
    assert list(nbr) == [1 + p for p in range(1, 2 * d + 1)]
    np.testing.assert_allclose(area, np.ones(2 * d), atol=1e-14)


def test_two_generators_split_the_square_at_the_bisector():
    a, b = 0.2, 0.7
    pts = np.array([[a, 0.5], [b, 0.5]])
    m = O.OracleMesh(pts, integrate=True)
    sig, r = m.vertices()
    # vertices: 4 corners + 2 points where the bisector x=(a+b)/2 meets y=0,1
    assert len(sig) == 6
    xm = 0.5 * (a + b)
    on_bisector = r[np.isclose(r[:, 0], xm, atol=1e-15)]
    assert len(on_bisector) == 2
    vol, area = m.polygon()
    np.testing.assert_allclose(vol, [xm, 1 - xm], atol=1e-15)
    offs, nbr = m.neighbors()
    # cell 1 (left): neighbour 2 (interface length 1) and the faces x=0 (plane 2),
    # y=1 (plane 3), y=0 (plane 4) as generators N+p = 4, 5, 6
    assert list(nbr[offs[0]:offs[1]]) == [2, 4, 5, 6]
    assert list(nbr[offs[1]:offs[2]]) == [1, 3, 5, 6]
    a1 = area[offs[0]:offs[1]]
    assert a1[0] == pytest.approx(1.0)


def test_box_offset_and_scale():
    pts = np.array([[1.5, -2.0, 3.2]])
    lo = np.array([1.0, -3.0, 3.0]); hi = np.array([2.0, -1.0, 4.0])
    m = O.OracleMesh(pts, lo=lo, hi=hi, integrate=True)
    vol, _ = m.polygon()
    assert vol[0] == pytest.approx(2.0, rel=1e-14)


@pytest.mark.parametrize("d,n", [(2, 1000), (3, 400), (4, 300), (5, 80)])
def test_vertices_pass_brute_force_empty_sphere(d, n):
    pts = D.uniform_points(d, n, 7 + d)
    m = O.OracleMesh(pts)
    sig, r = m.vertices()
    assert O.verify_vertices(pts, sig, r) == 0
    # each vertex: d+1 distinct sorted items, at least one generator
    assert np.all(np.diff(sig, axis=1) > 0)
    assert np.all(sig[:, 0] <= n)
    assert len({tuple(s) for s in sig}) == len(sig)


@pytest.mark.parametrize("d,n,tol", [(4, 1000, 1e-3), (4, 500, 1e-2), (5, 100, 1e-2)])
def test_reference_volume_sum_property(d, n, tol):
    """test/rcmethods.jl:3-13 (4D, 1000), test/basics.jl:42-46 (4D, 500), test/jld.jl:15-20 (5D, 100)."""
    pts = D.uniform_points(d, n, 100 + n)
    m = O.OracleMesh(pts, integrate=True)
    vol, area = m.polygon()
    assert abs(vol.sum() - 1.0) < tol
    assert abs(vol.sum() - 1.0) < 1e-11  # the exact integrator is exact up to rounding
    assert np.all(vol > 0)


@pytest.mark.parametrize("d,n", [(2, 500), (3, 300), (4, 150)])
def test_two_exploration_orders_agree(d, n):
    pts = D.uniform_points(d, n, 3)
    a = O.OracleMesh(pts, mode=0, integrate=True)
    b = O.OracleMesh(pts, mode=1, integrate=True)
    sa, ra = a.vertices()
    sb, rb = b.vertices()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(ra, rb)
    va, aa = a.polygon()
    vb, ab = b.polygon()
    np.testing.assert_allclose(va, vb, rtol=1e-12)
    # the reference's rule uses about one raycast per vertex (docs/src/index.md:93)
    st = b.stats()
    assert st["rays"] < 1.3 * len(sb)


def test_neighbours_and_areas_are_symmetric():
    pts = D.uniform_points(3, 300, 11)
    m = O.OracleMesh(pts, integrate=True)
    offs, nbr = m.neighbors()
    vol, area = m.polygon()
    n = len(pts)
    table = {}
    for i in range(n):
        for t in range(offs[i], offs[i + 1]):
            table[(i + 1, int(nbr[t]))] = area[t]
    for (i, k), a in table.items():
        if k <= n:
            assert (k, i) in table
            assert table[(k, i)] == a
    # sum of boundary facet areas = surface of the unit cube
    bsum = sum(a for (i, k), a in table.items() if k > n)
    assert bsum == pytest.approx(6.0, rel=1e-12)


def test_clustered_points_volume_sum():
    pts = D.clustered_points(5, 400, 2)
    m = O.OracleMesh(pts, integrate=True)
    sig, r = m.vertices()
    assert O.verify_vertices(pts, sig, r) == 0
    vol, _ = m.polygon()
    assert vol.sum() == pytest.approx(1.0, abs=1e-11)


def test_mc_matches_polygon_within_statistics():
    pts = D.uniform_points(3, 200, 5)
    m = O.OracleMesh(pts, integrate=True)
    vol, area = m.polygon()
    mvol, marea, vvar, avar = m.heuristic_mc(4000, 9)
    # raw per-cell estimator error within 5 sigma on nearly all cells
    z = np.abs(mvol - vol) / np.sqrt(np.maximum(vvar, 1e-300))
    assert np.mean(z < 5.0) > 0.97
    assert abs(mvol.sum() - 1.0) < 0.02


def test_philox_known_answers():
    """Random123 known-answer vectors of Philox4x32-10."""
    assert O.philox4x32([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox4x32([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox4x32([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_mc_directions_are_unit_and_deterministic():
    a = O.mc_directions(6, 17, 64, 3)
    b = O.mc_directions(6, 17, 64, 3)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, rtol=1e-14)
    c = O.mc_directions(6, 18, 64, 3)
    assert not np.allclose(a, c)


def test_sample_cells_counts_owned_vertices():
    pts = D.uniform_points(3, 400, 1)
    m = O.OracleMesh(pts)
    sig, _ = m.vertices()
    own, rays, sec = O.sample_cells(pts, np.arange(400))
    assert own == len(sig)
    assert rays > own and sec > 0
    assert math.isfinite(sec)


# ---- convex domains given by planes (Boundary(planes...), src/boundary.jl:94-131)

@pytest.mark.parametrize("d,n", [(2, 300), (3, 300), (4, 200), (5, 100)])
def test_rotated_cube_has_the_box_mesh(d, n):
    """A rigid motion of points and cube leaves the mesh unchanged: the same
    signatures (plane 2k = image of the box's plane 2k), coordinates moved by
    the rotation, the same volumes."""
    from _domains import rotate_points, rotated_cube
    X = D.uniform_points(d, n, 10 + d)
    Q, base, normal = rotated_cube(d, d)
    A = O.OracleMesh(X, integrate=True)
    B = O.OracleMesh(rotate_points(Q, X), planes=(base, normal), integrate=True)
    sa, ra = A.vertices()
    sb, rb = B.vertices()
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_allclose(rotate_points(Q, ra), rb, atol=1e-12)
    va, _ = A.polygon()
    vb, _ = B.polygon()
    np.testing.assert_allclose(va, vb, rtol=1e-10, atol=1e-15)
    assert O.verify_vertices(B.pts, sb, rb, planes=(base, normal)) == 0


@pytest.mark.parametrize("d,n", [(2, 200), (3, 200), (4, 200), (5, 100), (6, 40)])
def test_simplex_domain_volume(d, n):
    from _domains import simplex, simplex_points
    base, normal, vol = simplex(d)
    X = simplex_points(d, n, d)
    m = O.OracleMesh(X, planes=(base, normal), integrate=True)
    s, r = m.vertices()
    assert O.verify_vertices(X, s, r, planes=(base, normal)) == 0
    v, _ = m.polygon()
    assert abs(v.sum() - vol) < 1e-12 * max(1.0, vol) + 1e-15
    assert m.stats()["degenerate"] == 0


def test_hexagon_area_and_plane_ids():
    from _domains import points_in_planes, regular_polygon
    base, normal, area = regular_polygon(6)
    X = points_in_planes(base, normal, np.full(2, -1.0), np.full(2, 1.0), 400, 7)
    m = O.OracleMesh(X, planes=(base, normal), integrate=True)
    v, _ = m.polygon()
    assert abs(v.sum() - area) < 1e-12
    s, _ = m.vertices()
    planes_used = np.unique(s[s > len(X)]) - len(X)
    np.testing.assert_array_equal(planes_used, np.arange(1, 7))


def test_points_outside_planes_are_rejected():
    from _domains import simplex
    base, normal, _ = simplex(3)
    with pytest.raises(RuntimeError):
        O.OracleMesh(np.array([[0.2, 0.2, 0.2], [0.5, 0.5, 0.5]]), planes=(base, normal))


# ---- VoronoiData's derived views (orientations, boundary_nodes; src/voronoidata.jl:265-420)

@pytest.mark.parametrize("domain", ["box", "simplex"])
def test_orientations_are_facet_normals(domain):
    """Every vertex of cell i on the facet towards neighbour k lies on the
    bisector of x_i and x_i + o (o the orientation): (r - x_i - o/2) . o = 0.
    For plane neighbours x_i + o is the mirror image of x_i."""
    import hvgpu
    from _domains import simplex, simplex_points
    d = 3
    if domain == "box":
        X = D.uniform_points(d, 300, 5)
        b = hvgpu.cuboid(d, periodic=[])
        m = O.OracleMesh(X)
    else:
        base, normal, _ = simplex(d)
        X = simplex_points(d, 300, 5)
        b = hvgpu.Boundary(*[hvgpu.BC_Dirichlet(base[p], normal[p]) for p in range(len(base))])
        m = O.OracleMesh(X, planes=(base, normal))
    offs, nbr = m.neighbors()
    sig, r = m.vertices()
    o = hvgpu.orientations(X, offs, nbr, b)
    n = len(X)
    for i in range(0, n, 7):
        mine = np.any(sig == i + 1, axis=1)
        for t in range(offs[i], offs[i + 1]):
            rows = mine & np.any(sig == nbr[t], axis=1)
            assert rows.any()
            res = (r[rows] - X[i] - 0.5 * o[t]) @ o[t]
            assert np.max(np.abs(res)) < 1e-12
    bn = hvgpu.boundary_nodes(X, offs, nbr, b)
    for i, planes in list(bn.items())[:20]:
        for k, y in planes.items():
            np.testing.assert_allclose(y, hvgpu.reflect(X[i - 1], b, k - n), atol=1e-15)
    half = hvgpu.boundary_nodes(X, offs, nbr, b, onboundary=True)
    i, planes = next(iter(half.items()))
    for k, y in planes.items():
        np.testing.assert_allclose(y, 0.5 * (X[i - 1] + hvgpu.reflect(X[i - 1], b, k - n)), atol=1e-15)


# ---- periodic cuboids (cuboid(d), fully periodic by default, src/boundary.jl:510-534)

def _facet_pairs(P, n):
    """{(i, j, shift): area} of the periodic facets between generators."""
    out = {}
    for i in range(n):
        for t in range(P["offs"][i], P["offs"][i + 1]):
            j = int(P["nbr"][t])
            if j <= n:
                out[(i + 1, j, tuple(int(x) for x in P["shift"][t]))] = P["area"][t]
    return out


@pytest.mark.parametrize("d,n,per", [(2, 300, [1, 1]), (3, 300, [1, 1, 1]), (3, 200, [0, 1, 0]), (4, 200, [1, 1, 1, 1])])
def test_periodic_oracle_properties(d, n, per):
    """Volumes tile the torus; every facet (i, j, s) has its partner (j, i, -s)
    with the same area; the tessellation is invariant under translation mod L."""
    X = D.uniform_points(d, n, 40 + d)
    lo, hi = np.zeros(d), np.ones(d)
    P = O.periodic_mesh(X, lo, hi, per, integrate=True)
    assert abs(P["vol"].sum() - 1.0) < 1e-11
    fp = _facet_pairs(P, n)
    for (i, j, s), a in fp.items():
        b = fp[(j, i, tuple(-x for x in s))]
        assert abs(a - b) <= 1e-10 * max(a, 1e-300) + 1e-16
    t = np.where(np.asarray(per, dtype=bool), 0.3719, 0.0)
    Y = np.where(np.asarray(per, dtype=bool), (X + t) % 1.0, X)
    Q = O.periodic_mesh(Y, lo, hi, per, integrate=True)
    np.testing.assert_allclose(Q["vol"], P["vol"], rtol=1e-9, atol=1e-14)
    for i in range(0, n, 17):
        a = sorted(P["nbr"][P["offs"][i]:P["offs"][i + 1]])
        b = sorted(Q["nbr"][Q["offs"][i]:Q["offs"][i + 1]])
        assert a == b


# ---- committed golden fixtures (tests/golden/make_golden.py)

def _golden_names():
    import glob
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(here, "*.npz")))


@pytest.mark.parametrize("name", _golden_names())
def test_oracle_reproduces_golden(name):
    """The oracle still produces the committed fixtures: signatures and
    neighbours exactly, coordinates and integrals to rounding."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden as G
    ref = np.load(os.path.join(os.path.dirname(G.__file__), name + ".npz"))
    out = G.compute(name)
    np.testing.assert_array_equal(out["pts"], ref["pts"])
    np.testing.assert_array_equal(out["sig"], ref["sig"])
    np.testing.assert_allclose(out["r"], ref["r"], atol=1e-12)
    np.testing.assert_array_equal(out["offs"], ref["offs"])
    np.testing.assert_array_equal(out["nbr"], ref["nbr"])
    if "shift" in ref:
        np.testing.assert_array_equal(out["shift"], ref["shift"])
    np.testing.assert_allclose(out["vol"], ref["vol"], rtol=1e-12, atol=1e-16)
    np.testing.assert_allclose(out["area"], ref["area"], rtol=1e-12, atol=1e-16)


def test_reference_mc_directions_are_one_vector_per_batch():
    """The reference's new_directions! (src/mcintegrator.jl:82-95) keeps one
    direction for a whole batch of cells: every sample of a cell is the same,
    so the per-cell variance is zero and the volumes no longer tile the cube,
    while the i.i.d. estimator does to sampling accuracy."""
    X = D.uniform_points(3, 400, 9)
    m = O.OracleMesh(X)
    v, _, vv, _ = m.heuristic_mc(400, 3)
    r, _, rv, _ = m.heuristic_mc(400, 3, reference_directions=20)
    assert abs(v.sum() - 1.0) < 0.02
    assert np.all(rv <= 1e-12 * r ** 2) and np.all(vv > 1e-6 * v ** 2 / 400)
    assert abs(r.sum() - 1.0) > 0.05
    again, _, _, _ = m.heuristic_mc(400, 3)   # the switch is off again
    np.testing.assert_array_equal(again, v)


@pytest.mark.parametrize("d,n,seed", [(2, 800, 1), (3, 300, 2), (4, 200, 3), (5, 120, 4), (6, 50, 5)])
def test_certificate_accepts_voronoi_meshes_and_catches_errors(d, n, seed):
    """The search-independent certificate (empty spheres, two end points per
    edge, unique signatures) passes on the oracle's meshes and flags a dropped
    vertex, a duplicated one and a vertex whose signature lost a generator."""
    X = D.uniform_points(d, n, seed)
    s, r = O.OracleMesh(X).vertices()
    c = O.certify_mesh(X, s, r)
    assert all(c[k] == 0 for k in ("inside", "ties", "invalid", "open_edges", "duplicates"))
    assert c["max_coord_dev"] < 1e-12
    assert O.certify_mesh(X, s[1:], r[1:])["open_edges"] == d + 1
    assert O.certify_mesh(X, np.vstack([s, s[:1]]), np.vstack([r, r[:1]]))["duplicates"] == 1
    bad = s.copy()
    other = next(j for j in range(1, n + 1) if j not in bad[0])
    bad[0, 1] = other
    bad[0] = np.sort(bad[0])
    c = O.certify_mesh(X, bad, r)
    assert c["inside"] + c["invalid"] >= 1 and c["open_edges"] > 0


def test_certificate_on_plane_domains():
    from _domains import simplex, simplex_points
    base, normal, _ = simplex(3)
    X = simplex_points(3, 200, 7)
    s, r = O.OracleMesh(X, planes=(base, normal)).vertices()
    c = O.certify_mesh(X, s, r, planes=(base, normal))
    assert all(c[k] == 0 for k in ("inside", "ties", "invalid", "open_edges", "duplicates"))


def test_certificate_reports_lattice_ties():
    """More than d+1 co-spherical generators (a square lattice) are exact ties."""
    g = (np.arange(4) + 0.5) / 4
    X = np.array(np.meshgrid(g, g, indexing="ij")).reshape(2, -1).T.copy()
    sig = np.array([[1, 2, 5]])   # three of the four corners around (0.25, 0.25)
    c = O.certify_mesh(X, sig, np.array([[0.25, 0.25]]))
    assert c["ties"] == 1 and c["inside"] == 0


@pytest.mark.parametrize("d,n", [(2, 500), (3, 200), (4, 150), (5, 80)])
def test_polygon_cells_match_the_mesh_pass(d, n):
    """Cells integrated from their own polytope give the mesh pass's volumes and
    areas (which copies the lower cell's interfaces) to rounding."""
    X = D.uniform_points(d, n, 40 + d)
    m = O.OracleMesh(X, integrate=True)
    vol, area = m.polygon()
    ro, rn = m.neighbors()
    cells = np.arange(0, n, 3)
    v, offs, items, a = O.polygon_cells(X, cells)
    np.testing.assert_allclose(v, vol[cells], rtol=1e-12)
    for c, i in enumerate(cells):
        np.testing.assert_array_equal(items[offs[c]:offs[c + 1]], rn[ro[i]:ro[i + 1]])
        np.testing.assert_allclose(a[offs[c]:offs[c + 1]], area[ro[i]:ro[i + 1]], rtol=1e-11, atol=1e-15)


@pytest.mark.parametrize("d,n", [(2, 300), (3, 150), (4, 80)])
def test_oracle_integrand_quadrature(d, n):
    """The polygon quadrature of an integrand: a constant gives the areas and
    volumes; [1, x1, x2] integrates exactly over the cube in 2D and 3D (the
    reference's rule is the centroid rule on the facet simplices there)."""
    X = D.uniform_points(d, n, 50 + d)
    m = O.OracleMesh(X, integrate=True)
    vol, area = m.polygon()
    s, r = m.vertices()
    c = m.facet_centers()
    one = lambda P: np.ones((len(P), 1))  # noqa: E731
    I, B = m.polygon_functions(one(r), one(c), one(X))
    np.testing.assert_allclose(I[:, 0], area, rtol=1e-12)
    np.testing.assert_allclose(B[:, 0], vol, rtol=1e-12)
    lin = lambda P: np.stack([np.ones(len(P)), P[:, 0], P[:, 1]], axis=1)  # noqa: E731
    _, B = m.polygon_functions(lin(r), lin(c), lin(X))
    if d <= 3:
        np.testing.assert_allclose(B.sum(axis=0), [1.0, 0.5, 0.5], rtol=1e-12)
    else:
        assert abs(B.sum(axis=0)[1] - 0.5) < 0.01


def _lattice(d, k):
    g = (np.arange(k) + 0.5) / k
    return np.ascontiguousarray(np.stack(np.meshgrid(*([g] * d), indexing="ij"), -1).reshape(-1, d))


@pytest.mark.parametrize("d,k", [(2, 4), (3, 4), (4, 3)])
def test_generic_walk_of_lattices(d, k):
    """The reference's fraud case (test/fraud.jl:8-12, a 4 x 4 lattice) and
    its 3D/4D analogues: (k+1)^d grid-point vertices, interior ones with 2^d
    generators, 2d face neighbours per cell, cells of volume k^-d."""
    m = O.OracleMesh(_lattice(d, k), integrate=True, generic=True)
    offs, sig, r = m.vertices_csr()
    assert len(offs) - 1 == (k + 1) ** d
    assert np.diff(offs).max() == 2 ** d
    np.testing.assert_allclose(r * k, np.round(r * k), rtol=0, atol=1e-13)
    no, _ = m.neighbors()
    assert np.all(np.diff(no) == 2 * d)
    vol, area = m.polygon()
    np.testing.assert_allclose(vol, np.full(k ** d, float(k) ** -d), rtol=1e-13)
    np.testing.assert_allclose(area, np.full(len(area), float(k) ** (1 - d)), rtol=1e-13)


@pytest.mark.parametrize("d,n,seed", [(2, 150, 1), (3, 80, 2)])
def test_generic_walk_of_general_points_is_the_search(d, n, seed):
    """On points in general position the generic walk gives the per-cell search's mesh."""
    X = np.random.default_rng(seed).random((n, d))
    a = O.OracleMesh(X, integrate=True)
    b = O.OracleMesh(X, integrate=True, generic=True)
    sa, ra = a.vertices()
    ob, sb, rb = b.vertices_csr()
    np.testing.assert_array_equal(sb.reshape(-1, d + 1), sa)
    np.testing.assert_allclose(rb, ra, rtol=0, atol=1e-14)
    for x, y in zip(a.neighbors(), b.neighbors()):
        np.testing.assert_array_equal(x, y)
    va, aa = a.polygon()
    vb, ab = b.polygon()
    np.testing.assert_allclose(vb, va, rtol=1e-12)
    np.testing.assert_allclose(ab, aa, rtol=1e-11)
