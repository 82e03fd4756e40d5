"""Co-spherical generators (lattices): every vertex keeps all generators on its
sphere, as the reference's vertex database does (push!(mesh, sig => r),
src/abstractmesh.jl:111-127, with the tie sets of its inrange search and the
edges of FastEdgeIterator, src/edgeiterate.jl:82-110).  The reference's own
case is a 4 x 4 lattice of the unit square (test/fraud.jl:8-12); the 3D 4^3
and 4D 3^4 lattices follow it.  Against the oracle's generic walk
(binary128): signatures bit-exact, coordinates within 1e-13, neighbours
bit-exact, VI_POLYGON volumes and areas within 1e-12; every cell of a k^d
lattice has volume k^-d and the vertices are the grid points i/k.
HV_METHOD_GENERIC on points in general position must give the fast mesh."""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu


def lattice(d, k):
    g = (np.arange(k) + 0.5) / k
    return np.ascontiguousarray(np.stack(np.meshgrid(*([g] * d), indexing="ij"), -1).reshape(-1, d))


def build(hv, X, method=None):
    d = X.shape[1]
    prm = hv.make_params(hv.HV_METHOD_FAST if method is None else method)
    return hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), prm)


@pytest.mark.parametrize("d,k", [(2, 4), (2, 7), (3, 4), (3, 5), (4, 3)])
def test_lattice_matches_the_oracle(gpu_lib, d, k):
    hv = gpu_lib
    X = lattice(d, k)
    m = build(hv, X)
    ref = O.OracleMesh(X, integrate=True, generic=True)
    offs, sig, r = m.vertices_csr()
    ro, rs, rr = ref.vertices_csr()
    np.testing.assert_array_equal(offs, ro)
    np.testing.assert_array_equal(sig, rs)
    np.testing.assert_allclose(r, rr, rtol=0, atol=1e-13)
    assert len(offs) - 1 == (k + 1) ** d
    assert m.max_signature() == 2 ** d
    # the vertices are the grid points i/k
    np.testing.assert_allclose(r * k, np.round(r * k), rtol=0, atol=1e-12)
    no, nb = m.neighbors()
    rno, rnb = ref.neighbors()
    np.testing.assert_array_equal(no, rno)
    np.testing.assert_array_equal(nb, rnb)
    assert np.all(np.diff(no) == 2 * d)  # face neighbours only, no diagonal cells
    vol, area = m.polygon()
    rv, ra = ref.polygon()
    np.testing.assert_allclose(vol, rv, rtol=1e-12, atol=0)
    np.testing.assert_allclose(area, ra, rtol=1e-12, atol=0)
    np.testing.assert_allclose(vol, np.full(len(X), float(k) ** -d), rtol=1e-12)
    np.testing.assert_allclose(area, np.full(len(area), float(k) ** (1 - d)), rtol=1e-12)
    assert abs(vol.sum() - 1.0) < 1e-12


def test_fast_vertex_reads_refuse_long_signatures(gpu_lib):
    hv = gpu_lib
    m = build(hv, lattice(2, 4))
    with pytest.raises(hv.HVError) as e:
        m.vertices()
    assert e.value.code == hv._lib.HV_E_DEGENERATE


@pytest.mark.parametrize("d,n,seed", [(2, 300, 1), (3, 200, 2), (4, 100, 3)])
def test_generic_walk_of_general_points_is_the_fast_mesh(gpu_lib, d, n, seed):
    hv = gpu_lib
    X = D.uniform_points(d, n, seed)
    a = build(hv, X)
    b = build(hv, X, hv.HV_METHOD_GENERIC)
    sa, ra = a.vertices()
    ob, sb, rb = b.vertices_csr()
    assert np.all(np.diff(ob) == d + 1)
    np.testing.assert_array_equal(sb.reshape(-1, d + 1), sa)
    np.testing.assert_allclose(rb, ra, rtol=0, atol=1e-13)
    for x, y in zip(a.neighbors(), b.neighbors()):
        np.testing.assert_array_equal(x, y)
    va, aa = a.polygon()
    vb, ab = b.polygon()
    np.testing.assert_allclose(vb, va, rtol=1e-10, atol=0)
    np.testing.assert_allclose(ab, aa, rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("d,k,seed", [(2, 6, 5), (3, 4, 6)])
def test_lattice_with_moved_points(gpu_lib, d, k, seed):
    """A lattice with a few points moved: degenerate and simple vertices mixed."""
    hv = gpu_lib
    X = lattice(d, k)
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(X), size=len(X) // 4, replace=False)
    X[idx] += rng.uniform(-0.2, 0.2, size=(len(idx), d)) / k
    m = build(hv, X)
    ref = O.OracleMesh(X, integrate=True, generic=True)
    offs, sig, r = m.vertices_csr()
    ro, rs, rr = ref.vertices_csr()
    np.testing.assert_array_equal(offs, ro)
    np.testing.assert_array_equal(sig, rs)
    np.testing.assert_allclose(r, rr, rtol=0, atol=1e-13)
    for x, y in zip(m.neighbors(), ref.neighbors()):
        np.testing.assert_array_equal(x, y)
    vol, area = m.polygon()
    rv, ra = ref.polygon()
    np.testing.assert_allclose(vol, rv, rtol=1e-11, atol=0)
    np.testing.assert_allclose(area, ra, rtol=1e-10, atol=1e-15)
    assert abs(vol.sum() - 1.0) < 1e-12


def test_lattice_monte_carlo_and_voronoi_data(gpu_lib):
    hv = gpu_lib
    d, k = 3, 4
    X = lattice(d, k)
    geo = hv.VoronoiGeometry(X, hv.cuboid(d, periodic=[]), integrator=hv.VI_POLYGON)
    data = hv.VoronoiData(geo)
    assert len(data.vertex_sigs) == (k + 1) ** d
    assert max(len(s) for s in data.vertex_sigs) == 2 ** d
    np.testing.assert_allclose(data.volume, np.full(len(X), k ** -3.0), rtol=1e-12)
    m = build(hv, X)
    vol, area = m.heuristic_mc(2000, 7)
    assert abs(vol.sum() - 1.0) < 0.05
    assert np.all(np.abs(vol * k ** 3 - 1.0) < 0.25)


@pytest.mark.parametrize("d,n,seed", [(2, 2000, 1), (3, 3000, 2), (4, 3000, 3), (5, 1500, 4), (6, 600, 5)])
def test_device_verification_of_the_vertices(gpu_lib, d, n, seed):
    """hv_mesh_verify (verify_vertex / fraud_vertex, src/raycast.jl:477-502):
    no generator strictly inside any vertex's sphere and no extra generator on
    it, on uniform, clustered and lattice inputs; the vertex's own generators
    lie on its sphere to 1e-12."""
    hv = gpu_lib
    for X in (D.uniform_points(d, n, seed), D.clustered_points(d, n, seed)):
        v = build(hv, X).verify()
        assert v["inside"] == 0 and v["ties"] == 0 and v["max_dev"] < 1e-12, v
    if d <= 4:
        v = build(hv, lattice(d, 4)).verify()
        assert v["inside"] == 0 and v["ties"] == 0 and v["max_dev"] < 1e-12, v


@pytest.mark.parametrize("d,k,per", [(2, 4, [1, 1]), (2, 5, [1, 0]), (3, 3, [1, 1, 1]), (3, 4, [0, 1, 1])])
def test_periodic_lattice_matches_the_oracle(gpu_lib, d, k, per):
    """Periodic cuboids of lattice points (the reference's periodic_grid
    geometry): the images are co-spherical too; the public view keeps every
    generator of a vertex, against the oracle's generic walk of the same
    extended set (the GPU's image margin)."""
    hv = gpu_lib
    X = lattice(d, k)
    m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST), periodic=per)
    delta, ref, sh = m.periodic_images()
    P = O.periodic_mesh(X, np.zeros(d), np.ones(d), per, delta=delta, integrate=True, generic=True)
    offs, sig, r = m.vertices_csr()
    np.testing.assert_array_equal(offs, P["sig_offs"])
    np.testing.assert_array_equal(sig, P["sig"])
    np.testing.assert_allclose(r, P["r"], rtol=0, atol=1e-13)
    o, nb = m.neighbors()
    np.testing.assert_array_equal(o, P["offs"])
    np.testing.assert_array_equal(nb, P["nbr"])
    np.testing.assert_array_equal(m.periodic_shifts(), P["shift"])
    assert np.all(np.diff(o) == 2 * d)
    v, a = m.polygon()
    np.testing.assert_allclose(v, P["vol"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(a, P["area"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(v, np.full(len(X), float(k) ** -d), rtol=1e-12)


@pytest.mark.parametrize("d,k", [(2, 8), (3, 6)])
def test_lattice_in_a_simplex_domain(gpu_lib, d, k):
    """Lattice points in the simplex {x > 0, sum x < 1} (a plane domain): the
    walk starts at a corner of the domain polytope; the cells tile the simplex,
    every vertex's sphere is empty and carries all its generators."""
    import math
    hv = gpu_lib
    X = lattice(d, k)
    X = X[X.sum(axis=1) < 1.0 - 0.5 / k]
    base = np.array([np.zeros(d) for _ in range(d)] + [np.full(d, 1.0 / d)])
    normal = np.array([-np.eye(d)[q] for q in range(d)] + [np.ones(d)])
    m = hv.Mesh(hv.default_context(), np.ascontiguousarray(X), None, None, hv.make_params(hv.HV_METHOD_FAST),
                planes=(base, normal, None))
    assert m.max_signature() == 2 ** d
    v = m.verify()
    assert v["inside"] == 0 and v["ties"] == 0 and v["max_dev"] < 1e-12, v
    vol, _ = m.polygon()
    assert abs(vol.sum() - 1.0 / math.factorial(d)) < 1e-12
    inner = X.sum(axis=1) < 1.0 - 1.5 * d / k  # every face neighbour present, the square inside the simplex
    np.testing.assert_allclose(vol[inner], float(k) ** -d, rtol=1e-12)
