"""Serving loop (continuous batching) on the GPU, through the C ABI.

Requests of mixed dimension and size are submitted while others run; each
result must be bitwise identical to the same request served alone, and agree
with the oracle.
"""
import numpy as np
import pytest

import oracle as O
from hvgpu import datasets as D

pytestmark = pytest.mark.gpu


def _requests(k):
    rng = np.random.default_rng(5)
    out = []
    for rid in range(k):
        d = int(rng.integers(2, 6))
        n = int(np.exp(rng.uniform(np.log(50), np.log(800))))
        out.append((d, n, rid))
    return out


def test_results_identical_alone_and_in_the_mix(gpu_lib):
    from hvgpu.serve import Server
    reqs = _requests(12)
    alone = []
    with Server(slots=1) as s:
        for d, n, rid in reqs:
            t = s.submit(D.uniform_points(d, n, rid), integrator="polygon")
            alone.append(s.result(t))
    with Server(slots=4) as s:
        tickets = [s.submit(D.uniform_points(d, n, rid), integrator="polygon") for d, n, rid in reqs]
        mixed = [s.result(t) for t in tickets]
    for a, b in zip(alone, mixed):
        assert a["status"] == 0 and b["status"] == 0
        for key in ("sig", "r", "offs", "nbr", "vol", "area"):
            np.testing.assert_array_equal(a[key], b[key])
    # and against the oracle on a few of them
    for (d, n, rid), res in list(zip(reqs, mixed))[:4]:
        ref = O.OracleMesh(D.uniform_points(d, n, rid), integrate=True)
        np.testing.assert_array_equal(res["sig"], ref.vertices()[0])
        rv, ra = ref.polygon()
        np.testing.assert_allclose(res["vol"], rv, rtol=1e-10)


def test_server_reports_latency_and_errors(gpu_lib):
    from hvgpu.serve import Server
    with Server(slots=2) as s:
        bad = D.uniform_points(3, 40, 1)
        bad[0, 0] = 2.0
        t_bad = s.submit(bad)
        t_ok = s.submit(D.uniform_points(3, 40, 2))
        rb = s.result(t_bad)
        ro = s.result(t_ok)
        assert rb["status"] == -1
        assert ro["status"] == 0
        assert ro["latency_ms"] >= ro["service_ms"] >= 0.0


def test_admission_budget_serialises_large_requests(gpu_lib):
    from hvgpu.serve import Server
    import hvgpu
    with pytest.raises(hvgpu.HVError):
        with Server(slots=2, hbm_budget_bytes=1e6) as s:
            s.submit(D.uniform_points(4, 2000, 1))


def test_served_periodic_and_plane_domains(gpu_lib):
    """Periodic cuboids and plane domains through the server equal the direct builds."""
    from hvgpu.serve import Server
    from _domains import simplex, simplex_points
    hv = gpu_lib
    X = D.uniform_points(3, 600, 91)
    base, normal, _ = simplex(3)
    S = simplex_points(3, 600, 92)
    with Server(slots=4) as srv:
        tp = srv.submit(X, integrator="polygon", periodic=[1, 1, 1])
        ts = srv.submit(S, integrator="polygon", planes=(base, normal, np.zeros(4, dtype=np.int16)))
        tb = srv.submit(X, integrator="polygon")
        rp, rs, rb = srv.result(tp), srv.result(ts), srv.result(tb)
    assert rp["status"] == rs["status"] == rb["status"] == 0
    mp = hv.Mesh(hv.default_context(), X, np.zeros(3), np.ones(3), hv.make_params(hv.HV_METHOD_FAST),
                 periodic=[1, 1, 1])
    np.testing.assert_array_equal(rp["sig"], mp.vertices()[0])
    np.testing.assert_array_equal(rp["nbr"], mp.neighbors()[1])
    np.testing.assert_array_equal(rp["shift"], mp.periodic_shifts())
    np.testing.assert_array_equal(rp["vol"], mp.polygon()[0])
    assert abs(rp["vol"].sum() - 1.0) < 1e-11
    ms = hv.Mesh(hv.default_context(), S, None, None, hv.make_params(hv.HV_METHOD_FAST), planes=(base, normal, None))
    np.testing.assert_array_equal(rs["sig"], ms.vertices()[0])
    np.testing.assert_array_equal(rs["vol"], ms.polygon()[0])
    assert rs["shift"] is None and rb["shift"] is None


def test_lattice_requests_return_every_generator(gpu_lib):
    """A lattice request served next to general-position ones: its vertices
    carry all their co-spherical generators (a CSR in the result), as a direct
    build gives them."""
    from hvgpu.serve import Server
    hv = gpu_lib
    g = (np.arange(5) + 0.5) / 5
    lat = np.ascontiguousarray(np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3))
    with Server(slots=4) as s:
        tk = [s.submit(D.uniform_points(3, 300, 1), integrator="polygon"), s.submit(lat, integrator="polygon"),
              s.submit(D.uniform_points(4, 200, 2), integrator="polygon")]
        res = [s.result(t) for t in tk]
    assert all(r["status"] == 0 for r in res)
    m = hv.Mesh(hv.default_context(), lat, np.zeros(3), np.ones(3), hv.make_params(hv.HV_METHOD_FAST))
    offs, sig, r = m.vertices_csr()
    got = res[1]["sig"]
    assert len(got) == len(offs) - 1 and max(len(x) for x in got) == 8
    np.testing.assert_array_equal(np.concatenate(got), sig)
    np.testing.assert_array_equal(res[1]["r"], r)
    np.testing.assert_allclose(res[1]["vol"], np.full(len(lat), 0.2 ** 3), rtol=1e-12)
    assert res[0]["sig"].shape[1] == 4 and res[2]["sig"].shape[1] == 5
