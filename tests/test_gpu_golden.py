"""The GPU path against the committed golden fixtures (tests/golden), through
the C ABI: signatures, neighbours (and lattice shifts) bit-exact, coordinates
within COORD_TOL, VI_POLYGON volumes and areas within POLY_RTOL relative."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu

COORD_TOL = 1e-9
POLY_RTOL = 1e-10


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_gpu_matches_golden(gpu_lib, name):
    hv = gpu_lib
    ref = np.load(os.path.join(HERE, name + ".npz"))
    d, n, seed, dom = G.CASES[name]
    X = ref["pts"]
    params = hv.make_params(hv.HV_METHOD_FAST)
    if dom == "simplex":
        m = hv.Mesh(hv.default_context(), X, None, None, params, planes=(ref["base"], ref["normal"], None))
    elif dom == "periodic":
        m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), params, periodic=[1] * d)
    else:
        m = hv.Mesh(hv.default_context(), X, np.zeros(d), np.ones(d), params)
    s, r = m.vertices()
    if dom == "periodic":  # translates share a signature: match by coordinates
        assert s.shape == ref["sig"].shape
        groups = {}
        for k in range(len(ref["sig"])):
            groups.setdefault(tuple(ref["sig"][k]), []).append(ref["r"][k])
        for k in range(len(s)):
            cand = groups[tuple(s[k])]
            dist = [np.max(np.abs(r[k] - c)) for c in cand]
            j = int(np.argmin(dist))
            assert dist[j] < COORD_TOL
            cand.pop(j)
        np.testing.assert_array_equal(m.periodic_shifts(), ref["shift"])
    else:
        np.testing.assert_array_equal(s, ref["sig"])
        assert np.max(np.abs(r - ref["r"])) < COORD_TOL
    o, nb = m.neighbors()
    np.testing.assert_array_equal(o, ref["offs"])
    np.testing.assert_array_equal(nb, ref["nbr"])
    v, a = m.polygon()
    np.testing.assert_allclose(v, ref["vol"], rtol=POLY_RTOL, atol=1e-15)
    np.testing.assert_allclose(a, ref["area"], rtol=POLY_RTOL, atol=1e-15)
