"""Input generators and the C ABI surface (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from hvgpu import datasets as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_splitmix64_known_answers():
    # SplitMix64 with state 0 (Steele, Lea, Flood 2014)
    z = D.splitmix64(0, 0, 3)
    assert [int(x) for x in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_points_shape_range_determinism():
    a = D.uniform_points(4, 1000, 1)
    b = D.uniform_points(4, 1000, 1)
    assert a.shape == (1000, 4) and a.dtype == np.float64
    np.testing.assert_array_equal(a, b)
    assert np.all((a > 0) & (a < 1))
    assert not np.array_equal(a, D.uniform_points(4, 1000, 2))
    # prefix property: the first points do not depend on n
    np.testing.assert_array_equal(D.uniform_points(4, 10, 1), a[:10])


def test_clustered_points():
    p = D.clustered_points(5, 5000, 2)
    assert p.shape == (5000, 5)
    assert np.all((p > 0) & (p < 1))
    np.testing.assert_array_equal(p, D.clustered_points(5, 5000, 2))
    # mixture of 8 tight clusters: most points within 3 sigma of some centre
    assert p.std(axis=0).max() < 0.3


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "hvgpu.h")).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(hv_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def libhvgpu():
    import __graft_entry__ as g
    g.build()
    from hvgpu import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(libhvgpu):
    syms = _declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(libhvgpu, s), f"{s} declared in include/hvgpu.h but not exported"


def test_abi_argument_checks_need_no_gpu(libhvgpu):
    from hvgpu import _lib
    L = libhvgpu
    assert L.hv_version() == 10000
    p = _lib.Params()
    L.hv_params_default(ctypes.byref(p))
    assert p.method == _lib.HV_METHOD_FAST
    lo = np.zeros(2); hi = np.ones(2)
    out = ctypes.c_void_p()
    rc = L.hv_mesh_build(None, 2, 1, None, _lib.dptr(lo), _lib.dptr(hi), ctypes.byref(p), ctypes.byref(out))
    assert rc == _lib.HV_E_INVALID_ARG
    assert L.hv_mesh_free(None) == _lib.HV_E_INVALID_ARG
    assert L.hv_ctx_destroy(None) == _lib.HV_E_INVALID_ARG


def test_python_layer_fails_loudly_without_device(libhvgpu):
    import hvgpu
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(hvgpu.HVError):
        hvgpu.Context(0)


def test_cuboid_mirrors_reference_defaults():
    import hvgpu
    full = hvgpu.cuboid(3)  # the reference's default is fully periodic, partners named by 1-based index
    assert full.periodic == [1, 2, 3]
    assert [p.BC for p in full.planes] == [2, 1, 4, 3, 6, 5]
    part = hvgpu.cuboid(2, periodic=[2], neumann=[1])
    assert part.periodic_flags == [False, True]
    assert [p.BC for p in part.planes] == [hvgpu.Neumann, hvgpu.Dirichlet, 4, 3]
    b = hvgpu.cuboid(3, periodic=[], dimensions=[2, 1, 1], offset=[-1, 0, 0])
    np.testing.assert_array_equal(b.lo, [-1, 0, 0])
    np.testing.assert_array_equal(b.hi, [1, 1, 1])
    assert b.nplanes == 6
