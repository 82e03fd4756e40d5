"""The allocation-free Monte-Carlo entry point (collected last on purpose).

hv_integrate_heuristic_mc_noalloc serves callers that cannot allocate device
memory; its scratch is a static device array.  Called twice in a row through
the C ABI on caller-owned device buffers, it must reproduce the allocating
entry point hv_integrate_heuristic_mc within the Monte-Carlo tests' tolerance.
"""
import numpy as np
import pytest

from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

RTOL = 1e-4  # tolerance of the Monte-Carlo parity tests


def test_noalloc_mc_matches_allocating_entry_point(gpu_lib):
    import torch
    hv = gpu_lib
    d, n, ndir, seed = 4, 400, 300, 11
    pts = D.uniform_points(d, n, 23)
    mesh = hv.Mesh(hv.default_context(), pts, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    offs, nbr = mesh.neighbors()
    v_ref, a_ref = mesh.heuristic_mc(ndir, seed)
    dev = torch.device("cuda", hv.default_context().device)
    d_pts = torch.from_numpy(pts).to(dev)
    d_off = torch.from_numpy(offs.astype(np.int64)).to(dev)
    d_nbr = torch.from_numpy((nbr - 1).astype(np.int32)).to(dev)
    max_deg = int(np.diff(offs).max())
    for call in range(2):
        d_vol = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
        d_area = torch.full((len(nbr),), np.nan, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        hv._lib.heuristic_mc_noalloc(d, n, d_pts.data_ptr(), np.zeros(d), np.ones(d), d_off.data_ptr(),
                                     d_nbr.data_ptr(), len(nbr), max_deg, ndir, seed, d_vol.data_ptr(),
                                     d_area.data_ptr(), 0)
        torch.cuda.synchronize()
        np.testing.assert_allclose(d_vol.cpu().numpy(), v_ref, rtol=RTOL)
        np.testing.assert_allclose(d_area.cpu().numpy(), a_ref, rtol=RTOL, atol=1e-12)


def test_noalloc_mc_rejects_sizes_beyond_the_scratch(gpu_lib):
    import torch
    hv = gpu_lib
    n = 3_000_000  # 2n doubles alone exceed the 16 MiB scratch
    dev = torch.device("cuda", hv.default_context().device)
    dummy = torch.zeros(8, dtype=torch.float64, device=dev)
    with pytest.raises(hv.HVError) as e:
        hv._lib.heuristic_mc_noalloc(3, n, dummy.data_ptr(), np.zeros(3), np.ones(3), dummy.data_ptr(),
                                     dummy.data_ptr(), 10, 8, 10, 1, dummy.data_ptr(), dummy.data_ptr(), 0)
    assert e.value.code == hv._lib.HV_E_CAPACITY
