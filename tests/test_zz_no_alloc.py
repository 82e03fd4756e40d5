"""The allocation-free Monte-Carlo entry point (collected last on purpose).

hv_integrate_heuristic_mc_noalloc is for callers that cannot allocate device
memory (an application that already holds the device's whole memory budget, a
loop in which allocator calls are forbidden, a framework that hands out fixed
buffers); its scratch is a static device array.  Called twice in a row through
the C ABI on caller-owned device buffers, it must reproduce the allocating
entry point hv_integrate_heuristic_mc bit for bit: both run the same kernels
with the same Philox directions and a fixed summation order.  Invalid
neighbour lists and sizes beyond the scratch are rejected with an error code.
"""
import numpy as np
import pytest

from hvgpu import datasets as D

pytestmark = pytest.mark.gpu

SCRATCH = 16 << 20  # HV_NOALLOC_SCRATCH_BYTES
FIXED = 1536        # HV_NOALLOC_FIXED_BYTES


def _mesh_inputs(hv, d=4, n=400, seed=23):
    import torch
    pts = D.uniform_points(d, n, seed)
    mesh = hv.Mesh(hv.default_context(), pts, np.zeros(d), np.ones(d), hv.make_params(hv.HV_METHOD_FAST))
    offs, nbr = mesh.neighbors()
    dev = torch.device("cuda", hv.default_context().device)
    d_pts = torch.from_numpy(pts).to(dev)
    d_off = torch.from_numpy(offs.astype(np.int64)).to(dev)
    d_nbr = torch.from_numpy((nbr - 1).astype(np.int32)).to(dev)
    return mesh, pts, offs, nbr, dev, d_pts, d_off, d_nbr


def _call(hv, d, n, d_pts, d_off, d_nbr, nnbr, max_deg, ndir, seed, dev):
    import torch
    d_vol = torch.full((n,), np.nan, dtype=torch.float64, device=dev)
    d_area = torch.full((max(nnbr, 1),), np.nan, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    hv._lib.heuristic_mc_noalloc(d, n, d_pts.data_ptr(), np.zeros(d), np.ones(d), d_off.data_ptr(),
                                 d_nbr.data_ptr(), nnbr, max_deg, ndir, seed, d_vol.data_ptr(),
                                 d_area.data_ptr(), 0)
    torch.cuda.synchronize()
    return d_vol.cpu().numpy(), d_area.cpu().numpy()[:nnbr]


def test_noalloc_mc_matches_allocating_entry_point(gpu_lib):
    hv = gpu_lib
    d, n, ndir, seed = 4, 400, 300, 11
    mesh, pts, offs, nbr, dev, d_pts, d_off, d_nbr = _mesh_inputs(hv, d, n)
    v_ref, a_ref = mesh.heuristic_mc(ndir, seed)
    max_deg = int(np.diff(offs).max())
    for _ in range(2):  # the second call runs on the scratch the first one left behind
        vol, area = _call(hv, d, n, d_pts, d_off, d_nbr, len(nbr), max_deg, ndir, seed, dev)
        np.testing.assert_array_equal(vol, v_ref)
        np.testing.assert_array_equal(area, a_ref)


def test_noalloc_mc_rejects_rows_longer_than_max_degree(gpu_lib):
    hv = gpu_lib
    d, n = 4, 400
    mesh, pts, offs, nbr, dev, d_pts, d_off, d_nbr = _mesh_inputs(hv, d, n)
    max_deg = int(np.diff(offs).max())
    with pytest.raises(hv.HVError) as e:
        _call(hv, d, n, d_pts, d_off, d_nbr, len(nbr), max_deg - 8, 50, 1, dev)
    assert e.value.code == hv._lib.HV_E_INVALID_ARG
    # the scratch is usable again right after the error
    vol, _ = _call(hv, d, n, d_pts, d_off, d_nbr, len(nbr), max_deg, 50, 1, dev)
    assert np.all(np.isfinite(vol))


def test_noalloc_mc_rejects_invalid_neighbour_lists(gpu_lib):
    import torch
    hv = gpu_lib
    d, n = 3, 300
    mesh, pts, offs, nbr, dev, d_pts, d_off, d_nbr = _mesh_inputs(hv, d, n, seed=5)
    max_deg = int(np.diff(offs).max())
    # a plane id beyond the cuboid's 2d faces
    bad = (nbr - 1).astype(np.int32)
    bad[offs[1] - 1] = n + 2 * d
    with pytest.raises(hv.HVError) as e:
        _call(hv, d, n, d_pts, d_off, torch.from_numpy(bad).to(dev), len(nbr), max_deg, 50, 1, dev)
    assert e.value.code == hv._lib.HV_E_INVALID_ARG
    # a one-sided relation: cell 0's first real neighbour k no longer lists 0
    k = int(nbr[offs[0]] - 1)
    assert k < n
    row = (nbr[offs[k]:offs[k + 1]] - 1).tolist()
    assert 0 in row
    one_sided = (nbr - 1).astype(np.int32)
    pos = offs[k] + row.index(0)
    repl = next(j for j in range(1, n) if j != k and j not in row)
    one_sided[pos] = repl
    one_sided[offs[k]:offs[k + 1]].sort()
    with pytest.raises(hv.HVError) as e:
        _call(hv, d, n, d_pts, d_off, torch.from_numpy(one_sided).to(dev), len(nbr), max_deg, 50, 1, dev)
    assert e.value.code == hv._lib.HV_E_INVALID_ARG


def test_noalloc_mc_capacity_limit_is_exact(gpu_lib):
    """FIXED + 8 (2n + nnbr) bytes must fit: cells without neighbours give the
    largest n that fits, which runs (zero volumes), and n + 1, which is refused
    before any device work."""
    import torch
    hv = gpu_lib
    d = 2
    n_max = (SCRATCH - FIXED) // 16
    dev = torch.device("cuda", hv.default_context().device)
    pts = torch.full((n_max + 1, d), 0.5, dtype=torch.float64, device=dev)
    off = torch.zeros(n_max + 2, dtype=torch.int64, device=dev)
    nb = torch.zeros(1, dtype=torch.int32, device=dev)
    vol, _ = _call(hv, d, n_max, pts, off, nb, 0, 8, 1, 1, dev)
    assert vol.shape == (n_max,) and np.all(vol == 0.0)
    with pytest.raises(hv.HVError) as e:
        _call(hv, d, n_max + 1, pts, off, nb, 0, 8, 1, 1, dev)
    assert e.value.code == hv._lib.HV_E_CAPACITY


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
