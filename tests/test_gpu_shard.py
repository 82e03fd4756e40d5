"""One mesh split into shards (hv_mesh_build_shard), built one after the
other on one GPU and merged on the host (hvgpu.shard): the union of the
shards' vertex records is the single build's, bit for bit, and the neighbour
lists rebuilt from it are hv_mesh_neighbors'.  Every vertex comes from
exactly one shard.  (Running the shards on several GPUs at once changes
nothing in the records; that path is not measured on hardware here.)"""
import numpy as np
import pytest

from hvgpu import datasets as D

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d,n,seed,nranks", [(2, 3000, 1, 2), (3, 4000, 2, 3), (4, 20000, 1, 4),
                                             (5, 3000, 5, 2)])
def test_shards_merge_to_the_single_mesh(gpu_lib, d, n, seed, nranks):
    from hvgpu import shard as S
    hv = gpu_lib
    pts = D.uniform_points(d, n, seed)
    lo, hi = np.zeros(d), np.ones(d)
    ctx = hv.default_context()
    full = hv.Mesh(ctx, pts, lo, hi, hv.make_params(hv.HV_METHOD_FAST))
    fs, fr = full.vertices()
    fo, fn = full.neighbors()
    parts, kept = [], []
    for rank in range(nranks):
        m = hv.Mesh(ctx, pts, lo, hi, hv.make_params(hv.HV_METHOD_FAST), shard=(rank, nranks))
        s, r = m.vertices()
        assert m.stats()["vertices"] == len(s) > 0
        parts.append((s, r))
        kept.append(len(s))
        with pytest.raises(hv.HVError):
            m.polygon()
    assert sum(kept) == len(fs)
    ms, mr = S.merge_vertex_records(parts)
    np.testing.assert_array_equal(ms, fs)
    np.testing.assert_array_equal(mr, fr)
    mo, mn = S.neighbors_from_vertices(ms, n)
    np.testing.assert_array_equal(mo, fo)
    np.testing.assert_array_equal(mn, fn)


def test_shard_argument_errors(gpu_lib):
    hv = gpu_lib
    pts = D.uniform_points(3, 100, 1)
    for bad in ((2, 2), (-1, 2), (0, 0)):
        with pytest.raises(hv.HVError):
            hv.Mesh(hv.default_context(), pts, np.zeros(3), np.ones(3), hv.make_params(hv.HV_METHOD_FAST), shard=bad)
