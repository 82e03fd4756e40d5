"""One mesh split over ranks and merged (hvgpu.shard), on CPU with gloo.

Every rank holds the points and one contiguous range of a common generator
order.  The records a rank contributes are emulated from the oracle's mesh:
the rank visits every vertex with a generator in its range (the vertices of
its own cells, as the sharded GPU search does) and keeps those whose first
generator in that order lies in its range.  Two gloo ranks all-gather and
merge; the merged vertex set and the neighbour lists rebuilt from it must be
the single mesh's, and a vertex contributed twice must be caught.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _records(d, n, seed, rank, world):
    import oracle as O
    from hvgpu import datasets as D
    from hvgpu import shard as S
    pts = D.uniform_points(d, n, seed)
    sig, r = O.OracleMesh(pts).vertices()
    order = np.argsort(pts[:, 0] + 0.5 * pts[:, 1], kind="stable")  # any order shared by the ranks
    pos = np.empty(n, dtype=np.int64)
    pos[order] = np.arange(n)
    lo, hi = S.shard_ranges(n, world)[rank]
    real = sig <= n
    p = np.where(real, pos[np.clip(sig - 1, 0, n - 1)], n)   # position of every real generator
    visited = np.any(real & (p >= lo) & (p < hi), axis=1)
    owned = visited & (p.min(axis=1) >= lo) & (p.min(axis=1) < hi)
    return pts, sig, r, sig[owned], r[owned], sig[visited], r[visited]


def _rank(rank, world, port, out, d, n, seed):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle as O
        from hvgpu import shard as S
        pts, sig, r, osig, orr, vsig, vr = _records(d, n, seed, rank, world)
        msig, mr = S.all_gather_records(osig, orr)
        ok_set = np.array_equal(msig, sig) and np.array_equal(mr, r)
        offs, nbr = S.neighbors_from_vertices(msig, n)
        ro, rn = O.OracleMesh(pts).neighbors()
        ok_nbr = np.array_equal(offs, ro) and np.array_equal(nbr, rn)
        # contributing every visited vertex (no owner filter) repeats the shared ones
        try:
            S.all_gather_records(vsig, vr)
            caught = False
        except ValueError:
            caught = True
        out.put((rank, ok_set, ok_nbr, caught, len(osig), len(sig)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("d,n,seed", [(2, 400, 3), (3, 300, 4), (4, 150, 5)])
def test_two_ranks_merge_to_the_single_mesh(d, n, seed):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q, d, n, seed)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert all(ok_set and ok_nbr and caught for _, ok_set, ok_nbr, caught, _, _ in res)
    assert sum(k for *_, k, _ in res) == res[0][-1]          # every vertex kept by exactly one rank
    assert all(0 < k < tot for *_, k, tot in res)             # both ranks own part of the mesh


def test_shard_ranges_cover_the_order():
    from hvgpu import shard as S
    for n, w in ((10, 3), (7, 8), (100000, 4)):
        rg = S.shard_ranges(n, w)
        assert rg[0][0] == 0 and rg[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rg, rg[1:]))
        assert max(h - l for l, h in rg) - min(h - l for l, h in rg) <= 1
