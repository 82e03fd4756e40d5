"""One mesh split over several ranks (one GPU each), then merged.

The reference's multithreaded driver splits the cells of one mesh between
threads and merges their vertices in a shared database
(_voronoi(::MultiThread), src/sysvoronoi.jl:50-76).  Here the ranks split the
generators: every rank holds all points, orders them along the same Morton
curve (the library's internal order) and takes one contiguous range of that
order (hv_mesh_build_shard).  A rank's search visits only the vertices of its
own cells and keeps the vertices it owns: those whose smallest generator in
the Morton order lies in its range, so every vertex of the mesh is kept by
exactly one rank.  The one exchange is an all-gather of those vertex records;
the merge sorts them into the canonical order (lexicographic signatures) and
rebuilds the neighbour lists, which gives the single-GPU mesh bit for bit.
"""
from __future__ import annotations

import numpy as np


def shard_ranges(n: int, nranks: int):
    """Balanced contiguous ranges [lo, hi) of the internal (Morton) order."""
    edges = [(n * r) // nranks for r in range(nranks + 1)]
    return [(edges[r], edges[r + 1]) for r in range(nranks)]


def merge_vertex_records(parts):
    """Concatenates the (sig, r) records of all ranks and sorts them by
    signature.  Each vertex must come from exactly one rank (the owner rule);
    a repeated signature raises."""
    sigs = [np.asarray(s, dtype=np.int64) for s, _ in parts]
    rs = [np.asarray(r, dtype=np.float64) for _, r in parts]
    d1 = max((s.shape[1] for s in sigs if s.ndim == 2), default=1)
    sig = np.concatenate([s.reshape(-1, d1) for s in sigs], axis=0)
    r = np.concatenate([x.reshape(-1, d1 - 1) for x in rs], axis=0)
    order = np.lexsort(sig.T[::-1]) if len(sig) else np.zeros(0, dtype=np.int64)
    sig, r = sig[order], r[order]
    if len(sig) > 1 and np.any(np.all(sig[1:] == sig[:-1], axis=1)):
        raise ValueError("a vertex was contributed by more than one rank")
    return sig, r


def neighbors_from_vertices(sig, n: int):
    """Neighbour CSR of the cells 1..n from the vertex signatures (1-based,
    planes n+p): the sorted union of the other items of every vertex of the
    cell, the rule of neighbors_of_cell (src/neighbors.jl:219-258)."""
    sig = np.asarray(sig, dtype=np.int64)
    if sig.ndim != 2 or sig.shape[0] == 0:
        return np.zeros(n + 1, dtype=np.int64), np.zeros(0, dtype=np.int64)
    d1 = sig.shape[1]
    a = np.repeat(sig, d1, axis=1).reshape(-1)   # cell item, d1 times each
    b = np.tile(sig, (1, d1)).reshape(-1)         # every item of the same vertex
    keep = (a != b) & (a <= n)
    key = np.unique(a[keep] * (np.int64(1) << 32) + b[keep])
    cells = key >> 32
    nbr = key & ((np.int64(1) << 32) - 1)
    offs = np.cumsum(np.bincount(cells, minlength=n + 1)).astype(np.int64)  # cells are 1-based
    return offs, nbr


def all_gather_records(sig, r, group=None):
    """All-gather of every rank's owned vertex records over torch.distributed
    (NCCL between GPUs, gloo on the CPU); returns the merged mesh on every
    rank."""
    import torch.distributed as dist
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, (np.asarray(sig), np.asarray(r)), group=group)
    return merge_vertex_records(parts)
