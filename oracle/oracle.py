"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It restates HighVoronoi.jl's hot path on the CPU (see
hv_oracle.cpp for the reference file:line of every step) and is the checker
the CUDA library is compared against; it is never the thing measured for the
GPU numbers and never a fallback of the product.

Parity pin: parity unpinned against the reference's own outputs --
HighVoronoi.jl holds no golden vertex sets, neighbour lists or volumes and its
Julia code cannot run here.  The oracle is pinned against the reference's own property tests
(sum of volumes = domain volume, test/rcmethods.jl:3-13, test/basics.jl:42-46,
test/jld.jl:15-20), against analytic known-answer meshes and against a
brute-force empty-circumsphere check of every vertex (the model of
verify_mesh, src/abstractmesh.jl:221-254).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhvoracle.so")
_lock = threading.Lock()
_lib = None


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "rays", "descents", "descent_retries", "quad_rescores", "degenerate", "cell_vertices", "chains")]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    src = os.path.join(_HERE, "hv_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", _HERE, "-s"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            P, I64, D, I, U64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_double, ctypes.c_int, ctypes.c_uint64
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int64)
            L.hvo_build.argtypes = [I, I64, dp, dp, dp, U64, I, I, I, ctypes.POINTER(P)]
            L.hvo_build.restype = I
            L.hvo_build_planes.argtypes = [I, I64, dp, I, dp, dp, U64, I, I, I, ctypes.POINTER(P)]
            L.hvo_build_planes.restype = I
            L.hvo_verify_vertices_planes.argtypes = [I, I64, dp, I, dp, dp, I64, ip, dp, D]
            L.hvo_verify_vertices_planes.restype = I64
            L.hvo_num_vertices.argtypes = [P]; L.hvo_num_vertices.restype = I64
            L.hvo_build_generic.argtypes = [I, I64, dp, dp, dp, I, ctypes.POINTER(P)]
            L.hvo_build_generic.restype = I
            L.hvo_sig_total.argtypes = [P]; L.hvo_sig_total.restype = I64
            L.hvo_vertices_csr.argtypes = [P, ip, ip, dp]; L.hvo_vertices_csr.restype = None
            L.hvo_num_neighbors.argtypes = [P]; L.hvo_num_neighbors.restype = I64
            L.hvo_vertices.argtypes = [P, ip, dp]; L.hvo_vertices.restype = None
            L.hvo_neighbors.argtypes = [P, ip, ip]; L.hvo_neighbors.restype = None
            L.hvo_polygon.argtypes = [P, dp, dp]; L.hvo_polygon.restype = I
            L.hvo_heuristic_mc.argtypes = [P, I, U64, I, dp, dp, dp, dp]; L.hvo_heuristic_mc.restype = I
            L.hvo_get_stats.argtypes = [P, ctypes.POINTER(Stats)]; L.hvo_get_stats.restype = None
            L.hvo_last_error.argtypes = []; L.hvo_last_error.restype = ctypes.c_char_p
            L.hvo_free.argtypes = [P]; L.hvo_free.restype = None
            L.hvo_sample_cells.argtypes = [I, I64, dp, dp, dp, U64, I, I64, ip, ip, ip, dp]
            L.hvo_sample_cells.restype = I
            L.hvo_verify_vertices.argtypes = [I, I64, dp, dp, dp, I64, ip, dp, D]
            L.hvo_verify_vertices.restype = I64
            L.hvo_polygon_functions.argtypes = [P, I, dp, dp, dp, I, dp, dp]
            L.hvo_polygon_functions.restype = I
            L.hvo_facet_centers.argtypes = [P, dp]; L.hvo_facet_centers.restype = I
            L.hvo_heuristic_functions.argtypes = [P, I, dp, dp, dp, dp, I, dp, dp]
            L.hvo_heuristic_functions.restype = I
            L.hvo_mesh_from_csr.argtypes = [I, I64, dp, dp, dp, ip, ip, ctypes.POINTER(P)]
            L.hvo_mesh_from_csr.restype = I
            L.hvo_polygon_cells.argtypes = [I, I64, dp, dp, dp, U64, I, I64, ip, I64, dp, ip, ip, dp]
            L.hvo_polygon_cells.restype = I
            L.hvo_certify_mesh.argtypes = [I, I64, dp, dp, dp, I, dp, dp, I64, ip, dp, I, ip, dp]
            L.hvo_certify_mesh.restype = I
            u32p = ctypes.POINTER(ctypes.c_uint32)
            L.hvo_philox4x32.argtypes = [u32p, u32p, u32p]; L.hvo_philox4x32.restype = None
            L.hvo_mc_directions.argtypes = [I, I64, I, U64, dp]; L.hvo_mc_directions.restype = None
            L.hvo_set_mc_reference_directions.argtypes = [I]; L.hvo_set_mc_reference_directions.restype = None
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


class OracleMesh:
    """Result of one oracle mesh build (1-based reference index conventions)."""

    def __init__(self, pts, lo=None, hi=None, seed=0, nthreads=0, mode=0, integrate=False, planes=None,
                 csr=None, generic=False):
        """Box [lo, hi] (default unit cube), or the convex domain of
        ``planes = (base, normal)``, (P, d) arrays each.  ``csr = (offs, nbr)``
        (1-based neighbours) skips the search and holds only those neighbour
        lists, for running the integrators on another mesh's lists.
        ``generic=True`` (box only) walks the vertex graph with vertices of any
        number of generators (lattices); read them with vertices_csr()."""
        L = lib()
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.n, self.d = pts.shape
        self.pts = pts
        h = ctypes.c_void_p()
        if csr is not None:
            self.lo = np.ascontiguousarray(np.zeros(self.d) if lo is None else lo, dtype=np.float64)
            self.hi = np.ascontiguousarray(np.ones(self.d) if hi is None else hi, dtype=np.float64)
            offs = np.ascontiguousarray(csr[0], dtype=np.int64)
            nbr = np.ascontiguousarray(csr[1], dtype=np.int64)
            rc = L.hvo_mesh_from_csr(self.d, self.n, _dp(pts), _dp(self.lo), _dp(self.hi), _ip(offs), _ip(nbr),
                                     ctypes.byref(h))
        elif generic:
            self.lo = np.ascontiguousarray(np.zeros(self.d) if lo is None else lo, dtype=np.float64)
            self.hi = np.ascontiguousarray(np.ones(self.d) if hi is None else hi, dtype=np.float64)
            rc = L.hvo_build_generic(self.d, self.n, _dp(pts), _dp(self.lo), _dp(self.hi), 1 if integrate else 0,
                                     ctypes.byref(h))
        elif planes is not None:
            base = np.ascontiguousarray(planes[0], dtype=np.float64)
            normal = np.ascontiguousarray(planes[1], dtype=np.float64)
            self.lo = self.hi = None
            rc = L.hvo_build_planes(self.d, self.n, _dp(pts), base.shape[0], _dp(base), _dp(normal), seed,
                                    nthreads, mode, 1 if integrate else 0, ctypes.byref(h))
        else:
            self.lo = np.ascontiguousarray(np.zeros(self.d) if lo is None else lo, dtype=np.float64)
            self.hi = np.ascontiguousarray(np.ones(self.d) if hi is None else hi, dtype=np.float64)
            rc = L.hvo_build(self.d, self.n, _dp(pts), _dp(self.lo), _dp(self.hi), seed, nthreads, mode,
                             1 if integrate else 0, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle build failed ({rc}): {L.hvo_last_error().decode()}")
        self._h = h
        self.integrated = integrate

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().hvo_free(h)
            self._h = None

    def vertices(self):
        L = lib()
        V = L.hvo_num_vertices(self._h)
        sig = np.zeros((V, self.d + 1), dtype=np.int64)
        r = np.zeros((V, self.d), dtype=np.float64)
        if V:
            L.hvo_vertices(self._h, _ip(sig), _dp(r))
        return sig, r

    def vertices_csr(self):
        """(offs (V+1), sig (1-based, sorted per vertex), r (V, d)) for vertices
        of any number of generators, in lexicographic order of their signatures."""
        L = lib()
        V = L.hvo_num_vertices(self._h)
        S = L.hvo_sig_total(self._h)
        offs = np.zeros(V + 1, dtype=np.int64)
        sig = np.zeros(max(S, 1), dtype=np.int64)
        r = np.zeros((V, self.d), dtype=np.float64)
        if V:
            L.hvo_vertices_csr(self._h, _ip(offs), _ip(sig), _dp(r))
        return offs, sig[:S], r

    def neighbors(self):
        L = lib()
        E = L.hvo_num_neighbors(self._h)
        offs = np.zeros(self.n + 1, dtype=np.int64)
        nbr = np.zeros(max(E, 1), dtype=np.int64)
        L.hvo_neighbors(self._h, _ip(offs), _ip(nbr))
        return offs, nbr[:E]

    def polygon(self):
        L = lib()
        E = L.hvo_num_neighbors(self._h)
        vol = np.zeros(self.n)
        area = np.zeros(max(E, 1))
        if L.hvo_polygon(self._h, _dp(vol), _dp(area)) != 0:
            raise RuntimeError(L.hvo_last_error().decode())
        return vol, area[:E]

    def facet_centers(self):
        """(nnbr, d) centres (vertex means) of the facets, aligned with neighbors()."""
        L = lib()
        E = L.hvo_num_neighbors(self._h)
        c = np.zeros((max(E, 1), self.d))
        if L.hvo_facet_centers(self._h, _dp(c)) != 0:
            raise RuntimeError(L.hvo_last_error().decode())
        return c[:E]

    def polygon_functions(self, fv, fc, fx, bulk=True):
        """Interface (nnbr, p) and cell (n, p) integrals of a function given by
        its values fv at the vertices, fc at the facet centres and fx at the
        generators (the reference's Polygon_Integrator with an integrand)."""
        L = lib()
        fv = np.ascontiguousarray(np.asarray(fv, dtype=np.float64).reshape(len(fv), -1))
        p = fv.shape[1]
        fc = np.ascontiguousarray(np.asarray(fc, dtype=np.float64).reshape(-1, p))
        fx = np.ascontiguousarray(np.asarray(fx, dtype=np.float64).reshape(-1, p))
        E = L.hvo_num_neighbors(self._h)
        iface = np.zeros((max(E, 1), p))
        blk = np.zeros((self.n, p))
        if L.hvo_polygon_functions(self._h, p, _dp(fv), _dp(fc), _dp(fx), 1 if bulk else 0, _dp(iface), _dp(blk)) != 0:
            raise RuntimeError(L.hvo_last_error().decode())
        return iface[:E], blk

    def heuristic_functions(self, area, fv, fc, fx, bulk=True):
        """The heuristic integrand rule on the interface areas ``area``."""
        L = lib()
        fv = np.ascontiguousarray(np.asarray(fv, dtype=np.float64).reshape(len(fv), -1))
        p = fv.shape[1]
        fc = np.ascontiguousarray(np.asarray(fc, dtype=np.float64).reshape(-1, p))
        fx = np.ascontiguousarray(np.asarray(fx, dtype=np.float64).reshape(-1, p))
        area = np.ascontiguousarray(area, dtype=np.float64)
        E = L.hvo_num_neighbors(self._h)
        iface = np.zeros((max(E, 1), p))
        blk = np.zeros((self.n, p))
        if L.hvo_heuristic_functions(self._h, p, _dp(area), _dp(fv), _dp(fc), _dp(fx), 1 if bulk else 0,
                                     _dp(iface), _dp(blk)) != 0:
            raise RuntimeError(L.hvo_last_error().decode())
        return iface[:E], blk

    def heuristic_mc(self, ndir, seed, nthreads=0, reference_directions=0):
        """i.i.d. directions per cell; ``reference_directions=r`` (> 0) instead
        reproduces the reference's batches (one direction for every sample of r
        consecutive cells, src/mcintegrator.jl:82-107), for documentation."""
        L = lib()
        with _lock:
            L.hvo_set_mc_reference_directions(int(reference_directions))
            try:
                return self._heuristic_mc(L, ndir, seed, nthreads)
            finally:
                L.hvo_set_mc_reference_directions(0)

    def _heuristic_mc(self, L, ndir, seed, nthreads):
        E = L.hvo_num_neighbors(self._h)
        vol = np.zeros(self.n)
        area = np.zeros(max(E, 1))
        vv = np.zeros(self.n)
        av = np.zeros(max(E, 1))
        if L.hvo_heuristic_mc(self._h, ndir, seed, nthreads, _dp(vol), _dp(area), _dp(vv), _dp(av)) != 0:
            raise RuntimeError(L.hvo_last_error().decode())
        return vol, area[:E], vv, av[:E]

    def stats(self):
        st = Stats()
        lib().hvo_get_stats(self._h, ctypes.byref(st))
        return {n: getattr(st, n) for n, _ in Stats._fields_}


def verify_vertices(pts, sig, r, lo=None, hi=None, rel_tol=1e-9, planes=None):
    """Brute-force empty-sphere check; returns the number of bad vertices."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, d = pts.shape
    sig = np.ascontiguousarray(sig, dtype=np.int64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    if planes is not None:
        base = np.ascontiguousarray(planes[0], dtype=np.float64)
        normal = np.ascontiguousarray(planes[1], dtype=np.float64)
        return lib().hvo_verify_vertices_planes(d, n, _dp(pts), base.shape[0], _dp(base), _dp(normal),
                                                sig.shape[0], _ip(sig), _dp(r), rel_tol)
    lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
    hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
    sig = np.ascontiguousarray(sig, dtype=np.int64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    return lib().hvo_verify_vertices(d, n, _dp(pts), _dp(lo), _dp(hi), sig.shape[0], _ip(sig), _dp(r), rel_tol)


def sample_cells(pts, cells, seed=0, nthreads=0, lo=None, hi=None):
    """CPU-baseline sample: (owned vertices, rays, seconds) for the listed cells."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, d = pts.shape
    lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
    hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    own = ctypes.c_int64(); rays = ctypes.c_int64(); sec = ctypes.c_double()
    rc = lib().hvo_sample_cells(d, n, _dp(pts), _dp(lo), _dp(hi), seed, nthreads, cells.shape[0], _ip(cells),
                                ctypes.byref(own), ctypes.byref(rays), ctypes.byref(sec))
    if rc != 0:
        raise RuntimeError(lib().hvo_last_error().decode())
    return own.value, rays.value, sec.value


def polygon_cells(pts, cells, lo=None, hi=None, seed=0, nthreads=0):
    """VI_POLYGON of the listed cells (0-based), each from its own polytope:
    (vol[ncells], offs[ncells+1], items (1-based neighbours), areas)."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, d = pts.shape
    lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
    hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int64)
    m = cells.shape[0]
    cap = max(64, 8 * (d + 1) * 40 * m)
    while True:
        vol = np.zeros(m)
        offs = np.zeros(m + 1, dtype=np.int64)
        items = np.zeros(cap, dtype=np.int64)
        area = np.zeros(cap)
        rc = lib().hvo_polygon_cells(d, n, _dp(pts), _dp(lo), _dp(hi), seed, nthreads, m, _ip(cells), cap,
                                     _dp(vol), _ip(offs), _ip(items), _dp(area))
        if rc == -4:
            cap = int(offs[-1])
            continue
        if rc != 0:
            raise RuntimeError(lib().hvo_last_error().decode())
        return vol, offs, items[:offs[-1]], area[:offs[-1]]


def certify_mesh(pts, sig, r, lo=None, hi=None, planes=None, nthreads=0):
    """Certificate of a vertex list that does not use the oracle's search: an
    exact empty-sphere test of every vertex (kd-tree ball query, binary128 near
    the sphere), exactly two end points per edge, no duplicate signature.
    Returns a dict of violation counts (all zero for a Voronoi mesh), the
    binary128 re-decisions and the largest coordinate deviation."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, d = pts.shape
    sig = np.ascontiguousarray(sig, dtype=np.int64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
    hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
    if planes is not None:
        base = np.ascontiguousarray(planes[0], dtype=np.float64)
        normal = np.ascontiguousarray(planes[1], dtype=np.float64)
        np_ = base.shape[0]
    else:
        base = normal = np.zeros(d)
        np_ = 0
    out = np.zeros(6, dtype=np.int64)
    dev = ctypes.c_double()
    rc = lib().hvo_certify_mesh(d, n, _dp(pts), _dp(lo), _dp(hi), np_, _dp(base), _dp(normal), sig.shape[0],
                                _ip(sig), _dp(r), nthreads, _ip(out), ctypes.byref(dev))
    if rc != 0:
        raise RuntimeError(lib().hvo_last_error().decode())
    keys = ("inside", "ties", "invalid", "open_edges", "duplicates", "quad_decisions")
    res = {k: int(v) for k, v in zip(keys, out)}
    res["max_coord_dev"] = dev.value
    return res


def philox4x32(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().hvo_philox4x32(c, k, o)
    return list(o)


def mc_directions(d, cell, ndir, seed):
    out = np.zeros((ndir, d))
    lib().hvo_mc_directions(d, cell, ndir, seed, _dp(out))
    return out


# ---- periodic cuboids: the oracle's mesh of the generators and their periodic
# images in the widened box, reduced to the original cells (the same
# construction as the reference's periodize!, src/domain.jl:139-213)

def _codes(d):
    c = np.arange(3 ** d)
    return np.stack([(c // 3 ** k) % 3 - 1 for k in range(d)], axis=1)  # (3^d, d) shifts


def periodic_images(pts, lo, hi, periodic, delta):
    """Images x + s*L strictly inside the box widened by delta on the periodic
    axes, in (point, shift code) order: (images, 0-based originals, shifts)."""
    pts = np.asarray(pts, dtype=np.float64)
    n, d = pts.shape
    lo, hi, delta = (np.asarray(a, dtype=np.float64) for a in (lo, hi, delta))
    L = hi - lo
    per = np.asarray(periodic, dtype=bool)
    S = _codes(d)
    S = S[np.all((S == 0) | per, axis=1) & np.any(S != 0, axis=1)]
    Y = pts[:, None, :] + S[None, :, :] * L
    moved = S[None, :, :] != 0
    ok = np.all(~moved | ((Y > lo - delta) & (Y < hi + delta)), axis=2)
    ii, cc = np.nonzero(ok)  # row-major: point-major, codes ascending
    return Y[ii, cc], ii, S[cc]


def periodic_margin_ok(ext_sig, ext_r, ext_pts, n, n_ext, lo, hi, periodic, delta):
    """Every vertex of an original cell has its circumsphere inside the widened
    box and holds no widened periodic face."""
    pub = ext_sig[:, 0] <= n
    s, r = ext_sig[pub], ext_r[pub]
    per = np.asarray(periodic, dtype=bool)
    planes = s > n_ext
    if np.any(planes & per[np.clip((s - n_ext - 1) // 2, 0, len(per) - 1)]):
        return False
    R = np.linalg.norm(r - ext_pts[s[:, 0] - 1], axis=1)[:, None] * (1 + 1e-12) + 1e-12
    lo, hi, delta = (np.asarray(a, dtype=np.float64) for a in (lo, hi, delta))
    inside = (r - R > lo - delta) & (r + R < hi + delta)
    return bool(np.all(inside[:, per]))


def _margin_ok_csr(eoff, esig, er, ext_pts, n, n_ext, lo, hi, periodic, delta):
    """periodic_margin_ok for vertices of any number of generators (CSR rows)."""
    per = np.asarray(periodic, dtype=bool)
    lo, hi, delta = (np.asarray(a, dtype=np.float64) for a in (lo, hi, delta))
    for v in range(len(eoff) - 1):
        s = esig[eoff[v]:eoff[v + 1]]
        if s[0] > n:
            continue
        pl = s[s > n_ext]
        if np.any(per[(pl - n_ext - 1) // 2]):
            return False
        R = np.linalg.norm(er[v] - ext_pts[s[0] - 1]) * (1 + 1e-12) + 1e-12
        if not np.all(((er[v] - R > lo - delta) & (er[v] + R < hi + delta))[per]):
            return False
    return True


def periodic_mesh(pts, lo, hi, periodic, delta=None, integrate=False, nthreads=0, generic=False):
    """The periodic tessellation of ``pts`` in the cuboid [lo, hi] (periodic
    axes flagged) from the oracle's mesh of the extended generator set.  With
    delta None the margin grows from 1.5 spacings by 1.5 until certified.
    Returns a dict: delta, sig (V, d+1) 1-based original ids (rows sorted),
    r, offs, nbr (1-based, sorted by (id, shift code)), shift (nnbr, d) and,
    if integrate, vol and area.  generic=True meshes the extended set with the
    generic walk (lattices): sig is then a CSR, sig_offs (V+1) and sig."""
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, d = pts.shape
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    per = np.asarray(periodic, dtype=bool)
    L = hi - lo
    spacing = (np.prod(L) / n) ** (1.0 / d)
    grow = 1.5
    while True:
        dl = np.where(per, np.minimum(grow * spacing, 0.999 * L), 0.0) if delta is None else np.asarray(delta)
        img, ref, sh = periodic_images(pts, lo, hi, per, dl)
        ext = np.vstack([pts, img])
        n_ext = len(ext)
        M = OracleMesh(ext, lo=lo - dl, hi=hi + dl, integrate=integrate, nthreads=nthreads, generic=generic)
        if generic:
            eoff, esig, er = M.vertices_csr()
            ok = _margin_ok_csr(eoff, esig, er, ext, n, n_ext, lo, hi, per, dl)
        else:
            es, er = M.vertices()
            ok = periodic_margin_ok(es, er, ext, n, n_ext, lo, hi, per, dl)
        if delta is not None or ok:
            break
        if np.all(dl[per] >= 0.999 * L[per]):
            raise RuntimeError("too few generators for the periodic image margin")
        grow *= 1.5
    center = (3 ** d - 1) // 2
    codes = np.full(n_ext + 2 * d + 1, center, dtype=np.int64)
    ids = np.arange(n_ext + 2 * d + 1, dtype=np.int64)   # 1-based ext id -> public id
    weights = 3 ** np.arange(d)
    codes[n + 1:n_ext + 1] = (sh + 1) @ weights
    ids[n + 1:n_ext + 1] = ref + 1
    ids[n_ext + 1:] = n + np.arange(1, 2 * d + 1)
    if generic:
        rows = [np.sort(ids[esig[eoff[v]:eoff[v + 1]]]) for v in range(len(eoff) - 1) if esig[eoff[v]] <= n]
        pr = er[np.array([esig[eoff[v]] <= n for v in range(len(eoff) - 1)], dtype=bool)]
        psig_offs = np.concatenate([[0], np.cumsum([len(x) for x in rows])]).astype(np.int64)
        psig = np.concatenate(rows) if rows else np.zeros(0, dtype=np.int64)
    else:
        pub = es[:, 0] <= n
        psig = np.sort(ids[es[pub]], axis=1)
        pr = er[pub]
    eo, en = M.neighbors()
    offs = eo[:n + 1].copy()
    tot = int(offs[-1])
    key = ids[en[:tot]] * 1024 + codes[en[:tot]]
    row = np.repeat(np.arange(n), np.diff(offs))
    order = np.lexsort((key, row))
    nbr = ids[en[:tot]][order]
    c = codes[en[:tot]][order]
    shift = np.stack([(c // 3 ** k) % 3 - 1 for k in range(d)], axis=1).astype(np.int8)
    out = dict(delta=dl, sig=psig, r=pr, offs=offs, nbr=nbr, shift=shift, nimages=len(img), ref=ref + 1, ref_shift=sh)
    if generic:
        out["sig_offs"] = psig_offs
    if integrate:
        vol, area = M.polygon()
        out["vol"] = vol[:n]
        out["area"] = area[:tot][order]
    return out
