"""ctypes binding of libhvgpu (include/hvgpu.h).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "_build", "libhvgpu.so")

HV_OK = 0
HV_E_INVALID_ARG = -1
HV_E_OOM = -2
HV_E_CAPACITY = -3
HV_E_DEGENERATE = -4
HV_E_TIMEOUT = -5
HV_E_CUDA = -6
HV_E_INTERNAL = -7
HV_METHOD_FAST = 0
HV_METHOD_PLAIN = 1
HV_METHOD_GENERIC = 2  # vertices of any number of generators (lattices)

_ERRNAMES = {
    HV_E_INVALID_ARG: "HV_E_INVALID_ARG", HV_E_OOM: "HV_E_OOM", HV_E_CAPACITY: "HV_E_CAPACITY",
    HV_E_DEGENERATE: "HV_E_DEGENERATE", HV_E_TIMEOUT: "HV_E_TIMEOUT", HV_E_CUDA: "HV_E_CUDA",
    HV_E_INTERNAL: "HV_E_INTERNAL",
}


class HVError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("knn", ctypes.c_int), ("leaf_size", ctypes.c_int),
                ("rays_per_warp", ctypes.c_int), ("seed_stride", ctypes.c_int), ("edge_dedup", ctypes.c_int),
                ("seed", ctypes.c_uint64), ("capacity_factor", ctypes.c_double)]


STAT_FIELDS = ("vertices", "rays", "fallback_rays", "uncertified", "insecure", "dd_rescores", "degenerate",
               "descents", "descent_retries", "levels", "edges_closed", "capacity_retries", "launches")
TIME_FIELDS = ("ms_prepare", "ms_search", "ms_total", "ms_knn", "ms_descent", "ms_expand", "ms_fallback",
               "ms_centers", "ms_canonical")
POLY_FIELDS = ("ms_poly_incidence", "ms_poly_facets", "ms_poly_big", "ms_poly_total")
FALLBACK_FIELDS = ("fallback_tree_rays", "fallback_nodes", "fallback_leaves", "fallback_points", "ambiguous_sets")
LATTICE_FIELDS = ("poly_faces", "poly_terms", "poly_term_flops")


class Stats(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int64) for n in STAT_FIELDS] + [(n, ctypes.c_double) for n in TIME_FIELDS] +
                [("poly_big_facets", ctypes.c_int64)] + [(n, ctypes.c_double) for n in POLY_FIELDS] +
                [(n, ctypes.c_int64) for n in FALLBACK_FIELDS] + [(n, ctypes.c_int64) for n in LATTICE_FIELDS])


class DeviceViews(ctypes.Structure):
    """hv_device_views: device pointers into a mesh's own arrays."""
    _fields_ = [("d", ctypes.c_int), ("n", ctypes.c_int64), ("nverts", ctypes.c_int64), ("nnbr", ctypes.c_int64),
                ("ncell_vertices", ctypes.c_int64), ("sig", ctypes.c_void_p), ("r", ctypes.c_void_p),
                ("nbr_off", ctypes.c_void_p), ("nbr", ctypes.c_void_p), ("vtx_off", ctypes.c_void_p),
                ("vtx", ctypes.c_void_p), ("pts", ctypes.c_void_p), ("stream", ctypes.c_void_p)]


class CudaArray:
    """A device array exposing ``__cuda_array_interface__`` (v3), so
    torch.as_tensor / CuPy / Numba view it without a copy.  It keeps the owning
    mesh alive.  The memory is the mesh's own: read it, do not write it (the
    interface's read-only flag stays False because torch rejects it)."""

    def __init__(self, ptr: int, shape, typestr: str, owner, stream: int | None = None):
        self.ptr, self.shape, self.typestr, self.owner = int(ptr or 0), tuple(int(x) for x in shape), typestr, owner
        self.stream = stream

    @property
    def __cuda_array_interface__(self):
        iface = {"shape": self.shape, "typestr": self.typestr, "data": (self.ptr, False), "version": 3,
                 "strides": None}
        if self.stream:
            iface["stream"] = int(self.stream)
        return iface


_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Loads libhvgpu.so from the package's build folder (raises if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise HVError(HV_E_INTERNAL, f"libhvgpu.so not built ({p}); run highvoronoi.jl_gb300/build.py")
        L = ctypes.CDLL(p)
        I, I64, U64, P = ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int64)
        L.hv_version.argtypes = []; L.hv_version.restype = I
        L.hv_params_default.argtypes = [ctypes.POINTER(Params)]; L.hv_params_default.restype = None
        L.hv_ctx_create.argtypes = [I, ctypes.POINTER(P)]; L.hv_ctx_create.restype = I
        L.hv_ctx_destroy.argtypes = [P]; L.hv_ctx_destroy.restype = I
        L.hv_last_error.argtypes = [P]; L.hv_last_error.restype = ctypes.c_char_p
        L.hv_ctx_stream.argtypes = [P]; L.hv_ctx_stream.restype = P
        L.hv_mesh_build.argtypes = [P, I, I64, P, dp, dp, ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.hv_mesh_build.restype = I
        L.hv_mesh_build_device.argtypes = [P, I, I64, P, dp, dp, ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.hv_mesh_build_device.restype = I
        i16p = ctypes.POINTER(ctypes.c_int16)
        L.hv_mesh_build_planes.argtypes = [P, I, I64, P, I, dp, dp, i16p, ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.hv_mesh_build_planes.restype = I
        L.hv_mesh_build_planes_device.argtypes = [P, I, I64, P, I, dp, dp, i16p, ctypes.POINTER(Params),
                                                  ctypes.POINTER(P)]
        L.hv_mesh_build_planes_device.restype = I
        L.hv_mesh_counts.argtypes = [P, ip, ip]; L.hv_mesh_counts.restype = I
        L.hv_autotune.argtypes = [P, I, I64, P, dp, dp, ctypes.POINTER(Params)]; L.hv_autotune.restype = I
        L.hv_mesh_vertices.argtypes = [P, ip, dp]; L.hv_mesh_vertices.restype = I
        L.hv_mesh_signature_total.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int)]
        L.hv_mesh_signature_total.restype = I
        L.hv_mesh_vertices_csr.argtypes = [P, ip, ip, dp]; L.hv_mesh_vertices_csr.restype = I
        L.hv_mesh_verify.argtypes = [P, ip, ip, dp]; L.hv_mesh_verify.restype = I
        L.hv_mesh_neighbors.argtypes = [P, ip, ip]; L.hv_mesh_neighbors.restype = I
        L.hv_integrate_polygon.argtypes = [P, dp, dp]; L.hv_integrate_polygon.restype = I
        L.hv_integrate_heuristic_mc.argtypes = [P, I, U64, dp, dp]; L.hv_integrate_heuristic_mc.restype = I
        L.hv_mesh_stats.argtypes = [P, ctypes.POINTER(Stats)]; L.hv_mesh_stats.restype = I
        L.hv_mesh_free.argtypes = [P]; L.hv_mesh_free.restype = I
        L.hv_mesh_cell_vertices.argtypes = [P, ip, ip]; L.hv_mesh_cell_vertices.restype = I
        i32p = ctypes.POINTER(ctypes.c_int32)
        i8p = ctypes.POINTER(ctypes.c_int8)
        L.hv_mesh_build_periodic.argtypes = [P, I, I64, P, dp, dp, i32p, ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.hv_mesh_build_periodic.restype = I
        L.hv_mesh_build_periodic_device.argtypes = [P, I, I64, P, dp, dp, i32p, ctypes.POINTER(Params),
                                                    ctypes.POINTER(P)]
        L.hv_mesh_build_periodic_device.restype = I
        L.hv_mesh_facet_centers.argtypes = [P, dp]; L.hv_mesh_facet_centers.restype = I
        L.hv_integrate_polygon_functions.argtypes = [P, I, dp, dp, dp, dp, dp]
        L.hv_integrate_polygon_functions.restype = I
        L.hv_integrate_heuristic_functions.argtypes = [P, I, dp, dp, dp, dp, dp, dp]
        L.hv_integrate_heuristic_functions.restype = I
        L.hv_mesh_refine.argtypes = [P, I64, P, ctypes.POINTER(P)]; L.hv_mesh_refine.restype = I
        L.hv_mesh_refine_device.argtypes = [P, I64, P, ctypes.POINTER(P)]; L.hv_mesh_refine_device.restype = I
        L.hv_mesh_build_shard.argtypes = [P, I, I64, P, dp, dp, I, I, ctypes.POINTER(Params), ctypes.POINTER(P)]
        L.hv_mesh_build_shard.restype = I
        L.hv_mesh_build_shard_device.argtypes = [P, I, I64, P, dp, dp, I, I, ctypes.POINTER(Params),
                                                 ctypes.POINTER(P)]
        L.hv_mesh_build_shard_device.restype = I
        L.hv_mesh_periodic_shifts.argtypes = [P, i8p]; L.hv_mesh_periodic_shifts.restype = I
        L.hv_mesh_periodic_images.argtypes = [P, ip, dp, ip, i8p]; L.hv_mesh_periodic_images.restype = I
        L.hv_mesh_device_views.argtypes = [P, ctypes.POINTER(DeviceViews)]; L.hv_mesh_device_views.restype = I
        L.hv_integrate_polygon_device.argtypes = [P, P, P]; L.hv_integrate_polygon_device.restype = I
        L.hv_integrate_heuristic_mc_device.argtypes = [P, I, U64, P, P]
        L.hv_integrate_heuristic_mc_device.restype = I
        L.hv_integrate_heuristic_mc_noalloc.argtypes = [I, I64, P, dp, dp, P, P, I64, I, I, U64, P, P, P]
        L.hv_integrate_heuristic_mc_noalloc.restype = I
        _lib = L
        return L


def dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def heuristic_mc_noalloc(d, n, d_pts, lo, hi, d_nbr_off, d_nbr, nnbr, max_degree, ndir, seed, d_vol, d_area,
                        stream=0):
    """hv_integrate_heuristic_mc_noalloc on caller-owned device buffers (raw
    pointers); raises HVError on a non-zero return code."""
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    rc = load().hv_integrate_heuristic_mc_noalloc(d, n, d_pts, dptr(lo), dptr(hi), d_nbr_off, d_nbr, nnbr,
                                                  max_degree, ndir, seed, d_vol, d_area, stream)
    if rc != HV_OK:
        msg = {HV_E_CAPACITY: "1536 bytes + 2n + nnbr doubles exceed the static scratch",
               HV_E_INVALID_ARG: "invalid argument, a row longer than max_degree, an item outside "
                                 "0..n+2d-1, or a neighbour relation that is not symmetric"}.get(rc, "CUDA error")
        raise HVError(rc, "hv_integrate_heuristic_mc_noalloc: " + msg)


class Context:
    """One CUDA device + one stream (hv_ctx)."""

    def __init__(self, device: int = 0):
        L = load()
        h = ctypes.c_void_p()
        rc = L.hv_ctx_create(device, ctypes.byref(h))
        if rc != HV_OK:
            raise HVError(rc, f"hv_ctx_create(device={device}) failed: no usable CUDA device")
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def stream(self) -> int:
        """cudaStream_t of this context (as an integer handle)."""
        return load().hv_ctx_stream(self._h) or 0

    def error(self) -> str:
        return load().hv_last_error(self._h).decode()

    def autotune(self, d: int, n: int, pts=None, lo=None, hi=None) -> dict:
        """Runs hv_autotune; the winner is cached in this context per (d, log2 n)."""
        lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
        hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
        p = Params()
        ptr = None
        if pts is not None:
            pts = np.ascontiguousarray(pts, dtype=np.float64)
            ptr = pts.ctypes.data_as(ctypes.c_void_p)
        self.check(load().hv_autotune(self._h, d, n, ptr, dptr(lo), dptr(hi), ctypes.byref(p)), "hv_autotune")
        return {k: getattr(p, k) for k, _ in Params._fields_}

    def check(self, rc: int, what: str):
        if rc != HV_OK:
            raise HVError(rc, f"{what}: {self.error()}")

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().hv_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("HV_DEVICE", "0")))
    return _default_ctx


def make_params(method: int = HV_METHOD_FAST, **kw) -> Params:
    p = Params()
    load().hv_params_default(ctypes.byref(p))
    p.method = method
    for k, v in kw.items():
        if v is not None:
            setattr(p, k, v)
    return p


class Mesh:
    """A mesh built on the device (hv_mesh).  Results are copied out on demand."""

    def __init__(self, ctx: Context, pts: np.ndarray, lo, hi, params: Params, device_ptr: int | None = None,
                 planes=None, periodic=None, shard=None):
        """Box domain [lo, hi] (``periodic``: d flags of periodic axes), or
        (lo = hi = None) the convex domain of ``planes = (base, normal, bc)``:
        (P, d) base points, (P, d) outer normals and P boundary-condition codes
        (or None).  ``shard = (rank, nranks)``: one shard of the box mesh
        split over ranks (hv_mesh_build_shard; merge with hvgpu.shard)."""
        L = load()
        self.ctx = ctx
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.n, self.d = pts.shape if device_ptr is None else (int(pts[0]), int(pts[1]))
        self._pts = pts if device_ptr is None else None
        h = ctypes.c_void_p()
        self.periodic = None
        if shard is not None:
            self.planes = None
            self.lo = np.ascontiguousarray(lo, dtype=np.float64)
            self.hi = np.ascontiguousarray(hi, dtype=np.float64)
            rank, nranks = int(shard[0]), int(shard[1])
            if device_ptr is None:
                rc = L.hv_mesh_build_shard(ctx.handle, self.d, self.n, pts.ctypes.data_as(ctypes.c_void_p),
                                           dptr(self.lo), dptr(self.hi), rank, nranks, ctypes.byref(params),
                                           ctypes.byref(h))
            else:
                rc = L.hv_mesh_build_shard_device(ctx.handle, self.d, self.n, ctypes.c_void_p(device_ptr),
                                                  dptr(self.lo), dptr(self.hi), rank, nranks, ctypes.byref(params),
                                                  ctypes.byref(h))
            ctx.check(rc, "hv_mesh_build_shard")
            self._h = h
            return
        if periodic is not None and any(periodic):
            flags = np.ascontiguousarray([1 if f else 0 for f in periodic], dtype=np.int32)
            if flags.shape[0] != self.d:
                raise ValueError("periodic needs one flag per axis")
            self.periodic = flags.astype(bool)
            self.lo = np.ascontiguousarray(lo, dtype=np.float64)
            self.hi = np.ascontiguousarray(hi, dtype=np.float64)
            self.planes = None
            fp = flags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            if device_ptr is None:
                rc = L.hv_mesh_build_periodic(ctx.handle, self.d, self.n, pts.ctypes.data_as(ctypes.c_void_p),
                                              dptr(self.lo), dptr(self.hi), fp, ctypes.byref(params), ctypes.byref(h))
            else:
                rc = L.hv_mesh_build_periodic_device(ctx.handle, self.d, self.n, ctypes.c_void_p(device_ptr),
                                                     dptr(self.lo), dptr(self.hi), fp, ctypes.byref(params),
                                                     ctypes.byref(h))
            ctx.check(rc, "hv_mesh_build_periodic")
            self._h = h
            return
        if planes is not None:
            base = np.ascontiguousarray(planes[0], dtype=np.float64)
            normal = np.ascontiguousarray(planes[1], dtype=np.float64)
            if base.shape != normal.shape or base.ndim != 2 or base.shape[1] != self.d:
                raise ValueError("plane bases and normals must be (P, d) arrays")
            bc = None if planes[2] is None else np.ascontiguousarray(planes[2], dtype=np.int16)
            bcp = None if bc is None else bc.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
            self.lo = self.hi = None
            self.planes = (base, normal, bc)
            if device_ptr is None:
                rc = L.hv_mesh_build_planes(ctx.handle, self.d, self.n, pts.ctypes.data_as(ctypes.c_void_p),
                                            base.shape[0], dptr(base), dptr(normal), bcp, ctypes.byref(params),
                                            ctypes.byref(h))
            else:
                rc = L.hv_mesh_build_planes_device(ctx.handle, self.d, self.n, ctypes.c_void_p(device_ptr),
                                                   base.shape[0], dptr(base), dptr(normal), bcp,
                                                   ctypes.byref(params), ctypes.byref(h))
            ctx.check(rc, "hv_mesh_build_planes")
            self._h = h
            return
        self.planes = None
        self.lo = np.ascontiguousarray(lo, dtype=np.float64)
        self.hi = np.ascontiguousarray(hi, dtype=np.float64)
        if device_ptr is None:
            rc = L.hv_mesh_build(ctx.handle, self.d, self.n, pts.ctypes.data_as(ctypes.c_void_p), dptr(self.lo),
                                 dptr(self.hi), ctypes.byref(params), ctypes.byref(h))
        else:
            rc = L.hv_mesh_build_device(ctx.handle, self.d, self.n, ctypes.c_void_p(device_ptr), dptr(self.lo),
                                        dptr(self.hi), ctypes.byref(params), ctypes.byref(h))
        ctx.check(rc, "hv_mesh_build")
        self._h = h

    def refined(self, xs) -> "Mesh":
        """hv_mesh_refine: a new mesh of this mesh's generators plus the rows of
        ``xs`` (numbered after them), searching only the new generators' cells.
        This mesh stays valid."""
        xs = np.ascontiguousarray(np.asarray(xs, dtype=np.float64).reshape(-1, self.d))
        h = ctypes.c_void_p()
        rc = load().hv_mesh_refine(self._h, xs.shape[0], xs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        self.ctx.check(rc, "hv_mesh_refine")
        m = Mesh.__new__(Mesh)
        m.ctx, m.n, m.d, m.periodic, m.planes = self.ctx, self.n + xs.shape[0], self.d, None, self.planes
        m.lo, m.hi = self.lo, self.hi
        m._pts = None if getattr(self, "_pts", None) is None else np.vstack([self._pts, xs])
        m._h = h
        return m

    def counts(self, neighbors: bool = False):
        nv = ctypes.c_int64()
        nn = ctypes.c_int64()
        rc = load().hv_mesh_counts(self._h, ctypes.byref(nv), ctypes.byref(nn) if neighbors else None)
        self.ctx.check(rc, "hv_mesh_counts")
        return nv.value, (nn.value if neighbors else None)

    def vertices(self):
        V, _ = self.counts()
        sig = np.zeros((V, self.d + 1), dtype=np.int64)
        r = np.zeros((V, self.d), dtype=np.float64)
        self.ctx.check(load().hv_mesh_vertices(self._h, iptr(sig), dptr(r)), "hv_mesh_vertices")
        return sig, r

    def vertices_csr(self):
        """(offs (V+1), sig (1-based, ascending per vertex, back to back),
        r (V, d)): vertices of any number of generators -- a lattice puts 2^d
        points on one sphere -- in lexicographic order of their signatures."""
        V, _ = self.counts()
        tot = ctypes.c_int64()
        mx = ctypes.c_int()
        self.ctx.check(load().hv_mesh_signature_total(self._h, ctypes.byref(tot), ctypes.byref(mx)),
                       "hv_mesh_signature_total")
        offs = np.zeros(V + 1, dtype=np.int64)
        sig = np.zeros(max(tot.value, 1), dtype=np.int64)
        r = np.zeros((V, self.d), dtype=np.float64)
        self.ctx.check(load().hv_mesh_vertices_csr(self._h, iptr(offs), iptr(sig), dptr(r)), "hv_mesh_vertices_csr")
        return offs, sig[:tot.value], r

    def verify(self) -> dict:
        """The device check of the reference's verify_vertex: vertices with a
        generator strictly inside their sphere (``inside``, 0 for a correct
        mesh), with another generator on it (``ties``), and the largest relative
        deviation of a vertex's own generators from its sphere (``max_dev``)."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        dv = ctypes.c_double()
        self.ctx.check(load().hv_mesh_verify(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(dv)),
                       "hv_mesh_verify")
        return {"inside": a.value, "ties": b.value, "max_dev": dv.value}

    def max_signature(self) -> int:
        """Longest vertex signature (d+1 unless generators are co-spherical)."""
        tot = ctypes.c_int64()
        mx = ctypes.c_int()
        self.ctx.check(load().hv_mesh_signature_total(self._h, ctypes.byref(tot), ctypes.byref(mx)),
                       "hv_mesh_signature_total")
        return mx.value

    def neighbors(self):
        _, E = self.counts(neighbors=True)
        offs = np.zeros(self.n + 1, dtype=np.int64)
        nbr = np.zeros(max(E, 1), dtype=np.int64)
        self.ctx.check(load().hv_mesh_neighbors(self._h, iptr(offs), iptr(nbr)), "hv_mesh_neighbors")
        return offs, nbr[:E]

    def polygon(self):
        _, E = self.counts(neighbors=True)
        vol = np.zeros(self.n)
        area = np.zeros(max(E, 1))
        self.ctx.check(load().hv_integrate_polygon(self._h, dptr(vol), dptr(area)), "hv_integrate_polygon")
        return vol, area[:E]

    def facet_centers(self) -> np.ndarray:
        """(nnbr, d) centres of the facets (mean of their vertices), aligned
        with neighbors(): the facet nodes of the integrand quadrature."""
        _, E = self.counts(neighbors=True)
        c = np.zeros((max(E, 1), self.d))
        self.ctx.check(load().hv_mesh_facet_centers(self._h, dptr(c)), "hv_mesh_facet_centers")
        return c[:E]

    def polygon_functions(self, fv, fc, fx, bulk: bool = True):
        """Interface (nnbr, p) and cell (n, p) integrals of a function given by
        its values at the vertices (fv, rows of vertices()), the facet centres
        (fc) and the generators (fx)."""
        V, E = self.counts(neighbors=True)
        fv = np.ascontiguousarray(np.asarray(fv, dtype=np.float64).reshape(V, -1))
        p = fv.shape[1]
        fc = np.ascontiguousarray(np.asarray(fc, dtype=np.float64).reshape(E, p))
        fx = np.ascontiguousarray(np.asarray(fx, dtype=np.float64).reshape(self.n, p))
        iface = np.zeros((max(E, 1), p))
        blk = np.zeros((self.n, p)) if bulk else None
        rc = load().hv_integrate_polygon_functions(self._h, p, dptr(fv), dptr(fc), dptr(fx), dptr(iface),
                                                    dptr(blk) if bulk else None)
        self.ctx.check(rc, "hv_integrate_polygon_functions")
        return iface[:E], blk

    def heuristic_functions(self, area, fv, fc, fx, bulk: bool = True):
        """The reference's heuristic integrand rule (hv_integrate_heuristic_functions)
        on the interface areas ``area`` (e.g. from heuristic_mc)."""
        V, E = self.counts(neighbors=True)
        fv = np.ascontiguousarray(np.asarray(fv, dtype=np.float64).reshape(V, -1))
        p = fv.shape[1]
        fc = np.ascontiguousarray(np.asarray(fc, dtype=np.float64).reshape(E, p))
        fx = np.ascontiguousarray(np.asarray(fx, dtype=np.float64).reshape(self.n, p))
        area = np.ascontiguousarray(np.asarray(area, dtype=np.float64).reshape(E))
        iface = np.zeros((max(E, 1), p))
        blk = np.zeros((self.n, p)) if bulk else None
        rc = load().hv_integrate_heuristic_functions(self._h, p, dptr(area), dptr(fv), dptr(fc), dptr(fx),
                                                      dptr(iface), dptr(blk) if bulk else None)
        self.ctx.check(rc, "hv_integrate_heuristic_functions")
        return iface[:E], blk

    def integrate_function(self, f, bulk: bool = True, heuristic_area=None):
        """Evaluates ``f`` ((m, d) points -> (m,) or (m, p) values) at the
        quadrature nodes and returns the interface and cell integrals: the
        polygon rule, or with ``heuristic_area`` (the interface areas of the
        Monte-Carlo integrator) the heuristic rule."""
        _, r = self.vertices()
        c = self.facet_centers()
        x = self.points()

        def ev(P):
            y = np.asarray(f(P), dtype=np.float64)
            return y.reshape(len(P), -1)
        if heuristic_area is not None:
            return self.heuristic_functions(heuristic_area, ev(r), ev(c), ev(x), bulk)
        return self.polygon_functions(ev(r), ev(c), ev(x), bulk)

    def points(self) -> np.ndarray:
        """(n, d) generators in their original order (meshes built from host points)."""
        pts = getattr(self, "_pts", None)
        if pts is None:
            raise HVError(HV_E_INVALID_ARG, "the generators of a mesh built from device memory stay on the device")
        return pts

    def heuristic_mc(self, ndir: int, seed: int):
        _, E = self.counts(neighbors=True)
        vol = np.zeros(self.n)
        area = np.zeros(max(E, 1))
        rc = load().hv_integrate_heuristic_mc(self._h, ndir, seed, dptr(vol), dptr(area))
        self.ctx.check(rc, "hv_integrate_heuristic_mc")
        return vol, area[:E]

    def periodic_shifts(self) -> np.ndarray:
        """(nnbr, d) lattice shifts of the neighbour entries (zeros unless periodic)."""
        _, E = self.counts(neighbors=True)
        out = np.zeros((max(E, 1), self.d), dtype=np.int8)
        rc = load().hv_mesh_periodic_shifts(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int8)))
        self.ctx.check(rc, "hv_mesh_periodic_shifts")
        return out[:E]

    def periodic_images(self):
        """(margin delta (d), 1-based originals, (nimg, d) lattice shifts) of the images."""
        L = load()
        ni = ctypes.c_int64()
        delta = np.zeros(self.d)
        self.ctx.check(L.hv_mesh_periodic_images(self._h, ctypes.byref(ni), dptr(delta), None, None),
                       "hv_mesh_periodic_images")
        ref = np.zeros(max(ni.value, 1), dtype=np.int64)
        sh = np.zeros((max(ni.value, 1), self.d), dtype=np.int8)
        self.ctx.check(L.hv_mesh_periodic_images(self._h, ctypes.byref(ni), dptr(delta), iptr(ref),
                                                 sh.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))),
                       "hv_mesh_periodic_images")
        return delta, ref[:ni.value], sh[:ni.value]

    def cell_vertices(self):
        """(offs (n+1), 1-based vertex rows) of every cell, ascending."""
        offs = np.zeros(self.n + 1, dtype=np.int64)
        L = load()
        self.ctx.check(L.hv_mesh_cell_vertices(self._h, iptr(offs), None), "hv_mesh_cell_vertices")
        vtx = np.zeros(max(int(offs[-1]), 1), dtype=np.int64)
        self.ctx.check(L.hv_mesh_cell_vertices(self._h, iptr(offs), iptr(vtx)), "hv_mesh_cell_vertices")
        return offs, vtx[:int(offs[-1])]

    def device_views(self) -> dict:
        """Zero-copy device arrays of the mesh (0-based ids, planes n+p):
        sig, r, nbr_off, nbr, vtx_off, vtx, pts."""
        v = DeviceViews()
        self.ctx.check(load().hv_mesh_device_views(self._h, ctypes.byref(v)), "hv_mesh_device_views")
        d, st = v.d, v.stream
        return {
            "sig": CudaArray(v.sig, (v.nverts, d + 1), "<i4", self, st),
            "r": CudaArray(v.r, (v.nverts, d), "<f8", self, st),
            "nbr_off": CudaArray(v.nbr_off, (v.n + 1,), "<i8", self, st),
            "nbr": CudaArray(v.nbr, (v.nnbr,), "<i4", self, st),
            "vtx_off": CudaArray(v.vtx_off, (v.n + 1,), "<i8", self, st),
            "vtx": CudaArray(v.vtx, (v.ncell_vertices,), "<i4", self, st),
            "pts": CudaArray(v.pts, (v.n, d), "<f8", self, st),
        }

    def polygon_device(self, d_vol: int, d_area: int):
        """VI_POLYGON into caller device buffers (n and nnbr doubles)."""
        self.ctx.check(load().hv_integrate_polygon_device(self._h, ctypes.c_void_p(d_vol), ctypes.c_void_p(d_area)),
                       "hv_integrate_polygon_device")

    def heuristic_mc_device(self, ndir: int, seed: int, d_vol: int, d_area: int):
        rc = load().hv_integrate_heuristic_mc_device(self._h, ndir, seed, ctypes.c_void_p(d_vol),
                                                     ctypes.c_void_p(d_area))
        self.ctx.check(rc, "hv_integrate_heuristic_mc_device")

    def stats(self) -> dict:
        s = Stats()
        self.ctx.check(load().hv_mesh_stats(self._h, ctypes.byref(s)), "hv_mesh_stats")
        return {n: getattr(s, n) for n, _ in Stats._fields_}

    def free(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().hv_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
