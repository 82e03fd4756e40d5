"""Serving loop binding (hv_server_* in include/hvgpu.h).

The server keeps `slots` contexts (one CUDA stream + one worker thread each)
and admits queued mesh requests in arrival order as soon as a slot is idle and
the request's HBM estimate fits next to the running ones; their kernels overlap
on the device.  Results are pure functions of their request.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

INTEGRATORS = {None: 0, "none": 0, "polygon": 1, "heuristic_mc": 2}


class _Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("slots", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double)]


class _Request(ctypes.Structure):
    _fields_ = [("d", ctypes.c_int), ("n", ctypes.c_int64), ("pts", ctypes.c_void_p), ("lo", ctypes.c_void_p),
                ("hi", ctypes.c_void_p), ("integrator", ctypes.c_int), ("ndir", ctypes.c_int),
                ("mc_seed", ctypes.c_uint64), ("params", _lib.Params), ("periodic", ctypes.c_void_p),
                ("nplanes", ctypes.c_int), ("base", ctypes.c_void_p), ("normal", ctypes.c_void_p),
                ("bc", ctypes.c_void_p)]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("d", ctypes.c_int), ("n", ctypes.c_int64), ("nverts", ctypes.c_int64),
                ("nnbr", ctypes.c_int64), ("sig", ctypes.POINTER(ctypes.c_int64)),
                ("r", ctypes.POINTER(ctypes.c_double)), ("offs", ctypes.POINTER(ctypes.c_int64)),
                ("nbr", ctypes.POINTER(ctypes.c_int64)), ("vol", ctypes.POINTER(ctypes.c_double)),
                ("area", ctypes.POINTER(ctypes.c_double)), ("queue_ms", ctypes.c_double),
                ("service_ms", ctypes.c_double), ("latency_ms", ctypes.c_double), ("stats", _lib.Stats),
                ("shift", ctypes.POINTER(ctypes.c_int8)), ("sig_offs", ctypes.POINTER(ctypes.c_int64))]


def _bind():
    L = _lib.load()
    if getattr(L, "_hv_server_bound", False):
        return L
    P = ctypes.c_void_p
    L.hv_server_start.argtypes = [ctypes.POINTER(_Config), ctypes.POINTER(P)]; L.hv_server_start.restype = ctypes.c_int
    L.hv_server_submit.argtypes = [P, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_int64)]
    L.hv_server_submit.restype = ctypes.c_int
    L.hv_server_poll.argtypes = [P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]; L.hv_server_poll.restype = ctypes.c_int
    L.hv_server_wait.argtypes = [P, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(_Result)]
    L.hv_server_wait.restype = ctypes.c_int
    L.hv_server_release.argtypes = [P, ctypes.c_int64]; L.hv_server_release.restype = ctypes.c_int
    L.hv_server_stop.argtypes = [P]; L.hv_server_stop.restype = ctypes.c_int
    L._hv_server_bound = True
    return L


def _arr(ptr, count, dtype):
    if count <= 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True)


class Server:
    def __init__(self, device: int = 0, slots: int = 4, hbm_budget_bytes: float = 0.0):
        L = _bind()
        cfg = _Config(device, slots, hbm_budget_bytes)
        h = ctypes.c_void_p()
        rc = L.hv_server_start(ctypes.byref(cfg), ctypes.byref(h))
        if rc != _lib.HV_OK:
            raise _lib.HVError(rc, "hv_server_start failed")
        self._h = h

    def submit(self, pts, lo=None, hi=None, integrator=None, ndir=1000, mc_seed=0, method=_lib.HV_METHOD_FAST,
               periodic=None, planes=None, **params) -> int:
        """Queues one mesh request: the box [lo, hi] (default unit cube), with
        ``periodic`` (d flags) the periodic cuboid, or with ``planes = (base,
        normal, bc)`` the convex domain of those planes.  The arrays are copied."""
        pts = np.ascontiguousarray(pts, dtype=np.float64)
        n, d = pts.shape
        lo = np.ascontiguousarray(np.zeros(d) if lo is None else lo, dtype=np.float64)
        hi = np.ascontiguousarray(np.ones(d) if hi is None else hi, dtype=np.float64)
        q = _Request(d, n, pts.ctypes.data, lo.ctypes.data, hi.ctypes.data, INTEGRATORS[integrator], ndir, mc_seed,
                     _lib.make_params(method, **params))
        keep = []
        if periodic is not None:
            flags = np.ascontiguousarray([1 if f else 0 for f in periodic], dtype=np.int32)
            keep.append(flags)
            q.periodic = flags.ctypes.data
        if planes is not None:
            base = np.ascontiguousarray(planes[0], dtype=np.float64)
            normal = np.ascontiguousarray(planes[1], dtype=np.float64)
            keep += [base, normal]
            q.nplanes, q.base, q.normal = base.shape[0], base.ctypes.data, normal.ctypes.data
            if len(planes) > 2 and planes[2] is not None:
                bc = np.ascontiguousarray(planes[2], dtype=np.int16)
                keep.append(bc)
                q.bc = bc.ctypes.data
        t = ctypes.c_int64()
        rc = _bind().hv_server_submit(self._h, ctypes.byref(q), ctypes.byref(t))
        if rc != _lib.HV_OK:
            raise _lib.HVError(rc, "hv_server_submit failed")
        return t.value

    def done(self, ticket: int) -> bool:
        flag = ctypes.c_int()
        rc = _bind().hv_server_poll(self._h, ticket, ctypes.byref(flag))
        if rc != _lib.HV_OK:
            raise _lib.HVError(rc, "hv_server_poll failed")
        return bool(flag.value)

    def result(self, ticket: int, timeout_ms: float = -1.0, release: bool = True) -> dict:
        L = _bind()
        r = _Result()
        rc = L.hv_server_wait(self._h, ticket, timeout_ms, ctypes.byref(r))
        if rc != _lib.HV_OK:
            raise _lib.HVError(rc, "hv_server_wait failed")
        d, n, V, E = r.d, r.n, r.nverts, r.nnbr
        out = {"status": r.status, "queue_ms": r.queue_ms, "service_ms": r.service_ms, "latency_ms": r.latency_ms}
        if r.status == _lib.HV_OK:
            if r.sig_offs:  # co-spherical generators: one array per vertex
                so = _arr(r.sig_offs, V + 1, np.int64)
                flat = _arr(r.sig, int(so[-1]), np.int64)
                sig = [flat[so[v]:so[v + 1]] for v in range(V)]
            else:
                sig = _arr(r.sig, V * (d + 1), np.int64).reshape(V, d + 1)
            out.update({
                "sig": sig,
                "r": _arr(r.r, V * d, np.float64).reshape(V, d),
                "offs": _arr(r.offs, n + 1, np.int64),
                "nbr": _arr(r.nbr, E, np.int64),
                "vol": _arr(r.vol, n, np.float64) if r.vol else None,
                "area": _arr(r.area, E, np.float64) if r.area else None,
                "stats": {k: getattr(r.stats, k) for k, _ in _lib.Stats._fields_},
                "shift": _arr(r.shift, E * d, np.int8).reshape(E, d) if r.shift else None,
            })
        if release:
            L.hv_server_release(self._h, ticket)
        return out

    def stop(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _bind().hv_server_stop(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
