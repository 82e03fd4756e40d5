"""Host-side mirror of HighVoronoi.jl's user API for the GPU path.

    VoronoiGeometry(xs, cuboid(d, periodic=[]); search_settings=dict(method=RCGPU),
                    integrator=VI_POLYGON)           src/geometry.jl:139-201
    VoronoiData(geometry)                            src/voronoidata.jl:545-700
    cuboid(dim; dimensions, periodic, offset)        src/boundary.jl:518-534

The names, argument meanings and conventions (1-based generators, boundary
plane p as generator N+p, sorted signatures, neighbour lists with the planes
last) are the reference's.  Every computation runs in libhvgpu.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass
class Boundary:
    """Axis-aligned box [offset, offset + dimensions] with Dirichlet planes."""
    lo: np.ndarray
    hi: np.ndarray
    periodic: list = field(default_factory=list)

    @property
    def dim(self) -> int:
        return int(self.lo.shape[0])

    @property
    def nplanes(self) -> int:
        return 2 * self.dim


def cuboid(dim: int, dimensions=None, periodic=None, neumann=(), offset=None) -> Boundary:
    """The reference's cuboid (src/boundary.jl:518-534).  Its default is fully
    periodic (periodic=1:dim); only non-periodic boxes run on the GPU path, so
    pass ``periodic=[]`` as the reference's own tests and benchmarks do
    (test/rcmethods.jl:4, src/statistics.jl:107).  Plane 2k-1 is the upper face
    of axis k and plane 2k the lower face, as in the reference."""
    dims = np.ones(dim) if dimensions is None else np.asarray(dimensions, dtype=np.float64)
    off = np.zeros(dim) if offset is None else np.asarray(offset, dtype=np.float64)
    per = list(range(1, dim + 1)) if periodic is None else list(periodic)
    if per:
        raise NotImplementedError("periodic boundaries are not part of the GPU mesh path; use periodic=[]")
    # Neumann and Dirichlet planes give the same mesh; the flag only matters to the FV layer.
    del neumann
    return Boundary(lo=off.copy(), hi=off + dims, periodic=per)


@dataclass(frozen=True)
class RaycastMethod:
    name: str
    code: int

    def __repr__(self):
        return self.name


# Beside the reference's RCOriginal / RCNonGeneral / RCCombined (src/raycast-types.jl:244-285).
RCGPU = RaycastMethod("RCGPU", _lib.HV_METHOD_FAST)
RCGPUPlain = RaycastMethod("RCGPUPlain", _lib.HV_METHOD_PLAIN)

VI_GEOMETRY = "VI_GEOMETRY"
VI_POLYGON = "VI_POLYGON"
# The reference's memoised exact integrator (src/fastpolyintegrator.jl:4-476): the same cell
# volumes and interface areas as VI_POLYGON, which the GPU computes the same way for both.
VI_FAST_POLYGON = "VI_FAST_POLYGON"
VI_HEURISTIC_MC = "VI_HEURISTIC_MC"


class VoronoiGeometry:
    """Vertex search (and optionally integration) of the Voronoi mesh of ``xs``.

    ``xs`` is an (n, d) array (row i = generator i+1) or a list of points.
    ``search_settings`` accepts ``method`` (RCGPU default, RCGPUPlain), the
    GPU knobs ``knn``, ``leaf_size``, ``seed_stride``, ``edge_dedup``,
    ``capacity_factor``, ``seed``, and ``autotune=True`` (tune the knobs for
    this (d, n) once per context).  ``mc_accurate=(ndir, 1, recycle)`` sets the
    directions per cell of VI_HEURISTIC_MC (src/geometry.jl:70-72).
    """

    def __init__(self, xs, b: Boundary | None = None, *, search_settings=None, integrator=VI_GEOMETRY,
                 mc_accurate=(1000, 1, 20), mc_seed: int = 0, context: _lib.Context | None = None,
                 silence: bool = True):
        pts = np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
        if pts.ndim != 2:
            raise ValueError("xs must be an (n, d) array")
        n, d = pts.shape
        if b is None:
            raise ValueError("a bounded domain is required: pass cuboid(d, periodic=[])")
        if b.dim != d:
            raise ValueError("dimension of the boundary and of the points differ")
        ss = dict(search_settings or {})
        method = ss.pop("method", RCGPU)
        if not isinstance(method, RaycastMethod):
            raise ValueError(f"unsupported raycast method {method!r} on the GPU path")
        autotune = bool(ss.pop("autotune", False))
        allowed = {"knn", "leaf_size", "seed_stride", "edge_dedup", "capacity_factor", "seed", "rays_per_warp"}
        unknown = set(ss) - allowed
        if unknown:
            raise ValueError(f"unknown search settings {sorted(unknown)}")
        self.ctx = context or _lib.default_context()
        self.boundary = b
        self.nodes = pts
        self.method = method
        if autotune and method.code == _lib.HV_METHOD_FAST:
            # tuned on synthetic points of the same (d, n); cached in the context
            self.ctx.autotune(d, n, lo=b.lo, hi=b.hi)
        self.params = _lib.make_params(method.code, **ss)
        self.mesh = _lib.Mesh(self.ctx, pts, b.lo, b.hi, self.params)
        self.integrator = integrator
        self._volumes = None
        self._areas = None
        if integrator in (VI_POLYGON, VI_FAST_POLYGON):
            self._volumes, self._areas = self.mesh.polygon()
        elif integrator == VI_HEURISTIC_MC:
            self._volumes, self._areas = self.mesh.heuristic_mc(int(mc_accurate[0]), int(mc_seed))
        elif integrator != VI_GEOMETRY:
            raise ValueError(f"unsupported integrator {integrator!r} on the GPU path")
        if not silence:
            print(f"VoronoiGeometry: {self.mesh.stats()['vertices']} vertices")

    @property
    def dimension(self) -> int:
        return self.nodes.shape[1]

    def stats(self) -> dict:
        return self.mesh.stats()


class VoronoiData:
    """Read view of a VoronoiGeometry (src/voronoidata.jl:545-700).

    ``vertices``: (V, d+1) sorted 1-based signatures and (V, d) coordinates;
    ``neighbors[i]``: sorted 1-based neighbours of generator i+1 (planes as
    N+p); ``volume[i]`` and ``area[i]`` (aligned with ``neighbors[i]``) when the
    geometry was integrated.
    """

    def __init__(self, geo: VoronoiGeometry):
        self.nodes = geo.nodes
        self.boundary = geo.boundary
        self.vertex_sigs, self.vertex_coords = geo.mesh.vertices()
        offs, nbr = geo.mesh.neighbors()
        self.neighbor_offsets = offs
        self.neighbor_flat = nbr
        self.neighbors = [nbr[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
        self.volume = geo._volumes
        self.area = None
        if geo._areas is not None:
            self.area = [geo._areas[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]

    @property
    def vertices(self):
        return self.vertex_sigs, self.vertex_coords
