"""Host-side mirror of HighVoronoi.jl's user API for the GPU path.

    VoronoiGeometry(xs, cuboid(d, periodic=[]); search_settings=dict(method=RCGPU),
                    integrator=VI_POLYGON)           src/geometry.jl:139-201
    VoronoiData(geometry)                            src/voronoidata.jl:545-700
    cuboid(dim; dimensions, periodic, offset)        src/boundary.jl:510-534
    Boundary(planes...), BC_Dirichlet, BC_Neumann    src/boundary.jl:22-45,94-131

The names, argument meanings and conventions (1-based generators, boundary
plane p as generator N+p, sorted signatures, neighbour lists with the planes
last) are the reference's.  Every computation runs in libhvgpu.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _lib


# Boundary-condition codes of a plane (src/boundary.jl:2-3); a positive code
# names the periodic partner plane.
Dirichlet = 0
Neumann = -1


@dataclass
class Plane:
    """A boundary plane through ``base`` with outer normal ``normal``
    (src/boundary.jl:22-29); the domain side is (x - base) . normal < 0."""
    base: np.ndarray
    normal: np.ndarray
    BC: int = Dirichlet


def BC_Dirichlet(b, n) -> Plane:
    return Plane(np.asarray(b, dtype=np.float64), np.asarray(n, dtype=np.float64), Dirichlet)


def BC_Neumann(b, n) -> Plane:
    return Plane(np.asarray(b, dtype=np.float64), np.asarray(n, dtype=np.float64), Neumann)


def BC_Periodic(base1, base2, normal1):
    """Periodic plane pairs (src/boundary.jl:47-57) run on the GPU path only as
    the faces of a periodic cuboid: use ``cuboid(d, periodic=[...])``."""
    raise NotImplementedError("periodic planes are supported as cuboid(d, periodic=[...]) faces")


class Boundary:
    """A convex domain: the intersection of the half-spaces of its planes
    (src/boundary.jl:78-131).  ``Boundary(p1, p2, ...)`` takes Plane objects
    in the reference's order: plane p (1-based) is generator N+p.  A box made
    by ``cuboid`` also carries ``lo`` and ``hi`` and runs through the box
    entry point (exact single-coordinate plane arithmetic); any other domain
    runs through the plane entry point, where normals are scaled to unit length.
    Domains must be bounded with a non-empty interior; at most 64 planes."""

    def __init__(self, *planes: Plane, lo=None, hi=None, periodic=()):
        for p in planes:
            if not isinstance(p, Plane):
                raise TypeError("Boundary takes Plane objects (BC_Dirichlet / BC_Neumann)")
            if p.BC > 0 and lo is None:
                raise NotImplementedError("periodic planes are supported as cuboid(d, periodic=[...]) faces")
        self.planes = list(planes)
        self.lo = None if lo is None else np.asarray(lo, dtype=np.float64)
        self.hi = None if hi is None else np.asarray(hi, dtype=np.float64)
        self.periodic: list = sorted(int(k) for k in periodic)  # 1-based periodic axes

    @property
    def dim(self) -> int:
        return int(self.planes[0].normal.shape[0]) if self.planes else 0

    @property
    def nplanes(self) -> int:
        return len(self.planes)

    @property
    def is_box(self) -> bool:
        return self.lo is not None

    @property
    def periodic_flags(self):
        return [(k + 1) in self.periodic for k in range(self.dim)]

    def arrays(self):
        """(base (P, d), normal (P, d), BC (P,) int16) in plane order."""
        base = np.array([p.base for p in self.planes], dtype=np.float64)
        normal = np.array([p.normal for p in self.planes], dtype=np.float64)
        bc = np.array([p.BC for p in self.planes], dtype=np.int16)
        return base, normal, bc

    def __contains__(self, x) -> bool:
        """Membership as the reference tests it (src/boundary.jl:427-435)."""
        x = np.asarray(x, dtype=np.float64)
        return all(float(np.dot(p.base - x, p.normal)) >= 0.0 for p in self.planes)


def cuboid(dim: int, dimensions=None, periodic=None, neumann=(), offset=None) -> Boundary:
    """The reference's cuboid (src/boundary.jl:510-534), fully periodic by
    default (periodic=1:dim) like the reference's; ``periodic=[]`` gives the
    Dirichlet box the reference's own tests and benchmarks use
    (test/rcmethods.jl:4, src/statistics.jl:107).  Plane 2k-1 is the upper face
    of axis k and plane 2k the lower face, as in the reference; ``neumann``
    lists k for a Neumann upper face and -k for a Neumann lower face."""
    dims = np.ones(dim) if dimensions is None else np.asarray(dimensions, dtype=np.float64)
    off = np.zeros(dim) if offset is None else np.asarray(offset, dtype=np.float64)
    per = list(range(1, dim + 1)) if periodic is None else [int(k) for k in periodic]
    if any(not 1 <= k <= dim for k in per):
        raise ValueError("periodic axes are 1-based axis numbers")
    neu = set(int(k) for k in neumann)
    planes = []
    for k in range(dim):
        unit = np.zeros(dim)
        unit[k] = 1.0
        if (k + 1) in per:  # the partner plane's 1-based index (src/boundary.jl:517-520)
            planes.append(Plane(off + dims * unit, unit.copy(), 2 * k + 2))
            planes.append(Plane(off.copy(), -unit, 2 * k + 1))
            continue
        planes.append(Plane(off + dims * unit, unit.copy(), Neumann if (k + 1) in neu else Dirichlet))
        planes.append(Plane(off.copy(), -unit, Neumann if -(k + 1) in neu else Dirichlet))
    return Boundary(*planes, lo=off.copy(), hi=off + dims, periodic=per)


@dataclass(frozen=True)
class RaycastMethod:
    name: str
    code: int

    def __repr__(self):
        return self.name


# Beside the reference's RCOriginal / RCNonGeneral / RCCombined (src/raycast-types.jl:244-285).
RCGPU = RaycastMethod("RCGPU", _lib.HV_METHOD_FAST)
RCGPUPlain = RaycastMethod("RCGPUPlain", _lib.HV_METHOD_PLAIN)
# The reference's CPU raycast variants (src/raycast-types.jl:244-310) differ in
# speed, not in the tessellation they find (the unique Voronoi diagram of the
# generators in general position); on this path they all run the GPU search.
RCOriginal = RaycastMethod("RCOriginal", _lib.HV_METHOD_FAST)
RCOriginalSafety = RaycastMethod("RCOriginalSafety", _lib.HV_METHOD_FAST)
RCOriginalHP = RaycastMethod("RCOriginalHP", _lib.HV_METHOD_FAST)
RCNonGeneralFast = RaycastMethod("RCNonGeneralFast", _lib.HV_METHOD_FAST)
RCNonGeneralSkip = RaycastMethod("RCNonGeneralSkip", _lib.HV_METHOD_FAST)
RCNonGeneralHP = RaycastMethod("RCNonGeneralHP", _lib.HV_METHOD_FAST)
RCNonGeneralCutoff = RaycastMethod("RCNonGeneralCutoff", _lib.HV_METHOD_FAST)
RCCombined = RaycastMethod("RCCombined", _lib.HV_METHOD_FAST)
RCNonGeneral = RCNonGeneralHP
RCStandard = RCNonGeneral

VI_GEOMETRY = "VI_GEOMETRY"
VI_POLYGON = "VI_POLYGON"
# The reference's memoised exact integrator (src/fastpolyintegrator.jl:4-476): the same cell
# volumes and interface areas as VI_POLYGON, which the GPU computes the same way for both.
VI_FAST_POLYGON = "VI_FAST_POLYGON"
VI_HEURISTIC_MC = "VI_HEURISTIC_MC"
# VI_HEURISTIC_MC takes its volumes and areas from VI_MONTECARLO without an
# integrand (src/heuristic_mc.jl:10); without integrands the two give the same
# quantities, computed here by the GPU Monte-Carlo integrator.
VI_MONTECARLO = "VI_MONTECARLO"


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
                 silence: bool = True, integrand=None, bulk: bool = True):
        pts = np.ascontiguousarray(np.asarray(xs, dtype=np.float64))
        if pts.ndim != 2:
            raise ValueError("xs must be an (n, d) array")
        n, d = pts.shape
        if b is None:
            raise ValueError("a bounded domain is required: pass cuboid(d, periodic=[]) or Boundary(planes...)")
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
            # tuned on synthetic points of the same (d, n) in the domain's box; cached in the context
            if b.is_box:
                self.ctx.autotune(d, n, lo=b.lo, hi=b.hi)
            else:
                self.ctx.autotune(d, n, pts=pts, lo=pts.min(axis=0) - 1.0, hi=pts.max(axis=0) + 1.0)
        self.params = _lib.make_params(method.code, **ss)
        self.mesh = self._build(pts)
        self.integrator = integrator
        self.mc_accurate = mc_accurate
        self.mc_seed = mc_seed
        # integrand=f (points (m, d) -> values (m,) or (m, p)): interface and, with
        # bulk, cell integrals of f by VI_POLYGON's quadrature (src/polyintegrator.jl:80-123)
        self.integrand = integrand
        self.bulk = bulk
        if integrator not in (VI_GEOMETRY, VI_POLYGON, VI_FAST_POLYGON, VI_HEURISTIC_MC, VI_MONTECARLO):
            raise ValueError(f"unsupported integrator {integrator!r} on the GPU path")
        self._integrate()
        if not silence:
            print(f"VoronoiGeometry: {self.mesh.stats()['vertices']} vertices")

    def _build(self, pts):
        b = self.boundary
        if b.is_box and b.periodic:
            return _lib.Mesh(self.ctx, pts, b.lo, b.hi, self.params, periodic=b.periodic_flags)
        if b.is_box:
            return _lib.Mesh(self.ctx, pts, b.lo, b.hi, self.params)
        return _lib.Mesh(self.ctx, pts, None, None, self.params, planes=b.arrays())

    def _integrate(self):
        self._volumes = None
        self._areas = None
        self._iface_int = self._bulk_int = None
        if self.integrator in (VI_POLYGON, VI_FAST_POLYGON):
            self._volumes, self._areas = self.mesh.polygon()
            if self.integrand is not None:
                self._iface_int, self._bulk_int = self.mesh.integrate_function(self.integrand, self.bulk)
        elif self.integrator in (VI_HEURISTIC_MC, VI_MONTECARLO):
            self._volumes, self._areas = self.mesh.heuristic_mc(int(self.mc_accurate[0]), int(self.mc_seed))
            if self.integrand is not None and self.integrator == VI_HEURISTIC_MC:
                self._iface_int, self._bulk_int = self.mesh.integrate_function(self.integrand, self.bulk,
                                                                               heuristic_area=self._areas)

    def refine(self, xs, update: bool = True) -> "VoronoiGeometry":
        """refine!(VG, xs, update) (src/geometry.jl:404-433): appends the
        generators ``xs`` (numbered after the existing ones) and recomputes the
        mesh, and with ``update`` the integrals.  On box and plane domains the
        GPU searches only the new generators' cells and keeps the old vertices
        whose circumspheres stay empty (hv_mesh_refine), the reference's
        re-walk of the affected cells (src/meshrefine.jl:183); periodic
        cuboids search the enlarged set again.  The tessellation is unique, so
        both give the mesh of all points."""
        xs = np.asarray(xs, dtype=np.float64).reshape(-1, self.dimension)
        pts = np.ascontiguousarray(np.vstack([self.nodes, xs]))
        b = self.boundary
        mesh = None
        if not (b.is_box and b.periodic) and self.method.code == _lib.HV_METHOD_FAST:
            try:
                mesh = self.mesh.refined(xs)
            except _lib.HVError as e:  # co-spherical generators: a full build walks them
                if e.code != _lib.HV_E_DEGENERATE:
                    raise
        if mesh is None:
            mesh = self._build(pts)
        self.mesh.free()
        self.mesh, self.nodes = mesh, pts
        if update:
            self._integrate()
        else:
            self._volumes = self._areas = None
        return self

    @property
    def dimension(self) -> int:
        return self.nodes.shape[1]

    def stats(self) -> dict:
        return self.mesh.stats()


def refine(VG: "VoronoiGeometry", xs, update: bool = True) -> "VoronoiGeometry":
    """refine(VG, xs, update) (src/geometry.jl:440-442): a refined copy; VG is unchanged."""
    g = VoronoiGeometry(VG.nodes, VG.boundary, search_settings=None, integrator=VI_GEOMETRY, context=VG.ctx)
    g.params, g.method = VG.params, VG.method
    g.integrator, g.mc_accurate, g.mc_seed = VG.integrator, VG.mc_accurate, VG.mc_seed
    return g.refine(xs, update)


def _unit_planes(boundary: Boundary):
    base, normal, _ = boundary.arrays()
    normal = normal / np.linalg.norm(normal, axis=1, keepdims=True)
    return normal, np.einsum("pk,pk->p", normal, base)


def reflect(x, boundary: Boundary, plane: int):
    """Mirror image of ``x`` across plane ``plane`` (1-based), as the
    reference's reflect (src/boundary.jl:206-211) with the unit normal."""
    normal, off = _unit_planes(boundary)
    nrm = normal[plane - 1]
    x = np.asarray(x, dtype=np.float64)
    return x + 2.0 * nrm * (off[plane - 1] - float(np.dot(nrm, x)))


def orientations(nodes, offs, nbr, boundary: Boundary, onboundary: bool = False, shifts=None):
    """For every neighbour k of cell i the vector from x_i to x_k (to its
    periodic image x_k + s*L with ``shifts`` s), or to the mirror image of x_i
    across a boundary plane (half of it if ``onboundary``), aligned with the
    neighbour CSR (the reference's Orientations, src/voronoidata.jl:265-283)."""
    nodes = np.asarray(nodes, dtype=np.float64)
    n = nodes.shape[0]
    cell = np.repeat(np.arange(n), np.diff(offs))
    nbr = np.asarray(nbr, dtype=np.int64)
    out = np.empty((len(nbr), nodes.shape[1]))
    gen = nbr <= n
    out[gen] = nodes[nbr[gen] - 1] - nodes[cell[gen]]
    if shifts is not None and boundary.is_box:
        out[gen] += np.asarray(shifts, dtype=np.float64)[gen] * (boundary.hi - boundary.lo)
    if (~gen).any():
        normal, off = _unit_planes(boundary)
        p = nbr[~gen] - n - 1
        x = nodes[cell[~gen]]
        h = off[p] - np.einsum("ek,ek->e", normal[p], x)
        out[~gen] = (1.0 if onboundary else 2.0) * h[:, None] * normal[p]
    return out


def boundary_nodes(nodes, offs, nbr, boundary: Boundary, onboundary: bool = False, shifts=None) -> dict:
    """{i: {N+p: mirror of x_i across plane p}} (1-based keys) for every cell
    touching a boundary plane; the projection onto the plane if ``onboundary``
    (the reference's BNodesDictDict, src/voronoidata.jl:354-420)."""
    nodes = np.asarray(nodes, dtype=np.float64)
    n = nodes.shape[0]
    o = orientations(nodes, offs, nbr, boundary, onboundary, shifts)
    res: dict = {}
    for i in range(n):
        for t in range(int(offs[i]), int(offs[i + 1])):
            k = int(nbr[t])
            if k > n:
                res.setdefault(i + 1, {})[k] = nodes[i] + o[t]
    return res


class VoronoiData:
    """Read view of a VoronoiGeometry (src/voronoidata.jl:545-700).

    ``vertices[i]``: the vertices of cell i+1 as (sorted 1-based signature,
    coordinates) pairs; ``vertex_sigs`` / ``vertex_coords``: all vertices, rows
    sorted by signature; ``neighbors[i]``: sorted 1-based neighbours of
    generator i+1 (planes as N+p); ``orientations[i]``: vectors to the
    neighbours (mirror images for planes); ``boundary_nodes``: mirror images of
    the generators across the planes they touch; ``volume[i]`` and ``area[i]``
    (aligned with ``neighbors[i]``) when the geometry was integrated.  On a
    periodic cuboid the neighbour entries carry lattice shifts (``shifts[i]``,
    used by ``orientations``), ``offset`` counts the periodic images the search
    added, ``references`` (1-based originals) and ``reference_shifts`` (their
    translation vectors) describe them; otherwise ``offset`` is 0.  There are
    no infinite edges (``boundary_vertices``).  With ``integrand=f`` and
    VI_POLYGON or VI_HEURISTIC_MC, ``bulk_integral[i]`` (p values) and
    ``interface_integral[i]`` ((deg, p), aligned with ``neighbors[i]``) hold the
    integrals of f with the reference's polygon quadrature or its heuristic
    rule on the Monte-Carlo areas (box and plane domains).
    """

    def __init__(self, geo: VoronoiGeometry, onboundary: bool = False):
        self.geometry = geo
        self.nodes = geo.nodes
        self.boundary = geo.boundary
        voff, vsig, self.vertex_coords = geo.mesh.vertices_csr()
        width = np.diff(voff)
        if width.size == 0 or np.all(width == geo.mesh.d + 1):
            self.vertex_sigs = vsig.reshape(-1, geo.mesh.d + 1)
        else:  # co-spherical generators (a lattice): every generator on the vertex's sphere
            self.vertex_sigs = [vsig[voff[v]:voff[v + 1]] for v in range(width.size)]
        offs, nbr = geo.mesh.neighbors()
        self.neighbor_offsets = offs
        self.neighbor_flat = nbr
        self.neighbors = [nbr[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
        voffs, vtx = geo.mesh.cell_vertices()
        self.vertex_offsets, self.vertex_flat = voffs, vtx
        self.vertices = [[(self.vertex_sigs[v - 1], self.vertex_coords[v - 1]) for v in vtx[voffs[i]:voffs[i + 1]]]
                         for i in range(len(voffs) - 1)]
        shifts = geo.mesh.periodic_shifts() if geo.mesh.periodic is not None else None
        self.shifts = None if shifts is None else [shifts[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
        o = orientations(self.nodes, offs, nbr, self.boundary, onboundary, shifts)
        self.orientations = [o[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
        self.boundary_nodes = boundary_nodes(self.nodes, offs, nbr, self.boundary, onboundary, shifts)
        self.boundary_nodes_on_boundary = onboundary
        self.boundary_vertices: dict = {}
        self.offset = 0
        self.references = np.zeros(0, dtype=np.int64)
        self.reference_shifts = np.zeros((0, self.nodes.shape[1]))
        if geo.mesh.periodic is not None:
            _, ref, sh = geo.mesh.periodic_images()
            self.offset = len(ref)
            self.references = ref
            self.reference_shifts = sh * (self.boundary.hi - self.boundary.lo)
        self.bulk_integral = None
        self.interface_integral = None
        if getattr(geo, "_iface_int", None) is not None:
            ii = geo._iface_int
            self.interface_integral = [ii[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
            if geo._bulk_int is not None:
                self.bulk_integral = [geo._bulk_int[i] for i in range(len(offs) - 1)]
        self.volume = geo._volumes
        self.area = None
        if geo._areas is not None:
            self.area = [geo._areas[offs[i]:offs[i + 1]] for i in range(len(offs) - 1)]
