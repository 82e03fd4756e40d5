"""hvgpu -- GB300 (sm_103a) mesh-generation hot path of HighVoronoi.jl.

The compute path is libhvgpu (C ABI, include/hvgpu.h); this package is the
Python host side that mirrors the reference's VoronoiGeometry / VoronoiData API.
"""
from ._lib import (HV_METHOD_FAST, HV_METHOD_GENERIC, HV_METHOD_PLAIN, Context, HVError, Mesh, default_context, load,  # noqa: F401
                   make_params)
from .geometry import (RCGPU, RCCombined, RCGPUPlain, RCNonGeneral, RCNonGeneralCutoff, RCNonGeneralFast,  # noqa: F401
                       RCNonGeneralHP, RCNonGeneralSkip, RCOriginal, RCOriginalHP, RCOriginalSafety, RCStandard,
                       VI_FAST_POLYGON, VI_GEOMETRY, VI_HEURISTIC_MC, VI_MONTECARLO, VI_POLYGON,
                       BC_Dirichlet, BC_Neumann, BC_Periodic, Boundary, Dirichlet, Neumann, Plane, RaycastMethod,
                       VoronoiData, VoronoiGeometry, boundary_nodes, cuboid, orientations, refine, reflect)
from . import datasets  # noqa: F401

__version__ = "1.0.0"
