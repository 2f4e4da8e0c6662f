"""GB300-native (sm_103a) geometry evaluation for tetraloma (tbetcke/gridcl) meshes.

For every cell block of a mesh the native library gathers each cell's geometry nodes through
the dofmap and contracts them with the Lagrange basis and its reference gradients at the
quadrature points, producing physical points, Jacobians, det J (or the area element and unit
normals on manifolds) and the (pseudo-)inverse Jacobian, in the reference's tiled QuadField
layout. The C ABI is ``include/tlgeom.h``; this package is its host-side mirror of
tetraloma-geometry's API.
"""

from ._lib import GridError, lib
from .geometry import (
    AdjointBatch,
    Batch,
    CoordinateElement,
    Geometry,
    GeometryBlock,
    PointSet,
    QuadField,
    QuadRule,
    detj_block,
    facet_normals_block,
    facet_point_set,
    fd_check,
    geometric_factors_block,
    jacobians_block,
    measure_block,
    node_incidence,
    normals_block,
    physical_points_block,
    pseudo_inverse_block,
    pull_back_block,
    vjp_block,
)
from .strategy import (get_strategy, last_kernel_family, last_launch_family, record_strategies, set_strategy,
                       with_strategy)
from . import meshes, refcell

__all__ = [
    "AdjointBatch", "Batch", "CoordinateElement", "Geometry", "GeometryBlock", "GridError", "PointSet", "QuadField",
    "QuadRule", "detj_block", "facet_normals_block", "facet_point_set", "fd_check",
    "geometric_factors_block", "jacobians_block", "lib", "measure_block", "meshes", "normals_block",
    "node_incidence", "physical_points_block", "pseudo_inverse_block", "pull_back_block", "refcell", "vjp_block",
    "get_strategy", "last_kernel_family", "last_launch_family", "record_strategies", "set_strategy",
    "with_strategy",
]
