"""Signed distance functions and mesh utilities (geometry/ of the reference)."""
from .signed_distance_functions import (
    Ball,
    Cube,
    Cylinder,
    Difference,
    Disk,
    GridSDF,
    Intersection,
    Prism,
    Rectangle,
    Repeat,
    Torus,
    Union,
    corners,
    dball,
    dblock,
    drectangle,
)
from .utils import (
    calc_circumsphere_grad,
    calc_dihedral_angles,
    delete_boundary_entities,
    fix_mesh,
    get_boundary_edges,
    get_boundary_facets,
    get_boundary_vertices,
    laplacian2_fixed_point,
    simp_qual,
    simp_vol,
    unique_edges,
)

__all__ = [
    "Ball", "Cube", "Cylinder", "Difference", "Disk", "GridSDF", "Intersection",
    "Prism", "Rectangle", "Repeat", "Torus", "Union", "corners", "dball", "dblock",
    "drectangle", "calc_circumsphere_grad", "calc_dihedral_angles",
    "delete_boundary_entities", "fix_mesh", "get_boundary_edges",
    "get_boundary_facets", "get_boundary_vertices", "laplacian2_fixed_point",
    "simp_qual", "simp_vol", "unique_edges",
]
