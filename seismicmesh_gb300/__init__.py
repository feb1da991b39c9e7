"""GB300-native DistMesh engine with the SeismicMesh Python API.

generate_mesh / sliver_removal, the SDF classes and the sizing calls run on
hand-written sm_103a CUDA kernels (libdmgb.so, C ABI in include/dmgb.h).
"""
from . import geometry, sizing, synthetic
from .generation import generate_mesh, generate_meshes, sliver_removal
from .geometry import (
    Ball,
    Cube,
    Cylinder,
    Difference,
    Disk,
    GridSDF,
    Intersection,
    Isosurface,
    NeuralSDF,
    Prism,
    Rectangle,
    Repeat,
    Torus,
    Union,
)
from .sizing import (
    SizeFunction,
    get_sizing_function_from_segy,
    plot_sizing_function,
    read_velocity_model,
    read_velocity_model_to_device,
    write_velocity_model,
)

__version__ = "1.0.0"

__all__ = [
    "generate_mesh", "generate_meshes", "sliver_removal", "geometry", "sizing", "Ball", "Cube", "Cylinder",
    "Difference", "Disk", "GridSDF", "Intersection", "Prism", "Rectangle", "Repeat",
    "Torus", "Union", "SizeFunction", "get_sizing_function_from_segy",
    "plot_sizing_function", "read_velocity_model", "read_velocity_model_to_device",
    "write_velocity_model", "Isosurface",
    "NeuralSDF", "synthetic",
]
