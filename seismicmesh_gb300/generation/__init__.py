"""DistMesh generation on the GPU (generation/ of the reference)."""
from .mesh_generator import generate_mesh, sliver_removal

__all__ = ["generate_mesh", "sliver_removal"]
