"""DistMesh generation on the GPU (generation/ of the reference), and
generate_meshes: many independent problems stepped together."""
from .batch import generate_meshes
from .mesh_generator import generate_mesh, sliver_removal

__all__ = ["generate_mesh", "generate_meshes", "sliver_removal"]
