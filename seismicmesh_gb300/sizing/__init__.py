"""Mesh size functions (sizing/ of the reference)."""
from .mesh_size_function import (
    GridSizing,
    get_sizing_function_from_segy,
    plot_sizing_function,
    read_velocity_model,
    read_velocity_model_to_device,
    write_velocity_model,
)
from .size_function import SizeFunction

__all__ = [
    "GridSizing",
    "SizeFunction",
    "get_sizing_function_from_segy",
    "plot_sizing_function",
    "read_velocity_model",
    "read_velocity_model_to_device",
    "write_velocity_model",
]
