"""bskit_gb300 -- GB300-native FFT bispectrum estimator with bskit's measurement API.

``from bskit_gb300 import *`` gives the same names bskit exports for this path
(``FFTBispectrum`` and the bin-list generators); the arithmetic runs in the
sm_103a CUDA library ``libbskit_gb300.so`` through its C ABI.
"""
from .bins import (generate_bin_edge_list, generate_equilateral_triangle_bin_list,
                   generate_isosceles_triangle_bin_list, generate_squeezed_triangle_bin_list,
                   generate_triangle_bin_list, geometric_k_mean, triangle_indices_to_edges)
from .bigfile import BigFileMesh
from .mesh import ArrayMesh, as_mesh

__version__ = "0.1.0"

__all__ = [
    "FFTBispectrum", "ArrayMesh", "BigFileMesh", "as_mesh", "Plan", "TriangleSet",
    "generate_bin_edge_list", "generate_equilateral_triangle_bin_list",
    "generate_isosceles_triangle_bin_list", "generate_squeezed_triangle_bin_list",
    "generate_triangle_bin_list", "geometric_k_mean", "triangle_indices_to_edges",
]


def __getattr__(name):
    # torch-dependent pieces load lazily so that the host-side bin logic imports anywhere
    if name == "FFTBispectrum":
        from .bispectrum import FFTBispectrum
        return FFTBispectrum
    if name in ("Plan", "TriangleSet"):
        from . import engine
        return getattr(engine, name)
    raise AttributeError(name)
