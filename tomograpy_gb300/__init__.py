"""tomograpy_gb300 -- TomograPy's Siddon conic projector on NVIDIA GB300 (sm_103a).

A drop-in for the hot path of TomograPy (``tomograpy.projector``,
``backprojector``, ``projector4d``, ``backprojector4d``, ``obstacle="sun"``,
the ``lo_wrapper`` linear operators): the same Python API over hand-written
CUDA kernels reached through a C ABI (``include/tomograpy_gb300.h``).
"""
from . import headers, simu, solar, synthetic
from .headers import (INF, apply_rotation, array_to_dict, centered_cubic_map, centered_cubic_map_header,
                      centered_image, centered_image_header, centered_stack, dataarray_from_header,
                      dict_to_array, fov, full_intersection_parameters, full_rotation_matrix,
                      full_unit_vector, header_rotation_matrix, intersect_cube, map_borders, rotation_matrix)
from .infoarray import InfoArray
from .siddon import (C_full_intersection_parameters, C_full_unit_vector, backprojector, backprojector4d,
                     check_projector_inputs, conic_image_backprojector, conic_image_projector, projector,
                     projector4d, ray_projector)

version = "0.1.0"
