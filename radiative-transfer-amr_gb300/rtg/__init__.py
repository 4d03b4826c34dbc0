"""rtg -- GB300-native steady monochromatic radiative-transfer DG solve.

Drop-in for the reference's ``rt.Problem`` (src/rt) on the reference's hp mesh
(src/dg/mesh).  Compute runs in librtg.so (CUDA, sm_103a) behind a C ABI
(include/rtg.h); this package is the Python host side."""

from .mesh import Mesh, Column, Cell, from_file as mesh_from_file
from .projection import Projection, from_file as projection_from_file
from .problem import Problem, DeviceContext, DeviceOperator
from .error_indicator import ErrorIndicator, ErrorIndicatorColumn, ErrorIndicatorCell

__all__ = ["Mesh", "Column", "Cell", "mesh_from_file", "Projection", "projection_from_file",
           "Problem", "DeviceContext", "DeviceOperator", "ErrorIndicator", "ErrorIndicatorColumn",
           "ErrorIndicatorCell"]
