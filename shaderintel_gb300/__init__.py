"""shaderintel_gb300 — a GB300-native (sm_103a) MLS-MPM substep behind ShaderIntel's MPM solver API.

The CUDA library (libsi_cuda, C ABI in include/si_cuda.h) holds the kernels and the runtime; this
package is the host side over it, mirroring the reference's JavaScript MPM object.
"""
from ._lib import SIError, lib
from .mpm import FLUID, JELLY, MATERIALS, MPM, MPM_KINDS, SAND, SNOW, World, body_record, material_row, sample_shape

__all__ = ["MPM", "World", "SIError", "MATERIALS", "MPM_KINDS", "FLUID", "JELLY", "SNOW", "SAND", "lib",
           "material_row", "sample_shape", "body_record"]
