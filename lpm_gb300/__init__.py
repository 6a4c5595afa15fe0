"""lpm_gb300: GB300-native (sm_103a) direct-summation Biot-Savart path of LPM.

The compute path is the CUDA library ``_lib/liblpm_gb300.so`` behind the C
ABI in ``include/lpm_gb300.h``; this package is its Python host layer:

- ``core``      ctypes binding, contexts, mesh and initial-condition helpers
- ``functors``  one call per reference Kokkos functor launch
- ``bve``       BVESphere / BVERK4
- ``ic2d``      Incompressible2D / Incompressible2DRK2
- ``build``     nvcc build of the library
"""
from .core import (FP32C, FP64, PLANE, SPHERE, Context, LpmError, build_mesh, default_context,
                   eval_ic, lib, mesh_sizes)

__all__ = ["FP32C", "FP64", "PLANE", "SPHERE", "Context", "LpmError", "build_mesh",
           "default_context", "eval_ic", "lib", "mesh_sizes"]
