"""lpm_gb300: GB300-native (sm_103a) direct-summation Biot-Savart path of LPM.

The compute path is the CUDA library ``_lib/liblpm_gb300.so`` behind the C
ABI in ``include/lpm_gb300.h``; this package is its Python host layer:

- ``core``      ctypes binding, contexts, mesh and initial-condition helpers
                (host and device meshes, face vertex lists)
- ``functors``  one call per reference Kokkos functor launch (BVE,
                incompressible 2D, planar and spherical SWE sums)
- ``bve``       BVESphere / BVERK4
- ``ic2d``      Incompressible2D / Incompressible2DRK2
- ``ensemble``  many independent BVE problems in one persistent launch
- ``farfield``  octree far field with the learned correction
- ``vtk``       VTK PolyData output of a panel mesh
- ``partition`` target and problem sharding across ranks
- ``build``     nvcc build of the library
"""
from .core import (FP32C, FP64, FP64_CHORD, FP64_EXACT, PLANE, SPHERE, Context, LpmError, build_mesh,
                   build_mesh_device, default_context, eval_ic, lib, mesh_face_vertices,
                   mesh_sizes)

__all__ = ["FP32C", "FP64", "FP64_CHORD", "FP64_EXACT", "PLANE", "SPHERE", "Context", "LpmError",
           "build_mesh", "build_mesh_device", "default_context", "eval_ic", "lib",
           "mesh_face_vertices", "mesh_sizes"]
