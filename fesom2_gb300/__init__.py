"""fesom2_gb300 -- FESOM2's tracer-transport step on one GB300 (sm_103a).

Packages:
  * ``mesh``  -- synthetic FESOM2 meshes and step inputs (channel, icosahedral sphere)
  * ``gpu``   -- ctypes binding of libfesom_gpu.so, the C ABI of include/fesom_gpu.h
  * ``build`` -- in-tree nvcc build of the library
"""
from . import mesh  # noqa: F401

__all__ = ["mesh", "gpu", "build"]
