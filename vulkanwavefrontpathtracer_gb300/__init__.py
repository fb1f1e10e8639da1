"""GB300-native wavefront path tracer.

The compute path is libwfpt.so (hand-written sm_103a CUDA kernels behind the
C ABI in include/wfpt.h); this package holds its sources (csrc/), the build
recipe (build.py) and the Python host interface (api.py) that mirrors the
reference's RayGen / Tracer / Renderer stage interface.
"""
from . import _lib, api
from ._lib import (BVH2_FP32, BVH8_Q8, MORTON_6D48, MORTON_6D64, MORTON_AILA32, PATH_RAYS, PRIMARY_RAYS,
                   SHADOW_RAYS, WfptError)

__all__ = ["_lib", "api", "BVH2_FP32", "BVH8_Q8", "MORTON_AILA32", "MORTON_6D48", "MORTON_6D64", "PRIMARY_RAYS",
           "SHADOW_RAYS", "PATH_RAYS", "WfptError"]
