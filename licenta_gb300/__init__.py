"""GB300-native cloth-step engine (PBD + LBVH self-collision).

The compute path is the CUDA library built from licenta_gb300/csrc (C ABI in
include/lc/lc.h); this package is its Python binding.  Importing it does not
need a GPU; stepping a cloth does.
"""
from . import _ffi
from ._ffi import LcError, ClothParams, default_params, default_options, LC_MORTON_REF63, LC_MORTON_K30
from .cloth import ClothBatch, ClothBatchGroup, CudaDeformableBody, Lbvh, Narrowphase
from .scenes import ClothSpec

__all__ = [
    "_ffi", "LcError", "ClothParams", "default_params", "default_options", "LC_MORTON_REF63", "LC_MORTON_K30",
    "ClothBatch", "ClothBatchGroup", "CudaDeformableBody", "Lbvh", "Narrowphase", "ClothSpec",
]
