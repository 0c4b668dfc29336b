"""voxelis_gb300: a GB300-native (sm_103a) implementation of voxelis' batched SVO-DAG
edit-and-intern path (VoxTree::apply_batch + VoxInterner hash-consing), VoxTree::get and dense-chunk
construction, behind a C ABI (include/voxelis_gb300.h) and this host mirror of the reference API.
"""
from ._abi import (  # noqa: F401
    VX_MEM_DEVICE, VX_MEM_HOST, VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P3, VX_PATCH_P4, VX_PATCH_P5,
    ReferencePanic, ReferenceUB, VoxelisError,
)
from .api import Batch, VoxInterner, VoxTree  # noqa: F401
