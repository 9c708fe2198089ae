"""GB300-native volumetric fusion hot path of MeshHashing.

Spatial hash + block allocation, simple TSDF and Bayesian PSDF integration,
per-block marching cubes with shared vertices, and the trilinear raycaster,
as hand-written sm_103a CUDA kernels behind the C ABI in include/meshhash.h.
"""
from ._abi import MhParams, MhStats, STATUS_NAMES  # noqa: F401
from ._lib import MeshHashError, load  # noqa: F401
from .volume import Volume, default_params, hash_bucket, launch_count  # noqa: F401
from .batch import Batch  # noqa: F401
