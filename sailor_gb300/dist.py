"""Import path mirror of the reference: ``from c_lib.VoxelEncoding.dist import
VoxelEncoding`` becomes ``from sailor_gb300.dist import VoxelEncoding``."""
from . import voxel_encoding as VoxelEncoding  # noqa: F401
