"""sailor_gb300: SAILOR's VoxelEncoding hot path as sm_103a CUDA kernels.

TSDF fusion -> two-level brick tree -> ray/tree intersection -> adaptive
sampling -> compositing, plus adjoints for compositing and trilinear
gathers, behind the reference's Python op signatures (``dist.VoxelEncoding``
and ``voxel_encoding_helper``).  The kernels live in ``libsailor_gb300.so``
(C ABI: include/sailor_gb300.h); importing an op without it raises.
"""
__version__ = "0.1.0"
