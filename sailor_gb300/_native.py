"""ctypes binding of libsailor_gb300.so (the C ABI in include/sailor_gb300.h).

The library is required: importing this module raises ImportError when the
shared object is missing or lacks an entry point, so no operation of the
package can run without the CUDA kernels.
"""
import ctypes as C
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsailor_gb300.so")

SG_FLAG_HIT_OVERFLOW = 1
SG_FLAG_TREE_CAPACITY = 2
SG_FLAG_RECORD_CAPACITY = 4
# leading counters of the deterministic reduction's workspace
SG_DET_COUNTERS = 8
SG_DET_RAYS_WITH_HITS, SG_DET_SLOTS_NEEDED, SG_DET_SLOTS, SG_DET_CELLS, SG_DET_RECORDS = 0, 1, 2, 3, 4

EXPORTS = (
    "sg_mask_words", "sg_status_string", "sg_version", "sg_auto_bbox", "sg_fuse_tsdf",
    "sg_brick_occupancy", "sg_tree_scratch_bytes", "sg_tree_build", "sg_tree_nodes", "sg_intersect",
    "sg_sample_coarse", "sg_sort_samples", "sg_composite_fwd", "sg_composite_bwd",
    "sg_trilerp_nodes_fwd", "sg_trilerp_nodes_bwd", "sg_sample_sorted", "sg_grid_gather",
    "sg_render_fused", "sg_tune_set", "sg_tune_get", "sg_tree_build_static",
    "sg_grid_scatter", "sg_fuse_tsdf_views", "sg_intersect_segments", "sg_render_segments_fwd",
    "sg_render_segments_bwd", "sg_render_segments_train",
    "sg_camera_params", "sg_rays_from_cameras", "sg_segment_rays", "sg_zero_near_nodes",
    "sg_project_sampled_xyz", "sg_project_gather", "sg_train_det_workspace_bytes", "sg_render_segments_train_det",
    "sg_sort_pairs_scratch_bytes", "sg_sort_pairs", "sg_octree_scratch_bytes", "sg_octree_build",
    "sg_octree_nodes", "sg_octree_traversal", "sg_sample_fine", "sg_nerf_param_count", "sg_nerf_density",
)


class SgTree(C.Structure):
    _fields_ = [("B", C.c_int), ("Dt", C.c_int), ("Db", C.c_int), ("rate", C.c_int),
                ("base_top", C.c_int), ("base_bot", C.c_int), ("cap_top", C.c_int), ("cap_bot", C.c_int),
                ("brick_node", C.c_void_p), ("brick_mask", C.c_void_p), ("top_key", C.c_void_p),
                ("top_child_base", C.c_void_p), ("bot_key", C.c_void_p), ("bot_parent", C.c_void_p),
                ("counts", C.c_void_p), ("voxel_size", C.c_void_p), ("vol_bbox", C.c_void_p),
                ("brick_box", C.c_void_p)]


SG_MAX_LEVELS = 12
_LV = C.c_int * SG_MAX_LEVELS
_LP = C.c_void_p * SG_MAX_LEVELS


class SgOctree(C.Structure):
    _fields_ = [("B", C.c_int), ("L", C.c_int), ("rate", C.c_int), ("dim", _LV), ("base", _LV), ("cap", _LV),
                ("vol", _LP), ("key", _LP), ("parent", _LP), ("child_base", _LP), ("nchild", _LP),
                ("counts", C.c_void_p), ("voxel_size", C.c_void_p), ("vol_bbox", C.c_void_p)]


class SgViews(C.Structure):
    _fields_ = [("max_views", C.c_int), ("view_begin", C.c_void_p), ("view_hw", C.c_void_p),
                ("view_offset", C.c_void_p), ("K", C.c_void_p), ("RT", C.c_void_p), ("depth", C.c_void_p),
                ("color", C.c_void_p), ("block_offset", C.c_void_p), ("depth_blocks", C.c_void_p)]


class SgRaySegments(C.Structure):
    _fields_ = [("count", C.c_int), ("total", C.c_int), ("ray_begin", C.c_void_p), ("frame", C.c_void_p),
                ("samples", C.c_void_p), ("cameras", C.c_void_p), ("widths", C.c_void_p)]


class SgRenderArgs(C.Structure):
    _fields_ = [("ori", C.c_void_p), ("dir", C.c_void_p), ("hit_idx", C.c_void_p), ("hit_t0", C.c_void_p),
                ("hit_t1", C.c_void_p), ("hit_count", C.c_void_p), ("valid_len", C.c_void_p), ("W", C.c_int),
                ("S", C.c_int), ("rands", C.c_void_p), ("rand_const", C.c_float), ("rand_seed", C.c_ulonglong),
                ("tsdf", C.c_void_p), ("D", C.c_int), ("sdf_scale", C.c_float), ("sdf_s", C.c_float),
                ("feat", C.c_void_p), ("Df", C.c_int), ("C", C.c_int), ("feat_bbox", C.c_void_p),
                ("feat_vs", C.c_void_p), ("head", C.c_void_p), ("t_thres", C.c_float)]



class SgFeatureMap(C.Structure):
    _fields_ = [("data", C.c_void_p), ("stride", C.c_longlong * 4), ("C", C.c_int), ("H", C.c_int),
                ("W", C.c_int), ("out", C.c_void_p)]


class SgProjGather(C.Structure):
    _fields_ = [("grids_in", C.c_void_p), ("depth_in", C.c_void_p),
                ("points", C.c_void_p), ("points_stride", C.c_longlong * 3), ("points_div", C.c_int),
                ("p_depths", C.c_void_p), ("p_depths_stride", C.c_longlong * 2), ("K", C.c_void_p),
                ("R", C.c_void_p), ("T", C.c_void_p), ("n_images", C.c_int), ("num_points", C.c_int),
                ("depth_thres", C.c_float), ("min_d", C.c_float), ("max_d", C.c_float), ("half_res", C.c_float),
                ("ori_pts", C.c_void_p), ("grids", C.c_void_p), ("depth", C.c_void_p), ("n_maps", C.c_int),
                ("maps", SgFeatureMap * 4), ("psdf_map", C.c_int), ("psdf_clip", C.c_float),
                ("psdf_scale", C.c_float), ("psdf", C.c_void_p)]

def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(the package has no CPU implementation)")
    lib = C.CDLL(LIB_PATH)
    missing = [n for n in EXPORTS if not hasattr(lib, n)]
    if missing:
        raise ImportError(f"{LIB_PATH} lacks entry points: {missing}")
    i, f, p, sz = C.c_int, C.c_float, C.c_void_p, C.c_size_t
    lib.sg_status_string.restype = C.c_char_p
    lib.sg_status_string.argtypes = [i]
    lib.sg_mask_words.argtypes = [i]
    lib.sg_auto_bbox.argtypes = [p, p, p, p, i, i, i, i, i, f, p, p, p, p]
    lib.sg_fuse_tsdf.argtypes = [p, p, p, p, i, i, i, i, i, i, i, p, p, f, f, f, f, p, p, p, p, p, p]
    lib.sg_brick_occupancy.argtypes = [p, i, i, i, p, p, p]
    lib.sg_tree_scratch_bytes.argtypes = [i, i]
    lib.sg_tree_scratch_bytes.restype = sz
    lib.sg_tree_build.argtypes = [C.POINTER(SgTree), p, p, p, sz, p, p]
    lib.sg_tree_build_static.argtypes = [C.POINTER(SgTree), p, p, p, p]
    lib.sg_tree_nodes.argtypes = [C.POINTER(SgTree), i, p, p]
    lib.sg_intersect.argtypes = [C.POINTER(SgTree), p, p, i, i, i, i, i, i, p, p, p, p, p, p, p]
    lib.sg_sample_coarse.argtypes = [C.POINTER(SgTree), p, p, p, i, i, p, p, i, i, i, p, p, p]
    lib.sg_sort_samples.argtypes = [p, i, i, p, p, p]
    lib.sg_composite_fwd.argtypes = [p, p, p, p, i, i, i, f, i, p, p, p, p, p]
    lib.sg_composite_bwd.argtypes = [p] * 12 + [i, i, i, f, i, i, p, p, p]
    lib.sg_sample_sorted.argtypes = [C.POINTER(SgTree), p, p, p, p, i, i, p, f, p, i, i, i, p, p, p]
    lib.sg_grid_gather.argtypes = [p, p, p, i, i, i, p, i, i, p, p, i, f, f, p, p]
    lib.sg_grid_scatter.argtypes = [p, p, p, i, i, i, p, p, i, i, p, p, i, f, f, p, p]
    lib.sg_render_fused.argtypes = [C.POINTER(SgTree), p, p, p, p, i, i, p, f, p, i, i, i, p, p, p, i, f, f, p, i,
                                    p, p, f, p, p, p, p, p, p, p]
    T, V, G, A = C.POINTER(SgTree), C.POINTER(SgViews), C.POINTER(SgRaySegments), C.POINTER(SgRenderArgs)
    lib.sg_fuse_tsdf_views.argtypes = [V, i, i, p, p, f, f, f, f, p, p, p, p, p, p]
    lib.sg_intersect_segments.argtypes = [T, G, p, p, i, p, p, p, p, p, p, p]
    lib.sg_render_segments_fwd.argtypes = [T, G, A, p, p, p, p, p, p, p]
    lib.sg_render_segments_bwd.argtypes = [T, G, A, p, p, p, p, p, p, p, p, p]
    lib.sg_render_segments_train.argtypes = [T, G, A, p, f, p, p, p, p, p, p, p, p]
    ll = C.c_longlong
    lib.sg_train_det_workspace_bytes.argtypes = [ll, i, i, ll]
    lib.sg_train_det_workspace_bytes.restype = sz
    lib.sg_render_segments_train_det.argtypes = [T, G, A, i, p, p, p, f, p, p, p, p, p, p, p, p, sz, ll, p, p]
    lib.sg_sort_pairs_scratch_bytes.argtypes = [ll]
    lib.sg_sort_pairs_scratch_bytes.restype = sz
    lib.sg_sort_pairs.argtypes = [p, p, ll, i, p, p, p, p, p, sz, p]
    lib.sg_camera_params.argtypes = [p, p, p, i, p, p]
    lib.sg_rays_from_cameras.argtypes = [p, p, p, i, i, i, i, p, p]
    lib.sg_segment_rays.argtypes = [C.POINTER(SgRaySegments), p, p, p]
    lib.sg_zero_near_nodes.argtypes = [C.POINTER(SgTree), p, i, p]
    lib.sg_project_sampled_xyz.argtypes = [C.POINTER(SgTree), p, p, p, p, p, p, i, i, i, i, i, i, i, p, p, p]
    lib.sg_project_gather.argtypes = [C.POINTER(SgProjGather), p]
    lib.sg_tune_set.argtypes = [i, i]
    lib.sg_tune_get.argtypes = [i]
    O = C.POINTER(SgOctree)
    lib.sg_octree_scratch_bytes.argtypes = [O]
    lib.sg_octree_scratch_bytes.restype = sz
    lib.sg_octree_build.argtypes = [O, p, sz, p, p]
    lib.sg_octree_nodes.argtypes = [O, i, p, p]
    lib.sg_octree_traversal.argtypes = [O, p, p, i, i, i, i, i, i, p, p, p, p, p, p, p, p, p, p, p]
    lib.sg_sample_fine.argtypes = [O, p, p, p, i, i, p, p, i, i, p, p, p]
    lib.sg_nerf_param_count.argtypes = []
    lib.sg_nerf_param_count.restype = sz
    lib.sg_nerf_density.argtypes = [p, p, p, p, i, i, i, p, p, p, p]
    lib.sg_trilerp_nodes_fwd.argtypes = [C.POINTER(SgTree), p, p, p, p, p, i, i, i, p, p]
    lib.sg_trilerp_nodes_bwd.argtypes = [C.POINTER(SgTree), p, p, p, p, p, i, i, i, p, p]
    return lib


lib = _load()


def check(rc, what=""):
    if rc != 0:
        raise RuntimeError(f"sailor_gb300 {what}: {lib.sg_status_string(rc).decode()} (status {rc})")


def ptr(t):
    """Device address of a tensor (None -> NULL)."""
    if t is None:
        return None
    return C.c_void_p(t.data_ptr())


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def mask_words(rate):
    return lib.sg_mask_words(int(rate))
