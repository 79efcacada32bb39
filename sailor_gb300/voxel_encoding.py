"""Drop-in replacement of SAILOR's ``VoxelEncoding`` extension module.

The reference exposes these names from a pybind11 extension
(c_lib/VoxelEncoding/src/binding.cpp:17-74); SRONet imports it as
``from c_lib.VoxelEncoding.dist import VoxelEncoding`` and calls the
functions and the ``MultiLayerOctree`` class below with the same arguments.
Here every call goes through the C ABI of ``libsailor_gb300.so`` on the
current CUDA stream; there is no CPU path.

Ownership follows the reference: outputs are new tensors, occupancy volumes
are rewritten in place by ``build_multi_res_volumes`` / ``build_octree``, and
``MultiLayerOctree`` keeps references to the volumes, ``voxel_size`` and
``vol_bbox`` given to ``init_octree``.  Invalid inputs raise RuntimeError
(the reference's TORCH_CHECK); launch failures raise RuntimeError instead of
the reference's exit(-1).
"""
import ctypes as C

import torch

from . import _native as N

__all__ = ["rays_calculating", "integrate", "get_origin_bbox", "integrate_in_box", "build_multi_res_volumes",
           "volume_rendering_training_forward",
           "volume_rendering_training_backward", "volume_rendering_occ_forward", "MultiLayerOctree"]


def _cuda(t, name, dtype=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} input must be a cuda tensor")
    if dtype is not None and t.dtype != dtype:
        raise RuntimeError(f"{name} must be {dtype}, got {t.dtype}")
    return t


def _in(t, name, dtype=torch.float32):
    """Input tensor: CUDA, converted to dtype and made contiguous (a copy if needed)."""
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} input must be a cuda tensor")
    return t.to(dtype).contiguous()


def _inplace(t, name, dtype):
    _cuda(t, name, dtype)
    if not t.is_contiguous():
        raise RuntimeError(f"{name} input must be contiguous.")
    return t


class _Dev:
    """Make `device` current; the reference calls cudaSetDevice(device).
    Tensor checks run first, so a CPU tensor raises the reference's message
    even on a machine without a GPU."""

    def __init__(self, device, *tensors):
        for t in tensors:
            if isinstance(t, torch.Tensor) and not t.is_cuda:
                raise RuntimeError("input must be a cuda tensor")
        self.d = torch.device("cuda", int(device)) if not isinstance(device, torch.device) else device

    def __enter__(self):
        self.ctx = torch.cuda.device(self.d)
        self.ctx.__enter__()

    def __exit__(self, *a):
        self.ctx.__exit__(*a)


# --------------------------------------------------------------------------
# fusion: fusion_cuda_integrate (fusion_kernel.cu:600-727)
# --------------------------------------------------------------------------
def rays_calculating(cam_intr, cam_R, cam_T, load_size, device):
    """Per-pixel rays [B, N, load_size, load_size, 6] (origin, unit
    direction) of cameras K [B,N,3,3], R [B,N,3,3], T [B,N,3]
    (sampling_kernel.cu:674-731)."""
    with _Dev(device, cam_intr, cam_R, cam_T):
        K = _in(cam_intr, "cam_intr")
        R = _in(cam_R, "cam_R")
        T = _in(cam_T, "cam_T")
        B, Nv = K.shape[0], K.shape[1]
        H = int(load_size)
        out = torch.empty((B, Nv, H, H, 6), dtype=torch.float32, device=K.device)
        N.check(N.lib.sg_rays_from_cameras(N.ptr(K), N.ptr(R), N.ptr(T), B, Nv, H, H, N.ptr(out), N.stream()),
                "rays_calculating")
        return out


def integrate(occupied_vol, num_occ_voxel, cam_intr, cam_pose, cam_R, cam_T, color_ims, depth_ims, mask_ims,
              obs_weight, th_bbox, trunc_weight, tsdf_th_low, tsdf_th_high, device):
    """TSDF fusion over the data-driven cubic box of the depth points.

    Returns (tsdf, weight, color, vol_origin, vol_bbox, voxel_size); writes
    occupied_vol [B,Dx,Dy,Dz] (local id or -1) and adds the occupied count
    to num_occ_voxel [B] / [B,1], as the reference does."""
    with _Dev(device, depth_ims, cam_intr, cam_R, cam_T):
        depth = _in(depth_ims, "depth_ims")
        B, Nv, H, W = depth.shape
        K = _in(cam_intr, "cam_intr").view(B, Nv, 3, 3)
        R = _in(cam_R, "cam_R").view(B, Nv, 3, 3)
        T = _in(cam_T, "cam_T").view(B, Nv, 3)
        D = occupied_vol.shape[1]
        vol_origin = torch.empty((B, 3, 2), device=depth.device)
        vol_bbox = torch.empty((B, 3, 2), device=depth.device)
        voxel_size = torch.empty((B, 1), device=depth.device)
        N.check(N.lib.sg_auto_bbox(N.ptr(depth), N.ptr(K), N.ptr(R), N.ptr(T), B, Nv, H, W, D, float(th_bbox),
                                   N.ptr(vol_origin), N.ptr(vol_bbox), N.ptr(voxel_size), N.stream()),
                "auto bbox")
        out = integrate_in_box(occupied_vol, num_occ_voxel, cam_intr, cam_pose, color_ims, depth_ims, vol_bbox,
                               voxel_size, obs_weight, trunc_weight, tsdf_th_low, tsdf_th_high, device)
        return out[0], out[1], out[2], vol_origin, vol_bbox, voxel_size


def get_origin_bbox(depth_ims, cam_intr, cam_R, cam_T, th_bbox, device):
    """Bounding box [B, 3, 2] (min, max per axis) of the back-projected valid
    depth pixels, widened by th_bbox: the reference's get_origin_bbox
    (fusion_kernel.cu:473-534), the first steps of integrate."""
    with _Dev(device, depth_ims, cam_intr, cam_R, cam_T):
        depth = _in(depth_ims, "depth_ims")
        B, Nv, H, W = depth.shape
        K = _in(cam_intr, "cam_intr").view(B, Nv, 3, 3)
        R = _in(cam_R, "cam_R").view(B, Nv, 3, 3)
        T = _in(cam_T, "cam_T").view(B, Nv, 3)
        vol_origin = torch.empty((B, 3, 2), device=depth.device)
        vol_bbox = torch.empty((B, 3, 2), device=depth.device)  # the cubic box integrate goes on to take
        voxel_size = torch.empty((B, 1), device=depth.device)
        N.check(N.lib.sg_auto_bbox(N.ptr(depth), N.ptr(K), N.ptr(R), N.ptr(T), B, Nv, H, W, 2, float(th_bbox),
                                   N.ptr(vol_origin), N.ptr(vol_bbox), N.ptr(voxel_size), N.stream()),
                "origin bbox")
        return vol_origin


def integrate_in_box(occupied_vol, num_occ_voxel, cam_intr, cam_pose, color_ims, depth_ims, vol_bbox, voxel_size,
                     obs_weight, trunc_weight, tsdf_th_low, tsdf_th_high, device):
    """integrate_cuda over a given box (vol_bbox [B,3,2], voxel_size [B,1])."""
    with _Dev(device, depth_ims, color_ims, occupied_vol, num_occ_voxel):
        depth = _in(depth_ims, "depth_ims")
        B, Nv, H, W = depth.shape
        color = _in(color_ims, "color_ims").view(B, Nv, H, W)
        K = _in(cam_intr, "cam_intr").view(B, Nv, 3, 3)
        RT = _in(cam_pose, "cam_pose").view(B, Nv, 3, 4)
        occ = _inplace(occupied_vol, "occupied_vol", torch.int32)
        cnt = _inplace(num_occ_voxel, "num_occ_voxel", torch.int32)
        Dx, Dy, Dz = occ.shape[1:4]
        bb = _in(vol_bbox, "vol_bbox")
        vs = _in(voxel_size, "voxel_size")
        opts = dict(device=depth.device, dtype=torch.float32)
        tsdf = torch.empty((B, Dx, Dy, Dz), **opts)
        weight = torch.empty((B, Dx, Dy, Dz), **opts)
        colorv = torch.empty((B, Dx, Dy, Dz), **opts)
        N.check(N.lib.sg_fuse_tsdf(N.ptr(K), N.ptr(RT), N.ptr(color), N.ptr(depth), B, Nv, H, W, Dx, Dy, Dz,
                                   N.ptr(bb), N.ptr(vs), float(obs_weight), float(trunc_weight), float(tsdf_th_low),
                                   float(tsdf_th_high), N.ptr(tsdf), N.ptr(weight), N.ptr(colorv), N.ptr(occ),
                                   N.ptr(cnt), N.stream()), "fuse_tsdf")
        return tsdf, weight, colorv


# --------------------------------------------------------------------------
# coarse volumes: interface_build_m_res_volumes (octree.cpp:28-38)
# --------------------------------------------------------------------------
def build_multi_res_volumes(o_volumes, num_occupied_voxels, level, rate, device):
    """Fill o_volumes[i+1] (coarse occupancy) from o_volumes[i], in place."""
    with _Dev(device, *o_volumes, *num_occupied_voxels):
        for v in o_volumes:
            _inplace(v, "volume", torch.int32)
        for c in num_occupied_voxels:
            _inplace(c, "num_voxels", torch.int32)
        for i in range(int(level) - 1):
            fine, coarse = o_volumes[i], o_volumes[i + 1]
            B, Df = fine.shape[0], fine.shape[1]
            N.check(N.lib.sg_brick_occupancy(N.ptr(fine), B, Df, int(rate), N.ptr(coarse),
                                             N.ptr(num_occupied_voxels[i + 1]), N.stream()), "brick_occupancy")


# --------------------------------------------------------------------------
# compositing: volume_rendering.cu:525-787
# --------------------------------------------------------------------------
def _comp_shapes(sampled_depth, feats):
    B, Nr, S = sampled_depth.shape
    Cf = feats.shape[-1]
    return B, Nr, S, Cf


def volume_rendering_training_forward(sampled_depth, sampled_sort_idx, sigmas, feats, device, t_thresh,
                                      support_occ):
    with _Dev(device, sampled_depth, sampled_sort_idx, sigmas, feats):
        z = _in(sampled_depth, "sampled_depth")
        B, Nr, S, Cf = _comp_shapes(z, feats)
        si = _in(sampled_sort_idx, "sampled_sort_idx", torch.int32)
        sg = _in(sigmas, "sigmas")
        ft = _in(feats, "feats")
        opts = dict(device=z.device, dtype=torch.float32)
        of = torch.empty((B, Nr, Cf), **opts)
        od, ows, oa = (torch.empty((B, Nr, 1), **opts) for _ in range(3))
        N.check(N.lib.sg_composite_fwd(N.ptr(z), N.ptr(si), N.ptr(sg), N.ptr(ft), B * Nr, S, Cf, float(t_thresh),
                                       1 if support_occ else 0, N.ptr(of), N.ptr(od), N.ptr(ows), N.ptr(oa),
                                       N.stream()), "composite_fwd")
        return of, od, ows, oa


def volume_rendering_training_backward(grad_output_feats, grad_output_depths, grad_weight_sums, grad_output_alphas,
                                       output_feats, output_depths, output_ws, output_alphas, sampled_depth,
                                       sampled_sort_idx, sigmas, feats, device, t_thresh, support_occ,
                                       exact=False):
    """Reference gradient formula (exact=False) or the true derivative."""
    with _Dev(device, sampled_depth, sigmas, feats, grad_output_feats):
        z = _in(sampled_depth, "sampled_depth")
        B, Nr, S, Cf = _comp_shapes(z, feats)
        args = [_in(t, n) for t, n in ((grad_output_feats, "grad_output_feats"),
                                       (grad_output_depths, "grad_output_depths"),
                                       (grad_weight_sums, "grad_weight_sums"),
                                       (grad_output_alphas, "grad_output_alphas"),
                                       (output_feats, "output_feats"), (output_depths, "output_depths"),
                                       (output_ws, "output_ws"), (output_alphas, "output_alphas"))]
        si = _in(sampled_sort_idx, "sampled_sort_idx", torch.int32)
        sg = _in(sigmas, "sigmas")
        ft = _in(feats, "feats")
        gf = torch.empty((B, Nr, S, Cf), device=z.device)
        gs = torch.empty((B, Nr, S, 1), device=z.device)
        N.check(N.lib.sg_composite_bwd(*[N.ptr(a) for a in args], N.ptr(z), N.ptr(si), N.ptr(sg), N.ptr(ft),
                                       B * Nr, S, Cf, float(t_thresh), 1 if support_occ else 0,
                                       1 if exact else 0, N.ptr(gf), N.ptr(gs), N.stream()), "composite_bwd")
        return gf, gs


def volume_rendering_occ_forward(sampled_depth, occs, feats, device, t_thresh):
    """Pre-sorted occupancy compositing (volume_rendering_occ_kernel)."""
    with _Dev(device, sampled_depth, occs, feats):
        z = _in(sampled_depth, "sampled_depth")
        B, Nr, S, Cf = _comp_shapes(z, feats)
        sg = _in(occs, "occs")
        ft = _in(feats, "feats")
        opts = dict(device=z.device, dtype=torch.float32)
        of = torch.empty((B, Nr, Cf), **opts)
        od, ows, oa = (torch.empty((B, Nr, 1), **opts) for _ in range(3))
        N.check(N.lib.sg_composite_fwd(N.ptr(z), None, N.ptr(sg), N.ptr(ft), B * Nr, S, Cf, float(t_thresh), 1,
                                       N.ptr(of), N.ptr(od), N.ptr(ows), N.ptr(oa), N.stream()), "composite_occ")
        return of, od, ows, oa


# --------------------------------------------------------------------------
# MultiLayerOctree (include/octree.h:156-304, octree_kernel.cu:545-737,
# intersection_kernel.cu:828-895, sampling_kernel.cu:1251-1462)
# --------------------------------------------------------------------------
class MultiLayerOctree:
    """Brick tree with the reference class's methods.  Two levels (the
    shipped octree_level=2) build the two-level tree that the coarse
    traversal, sampling, trilinear and projection calls use; every depth
    from 2 to SG_MAX_LEVELS also builds the multi-level node tables that
    octree_traversal, ray_voxels_points_sampling and the node queries use."""

    def __init__(self, num_levels, batch_size, rate, device):
        self.num_levels = int(num_levels)
        self.batch_size = int(batch_size)
        self.rate = int(rate)
        self.device = torch.device("cuda", int(device))
        self._tree = None
        self._oct = None
        self._status = None  # SgStatus block, allocated by init_octree
        self._ostatus = None  # SgOctreeStatus block
        self.num_octree_nodes = 0

    # -- build -------------------------------------------------------------
    def init_octree(self, dense_volumes, total_num_occupied_voxels, num_occ_voxels_batches, octree_nodes_index,
                    vol_size, vol_bbox):
        L = len(dense_volumes)
        if L < 2 or L > N.SG_MAX_LEVELS:
            raise RuntimeError(f"MultiLayerOctree: {L} levels (2 to {N.SG_MAX_LEVELS} are supported)")
        if self.rate not in (2, 4, 8):
            raise RuntimeError(f"MultiLayerOctree: rate {self.rate} (2, 4 or 8 are supported)")
        with torch.cuda.device(self.device):
            self._vols = [_inplace(v, "volume", torch.int32) for v in dense_volumes]
            self._cnts = list(num_occ_voxels_batches)
            self.num_levels = L
            self.batch_size = self._vols[0].shape[0]
            self._totals = [int(x) for x in total_num_occupied_voxels]
            self._index = [int(x) for x in octree_nodes_index]
            self.num_octree_nodes = sum(self._totals)
            self.voxel_size = _in(vol_size, "voxel_size").view(-1)
            self.volume_bbox = _in(vol_bbox, "vol_bbox")
            dims = [int(v.shape[1]) for v in self._vols]
            for l in range(1, L):
                if dims[l - 1] != dims[l] * self.rate:
                    raise RuntimeError(f"volume dims {dims[l - 1]}/{dims[l]} do not match rate {self.rate}")
            dev = self.device
            i32 = dict(dtype=torch.int32, device=dev)
            self._status = torch.zeros(4, **i32)
            self._ostatus = torch.zeros(4, **i32)
            self._tree = None
            if L == 2:
                B, Db, Dt = self.batch_size, dims[0], dims[1]
                mw = N.mask_words(self.rate)
                cap_top, cap_bot = max(self._totals[1], 1), max(self._totals[0], 1)
                self._bufs = dict(
                    brick_node=torch.empty(B * Dt ** 3, **i32),
                    brick_mask=torch.empty(B * Dt ** 3 * mw, **i32),
                    top_key=torch.empty(cap_top, **i32), top_child_base=torch.empty(cap_top, **i32),
                    bot_key=torch.empty(cap_bot, **i32), bot_parent=torch.empty(cap_bot, **i32),
                    counts=torch.zeros(2, **i32), brick_box=torch.empty(6 * B, **i32),
                    scratch=torch.empty(int(N.lib.sg_tree_scratch_bytes(B, Dt)), dtype=torch.uint8, device=dev))
                b = self._bufs
                self._tree = N.SgTree(B, Dt, Db, self.rate, self._index[1], self._index[0], cap_top, cap_bot,
                                      b["brick_node"].data_ptr(), b["brick_mask"].data_ptr(),
                                      b["top_key"].data_ptr(), b["top_child_base"].data_ptr(),
                                      b["bot_key"].data_ptr(), b["bot_parent"].data_ptr(), b["counts"].data_ptr(),
                                      self.voxel_size.data_ptr(), self.volume_bbox.data_ptr(),
                                      b["brick_box"].data_ptr())
            # multi-level node tables: one run per level, capacity = its occupied count
            caps = [max(c, 0) for c in self._totals]
            ob = dict(counts=torch.zeros(L, **i32))
            for name in ("key", "parent", "child_base", "nchild"):
                ob[name] = [torch.empty(max(c, 1), **i32) for c in caps]
            o = N.SgOctree()
            o.B, o.L, o.rate = self.batch_size, L, self.rate
            for l in range(L):
                o.dim[l], o.base[l], o.cap[l] = dims[l], self._index[l], caps[l]
                o.vol[l] = self._vols[l].data_ptr()
                for name in ("key", "parent", "child_base", "nchild"):
                    getattr(o, name)[l] = ob[name][l].data_ptr()
            o.counts = ob["counts"].data_ptr()
            o.voxel_size = self.voxel_size.data_ptr()
            o.vol_bbox = self.volume_bbox.data_ptr()
            ob["scratch"] = torch.empty(max(int(N.lib.sg_octree_scratch_bytes(C.byref(o))), 16), dtype=torch.uint8,
                                        device=dev)
            self._oct, self._obufs = o, ob
            self._oct_stale = True

    def build_octree(self):
        if self._oct is None:
            raise RuntimeError("build_octree before init_octree")
        with torch.cuda.device(self.device):
            if self._tree is not None:
                s = self._bufs["scratch"]
                N.check(N.lib.sg_tree_build(C.byref(self._tree), N.ptr(self._vols[1]), N.ptr(self._vols[0]),
                                            N.ptr(s), s.numel(), N.ptr(self._status), N.stream()), "tree_build")
                self._oct_stale = True  # multi-level tables built on first use
            else:
                self._build_levels()

    def _build_levels(self):
        """The multi-level node tables.  Over a two-level tree already built
        they get the same ids (the volumes hold them; occupancy is still
        value > -1) and the build writes them again."""
        with torch.cuda.device(self.device):
            self._ostatus.zero_()
            s = self._obufs["scratch"]
            N.check(N.lib.sg_octree_build(C.byref(self._oct), N.ptr(s), s.numel(), N.ptr(self._ostatus),
                                          N.stream()), "octree_build")
        self._oct_stale = False

    def _levels(self):
        if self._oct is None:
            raise RuntimeError("multi-level query before init_octree")
        if getattr(self, "_oct_stale", True):
            self._build_levels()

    def _two_level(self, what):
        if self._tree is None:
            raise RuntimeError(f"{what}: supported on two-level trees (octree_level=2); this tree has "
                               f"{self.num_levels} levels")

    # -- queries -----------------------------------------------------------
    def voxel_traversal(self, ray_ori, ray_dir, n_max_hits_coarse, start_level, th_early_stop, is_training,
                        opt_num_intersected_voxels):
        self._two_level("voxel_traversal")
        if int(start_level) != 0:
            raise RuntimeError("voxel_traversal: only start_level 0 (the top level) is supported")
        with torch.cuda.device(self.device):
            ori = _in(ray_ori, "ray_ori")
            dr = _in(ray_dir, "ray_dir")
            Nr = ori.shape[1]
            B, W = self.batch_size, int(n_max_hits_coarse)
            idx = torch.empty((B, Nr, W), dtype=torch.int32, device=self.device)
            t0 = torch.empty((B, Nr, W), device=self.device)
            t1 = torch.empty((B, Nr, W), device=self.device)
            vl = torch.empty((B, Nr, 1), device=self.device)
            cnt = torch.empty((B, Nr), dtype=torch.int32, device=self.device)
            self._status[0:2].zero_()
            N.check(N.lib.sg_intersect(C.byref(self._tree), N.ptr(ori), N.ptr(dr), Nr, W, int(th_early_stop),
                                       int(opt_num_intersected_voxels), 1 if is_training else 0, 1, N.ptr(idx),
                                       N.ptr(t0), N.ptr(t1), N.ptr(vl), N.ptr(cnt), N.ptr(self._status),
                                       N.stream()), "intersect")
            self._last_W = W
            return idx, t0, t1, vl

    def ray_voxels_points_sampling_coarse(self, hits_idxs, min_depths, max_depths, uniform_rand_values,
                                          rays_valid_len, start_level, num_sampled):
        self._two_level("ray_voxels_points_sampling_coarse")
        with torch.cuda.device(self.device):
            st = self._status.tolist()  # the reference reads its max-hit counter here too
            if st[0] & N.SG_FLAG_HIT_OVERFLOW:
                raise RuntimeError(f"hit list overflow: a ray has {st[1]} hits, rows hold {self._last_W}")
            hi = _in(hits_idxs, "hits_idxs", torch.int32)
            B, Nr, W = hi.shape
            t0 = _in(min_depths, "min_depths")
            t1 = _in(max_depths, "max_depths")
            rd = _in(uniform_rand_values, "uniform_rand_values")
            vl = _in(rays_valid_len, "rays_valid_len")
            S = int(num_sampled)
            si = torch.empty((B, Nr, S), dtype=torch.int32, device=self.device)
            sz = torch.empty((B, Nr, S), device=self.device)
            N.check(N.lib.sg_sample_coarse(C.byref(self._tree), N.ptr(hi), N.ptr(t0), N.ptr(t1), Nr, W, N.ptr(rd),
                                           N.ptr(vl), S, self.num_levels, int(start_level), N.ptr(si), N.ptr(sz),
                                           N.stream()), "sample_coarse")
            return si, sz

    def sort_samplings(self, sampled_depths):
        with torch.cuda.device(self.device):
            z = _in(sampled_depths, "sampled_depths")
            srt = torch.empty_like(z)
            idx = torch.empty(z.shape, dtype=torch.int32, device=z.device)
            if z.numel() == 0:  # as torch.sort: empty in, empty out
                return srt, idx
            S = z.shape[-1]
            R = z.numel() // S
            N.check(N.lib.sg_sort_samples(N.ptr(z), R, S, N.ptr(srt), N.ptr(idx), N.stream()), "sort")
            return srt, idx

    def trilinear_aggregate_features(self, ray_ori, ray_dir, sampled_z, sampled_idx, input_feats):
        self._two_level("trilinear_aggregate_features")
        with torch.cuda.device(self.device):
            f = _in(input_feats, "input_feats")
            B, Cf, Nr, S, _ = f.shape
            out = torch.zeros((B, Cf, Nr, S), device=self.device)
            N.check(N.lib.sg_trilerp_nodes_fwd(C.byref(self._tree), N.ptr(_in(ray_ori, "ray_ori")),
                                               N.ptr(_in(ray_dir, "ray_dir")), N.ptr(_in(sampled_z, "sampled_z")),
                                               N.ptr(_in(sampled_idx, "sampled_idx", torch.int32)), N.ptr(f), Nr, S,
                                               Cf, N.ptr(out), N.stream()), "trilerp_fwd")
            return out

    def trilinear_aggregate_features_backward(self, ray_ori, ray_dir, sampled_z, sampled_idx, input_feats,
                                              grad_output):
        self._two_level("trilinear_aggregate_features_backward")
        with torch.cuda.device(self.device):
            g = _in(grad_output, "grad_output")
            B, Cf, Nr, S = g.shape
            gin = torch.empty((B, Cf, Nr, S, 8), device=self.device)
            N.check(N.lib.sg_trilerp_nodes_bwd(C.byref(self._tree), N.ptr(_in(ray_ori, "ray_ori")),
                                               N.ptr(_in(ray_dir, "ray_dir")), N.ptr(_in(sampled_z, "sampled_z")),
                                               N.ptr(_in(sampled_idx, "sampled_idx", torch.int32)), N.ptr(g), Nr, S,
                                               Cf, N.ptr(gin), N.stream()), "trilerp_bwd")
            return gin

    def project_sampled_xyz(self, ray_ori, ray_dir, sampled_z, sampled_idx, Ks, RTs, ori_w, ori_h, num_views,
                            record_corners=True):
        """Samples (and, with record_corners, their nodes' eight corners)
        projected into every view: (proj_xy [B,V,N,S,9,2] or [B,V,N,S,2]
        normalised to [-1, 1], proj_z [B,V,N,S,9,1] or [B,V,N,S,1] camera z);
        -1 where the sample has no node (sampling_kernel.cu:1333-1381)."""
        if record_corners and self._oct is None:
            raise RuntimeError("project_sampled_xyz with record_corners before init_octree")
        if record_corners:
            self._two_level("project_sampled_xyz with record_corners")
        with torch.cuda.device(self.device):
            z = _in(sampled_z, "sampled_z")
            idx = _in(sampled_idx, "sampled_idx", torch.int32)
            B, Nr, S = z.shape
            V = int(num_views)
            K = _in(Ks, "Ks")
            RT = _in(RTs, "RTs")
            if K.numel() != B * V * 9 or RT.numel() != B * V * 12:
                raise RuntimeError(f"Ks / RTs must hold [{B}, {V}] cameras")
            shape = (B, V, Nr, S, 9) if record_corners else (B, V, Nr, S)
            xy = torch.empty(shape + (2,), device=self.device)
            pz = torch.empty(shape + (1,), device=self.device)
            N.check(N.lib.sg_project_sampled_xyz(C.byref(self._tree) if self._tree is not None else None,
                                                 N.ptr(_in(ray_ori, "ray_ori")), N.ptr(_in(ray_dir, "ray_dir")),
                                                 N.ptr(z), N.ptr(idx), N.ptr(K), N.ptr(RT), B, V, Nr, S,
                                                 int(ori_w), int(ori_h), 1 if record_corners else 0, N.ptr(xy),
                                                 N.ptr(pz), N.stream()), "project_sampled_xyz")
            return xy, pz

    # -- node queries -----------------------------------------------------
    def get_nodes_tensor(self):
        with torch.cuda.device(self.device):
            out = torch.empty((self.num_octree_nodes, 6), device=self.device)
            if self._tree is not None:
                N.check(N.lib.sg_tree_nodes(C.byref(self._tree), self.num_octree_nodes, N.ptr(out), N.stream()),
                        "tree_nodes")
            else:
                self._levels()
                N.check(N.lib.sg_octree_nodes(C.byref(self._oct), self.num_octree_nodes, N.ptr(out),
                                              N.stream()), "octree_nodes")
            return out

    def get_num_nodes(self):
        return self.num_octree_nodes

    def get_num_nodes_valid(self):
        """Nodes built per level, top level first (the reference's
        queue_control: [#top nodes, #next level, ...])."""
        if self._tree is not None:
            return self._bufs["counts"].tolist()
        self._levels()
        return self._obufs["counts"].tolist()[::-1]

    def get_num_levels(self):
        return self.num_levels

    def get_batch_size(self):
        return self.batch_size

    def get_volume_dim(self):
        return [int(v.shape[1]) for v in self._vols]

    def tree_arrays(self):
        """Device node tables (brick map, masks, keys) for inspection."""
        return dict(self._bufs)

    def octree_traversal(self, ray_ori, ray_dir, n_max_hits_coarse, n_max_hits, start_level, th_early_stop,
                         opt_num_intersected_voxels):
        """(idx, min_depths, max_depths, valid_len [B,N,1], idx_c, min_depths_c,
        max_depths_c): the coarse DDA over level L-1-start_level, then the
        depth-first descent of each coarse node (intersection_kernel.cu:
        441-643, 722-826).  Fine rows hold each coarse node's entries
        together, in descent order; the reference's atomic appends leave the
        same entries in a run-dependent order."""
        if self._oct is None:
            raise RuntimeError("octree_traversal before init_octree")
        self._levels()
        start_level = int(start_level)
        if not 0 <= start_level < self.num_levels:
            raise RuntimeError(f"octree_traversal: start_level {start_level} outside [0, {self.num_levels})")
        with torch.cuda.device(self.device):
            ori = _in(ray_ori, "ray_ori")
            dr = _in(ray_dir, "ray_dir")
            Nr = ori.shape[1]
            B, Wc, Wf = self.batch_size, int(n_max_hits_coarse), int(n_max_hits)
            dev = self.device
            idx_c = torch.empty((B, Nr, Wc), dtype=torch.int32, device=dev)
            t0_c = torch.empty((B, Nr, Wc), device=dev)
            t1_c = torch.empty((B, Nr, Wc), device=dev)
            idx = torch.empty((B, Nr, Wf), dtype=torch.int32, device=dev)
            t0 = torch.empty((B, Nr, Wf), device=dev)
            t1 = torch.empty((B, Nr, Wf), device=dev)
            vl = torch.empty((B, Nr, 1), device=dev)
            cnt_c = torch.empty((B, Nr), dtype=torch.int32, device=dev)
            cnt = torch.empty((B, Nr), dtype=torch.int32, device=dev)
            self._ostatus.zero_()
            N.check(N.lib.sg_octree_traversal(C.byref(self._oct), N.ptr(ori), N.ptr(dr), Nr, start_level, Wc, Wf,
                                              int(th_early_stop), int(opt_num_intersected_voxels), N.ptr(idx_c),
                                              N.ptr(t0_c), N.ptr(t1_c), N.ptr(cnt_c), N.ptr(idx), N.ptr(t0),
                                              N.ptr(t1), N.ptr(cnt), N.ptr(vl), N.ptr(self._ostatus), N.stream()),
                    "octree_traversal")
            self._last_fine = (Wc, Wf)
            return idx, t0, t1, vl, idx_c, t0_c, t1_c

    def ray_voxels_points_sampling(self, hits_idxs, min_depths, max_depths, rays_valid_len, uniform_rand_values,
                                   start_level, num_sampled):
        """(sampled_idx, sampled_depths) [B,N,S] over fine rows
        (sampling_kernel.cu:911-1068, 1178-1248); unsorted, as the
        reference returns them."""
        if self._oct is None:
            raise RuntimeError("ray_voxels_points_sampling before init_octree")
        self._levels()
        with torch.cuda.device(self.device):
            st = self._ostatus.tolist()  # the reference reads its fine max-hit counter here too
            if st[0] & N.SG_FLAG_HIT_OVERFLOW:
                Wc, Wf = getattr(self, "_last_fine", (0, 0))
                raise RuntimeError(f"octree row overflow: a ray has {st[1]} coarse / {st[2]} fine entries, "
                                   f"rows hold {Wc} / {Wf}")
            hi = _in(hits_idxs, "hits_idxs", torch.int32)
            B, Nr, W = hi.shape
            t0 = _in(min_depths, "min_depths")
            t1 = _in(max_depths, "max_depths")
            vl = _in(rays_valid_len, "rays_valid_len")
            rd = _in(uniform_rand_values, "uniform_rand_values")
            S = int(num_sampled)
            if rd.numel() != B * Nr * S:
                raise RuntimeError(f"uniform_rand_values must hold [{B}, {Nr}, {S}] values")
            si = torch.empty((B, Nr, S), dtype=torch.int32, device=self.device)
            sz = torch.empty((B, Nr, S), device=self.device)
            N.check(N.lib.sg_sample_fine(C.byref(self._oct), N.ptr(hi), N.ptr(t0), N.ptr(t1), Nr, W, N.ptr(vl),
                                         N.ptr(rd), S, int(start_level), N.ptr(si), N.ptr(sz), N.stream()),
                    "sample_fine")
            return si, sz
