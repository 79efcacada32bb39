"""Drop-in mirror of SAILOR's ``c_lib/VoxelEncoding/voxel_encoding_helper.py``.

Same classes, functions and argument orders as the reference's Python op
layer (lines cited per object), with every CUDA call routed to
``sailor_gb300.dist.VoxelEncoding`` (the sm_103a kernels).  Additions over the
reference are marked as such: ``volume_render_exact`` (the true adjoint of
compositing) and ``integrate_depths(..., vol_bbox=, voxel_size=)`` (a fixed
box instead of the data-driven one).
"""
import torch
import torch.nn as nn
from torch.autograd import Function

from .dist import VoxelEncoding

MAX_VOL_DIST = 999999


def _dev_id(t):
    return t.device.index if t.device.index is not None else torch.cuda.current_device()


# voxel_encoding_helper.py:12-59
class _voxel_tri_interpolation(Function):

    @staticmethod
    def forward(ctx, octree, ray_ori, ray_dir, sampled_depths, sampled_idx, sampled_feats):
        assert (not ray_ori.requires_grad) and (not ray_dir.requires_grad) \
            and (not sampled_depths.requires_grad) and (not sampled_idx.requires_grad), "Not supported"
        sampled_feats = sampled_feats.float()
        ctx.octree = octree
        ctx.ray_ori, ctx.ray_dir = ray_ori, ray_dir
        ctx.sampled_depths, ctx.sampled_idx = sampled_depths, sampled_idx
        ctx.save_for_backward(sampled_feats)
        return octree.trilinear_aggregate_features(ray_ori, ray_dir, sampled_depths, sampled_idx, sampled_feats)

    @staticmethod
    def backward(ctx, grad_output_feats):
        sampled_feats, = ctx.saved_tensors
        grad = ctx.octree.trilinear_aggregate_features_backward(
            ctx.ray_ori, ctx.ray_dir, ctx.sampled_depths, ctx.sampled_idx, sampled_feats,
            grad_output_feats.contiguous())
        if not ctx.needs_input_grad[5]:
            grad = None
        return None, None, None, None, None, grad


voxel_trilinear_interpolation = _voxel_tri_interpolation.apply


# voxel_encoding_helper.py:62-80
class _volume_rendering_inference(Function):

    @staticmethod
    def forward(ctx, depths, sigmas, feats, t_thres=1e-4):
        return VoxelEncoding.volume_rendering_occ_forward(depths.float(), sigmas.float(), feats.float(),
                                                          _dev_id(depths), t_thres)

    @staticmethod
    def backward(ctx, grad_output_feats, grad_output_depths, grad_ws, grad_alphas):
        return None, None, None, None


volume_render_infer = _volume_rendering_inference.apply


# voxel_encoding_helper.py:83-127
class _volume_render_training(Function):

    @staticmethod
    def forward(ctx, depths, depth_sort_idxs, sigmas, feats, t_thres=1e-4, using_occ=True):
        depths, sigmas, feats = depths.float(), sigmas.float(), feats.float()
        ctx.depths, ctx.depth_sort_idxs = depths, depth_sort_idxs
        ctx.t_thres, ctx.using_occ = t_thres, using_occ
        outs = VoxelEncoding.volume_rendering_training_forward(depths, depth_sort_idxs, sigmas, feats,
                                                               _dev_id(depths), t_thres, using_occ)
        ctx.save_for_backward(sigmas, feats, *outs)
        return outs

    @staticmethod
    def backward(ctx, grad_output_feats, grad_output_depths, grad_ws, grad_alphas):
        sigmas, feats, of, od, ows, oa = ctx.saved_tensors
        gf, gs = VoxelEncoding.volume_rendering_training_backward(
            grad_output_feats, grad_output_depths, grad_ws, grad_alphas, of, od, ows, oa, ctx.depths,
            ctx.depth_sort_idxs, sigmas, feats, _dev_id(ctx.depths), ctx.t_thres, ctx.using_occ)
        return (None, None, gs if ctx.needs_input_grad[2] else None, gf if ctx.needs_input_grad[3] else None,
                None, None)


volume_render = _volume_render_training.apply


class _volume_render_exact(Function):
    """Addition: compositing whose backward is the true derivative of the
    forward (transmittance and prefix sums recomputed per ray from the inputs;
    no per-sample state saved).  Same forward as ``volume_render``."""

    @staticmethod
    def forward(ctx, depths, depth_sort_idxs, sigmas, feats, t_thres=1e-4, using_occ=False):
        depths, sigmas, feats = depths.float(), sigmas.float(), feats.float()
        ctx.depths, ctx.depth_sort_idxs = depths, depth_sort_idxs
        ctx.t_thres, ctx.using_occ = t_thres, using_occ
        outs = VoxelEncoding.volume_rendering_training_forward(depths, depth_sort_idxs, sigmas, feats,
                                                               _dev_id(depths), t_thres, using_occ)
        ctx.save_for_backward(sigmas, feats)
        return outs

    @staticmethod
    def backward(ctx, grad_output_feats, grad_output_depths, grad_ws, grad_alphas):
        sigmas, feats = ctx.saved_tensors
        z = torch.zeros(1, device=sigmas.device)
        B, Nr = ctx.depths.shape[:2]

        def g(t, shape):
            return torch.zeros(shape, device=sigmas.device) if t is None else t

        gf, gs = VoxelEncoding.volume_rendering_training_backward(
            g(grad_output_feats, (B, Nr, feats.shape[-1])), g(grad_output_depths, (B, Nr, 1)),
            g(grad_ws, (B, Nr, 1)), g(grad_alphas, (B, Nr, 1)), z, z, z, z, ctx.depths, ctx.depth_sort_idxs,
            sigmas, feats, _dev_id(ctx.depths), ctx.t_thres, ctx.using_occ, exact=True)
        return (None, None, gs if ctx.needs_input_grad[2] else None, gf if ctx.needs_input_grad[3] else None,
                None, None)


volume_render_exact = _volume_render_exact.apply


# voxel_encoding_helper.py:130-189: the reference's plain-PyTorch compositing
# (its training path, SRONet/BasicRenNet.py:314-316).
class _volume_render_torch(nn.Module):

    def forward(self, sampled_depths, sigma, feats, max_depths, valid_rays=None):
        B, Nr, S = sampled_depths.shape
        zz = sampled_depths.view(-1, S)
        density = sigma.view(-1, S)
        dists = zz[:, 1:] - zz[:, :-1]
        dists = torch.cat([dists, torch.zeros(dists.shape[0], 1, device=dists.device)], -1)  # last = 0
        energy = dists * density
        shifted = torch.cat([torch.zeros(dists.shape[0], 1, device=dists.device), energy], -1)
        alpha = 1 - torch.exp(-energy)
        trans = torch.exp(-torch.cumsum(shifted, dim=-1))
        weights = (alpha * trans[:, :-1]).view(B, Nr, S, 1)
        depths = torch.sum(weights * sampled_depths[..., None], -2)
        alphas = torch.sum(weights * alpha.view(B, Nr, S, 1), -2)
        feats = torch.sum(weights * feats, -2)
        ws = torch.sum(weights, -2)
        if valid_rays is not None:
            inv = (1 - valid_rays[..., None].int()).bool()
            depths[inv] = 0
            feats[inv.repeat(1, 1, feats.shape[-1])] = 0
            alphas[inv] = 0
            ws[inv] = 0
        return feats, depths, ws, alphas

    def forward_occ(self, sampled_depths, sigma, feats, max_depths, valid_rays=None):
        B, Nr, S = sampled_depths.shape
        alpha = sigma.view(-1, S)
        eps = 1e-6
        ones = torch.ones((alpha.shape[0], 1), device=alpha.device)
        weights = alpha * torch.cumprod(torch.cat([ones, 1. - alpha + eps], -1), -1)[:, :-1]
        weights = weights.view(B, Nr, S, 1)
        depths = torch.sum(weights * sampled_depths[..., None], -2)
        alphas = torch.sum(weights * alpha.view(B, Nr, S, 1), -2)
        feats = torch.sum(weights * feats, -2)
        ws = torch.sum(weights, -2)
        if valid_rays is not None:
            inv = (1 - valid_rays[..., None].int()).bool()
            depths[inv] = 0
            feats[inv.repeat(1, 1, feats.shape[-1])] = 0
            alphas[inv] = 0
            ws[inv] = 0
        return feats, depths, ws, alphas


volume_render_torch = _volume_render_torch()


# voxel_encoding_helper.py:206-294
class _integrate_depths(nn.Module):
    """Pack colours, fuse depths into the level-0 volume, build coarse levels."""

    def preprocess_data(self, batch_size, inputs_data):
        colors, depths, masks, Ks, RTs = inputs_data
        h, w = depths.shape[-2:]
        num_views = depths.shape[0] // batch_size
        colors = torch.floor(colors[:, 2] * 256.0 * 256.0 + colors[:, 1] * 256.0 + colors[:, 0])
        if len(depths.shape) == 4:
            depths = depths[:, 0]
        if len(masks.shape) == 4:
            masks = masks[:, 0]
        depths = depths.reshape(-1, num_views, h, w).contiguous()
        colors = colors.reshape(-1, num_views, h, w).contiguous()
        masks = masks.reshape(-1, num_views, h, w).contiguous().int()
        Ks = Ks.reshape(-1, num_views, 3, 3).contiguous()
        RTs = RTs.reshape(-1, num_views, 3, 4).contiguous()
        Rs = RTs[..., :3, :3].contiguous()
        Ts = RTs[..., :3, -1].contiguous()
        return colors, depths, masks, Ks, RTs, Rs, Ts

    def clear_vol_buf(self, volumes, _level_volumes):
        occ, cnt = volumes
        for i in range(_level_volumes):
            occ[i].fill_(-1)
            cnt[i].fill_(0)
        return occ, cnt

    @torch.no_grad()
    def forward(self, inputs_data, volumes, batch_size=1, _obs_weight=1.0, _th_bbox=0.025, _tsdf_th_low=8.0,
                _tsdf_th_high=8.0, _level_volumes=6, _volume_res_rate=2, build_octree=True, _trunc_weight=3.0,
                vol_bbox=None, voxel_size=None):
        colors, depths, masks, Ks, RTs, Rs, Ts = self.preprocess_data(batch_size, inputs_data)
        occ, cnt = self.clear_vol_buf(volumes, _level_volumes)
        gpu_id = _dev_id(colors)
        if vol_bbox is None:
            tsdf_vol, _, color_vol, vol_origin, vol_bbox, voxel_size = VoxelEncoding.integrate(
                occ[0], cnt[0], Ks, RTs, Rs, Ts, colors, depths, masks, _obs_weight, _th_bbox, _trunc_weight,
                _tsdf_th_low, _tsdf_th_high, gpu_id)
        else:  # addition: fixed box
            tsdf_vol, _, color_vol = VoxelEncoding.integrate_in_box(
                occ[0], cnt[0], Ks, RTs, colors, depths, vol_bbox, voxel_size, _obs_weight, _trunc_weight,
                _tsdf_th_low, _tsdf_th_high, gpu_id)
            vol_origin = vol_bbox
        if build_octree:
            VoxelEncoding.build_multi_res_volumes(occ, cnt, _level_volumes, _volume_res_rate, gpu_id)
        return occ, cnt, tsdf_vol, color_vol, vol_origin, vol_bbox, voxel_size


integrate_depths = _integrate_depths()


# voxel_encoding_helper.py:535-662
class OcTreeOptions(nn.Module):

    def __init__(self, levels=6, batch_size=1, rate=2, vol_dim=256, n_max_hits=512, device='cuda:0'):
        super().__init__()
        self._levels, self._batch_size, self._rate = levels, batch_size, rate
        self._gpu_id = torch.device(device).index or 0
        self._octree = VoxelEncoding.MultiLayerOctree(levels, batch_size, rate, self._gpu_id)
        self._vol_dim = (vol_dim, vol_dim, vol_dim)
        self._n_max_hits = n_max_hits
        self._n_max_hits_coarse = None

    @torch.no_grad()
    def _init_octree(self, _occupied_volumes, _num_occ_voxels, _voxel_size, _vol_bbox):
        self._vol_dim = _occupied_volumes[0].shape[-3:]
        assert len(_occupied_volumes) == self._levels and len(_num_occ_voxels) == self._levels
        totals, index = [], []
        for i, nv in enumerate(_num_occ_voxels):
            totals.append(int(torch.sum(nv)))
            index.append(sum(totals[:i]))
        self._octree.init_octree(_occupied_volumes, totals, _num_occ_voxels, index, _voxel_size, _vol_bbox)
        self._octree.build_octree()
        return totals, index

    @torch.no_grad()
    def _ray_intersection(self, _ray_ori, _ray_dir, _instersect_start_level=1, th_early_stop=-1,
                          only_voxel_traversal=True, is_training=False, opt_num_intersected_voxels=-1):
        # coarse rows: three cells per coarse-grid edge (voxel_encoding_helper.py:573)
        self._n_max_hits_coarse = self._vol_dim[0] * 3 // self._rate ** (self._levels - _instersect_start_level - 1)
        if only_voxel_traversal:
            self._n_max_hits_coarse = 1024
            return self._octree.voxel_traversal(_ray_ori, _ray_dir, self._n_max_hits_coarse,
                                                _instersect_start_level, th_early_stop, is_training,
                                                opt_num_intersected_voxels)
        return self._octree.octree_traversal(_ray_ori, _ray_dir, self._n_max_hits_coarse, self._n_max_hits,
                                             _instersect_start_level, th_early_stop, opt_num_intersected_voxels)

    @torch.no_grad()
    def _sort_sampling(self, sampled_depths):
        return self._octree.sort_samplings(sampled_depths)

    @torch.no_grad()
    def _ray_voxels_sampling_points(self, _idx, _min_depths, _max_depths, _ray_total_valid_len, _uniform_noise,
                                    _instersect_start_level, _n_sampled_points):
        return self._octree.ray_voxels_points_sampling(_idx, _min_depths, _max_depths, _ray_total_valid_len,
                                                       _uniform_noise, _instersect_start_level, _n_sampled_points)

    @torch.no_grad()
    def _ray_voxels_points_sampling_coarse(self, _idx, _min_depths, _max_depths, _uniform_noise,
                                           _ray_total_valid_len, _instersect_start_level, _n_sampled_points):
        return self._octree.ray_voxels_points_sampling_coarse(_idx, _min_depths, _max_depths, _uniform_noise,
                                                              _ray_total_valid_len, _instersect_start_level,
                                                              _n_sampled_points)

    def init_octree(self, occupied_volumes, num_occ_voxels, voxel_size, vol_bbox):
        return self._init_octree(occupied_volumes, num_occ_voxels, voxel_size, vol_bbox)

    def ray_intersection(self, ray_ori, ray_dir, instersect_start_level=1, th_early_stop=-1,
                         only_voxel_traversal=True, is_training=False, opt_num_intersected_voxels=-1):
        return self._ray_intersection(ray_ori, ray_dir, instersect_start_level, th_early_stop,
                                      only_voxel_traversal, is_training, opt_num_intersected_voxels)

    def ray_voxels_sampling_points(self, idx, min_depths, max_depths, ray_total_valid_len, uniform_noise,
                                   instersect_start_level=1, n_sampled_points=128):
        return self._ray_voxels_sampling_points(idx, min_depths, max_depths, ray_total_valid_len, uniform_noise,
                                                instersect_start_level, n_sampled_points)

    def ray_voxels_points_sampling_coarse(self, idx, min_depths, max_depths, uniform_noise, ray_total_valid_len,
                                          instersect_start_level=1, n_sampled_points=128):
        return self._ray_voxels_points_sampling_coarse(idx, min_depths, max_depths, uniform_noise,
                                                       ray_total_valid_len, instersect_start_level,
                                                       n_sampled_points)

    def sort_sampling(self, _sampled_depths):
        return self._sort_sampling(_sampled_depths)

    @torch.no_grad()
    def get_all_nodes(self):
        return self._octree.get_nodes_tensor()

    @torch.no_grad()
    def get_octree(self):
        return self._octree
