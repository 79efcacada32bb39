"""Differentiable trilinear gathers from dense per-voxel grids.

The reference's trilinear aggregation (``_voxel_tri_interpolation``,
c_lib/VoxelEncoding/voxel_encoding_helper.py:12-59) interpolates per-node
corner features; these Functions interpolate a dense grid instead and send
gradients back into that grid (``sg_grid_scatter``), so a feature grid or the
fused TSDF grid can be optimised through compositing.

Grids are channel-last ``[B, D, D, D, C]`` (C in 1, 3, 4, 8, 16; ``[B, D, D,
D]`` means C = 1) over each frame's ``vol_bbox [B, 3, 2]`` / ``voxel_size
[B]``; voxel (x, y, z) sits at ``bbox_min + (x, y, z) * voxel_size``.  The
point of sample (b, n, s) is ``ray_ori[b, n] + z[b, n, s] * ray_dir[b, n]``;
samples with z < 0 give 0 and receive no gradient.
"""
import torch
from torch.autograd import Function

from . import _native as N
from .voxel_encoding import _in


def _shapes(grid, ray_ori, sampled_depths):
    if grid.dim() == 4:
        grid = grid.unsqueeze(-1)
    if grid.dim() != 5 or grid.shape[1] != grid.shape[2] or grid.shape[1] != grid.shape[3]:
        raise RuntimeError("grid must be [B, D, D, D, C]")
    B, D, C = grid.shape[0], grid.shape[1], grid.shape[4]
    if ray_ori.shape[0] != B or sampled_depths.shape[:2] != ray_ori.shape[:2]:
        raise RuntimeError("ray_ori [B, N, 3] and sampled_depths [B, N, S] must share B and N with the grid")
    return grid, B, D, C, ray_ori.shape[1], sampled_depths.shape[2]


def _gather(grid, ray_ori, ray_dir, z, vol_bbox, voxel_size, mode, scale, s):
    grid, B, D, C, Nr, S = _shapes(grid, ray_ori, z)
    grid = _in(grid, "grid")
    ori, dirs, z = _in(ray_ori, "ray_ori"), _in(ray_dir, "ray_dir"), _in(z, "sampled_depths")
    bbox, vs = _in(vol_bbox, "vol_bbox"), _in(voxel_size, "voxel_size")
    out = torch.empty((B, Nr, S, C), dtype=torch.float32, device=z.device)
    with torch.cuda.device(z.device):
        N.check(N.lib.sg_grid_gather(N.ptr(ori), N.ptr(dirs), N.ptr(z), B, Nr, S, N.ptr(grid), D, C, N.ptr(bbox),
                                     N.ptr(vs), mode, float(scale), float(s), N.ptr(out), N.stream()),
                "grid_gather")
    return out, (grid, ori, dirs, z, bbox, vs)


def _scatter(saved, gout, mode, scale, s, grid_shape):
    grid, ori, dirs, z, bbox, vs = saved
    B, D, C = grid.shape[0], grid.shape[1], grid.shape[4]
    Nr, S = z.shape[1], z.shape[2]
    gout = gout.float().contiguous()
    ggrid = torch.zeros(grid.shape, dtype=torch.float32, device=grid.device)
    with torch.cuda.device(z.device):
        N.check(N.lib.sg_grid_scatter(N.ptr(ori), N.ptr(dirs), N.ptr(z), B, Nr, S, N.ptr(gout),
                                      N.ptr(grid) if mode == 1 else None, D, C, N.ptr(bbox), N.ptr(vs), mode,
                                      float(scale), float(s), N.ptr(ggrid), N.stream()), "grid_scatter")
    return ggrid.reshape(grid_shape)


class _GridGather(Function):
    @staticmethod
    def forward(ctx, grid, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size):
        out, saved = _gather(grid, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size, 0, 1.0, 1.0)
        ctx.saved = saved
        ctx.grid_shape = grid.shape
        return out

    @staticmethod
    def backward(ctx, gout):
        ggrid = _scatter(ctx.saved, gout, 0, 1.0, 1.0, ctx.grid_shape) if ctx.needs_input_grad[0] else None
        return ggrid, None, None, None, None, None


class _TsdfDensity(Function):
    @staticmethod
    def forward(ctx, tsdf, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size, scale, s):
        out, saved = _gather(tsdf, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size, 1, scale, s)
        ctx.saved, ctx.scale, ctx.s = saved, scale, s
        ctx.grid_shape = tsdf.shape
        return out[..., 0]

    @staticmethod
    def backward(ctx, gout):
        ggrid = None
        if ctx.needs_input_grad[0]:
            ggrid = _scatter(ctx.saved, gout.unsqueeze(-1), 1, ctx.scale, ctx.s, ctx.grid_shape)
        return ggrid, None, None, None, None, None, None, None


def grid_gather(grid, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size):
    """Trilinear features [B, N, S, C] of a dense grid at the samples;
    differentiable with respect to the grid."""
    return _GridGather.apply(grid, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size)


def tsdf_density(tsdf, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size, scale, s):
    """Density sigmoid(-t * scale / s) / s [B, N, S] of the trilinear TSDF t
    at the samples (scale: the truncation margin in metres that turns the
    normalised TSDF into metres; s: the density's length scale);
    differentiable with respect to the TSDF grid."""
    return _TsdfDensity.apply(tsdf, ray_ori, ray_dir, sampled_depths, vol_bbox, voxel_size, scale, s)
