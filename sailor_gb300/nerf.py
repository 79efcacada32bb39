"""FastNerf's occupancy network through the library's tensor-core kernel.

Drop-in for the FastNerf extension's ``infer_density`` binding
(c_lib/FastNerf/src/binding.cpp:9 -> infer_density_mlp,
c_lib/FastNerf/src/infer_mlp.cu:583-636): same arguments and result.
"""
import torch

from . import _native as N


def _in(t, name, dtype):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a cuda tensor")
    return t.to(dtype).contiguous()


def infer_density(points_z, points_tpsdf, sampled_feats_geo, net_params_density, batch_size, num_points, num_views,
                  device, return_geo=False):
    """points_z / points_tpsdf [B, V, ..., 1], sampled_feats_geo [B, V, ..., 16]
    (num_points entries per view), net_params_density float16
    [sg_nerf_param_count()].  Returns the densities [B, 1, num_points]
    (and, with return_geo, the geometry features [B, V, num_points, 8], which
    the reference computes and drops)."""
    B, Np, V = int(batch_size), int(num_points), int(num_views)
    with torch.cuda.device(torch.device("cuda", int(device))):
        z = _in(points_z, "points_z", torch.float32)
        tp = _in(points_tpsdf, "points_tpsdf", torch.float32)
        geo = _in(sampled_feats_geo, "sampled_feats_geo", torch.float32)
        params = _in(net_params_density, "net_params_density", torch.float16)
        if params.numel() != N.lib.sg_nerf_param_count():
            raise RuntimeError(f"net_params_density holds {params.numel()} values, the network "
                               f"{N.lib.sg_nerf_param_count()}")
        if z.numel() != B * V * Np or tp.numel() != B * V * Np or geo.numel() != B * V * Np * 16:
            raise RuntimeError(f"inputs must hold [{B}, {V}, {Np}] points (16 geometry features each)")
        dens = torch.empty((B, 1, Np), device=z.device)
        geo_out = torch.empty((B, V, Np, 8), device=z.device) if return_geo else None
        err = torch.zeros(1, dtype=torch.int32, device=z.device)
        N.check(N.lib.sg_nerf_density(N.ptr(params), N.ptr(z), N.ptr(tp), N.ptr(geo), B, Np, V, N.ptr(dens),
                                      N.ptr(geo_out), N.ptr(err), N.stream()), "nerf_density")
        if err.item():
            raise RuntimeError("nerf_density: a tensor-core wait timed out")
        return (dens, geo_out) if return_geo else dens


def occupancy_compositing(sorted_depths, occupancies, feats, t_thres, device):
    """FastNerf's occupancy compositing (volume_rendering_occ_kernel,
    c_lib/FastNerf/src/infer_mlp.cu:508-580): pre-sorted depths [B, R, S]
    (-1 for none), occupancies [B, R, S(, 1)] used as alphas, features
    [B, R, S, C] (C <= 32; FastNerf composites 30) -> (features [B, R, C],
    depths [B, R, 1]); rays whose last depth is negative give zeros, and a
    ray stops after the sample that takes its transmittance below t_thres."""
    from .voxel_encoding import volume_rendering_occ_forward
    occ = occupancies if occupancies.dim() == 4 else occupancies.unsqueeze(-1)
    f, d, _, _ = volume_rendering_occ_forward(sorted_depths, occ, feats, device, t_thres)
    return f, d
