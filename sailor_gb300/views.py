"""Projection of points into the source views and the gather of per-view 2D
feature maps at the projections: the step of SRONet's render after sampling.

Drop-ins, with the reference's arguments and results:

* ``proj_persp`` for ``utils_render.proj_persp``
  (utils_render/utils_render.py:380-414);
* ``forward_sample_feature`` for ``BasicRenNet.forward_sample_feature``
  (SRONet/BasicRenNet.py:245-259): four ``F.grid_sample`` calls
  (bilinear, align_corners=True, zero padding) and the clamped depth
  difference t_psdf;

and the fused form ``project_sample_features``, both steps in one launch
(the projected grids never leave the SM).  Every call runs
``sg_project_gather`` of ``libsailor_gb300.so`` on the current CUDA stream;
there is no CPU path.  Feature maps are read through their strides, so NCHW
tensors and channels-last ones (``memory_format=torch.channels_last``, read
with 16-byte vectors when C % 4 == 0) both work.
"""
import ctypes as C

import torch

from . import _native as N

__all__ = ["proj_persp", "forward_sample_feature", "project_sample_features"]

PSDF_CLIP = 0.01  # clamp of proj_z - sampled depth (BasicRenNet.py:250)


def _f32(t, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} input must be a cuda tensor")
    if t.dtype != torch.float32:
        raise RuntimeError(f"{name} must be float32, got {t.dtype}")
    return t


def _cams(K, R, T, n_images):
    K = _f32(K, "K").reshape(n_images, 9).contiguous()
    R = _f32(R, "R").reshape(n_images, 9).contiguous()
    T = _f32(T, "T").reshape(n_images, 3).contiguous()
    return K, R, T


def _map(a, img, N_pts):
    """SgFeatureMap of a [n_images, C, H, W] map and its [n_images, N, C] output."""
    if img.dim() != 4:
        raise RuntimeError("feature maps must be [n_images, C, H, W]")
    _f32(img, "feature map")
    n, Cm, H, W = img.shape
    out = torch.empty((n, N_pts, Cm), device=img.device)
    m = N.SgFeatureMap()
    m.data = img.data_ptr()
    for k in range(4):
        m.stride[k] = img.stride(k)
    m.C, m.H, m.W = Cm, H, W
    m.out = out.data_ptr()
    return m, out


def _launch(a, keep):
    N.check(N.lib.sg_project_gather(C.byref(a), N.stream()), "project_gather")
    return keep


def _persp_args(a, points, K, R, T, p_depths, n_views, depth_thres, min_d, max_d, res):
    pts = _f32(points, "points")
    if pts.dim() != 3 or pts.shape[1] != 3:
        raise RuntimeError("points must be [batch, 3, N]")
    n_images = K.shape[0] if K.dim() == 3 else K.numel() // 9
    Bp = pts.shape[0]
    if p_depths is not None:
        div = n_views  # proj_persp repeats the points over the views
        if Bp * n_views != n_images:
            raise RuntimeError(f"points batch {Bp} x {n_views} views != {n_images} cameras")
    elif Bp == n_images:
        div = 1
    elif Bp == 1:
        div = n_images  # broadcast
    else:
        raise RuntimeError(f"points batch {Bp} does not broadcast against {n_images} cameras")
    Kc, Rc, Tc = _cams(K, R, T, n_images)
    a.points = pts.data_ptr()
    a.points_stride[0], a.points_stride[1], a.points_stride[2] = pts.stride(0), pts.stride(1), pts.stride(2)
    a.points_div = div
    keep = [pts, Kc, Rc, Tc]
    if p_depths is not None:
        pd = _f32(p_depths, "p_depths")
        a.p_depths = pd.data_ptr()
        a.p_depths_stride[0], a.p_depths_stride[1] = pd.stride(0), pd.stride(-1)
        keep.append(pd)
    a.K, a.R, a.T = Kc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()
    a.n_images, a.num_points = n_images, pts.shape[2]
    a.depth_thres, a.min_d, a.max_d = float(depth_thres), float(min_d), float(max_d)
    a.half_res = float(int(res) // 2)
    a.psdf_map = -1
    return keep


def proj_persp(points, K, R, T, p_depths, n_views, depth_thres=0.01, min_d=0.1, max_d=4.0, res=512):
    """points [batch, 3, N]; K, R [batch*n_views, 3, 3]; T [batch*n_views, 3, 1]
    -> (ori_pts [n_images, 3, N] = R p + T, grids [n_images, 2, N] in
    [-1, 1] (-2: behind depth_thres, or p_depth outside [min_d, max_d]),
    depth [n_images, 1, N] (-2 for the latter))."""
    a = N.SgProjGather()
    keep = _persp_args(a, points, K, R, T, p_depths, n_views, depth_thres, min_d, max_d, res)
    dev = points.device
    n, Np = a.n_images, a.num_points
    ori = torch.empty((n, 3, Np), device=dev)
    grids = torch.empty((n, 2, Np), device=dev)
    depth = torch.empty((n, 1, Np), device=dev)
    a.ori_pts, a.grids, a.depth = ori.data_ptr(), grids.data_ptr(), depth.data_ptr()
    _launch(a, keep)
    return ori, grids, depth


def forward_sample_feature(feats_geo, depths, feats_rgb, rgbs_n, xy, z):
    """Maps [n_images, C, H, W]; xy [n_images, N, 1, 2] grids; z [n_images, 1, N]
    -> (geo [n_images, N, Cg], rgb feats [n_images, N, Cr], t_psdf
    [n_images, N, 1] = clamp(z - depth sample, -0.01, 0.01) / 0.01, rgbs
    [n_images, N, 3])."""
    grid = _f32(xy, "xy")
    n = grid.shape[0]
    Np = grid.numel() // (2 * n)
    g = grid.reshape(n, Np, 2).contiguous()
    zz = _f32(z, "z").reshape(n, Np).contiguous()
    a = N.SgProjGather()
    a.grids_in, a.depth_in = g.data_ptr(), zz.data_ptr()
    a.n_images, a.num_points = n, Np
    outs, keep = [], [g, zz]
    for i, img in enumerate((feats_geo, depths, feats_rgb, rgbs_n)):
        m, o = _map(a, img, Np)
        a.maps[i] = m
        outs.append(o)
        keep.append(img)
    a.n_maps = 4
    psdf = torch.empty((n, Np, 1), device=g.device)
    a.psdf_map, a.psdf_clip, a.psdf_scale, a.psdf = 1, PSDF_CLIP, 1.0 / PSDF_CLIP, psdf.data_ptr()
    _launch(a, keep)
    return outs[0], outs[2], psdf, outs[3]


def project_sample_features(points, K, R, T, p_depths, n_views, feats_geo, depths, feats_rgb, rgbs_n,
                            depth_thres=0.01, min_d=0.1, max_d=4.0, res=512, want_grids=False):
    """proj_persp + forward_sample_feature in one launch.  Returns
    (proj_z [n_images, 1, N], geo, rgb feats, t_psdf, rgbs) as the two
    reference calls give them, and the grids [n_images, 2, N] when
    want_grids."""
    a = N.SgProjGather()
    keep = _persp_args(a, points, K, R, T, p_depths, n_views, depth_thres, min_d, max_d, res)
    dev = points.device
    n, Np = a.n_images, a.num_points
    depth = torch.empty((n, 1, Np), device=dev)
    a.depth = depth.data_ptr()
    grids = None
    if want_grids:
        grids = torch.empty((n, 2, Np), device=dev)
        a.grids = grids.data_ptr()
    outs = []
    for i, img in enumerate((feats_geo, depths, feats_rgb, rgbs_n)):
        m, o = _map(a, img, Np)
        a.maps[i] = m
        outs.append(o)
        keep.append(img)
    a.n_maps = 4
    psdf = torch.empty((n, Np, 1), device=dev)
    a.psdf_map, a.psdf_clip, a.psdf_scale, a.psdf = 1, PSDF_CLIP, 1.0 / PSDF_CLIP, psdf.data_ptr()
    _launch(a, keep)
    res_ = (depth, outs[0], outs[2], psdf, outs[3])
    return res_ + (grids,) if want_grids else res_
