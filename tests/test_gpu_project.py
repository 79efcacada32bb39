"""GPU checks of the projection into the source views and the 2D feature
gather (sailor_gb300.views, MultiLayerOctree.project_sampled_xyz).

* project_sampled_xyz (sampling_kernel.cu:1333-1381) against the oracle's
  restatement of project_xyz (itself bit-exact against the reference
  kernel's output, tests/golden/ref_project.npz) on the tree and samples of
  the drop-in chain: bit for bit with half image sizes that are powers of
  two; otherwise within one ulp (the reference normalises in double
  precision) and nearly all bit for bit; -1 where a sample has no node;
* proj_persp (utils_render.py:380-414) against the oracle's float64
  restatement: within 1e-5, and the -2 markers exactly;
* forward_sample_feature (BasicRenNet.py:245-259) against torch's own
  F.grid_sample (align_corners=True) and clamp on the GPU: features within
  1e-5, t_psdf (a difference scaled by 100) within 1e-4; against the
  oracle's float64 grid_sample within 1e-4 (float32 pixel coordinates);
* channels-last maps give the NCHW results bit for bit, and the fused
  project_sample_features gives the two separate calls' results bit for bit.
"""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

CASES = [
    dict(name="r8_D128", seed=31, res=192, D=128, rate=8, S=48, tres=64, prims=12, batch=1),
    dict(name="r2_D64_b2", seed=32, res=128, D=64, rate=2, S=32, tres=48, prims=8, batch=2),
]


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


@pytest.fixture(scope="module", params=CASES, ids=[c["name"] for c in CASES])
def chain(request):
    from test_gpu_parity import gpu_chain
    c = request.param
    B = c["batch"]
    sc = syn.make_scene(seed=c["seed"], n_views=4, res=c["res"], n_prims=c["prims"], D=c["D"], trunc=0.03, batch=B)
    ori, dirs = syn.target_rays(seed=c["seed"], res=c["tres"], batch=B)
    rands = np.random.default_rng(c["seed"]).random((B, ori.shape[1], c["S"]), dtype=np.float32)
    g = gpu_chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, 1024)
    ref = orc.chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, W=1024, trunc_weight=sc["trunc_weight"])
    assert (g["si"] >= 0).mean() > 0.05 and (g["si"] < 0).any()
    return dict(c=c, sc=sc, ori=ori, dirs=dirs, g=g, ref=ref)


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-2 ** 31) - ia, ia)
    ib = np.where(ib < 0, np.int64(-2 ** 31) - ib, ib)
    return np.abs(ia - ib)


@pytest.mark.parametrize("w,h,corners", [(512, 512, True), (640, 480, True), (1024, 1024, False)])
def test_project_sampled_xyz_matches_oracle(chain, w, h, corners):
    g, sc = chain["g"], chain["sc"]
    B, V = sc["K"].shape[:2]
    xy, pz = g["octree"].project_sampled_xyz(_t(chain["ori"]), _t(chain["dirs"]), _t(g["sz"]),
                                             _t(g["si"], torch.int32), _t(sc["K"]), _t(sc["RT"]), w, h, V,
                                             record_corners=corners)
    torch.cuda.synchronize()
    table = orc.node_corner_table(chain["ref"]["tree"], sc["voxel_size"], sc["vol_bbox"]) if corners else None
    rxy, rz = orc.project_xyz(chain["ori"], chain["dirs"], g["sz"], g["si"], sc["K"], sc["RT"], w, h, corners=table)
    gxy = xy.cpu().numpy().reshape(rxy.shape)
    gz = pz.cpu().numpy().reshape(rz.shape)
    assert np.array_equal(gz.view(np.uint32), rz.view(np.uint32))  # camera z: float operations alone
    none = np.broadcast_to((g["si"] == -1)[:, None, :, :, None, None], gxy.shape)
    assert (gxy[none] == -1).all() and none.any() and (~none).any()
    if (w // 2) & (w // 2 - 1) == 0 and (h // 2) & (h // 2 - 1) == 0:
        assert np.array_equal(gxy.view(np.uint32), rxy.view(np.uint32))
    else:
        u = _ulps(gxy, rxy)
        assert u.max() <= 1 and (u == 0).mean() > 0.999


def _cams(sc):
    B, V = sc["K"].shape[:2]
    K = sc["K"].reshape(B * V, 3, 3)
    R = sc["RT"][..., :3].reshape(B * V, 3, 3)
    T = sc["RT"][..., 3:].reshape(B * V, 3, 1)
    return K, R, T, B, V


def _points(sc, seed, n=4096):
    """Points in the scene box, a few behind some cameras, and p_depths with
    some outside [0.1, 4.0]."""
    B = sc["K"].shape[0]
    rng = np.random.default_rng(seed)
    bb = sc["vol_bbox"]
    pts = np.empty((B, 3, n), np.float32)
    for b in range(B):
        lo, hi = bb[b, :, 0], bb[b, :, 1]
        pts[b] = (lo[:, None] + (hi - lo)[:, None] * rng.random((3, n))).astype(np.float32)
    pts[:, :, :16] *= np.float32(6.0)  # far outside: behind some of the ring cameras
    pd = rng.uniform(0.0, 4.5, (B, 1, n)).astype(np.float32)
    return pts, pd


@pytest.mark.parametrize("with_pd", [True, False])
def test_proj_persp_vs_oracle(chain, with_pd):
    from sailor_gb300.views import proj_persp
    sc = chain["sc"]
    K, R, T, B, V = _cams(sc)
    pts, pd = _points(sc, 5)
    if not with_pd:
        pts = np.repeat(pts, V, 0)  # one point set per view image
    ori, grids, depth = proj_persp(_t(pts), _t(K), _t(R), _t(T), _t(pd) if with_pd else None, V, res=sc["res"])
    rori, rgrids, rdepth = orc.proj_persp(pts, K, R, T, pd if with_pd else None, V, res=sc["res"])
    ori, grids, depth = ori.cpu().numpy(), grids.cpu().numpy(), depth.cpu().numpy()
    marked = rgrids == -2
    assert marked.any() and (~marked).any()
    assert (grids[marked] == -2).all() and (depth[rdepth == -2] == -2).all()
    assert np.abs(ori - rori).max() <= 1e-5 * max(1.0, np.abs(rori).max())
    assert np.abs(depth - rdepth).max() <= 1e-5 * max(1.0, np.abs(rdepth).max())
    ok = ~marked & (np.abs(rgrids) < 4.0)
    assert np.abs(grids - rgrids)[ok].max() <= 1e-5


def _maps(n, H, W, seed):
    rng = np.random.default_rng(seed)
    return [_t(rng.normal(0, 1, (n, C, H, W))) for C in (32, 1, 32, 3)]


def test_forward_sample_feature_vs_torch_and_oracle():
    from sailor_gb300.views import forward_sample_feature
    n, Np, H, W = 6, 3000, 96, 128
    rng = np.random.default_rng(7)
    maps = _maps(n, H, W, 8)
    maps[1] = _t(rng.uniform(1.0, 3.0, (n, 1, H, W)))  # depth map
    xy = rng.uniform(-1.2, 1.2, (n, Np, 1, 2)).astype(np.float32)
    xy[:, :40] = -2.0  # the invalid marker
    xy[:, 40:60, 0, 0] = 1.0  # the last column exactly
    z = rng.uniform(0.9, 3.1, (n, 1, Np)).astype(np.float32)
    z[:, :, :8] = -2.0
    geo, rgbf, psdf, rgbs = forward_sample_feature(*maps, _t(xy), _t(z))
    # torch on the GPU, as the reference calls it
    ref = [F.grid_sample(m, _t(xy), align_corners=True, mode="bilinear")[..., 0] for m in maps]
    ref_psdf = (torch.clamp(_t(z) - ref[1], -0.01, 0.01) * (1.0 / 0.01)).permute(0, 2, 1)
    for got, r in ((geo, ref[0]), (rgbf, ref[2]), (rgbs, ref[3])):
        assert (got - r.permute(0, 2, 1)).abs().max().item() <= 1e-5
    assert (psdf - ref_psdf).abs().max().item() <= 1e-4
    # float64 restatement: the float32 pixel coordinate ((x + 1) / 2 * (W - 1),
    # up to 127 here) carries ~1e-5 px of rounding, times neighbour
    # differences of O(1) in these N(0, 1) maps: within 1e-4 (torch's own
    # float32 grid_sample shows the same error)
    for got, m in ((geo, maps[0]), (rgbs, maps[3])):
        r = orc.grid_sample(m.cpu().numpy(), xy.reshape(n, Np, 2))
        assert np.abs(got.cpu().numpy() - r).max() <= 1e-4


def test_channels_last_and_fused_match(chain):
    from sailor_gb300.views import forward_sample_feature, proj_persp, project_sample_features
    sc = chain["sc"]
    K, R, T, B, V = _cams(sc)
    pts, pd = _points(sc, 9, n=5000)
    H = W = sc["res"]
    maps = _maps(B * V, H, W, 10)
    maps[1] = _t(np.random.default_rng(11).uniform(1.0, 3.0, (B * V, 1, H, W)))
    args = (_t(pts), _t(K), _t(R), _t(T), _t(pd), V)
    _, grids, depth = proj_persp(*args, res=sc["res"])
    xy = grids.permute(0, 2, 1).reshape(B * V, -1, 1, 2)
    sep = forward_sample_feature(*maps, xy, depth)
    cl = forward_sample_feature(*[m.contiguous(memory_format=torch.channels_last) for m in maps], xy, depth)
    fused = project_sample_features(*args, *maps, res=sc["res"], want_grids=True)
    torch.cuda.synchronize()
    assert torch.equal(fused[0], depth) and torch.equal(fused[5], grids)
    for a, b_, c in zip(sep, cl, fused[1:5]):
        assert torch.equal(a, b_) and torch.equal(a, c)
    assert sep[0].abs().max().item() > 0
