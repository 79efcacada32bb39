"""Error paths that the device reports (no GPU fault involved), and the
plain-PyTorch compositing mirror against the CUDA compositing.

* Hit-row overflow: rows narrower than a ray's hit count.  The traversal
  writes the first W hits (the oracle's first W, bit for bit) and never past
  the row, counts every hit, and reports SG_FLAG_HIT_OVERFLOW with the
  largest hit count in SgStatus (the oracle's count); the drop-in sampling
  call that reads those rows then raises RuntimeError (the reference has no
  check and reads a truncated row).  The batched intersection reports the
  same, and the render over overflowed rows reads only the first W hits.
* volume_render_torch (voxel_encoding_helper.py:132-186, the reference's
  training-path compositing: last delta 0, transmittance exp(-cumsum))
  equals the CUDA compositing kernel when the two conventions coincide: all
  samples valid and sorted, no early termination (t_thres 0), and the last
  sample's density 0 for the kernel (its alpha is then 0 under either last
  delta).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


@pytest.fixture(scope="module")
def scene():
    from test_gpu_parity import gpu_chain
    D, rate, S = 128, 4, 32
    sc = syn.make_scene(seed=71, n_views=4, res=192, n_prims=12, D=D, trunc=0.03)
    ori, dirs = syn.target_rays(seed=71, res=64)
    R = ori.shape[1]
    rands = np.full((1, R, S), 0.5, np.float32)
    g = gpu_chain(sc, D, rate, S, ori, dirs, rands, 256)
    ref = orc.chain(sc, D, rate, S, ori, dirs, rands, W=256, trunc_weight=sc["trunc_weight"])
    return dict(sc=sc, ori=ori, dirs=dirs, g=g, ref=ref, S=S, rands=rands)


def test_hit_row_overflow_drop_in(scene):
    from sailor_gb300 import _native as N
    g, h = scene["g"], scene["ref"]["hits"]
    octree = g["octree"]
    W = 4
    assert h["max_hits"] > W
    idx, t0, t1, vl = octree.voxel_traversal(_t(scene["ori"]), _t(scene["dirs"]), W, 0, -1, False, -1)
    torch.cuda.synchronize()
    st = octree._status.cpu().numpy()
    assert st[0] & N.SG_FLAG_HIT_OVERFLOW
    assert st[1] == h["max_hits"], (st[1], h["max_hits"])
    ok = h["flags"] == 0
    # the first W hits of every unflagged ray, and the -1 padding of shorter rows
    assert np.array_equal(idx.cpu().numpy()[ok], h["idx"][..., :W][ok])
    assert np.abs(t0.cpu().numpy()[ok] - h["t0"][..., :W][ok]).max() <= 1e-5  # __fdividef vs exact reciprocal
    # valid lengths count every hit, as the reference's do
    assert np.abs(vl.cpu().numpy()[..., 0][ok] - h["valid_len"][..., 0][ok]).max() <= 1e-4
    with pytest.raises(RuntimeError, match="overflow"):
        octree.ray_voxels_points_sampling_coarse(idx, t0, t1, _t(scene["rands"]), vl, 0, scene["S"])
    # wide rows again: the status is cleared and sampling runs
    idx, t0, t1, vl = octree.voxel_traversal(_t(scene["ori"]), _t(scene["dirs"]), 256, 0, -1, False, -1)
    octree.ray_voxels_points_sampling_coarse(idx, t0, t1, _t(scene["rands"]), vl, 0, scene["S"])
    assert not (octree._status[0].item() & N.SG_FLAG_HIT_OVERFLOW)


def test_hit_row_overflow_batched():
    """sg_intersect_segments with rows of 3 hits: the status carries the flag
    and the largest count, hit_count keeps the full count, the rows hold the
    first 3 hits of a wide-row run, and the forward render reads only
    those (its output equals a render of the wide rows cut to 3 hits)."""
    from sailor_gb300 import _native as N
    from sailor_gb300.batch import BatchPipeline
    w = syn.make_batch_workload(seed=4, n_frames=2, views=(2, 3), view_res=(96, 128), n_prims=8, D=64,
                                trunc=0.04, n_targets=2, target_res=(48, 64), target_S=(32, 64))
    view_hw = [[d.shape for d in fr["depth"]] for fr in w["frames"]]
    targets = [(t["frame"], t["ori"].shape[0], t["S"]) for t in w["targets"]]
    pipes = {}
    for Wh in (96, 3):
        bp = BatchPipeline(view_hw, targets, D=64, rate=4, C=3, W_hits=Wh)
        bp.load_views(w["frames"], w["vol_bbox"], w["voxel_size"], w["trunc_weight"])
        bp.load_rays([(t["ori"], t["dir"]) for t in w["targets"]])
        bp.set_fields(feat=torch.rand((bp.B, 64, 64, 64, 3), device="cuda", generator=torch.Generator(
            device="cuda").manual_seed(3)))
        bp.render_args(float(w["voxel_size"][0]) * w["trunc_weight"], sdf_s=0.01)
        bp.build()
        bp.intersect()
        torch.cuda.synchronize()
        pipes[Wh] = bp
    wide, narrow = pipes[96], pipes[3]
    cnt = wide.hit_count.cpu().numpy()
    assert cnt.max() > 3 and not (wide.status[0].item() & N.SG_FLAG_HIT_OVERFLOW)
    st = narrow.status.cpu().numpy()
    assert st[0] & N.SG_FLAG_HIT_OVERFLOW and st[1] == cnt.max()
    assert np.array_equal(narrow.hit_count.cpu().numpy(), cnt)
    k = np.minimum(cnt, 3)
    for name in ("hit_idx", "hit_t0", "hit_t1"):
        a, b = getattr(narrow, name).cpu().numpy(), getattr(wide, name).cpu().numpy()[:, :3]
        m = np.arange(3)[None, :] < k[:, None]
        assert np.array_equal(a[m], b[m]), name
    # the wide rows cut to 3 hits (count clamped) render like the narrow rows
    wide.hit_count.clamp_(max=3)
    wide.valid_len.copy_(narrow.valid_len)
    outs = []
    for bp in (narrow, wide):
        bp.forward()
        torch.cuda.synchronize()
        outs.append(bp.out_rgb.clone())
    assert torch.equal(outs[0], outs[1])


def test_volume_render_torch_matches_cuda():
    from sailor_gb300.dist import VoxelEncoding as VE
    from sailor_gb300.voxel_encoding_helper import volume_render_torch
    rng = np.random.default_rng(5)
    B, Nr, S = 2, 500, 48
    z = np.sort(rng.uniform(1.0, 3.0, (B, Nr, S)), -1).astype(np.float32)
    sig = rng.uniform(0, 60, (B, Nr, S, 1)).astype(np.float32)
    feats = rng.random((B, Nr, S, 3), dtype=np.float32)
    zt, st, ft = _t(z), _t(sig), _t(feats)
    tf, td, tw, ta = volume_render_torch(zt, st, ft, None)
    sig0 = sig.copy()
    sig0[..., -1, :] = 0.0  # the last alpha is 0 under either last delta
    idx = torch.arange(S, dtype=torch.int32, device="cuda").expand(B, Nr, S).contiguous()
    cf, cd, cw, ca = VE.volume_rendering_training_forward(zt, idx, _t(sig0), ft, 0, 0.0, False)
    torch.cuda.synchronize()
    assert (tf - cf).abs().max().item() <= 1e-5
    assert (td - cd).abs().max().item() <= 1e-5 * 3.0
    assert (tw - cw).abs().max().item() <= 1e-5
    assert (ta - ca).abs().max().item() <= 1e-5
    assert cw.max().item() > 0.5
