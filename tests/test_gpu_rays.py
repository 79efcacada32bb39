"""GPU checks of ray generation (rays_calculating, sampling_kernel.cu:674-731)
and of camera-defined ray segments in the batched pipeline.

* sg_rays_from_cameras against the oracle (itself bit-exact against the
  reference kernel's own output, tests/golden/ref_rays.npz): origins bit for
  bit; directions within one ulp (the reference normalises in double
  precision, the CUDA path in single), nearly all bit for bit;
* the drop-in VoxelEncoding.rays_calculating returns the same rays;
* a BatchPipeline whose targets are cameras (rays generated inside the
  intersection and render kernels, never stored) gives the same hits,
  outputs and gradients as one fed the generated rays as buffers.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


def _cameras(seed, B, N, H):
    rng = np.random.default_rng(seed)
    K, R, T = [], [], []
    for b in range(B):
        for v in range(N):
            if v % 2 == 0:
                K.append(syn.intrinsics(H))
                r, t = syn.ring_cameras(1, phase=rng.uniform(0, 6.3))[0]
            else:
                K.append(np.array([[rng.uniform(30, 60), rng.uniform(-2, 2), rng.uniform(15, 30)],
                                   [0.0, rng.uniform(30, 60), rng.uniform(15, 25)], [0.0, 0.0, 1.0]]))
                r, t = syn.look_at(rng.uniform(-3, 3, 3) + np.array([0, 0, 3.0]), rng.uniform(-0.3, 0.3, 3))
            R.append(r)
            T.append(t)
    f = lambda a, s: np.asarray(a, np.float32).reshape(s)  # noqa: E731
    return f(K, (B, N, 3, 3)), f(R, (B, N, 3, 3)), f(T, (B, N, 3))


def _ulps(a, b):
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-2 ** 31) - ia, ia)
    ib = np.where(ib < 0, np.int64(-2 ** 31) - ib, ib)
    return np.abs(ia - ib)


def test_rays_match_oracle():
    from sailor_gb300 import _native as N
    B, Nv, H, W = 2, 3, 40, 56
    K, R, T = _cameras(3, B, Nv, H)
    Kt, Rt, Tt = _t(K), _t(R), _t(T)
    out = torch.empty((B, Nv, H, W, 6), device="cuda")
    N.check(N.lib.sg_rays_from_cameras(N.ptr(Kt), N.ptr(Rt), N.ptr(Tt), B, Nv, H, W, N.ptr(out), N.stream()),
            "rays")
    got = out.cpu().numpy()
    ref = orc.rays(K, R, T, H, W)
    assert np.array_equal(got[..., :3].view(np.uint32), ref[..., :3].view(np.uint32))
    u = _ulps(got[..., 3:], ref[..., 3:])
    assert u.max() <= 1
    assert (u == 0).mean() > 0.99


def test_rays_calculating_dropin():
    from sailor_gb300.dist import VoxelEncoding as VE
    K, R, T = _cameras(4, 1, 2, 32)
    out = VE.rays_calculating(_t(K), _t(R), _t(T), 32, 0).cpu().numpy()
    ref = orc.rays(K, R, T, 32)
    assert out.shape == (1, 2, 32, 32, 6)
    assert np.array_equal(out[..., :3], ref[..., :3])
    assert _ulps(out[..., 3:], ref[..., 3:]).max() <= 1


def test_camera_segments_match_ray_buffers():
    from sailor_gb300 import _native as N
    from sailor_gb300.batch import BatchPipeline
    D, rate, C = 64, 4, 16
    w = syn.make_batch_workload(seed=7, n_frames=2, views=(2, 3), view_res=(96, 128), n_prims=8, D=D, trunc=0.04,
                                n_targets=3, target_res=(32, 96), target_S=(32, 64, 128))
    view_hw = [[d.shape for d in fr["depth"]] for fr in w["frames"]]
    targets = [(t["frame"], t["res"] ** 2, t["S"]) for t in w["targets"]]
    rng = np.random.default_rng(1)
    feat = _t(rng.normal(0, 0.5, (2, D, D, D, C)))
    head = _t(rng.normal(0, 0.5, (3, C)))
    R = sum(n for _, n, _ in targets)
    target_rgb = _t(rng.random((R, 3)))
    pipes = []
    for cam in (True, False):
        bp = BatchPipeline(view_hw, targets, D=D, rate=rate, C=C, W_hits=96,
                           target_widths=[t["res"] for t in w["targets"]] if cam else None)
        bp.load_views(w["frames"], w["vol_bbox"], w["voxel_size"], w["trunc_weight"])
        if cam:
            bp.load_cameras([t["K"] for t in w["targets"]], [t["R"] for t in w["targets"]],
                            [t["T"] for t in w["targets"]])
        else:
            rays = []
            for t in w["targets"]:
                out = torch.empty((1, 1, t["res"], t["res"], 6), device="cuda")
                Kt, Rt, Tt = _t(t["K"]), _t(t["R"]), _t(t["T"])  # held until the launch has read them
                N.check(N.lib.sg_rays_from_cameras(N.ptr(Kt), N.ptr(Rt), N.ptr(Tt), 1, 1, t["res"], t["res"],
                                                   N.ptr(out), N.stream()), "rays")
                torch.cuda.synchronize()
                rays.append((out[..., :3].reshape(-1, 3), out[..., 3:].reshape(-1, 3)))
            bp.load_rays(rays)
        bp.set_fields(feat=feat, head=head, target_rgb=target_rgb)
        bp.render_args(float(w["voxel_size"][0]) * w["trunc_weight"], sdf_s=0.01, rand_seed=3)
        bp.train_step()
        torch.cuda.synchronize()
        pipes.append(bp)
    a, b = pipes
    assert torch.equal(a.hit_count, b.hit_count) and torch.equal(a.valid_len, b.valid_len)
    for x, y in ((a.out_rgb, b.out_rgb), (a.out_depth, b.out_depth), (a.out_ws, b.out_ws), (a.out_loss, b.out_loss)):
        assert torch.equal(x, y)
    m = b.grad_feat.abs().max().item()
    assert m > 0 and (a.grad_feat - b.grad_feat).abs().max().item() <= 1e-5 * m
    assert a.out_ws.max().item() > 0.5


def test_rays_generated_inside_kernels_match_buffers():
    """Camera segments handed straight to the intersection kernel (each ray
    generated from its pixel in the kernel) reproduce the pipeline that writes
    the rays to buffers first (sg_segment_rays); the training pass then reads
    rays rewritten by sg_segment_rays."""
    import ctypes as C
    from sailor_gb300 import _native as N
    from sailor_gb300.batch import BatchPipeline
    D, rate, Cf = 64, 4, 16
    w = syn.make_batch_workload(seed=8, n_frames=2, views=(2, 3), view_res=(96, 128), n_prims=8, D=D, trunc=0.04,
                                n_targets=3, target_res=(32, 96), target_S=(32, 64, 128))
    view_hw = [[d.shape for d in fr["depth"]] for fr in w["frames"]]
    targets = [(t["frame"], t["res"] ** 2, t["S"]) for t in w["targets"]]
    rng = np.random.default_rng(2)
    bp = BatchPipeline(view_hw, targets, D=D, rate=rate, C=Cf, W_hits=96, target_widths=[t["res"] for t in w["targets"]])
    bp.load_views(w["frames"], w["vol_bbox"], w["voxel_size"], w["trunc_weight"])
    bp.load_cameras([t["K"] for t in w["targets"]], [t["R"] for t in w["targets"]], [t["T"] for t in w["targets"]])
    bp.set_fields(feat=_t(rng.normal(0, 0.5, (2, D, D, D, Cf))), head=_t(rng.normal(0, 0.5, (3, Cf))),
                  target_rgb=_t(rng.random((bp.R, 3))))
    bp.render_args(float(w["voxel_size"][0]) * w["trunc_weight"], sdf_s=0.01, rand_seed=5)
    bp.train_step()
    torch.cuda.synchronize()
    ref = [t.clone() for t in (bp.hit_count, bp.valid_len, bp.out_rgb, bp.out_loss, bp.grad_feat)]
    # again, rays from the cameras inside the kernels (no ray buffers read)
    bp.ori.fill_(float("nan"))
    bp.dirs.fill_(float("nan"))
    bp.grad_feat.zero_()
    N.check(N.lib.sg_intersect_segments(C.byref(bp.tree), C.byref(bp.cam_seg), None, None, bp.W, N.ptr(bp.hit_idx),
                                        N.ptr(bp.hit_t0), N.ptr(bp.hit_t1), N.ptr(bp.valid_len), N.ptr(bp.hit_count),
                                        N.ptr(bp.status), N.stream()), "intersect")
    N.check(N.lib.sg_segment_rays(C.byref(bp.cam_seg), N.ptr(bp.ori), N.ptr(bp.dirs), N.stream()), "segment_rays")
    N.check(N.lib.sg_render_segments_train(C.byref(bp.tree), C.byref(bp.seg), C.byref(bp.args),
                                           N.ptr(bp.target_rgb), 2.0 / (3.0 * bp.R), N.ptr(bp.out_rgb),
                                           N.ptr(bp.out_depth), N.ptr(bp.out_ws), N.ptr(bp.out_alpha),
                                           N.ptr(bp.out_loss), N.ptr(bp.grad_feat), None, N.stream()), "train")
    torch.cuda.synchronize()
    assert torch.equal(bp.hit_count, ref[0]) and torch.equal(bp.valid_len, ref[1])
    assert torch.equal(bp.out_rgb, ref[2]) and torch.equal(bp.out_loss, ref[3])
    m = ref[4].abs().max().item()
    assert m > 0 and (bp.grad_feat - ref[4]).abs().max().item() <= 1e-5 * m
