"""GPU checks of the batched launches (segment tables) in
sailor_gb300.batch.BatchPipeline, on a small uneven workload: frames with
different view counts and mixed view resolutions, targets with different ray
counts and sample counts (32 .. 128, every register-tile size).

* fusion over the view table is bit-identical to per-frame sg_fuse_tsdf
  (views zero-padded to one size: a pixel in the padding has depth 0 and is
  rejected exactly like a pixel outside the image);
* the batched tree / intersection / sampling give the oracle's samples
  (bit-exact on unflagged rays), with constant and hashed jitter;
* the fused forward equals the modular chain grid_gather -> head ->
  tsdf_density -> compositing on the same samples (within 1e-5);
* the fused backward's grid and per-sample gradients equal float64-checked
  autograd of that modular chain (within 1e-4 of the largest gradient);
* a CUDA-graph replay of train_step reproduces the eager step.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

D, RATE, CF = 64, 4, 16


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


@pytest.fixture(scope="module")
def work():
    w = syn.make_batch_workload(seed=2, n_frames=3, views=(2, 4), view_res=(96, 128), n_prims=8, D=D,
                                trunc=0.04, n_targets=5, target_res=(48, 96), target_S=(32, 48, 64, 96, 128))
    return w


def _pipeline(w, C=CF, W_hits=96, seed=0):
    from sailor_gb300.batch import BatchPipeline
    view_hw = [[d.shape for d in fr["depth"]] for fr in w["frames"]]
    targets = [(t["frame"], t["ori"].shape[0], t["S"]) for t in w["targets"]]
    bp = BatchPipeline(view_hw, targets, D=D, rate=RATE, C=C, W_hits=W_hits)
    bp.load_views(w["frames"], w["vol_bbox"], w["voxel_size"], w["trunc_weight"])
    bp.load_rays([(t["ori"], t["dir"]) for t in w["targets"]])
    rng = np.random.default_rng(4)
    bp.set_fields(feat=_t(rng.normal(0, 0.5, (len(view_hw), D, D, D, C))),
                  head=_t(rng.normal(0, 0.5, (3, C))) if C != 3 else None,
                  target_rgb=_t(rng.random((bp.R, 3))))
    trunc_m = float(w["voxel_size"][0]) * w["trunc_weight"]
    bp.render_args(trunc_m, sdf_s=0.01, t_thres=1e-4, rand_seed=seed)
    bp.build()
    bp.intersect()
    torch.cuda.synchronize()
    return bp


def test_fuse_views_matches_per_frame(work):
    from sailor_gb300 import _native as N
    bp = _pipeline(work)
    for b, fr in enumerate(work["frames"]):
        hmax = max(d.shape[0] for d in fr["depth"])
        nv = len(fr["depth"])
        dep = np.zeros((1, nv, hmax, hmax), np.float32)
        col = np.zeros((1, nv, hmax, hmax), np.float32)
        for v in range(nv):
            h, w_ = fr["depth"][v].shape
            dep[0, v, :h, :w_] = fr["depth"][v]
            col[0, v, :h, :w_] = fr["color"][v]
        K, RT = _t(np.stack(fr["K"])[None]), _t(np.stack(fr["RT"])[None])
        dep_t, col_t = _t(dep), _t(col)
        out = [torch.empty((1, D, D, D), device="cuda") for _ in range(3)]
        occ = torch.empty((1, D, D, D), dtype=torch.int32, device="cuda")
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        bb, vs = _t(work["vol_bbox"][b:b + 1]), _t(work["voxel_size"][b:b + 1])
        N.check(N.lib.sg_fuse_tsdf(N.ptr(K), N.ptr(RT), N.ptr(col_t), N.ptr(dep_t), 1, nv, hmax, hmax, D, D, D,
                                   N.ptr(bb), N.ptr(vs), 1.0, work["trunc_weight"], 13.5, 13.5, N.ptr(out[0]),
                                   N.ptr(out[1]), N.ptr(out[2]), N.ptr(occ), N.ptr(cnt), N.stream()), "fuse")
        torch.cuda.synchronize()
        assert torch.equal(out[0][0], bp.tsdf[b])
        assert torch.equal(out[1][0], bp.weight[b])
        assert torch.equal(out[2][0], bp.colorv[b])
        # the tree build rewrote kept voxels to node ids; occupancy signs stay
        assert torch.equal(occ[0] >= 0, bp.occ0[b] >= 0)
        assert int(cnt[0]) == int(bp.cnt[0, b])
    assert int(bp.status[0]) == 0


def test_fusion_block_culling_with_nan_and_far_views(work):
    """Fusion through the depth-block maps against the oracle, bit for bit,
    with NaN depths (valid to the integrator, so they must stop a view from
    being culled), depths beyond the valid range and a view whose camera is
    moved far behind the volume."""
    from sailor_gb300.batch import BatchPipeline
    rng = np.random.default_rng(9)
    frames = []
    for fr in work["frames"]:
        dep = [d.copy() for d in fr["depth"]]
        for d in dep:
            m = rng.random(d.shape) < 0.01
            d[m] = np.nan
            d[rng.random(d.shape) < 0.01] = 4.5
        RT = [r.copy() for r in fr["RT"]]
        RT[0][:, 3] = RT[0][:, 3] + np.float32(40.0)  # the volume is behind or outside this view
        frames.append(dict(fr, depth=dep, RT=RT))
    view_hw = [[d.shape for d in fr["depth"]] for fr in frames]
    targets = [(t["frame"], t["ori"].shape[0], t["S"]) for t in work["targets"]]
    bp = BatchPipeline(view_hw, targets, D=D, rate=RATE, C=CF, W_hits=96)
    bp.load_views(frames, work["vol_bbox"], work["voxel_size"], work["trunc_weight"])
    bp.build()
    torch.cuda.synchronize()
    for b, fr in enumerate(frames):
        K = np.stack(fr["K"])[None]
        RT = np.stack(fr["RT"])[None]
        hmax = max(d.shape[0] for d in fr["depth"])
        nv = len(fr["depth"])
        dep = np.zeros((1, nv, hmax, hmax), np.float32)
        col = np.zeros((1, nv, hmax, hmax), np.float32)
        for v in range(nv):
            h, w_ = fr["depth"][v].shape
            dep[0, v, :h, :w_] = fr["depth"][v]
            col[0, v, :h, :w_] = fr["color"][v]
        ref = orc.integrate(K, RT, col, dep, D, work["vol_bbox"][b:b + 1], work["voxel_size"][b:b + 1], 1.0,
                            work["trunc_weight"], 13.5, 13.5)
        for got, key in ((bp.tsdf[b], "tsdf"), (bp.weight[b], "weight"), (bp.colorv[b], "color")):
            assert np.array_equal(got.cpu().numpy().view(np.uint32), ref[key][0].view(np.uint32)), key
        assert np.isnan(dep).any()


def _hash_uniform(seed, r, q):
    x = (np.uint64(seed) + r.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15) + q.astype(np.uint64))
    x ^= x >> np.uint64(30)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(27)
    x *= np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    return (x >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)


@pytest.mark.parametrize("seed", [0, 12345])
def test_batched_samples_match_oracle(work, seed):
    """Sorted samples of every target (its own frame and S) against the
    oracle's sampling + sort on the same hit rows."""
    bp = _pipeline(work, seed=seed)
    Sm = bp.S
    z = torch.empty((bp.R, Sm), device="cuda")
    node = torch.empty((bp.R, Sm), dtype=torch.int32, device="cuda")
    bp.forward(z, node)
    torch.cuda.synchronize()
    z, node = z.cpu().numpy(), node.cpu().numpy()
    cnt = bp.hit_count.cpu().numpy()
    assert cnt.max() <= bp.W and int(bp.status[0]) == 0
    idx = bp.hit_idx.cpu().numpy().copy()
    t0, t1 = bp.hit_t0.cpu().numpy().copy(), bp.hit_t1.cpu().numpy().copy()
    vlen = bp.valid_len.cpu().numpy()
    col = np.arange(bp.W)[None, :] >= cnt[:, None]
    idx[col], t0[col], t1[col] = -1, -1.0, -1.0
    tree = {"Dt": bp.Dt, "Db": D, "base_top": bp.B * D ** 3}
    checked = 0
    for t, (f, n, S) in enumerate(bp.targets):
        a, b = bp.ray_slices[t]
        hits = dict(idx=idx[None, a:b], t0=t0[None, a:b], t1=t1[None, a:b], valid_len=vlen[None, a:b],
                    max_hits=int(cnt[a:b].max(initial=0)), flags=np.zeros((1, n), np.int32))
        r = np.arange(a, b)[:, None]
        q = np.arange(S)[None, :]
        rands = _hash_uniform(seed, r, q) if seed else np.full((n, S), 0.5, np.float32)
        sidx, sz, flags = orc.sample_coarse(tree, hits, rands[None], bp.voxel_size.cpu().numpy()[f:f + 1], S)
        srt, order = orc.sort(sz)
        ok = flags[0] == 0
        got = z[a:b, :S]
        assert np.array_equal(got[ok].view(np.uint32), srt[0][ok].view(np.uint32)), (t, seed)
        nd = np.take_along_axis(sidx[0], order[0].astype(np.int64), 1)
        assert np.array_equal(node[a:b, :S][ok], nd[ok])
        assert (z[a:b, S:] == -1).all()
        checked += int(ok.sum())
    assert checked > 0.95 * bp.R


def _modular_chain(bp, z, w, t_thres, requires_grad=False):
    """Per target: grid_gather -> head -> tsdf_density -> exact compositing
    with the sorted samples z [R, S] of the fused forward."""
    from sailor_gb300.fields import grid_gather, tsdf_density
    from sailor_gb300.voxel_encoding_helper import volume_render_exact
    feat = bp.feat.detach().clone().requires_grad_(requires_grad)
    tsdf = bp.tsdf.detach().clone().requires_grad_(requires_grad)
    trunc_m = float(w["voxel_size"][0]) * w["trunc_weight"]
    outs, leaves = [], []
    for t, (f, n, S) in enumerate(bp.targets):
        a, b = bp.ray_slices[t]
        zz = z[a:b, :S][None].contiguous()
        o, d = bp.ori[a:b][None], bp.dirs[a:b][None]
        bb, vs = bp.vol_bbox[f:f + 1], bp.voxel_size[f:f + 1]
        fe = grid_gather(feat[f:f + 1], o, d, zz, bb, vs)
        rgb = (fe @ bp.head.T) if bp.C != 3 else fe
        sig = tsdf_density(tsdf[f:f + 1], o, d, zz, bb, vs, trunc_m, 0.01)
        if requires_grad:
            sig.retain_grad()
            rgb.retain_grad()
        idx = torch.arange(S, dtype=torch.int32, device="cuda").expand(1, n, S).contiguous()
        outs.append(volume_render_exact(zz, idx, sig[..., None], rgb, t_thres, False))
        leaves.append((sig, rgb))
    return outs, leaves, feat, tsdf


def test_fused_forward_matches_modular_chain(work):
    bp = _pipeline(work)
    z = torch.empty((bp.R, bp.S), device="cuda")
    node = torch.empty((bp.R, bp.S), dtype=torch.int32, device="cuda")
    bp.forward(z, node)
    outs, _, _, _ = _modular_chain(bp, z, work, 1e-4)
    for t in range(len(bp.targets)):
        a, b = bp.ray_slices[t]
        ref = outs[t]
        assert (bp.out_rgb[a:b] - ref[0][0]).abs().max().item() <= 1e-5
        assert (bp.out_depth[a:b] - ref[1][0, :, 0]).abs().max().item() <= 1e-5 * 4
        assert (bp.out_ws[a:b] - ref[2][0, :, 0]).abs().max().item() <= 1e-5
        assert (bp.out_alpha[a:b] - ref[3][0, :, 0]).abs().max().item() <= 1e-5
    assert bp.out_ws.max().item() > 0.5


def test_fused_backward_matches_modular_autograd(work):
    bp = _pipeline(work)
    R, S = bp.R, bp.S
    z = torch.empty((R, S), device="cuda")
    node = torch.empty((R, S), dtype=torch.int32, device="cuda")
    bp.forward(z, node)
    rng = np.random.default_rng(8)
    g = [_t(rng.normal(size=s)) for s in ((R, 3), (R,), (R,), (R,))]
    gs = torch.empty((R, S), device="cuda")
    gr = torch.empty((R, S, 3), device="cuda")
    bp.backward(*g, grad_sigma=gs, grad_rgb=gr)
    outs, leaves, feat, tsdf = _modular_chain(bp, z, work, 1e-4, requires_grad=True)
    loss = 0
    for t, o in enumerate(outs):
        a, b = bp.ray_slices[t]
        loss = loss + (o[0][0] * g[0][a:b]).sum() + (o[1][0, :, 0] * g[1][a:b]).sum() + \
            (o[2][0, :, 0] * g[2][a:b]).sum() + (o[3][0, :, 0] * g[3][a:b]).sum()
    loss.backward()
    for got, ref in ((bp.grad_feat, feat.grad), (bp.grad_tsdf, tsdf.grad)):
        m = ref.abs().max().item()
        assert m > 0
        assert (got - ref).abs().max().item() <= 1e-4 * m
    for t, (sig, rgb) in enumerate(leaves):
        a, b = bp.ray_slices[t]
        Sr = bp.targets[t][2]
        ms = sig.grad.abs().max().item()
        assert (gs[a:b, :Sr] - sig.grad[0]).abs().max().item() <= 1e-4 * max(ms, 1e-6)
        assert (gr[a:b, :Sr] - rgb.grad[0]).abs().max().item() <= 1e-5
        assert (gs[a:b, Sr:] == 0).all()


@pytest.mark.parametrize("train_tsdf", [False, True])
def test_train_step_graph_replay(work, train_tsdf):
    """A CUDA-graph replay of train_step gives the eager step's outputs and
    gradients bit for bit (the deterministic gradient reduction), after the
    grids held stale values where the step clears."""
    bp = _pipeline(work)
    bp.train_tsdf = train_tsdf
    bp.train_step()
    torch.cuda.synchronize()
    ref = [t.clone() for t in (bp.out_rgb, bp.out_depth, bp.tsdf, bp.grad_feat, bp.grad_tsdf, bp.out_loss)]
    assert ref[3].abs().max().item() > 0 and (not train_tsdf or ref[4].abs().max().item() > 0)
    g = bp.capture()
    near = torch.as_tensor(_near_node_voxels(bp.grad_bricks.cpu().numpy(), bp.B, bp.Dt, RATE), device="cuda")
    for _ in range(2):
        bp.out_rgb.zero_()
        bp.grad_feat.masked_fill_(near[..., None], 7.0)
        if train_tsdf:
            bp.grad_tsdf.masked_fill_(near, 7.0)
        g.replay()
        torch.cuda.synchronize()
        for got, r in zip((bp.out_rgb, bp.out_depth, bp.tsdf, bp.grad_feat, bp.grad_tsdf, bp.out_loss), ref):
            assert torch.equal(got, r)


def test_det_gradients_match_atomics_and_launch_shapes(work):
    """The deterministic reduction against the atomic scatter: outputs and
    loss bit for bit (the same per-ray pass), feature- and TSDF-grid
    gradients within 1e-5 of the largest; and the same gradients bit for bit
    under every training-pass grid size."""
    from sailor_gb300 import autotune
    bp = _pipeline(work)
    bp.train_tsdf = True
    bp.deterministic = False
    bp.train_step()
    torch.cuda.synchronize()
    ref = [t.clone() for t in (bp.out_rgb, bp.out_depth, bp.out_ws, bp.out_alpha, bp.out_loss, bp.grad_feat,
                               bp.grad_tsdf)]
    det = _pipeline(work)
    det.train_tsdf = True
    saved = autotune.current()
    outs = []
    try:
        for warps in (64, 7, 16):
            autotune.set_knob("render_warps", warps)
            det.zero_grads()
            det.train_step()
            torch.cuda.synchronize()
            outs.append([t.clone() for t in (det.out_rgb, det.out_depth, det.out_ws, det.out_alpha, det.out_loss,
                                             det.grad_feat, det.grad_tsdf)])
    finally:
        for k, v in saved.items():
            autotune.set_knob(k, v)
    for a, b in zip(outs[0][:5], ref[:5]):
        assert torch.equal(a, b)
    for a, b in zip(outs[0][5:], ref[5:]):
        m = b.abs().max().item()
        assert m > 0 and (a - b).abs().max().item() <= 1e-5 * m
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert torch.equal(a, b)


def test_record_capacity_reported(work):
    """Fewer record slots than the step's samples: the status carries
    SG_FLAG_RECORD_CAPACITY, nothing is written past the workspace, and the
    outputs are still the full step's."""
    from sailor_gb300 import _native as N
    full = _pipeline(work)
    full.train_step()
    torch.cuda.synchronize()
    assert not (full.status[0].item() & N.SG_FLAG_RECORD_CAPACITY)
    from sailor_gb300.batch import BatchPipeline
    view_hw = [[d.shape for d in fr["depth"]] for fr in work["frames"]]
    targets = [(t["frame"], t["ori"].shape[0], t["S"]) for t in work["targets"]]
    bp = BatchPipeline(view_hw, targets, D=D, rate=RATE, C=CF, W_hits=96, record_capacity=1000)
    bp.load_views(work["frames"], work["vol_bbox"], work["voxel_size"], work["trunc_weight"])
    bp.load_rays([(t["ori"], t["dir"]) for t in work["targets"]])
    bp.set_fields(feat=full.feat, head=full.head, target_rgb=full.target_rgb)
    bp.render_args(float(work["voxel_size"][0]) * work["trunc_weight"], sdf_s=0.01, t_thres=1e-4)
    bp.train_step()
    torch.cuda.synchronize()
    assert bp.status[0].item() & N.SG_FLAG_RECORD_CAPACITY
    assert torch.equal(bp.out_rgb, full.out_rgb)
    # the reduction's sizes: the same rays and slot needs; the capped
    # pipeline keeps the records of its first 1000 slots only
    a, c = full.reduction_sizes(), bp.reduction_sizes()
    hits = int((full.hit_count > 0).sum().item())
    assert a["rays_with_hits"] == c["rays_with_hits"] == hits
    assert a["slots_needed"] == c["slots_needed"] == a["slots"] > 1000 == c["slots"]
    assert 0 < a["cells"] <= a["records"] <= a["slots"] and a["cells"] > 100
    assert 0 < c["cells"] <= c["records"] <= 1000


@pytest.mark.parametrize("n,cap,bits", [(1, 16, 8), (5000, 8192, 12), (300000, 300000, 31), (70000, 100000, 20)])
def test_sort_pairs_stable(n, cap, bits):
    """sg_sort_pairs (the reduction's radix sort) against numpy's stable
    argsort: keys with many repeats, a live count below the capacity held
    in device memory, 1 to 4 passes."""
    from sailor_gb300 import _native as N
    rng = np.random.default_rng(n)
    keys = rng.integers(0, min(2 ** bits, 3 * n + 7), cap, dtype=np.int64).astype(np.uint32)
    kt = torch.as_tensor(keys.view(np.int32), device="cuda")
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    ko, vo, kt2, vt2 = (torch.full((cap,), -1, dtype=torch.int32, device="cuda") for _ in range(4))
    nb = int(N.lib.sg_sort_pairs_scratch_bytes(cap))
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    N.check(N.lib.sg_sort_pairs(N.ptr(kt), N.ptr(cnt), cap, bits, N.ptr(ko), N.ptr(vo), N.ptr(kt2), N.ptr(vt2),
                                N.ptr(scratch), nb, N.stream()), "sort_pairs")
    torch.cuda.synchronize()
    order = np.argsort(keys[:n], kind="stable")
    assert np.array_equal(vo.cpu().numpy()[:n].astype(np.int64), order)
    assert np.array_equal(ko.cpu().numpy()[:n].view(np.uint32), keys[:n][order])


def test_fused_train_step_matches_unfused(work):
    """sg_render_segments_train (forward + per-ray loss + backward in one
    pass) against the forward kernel, the loss gradient formed in torch, and
    the backward kernel: outputs within 1e-5 (only the summation order of
    the colour sums differs), loss = mean squared colour error, feature-grid
    gradient within 1e-5 of its largest value."""
    bp = _pipeline(work)
    bp.train_step_unfused()
    torch.cuda.synchronize()
    ref = [t.clone() for t in (bp.out_rgb, bp.out_depth, bp.out_ws, bp.out_alpha, bp.grad_feat)]
    mse = ((bp.out_rgb - bp.target_rgb) ** 2).mean().item()
    bp.train_step()
    torch.cuda.synchronize()
    for got, r in zip((bp.out_rgb, bp.out_depth, bp.out_ws, bp.out_alpha), ref[:4]):
        assert (got - r).abs().max().item() <= 1e-5 * max(1.0, r.abs().max().item())
    assert abs(bp.out_loss.sum().item() - mse) <= 1e-5 * max(mse, 1e-12) + 1e-9
    m = ref[4].abs().max().item()
    assert m > 0 and (bp.grad_feat - ref[4]).abs().max().item() <= 1e-5 * m


def _near_node_voxels(brick_node, B, Dt, rate):
    """Voxel mask [B, Db, Db, Db] of the bricks that are nodes or border one."""
    node = (brick_node.reshape(B, Dt, Dt, Dt) >= 0)
    pad = np.pad(node, ((0, 0), (1, 1), (1, 1), (1, 1)))
    near = np.zeros_like(node)
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                near |= pad[:, dx:dx + Dt, dy:dy + Dt, dz:dz + Dt]
    return near.repeat(rate, 1).repeat(rate, 2).repeat(rate, 3)


@pytest.mark.parametrize("C,aligned", [(16, True), (1, True), (3, False)])
def test_zero_near_nodes_exact(work, C, aligned):
    """sg_zero_near_nodes clears exactly the bricks that are nodes or border
    one (16-byte stores, and the scalar path for an unaligned grid)."""
    from sailor_gb300 import _native as N
    bp = _pipeline(work)
    B, Dt = bp.B, bp.Dt
    n = B * D ** 3 * C
    buf = torch.ones(n + 1, device="cuda")
    grid = buf[:n] if aligned else buf[1:]
    N.check(N.lib.sg_zero_near_nodes(_byref(bp.tree), N.ptr(grid), C, N.stream()), "zero_near_nodes")
    torch.cuda.synchronize()
    near = _near_node_voxels(bp.brick_node.cpu().numpy(), B, Dt, RATE)
    assert 0 < near.mean() < 1
    expect = np.repeat(np.where(near, 0.0, 1.0).astype(np.float32)[..., None], C, -1).reshape(-1)
    assert np.array_equal(grid.cpu().numpy(), expect)


def _byref(x):
    return C.byref(x)


@pytest.mark.parametrize("train_tsdf", [False, True])
def test_train_step_clears_previous_gradients(work, train_tsdf):
    """Two training steps on different scenes (the second's depths scaled, so
    its tree differs): the second step's gradients (feature grid, and TSDF
    grid when trained) equal a fresh pipeline's, although the first left
    gradients outside the second's node bricks."""
    frames2 = [dict(fr, depth=[(d * 0.9).astype(np.float32) for d in fr["depth"]]) for fr in work["frames"]]
    bp = _pipeline(work)
    bp.train_tsdf = train_tsdf
    bp.train_step()
    torch.cuda.synchronize()
    g1 = bp.grad_feat.clone()
    nodes1 = bp.brick_node.clone()
    bp.load_views(frames2, work["vol_bbox"], work["voxel_size"], work["trunc_weight"])
    bp.train_step()
    torch.cuda.synchronize()
    assert not torch.equal(nodes1, bp.brick_node)
    near2 = torch.as_tensor(_near_node_voxels(bp.brick_node.cpu().numpy(), bp.B, bp.Dt, RATE), device="cuda")
    assert (g1.abs().sum(-1) * (~near2)).max().item() > 0  # stale values a dense-only scheme would keep
    fresh = _pipeline(work)
    fresh.train_tsdf = train_tsdf
    fresh.load_views(frames2, work["vol_bbox"], work["voxel_size"], work["trunc_weight"])
    fresh.train_step()
    torch.cuda.synchronize()
    m = fresh.grad_feat.abs().max().item()
    assert m > 0 and (bp.grad_feat - fresh.grad_feat).abs().max().item() <= 1e-5 * m
    assert torch.equal(bp.out_rgb, fresh.out_rgb)
    if train_tsdf:
        mt = fresh.grad_tsdf.abs().max().item()
        assert mt > 0 and (bp.grad_tsdf - fresh.grad_tsdf).abs().max().item() <= 1e-5 * mt


@pytest.mark.parametrize("seed", [0, 77])
def test_parity_batch_against_oracle(work, seed):
    """bench.parity_batch on the small workload: fusion of every frame bit for
    bit; traversal rows equal the oracle's on every unflagged ray
    (t-intervals within 1e-5); samples equal the oracle's sampling of the
    same rows bit for bit (constant and hashed jitter); the training pass's
    colour, depth, weight sum and alpha within 1e-5 of the float64 oracle
    render; the feature-grid gradient within a relative 1e-4 of float64
    central differences (h = 1e-4) of the oracle's loss."""
    import bench
    bp = _pipeline(work, seed=seed)
    bp.train_step()
    torch.cuda.synchronize()
    bcfg = dict(frames=bp.B, D=D, rate=RATE, C=CF, sdf_s=0.01)
    par = bench.parity_batch(bp, work, bcfg, seed, n_hit=64, n_all=16, n_fd_entries=24)
    print(par)
    assert par["fusion_frames_bit_exact"]
    tr = par["traversal"]
    assert tr["unflagged_row_mismatches"] == 0 and tr["rays_flagged"] < 0.2 * par["rays"]
    assert tr["t_max_abs_err"] <= 1e-5
    assert par["sample_mismatches"] == 0 and par["composite_rays_flagged"] < 0.01 * par["rays"]
    assert par["composite_within_atol"], par["composite_max_abs_err"]
    assert par["grad_fd"]["max_abs_fd"] > 0 and par["grad_fd"]["rel_err"] <= 1e-4, par["grad_fd"]


def test_train_steps_from_host_matches_serial(work):
    """BatchPipeline.train_steps_from_host (each step's inputs uploaded on a
    copy stream beside the previous step, outputs read back beside the next)
    gives, step by step, the outputs of copy-in -> train_step -> copy-out in
    sequence bit for bit, eagerly and through a graph replay, with inputs
    that differ from step to step; the gradient grids end as the last
    step's.  Host tensors that are not pinned, of another shape, or not
    inputs of this pipeline are refused."""
    bp = _pipeline(work)
    rng = np.random.default_rng(21)
    base = dict(depth=bp.depth.cpu(), color=bp.color.cpu(), K=bp.K.cpu(), RT=bp.RT.cpu(), ori=bp.ori.cpu(),
                dirs=bp.dirs.cpu())
    steps = []
    for q in range(4):
        inp = {k: v.clone() for k, v in base.items()}
        inp["depth"] *= 1.0 + 0.01 * q
        inp["target_rgb"] = torch.as_tensor(rng.random((bp.R, 3), dtype=np.float32))
        steps.append({k: v.contiguous().pin_memory() for k, v in inp.items()})
    # serial reference
    ref = []
    for inp in steps:
        for k, v in inp.items():
            getattr(bp, k).copy_(v)
        bp.train_step()
        torch.cuda.synchronize()
        ref.append((bp.out_rgb.cpu(), bp.out_loss.cpu(), bp.out_depth.cpu()))
    ref_grad = bp.grad_feat.clone()
    g = bp.capture()
    for graph in (None, g):
        outs = [dict(out_rgb=torch.empty((bp.R, 3)).pin_memory(), out_loss=torch.empty(bp.R).pin_memory(),
                     out_depth=torch.empty(bp.R).pin_memory()) for _ in steps]
        bp.train_steps_from_host(list(zip(steps, outs)), graph)
        torch.cuda.synchronize()
        for o, r in zip(outs, ref):
            assert torch.equal(o["out_rgb"], r[0]) and torch.equal(o["out_loss"], r[1])
            assert torch.equal(o["out_depth"], r[2])
        assert torch.equal(bp.grad_feat, ref_grad)
    assert not torch.equal(ref[0][1], ref[1][1])  # the steps did differ
    out = dict(out_rgb=torch.empty((bp.R, 3)).pin_memory())
    for bad, match in ((dict(depth=base["depth"]), "pinned"),
                       (dict(depth=base["depth"][:-1].contiguous().pin_memory()), "expected"),
                       (dict(tK=torch.zeros(len(work["targets"]), 3, 3).pin_memory()), "not an input"),
                       (dict(weight=base["depth"].pin_memory()), "not one of")):
        with pytest.raises(ValueError, match=match):
            bp.train_steps_from_host([(bad, out)])
