"""GPU parity: each sm_103a stage against the CPU oracle on seeded scenes.

Bars (stated per test): bit-exact for occupancy, node ids, hit lists, sample
counts/indices and the integer-valued colour/weight volumes; TSDF bit-exact;
t-intervals, composited values and gradients within 1e-5 absolute of the
FP64 oracle.  Rays the oracle flags (a decision within a relative 1e-5 of a
tie, where the GPU's __fdividef reciprocal may decide differently from the
CPU's exact one) are excluded from the bit-exact hit/sample comparisons and
counted.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

ATOL = 1e-5


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


def gpu_chain(sc, D, rate, S, ori, dirs, rands, W, th_early_stop=-1, opt_num=-1, is_training=False):
    from sailor_gb300.dist import VoxelEncoding as VE
    B = sc["depths"].shape[0]
    Dt = D // rate
    occ0 = torch.full((B, D, D, D), -1, dtype=torch.int32, device="cuda")
    occ1 = torch.full((B, Dt, Dt, Dt), -1, dtype=torch.int32, device="cuda")
    cnt0 = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
    cnt1 = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
    tsdf, weight, color = VE.integrate_in_box(occ0, cnt0, _t(sc["K"]), _t(sc["RT"]), _t(sc["colors"]),
                                              _t(sc["depths"]), _t(sc["vol_bbox"]), _t(sc["voxel_size"]), 1.0,
                                              sc["trunc_weight"], 13.5, 13.5, 0)
    out = dict(tsdf=tsdf.cpu().numpy(), weight=weight.cpu().numpy(), color=color.cpu().numpy(),
               occ0=occ0.cpu().numpy(), cnt0=cnt0.cpu().numpy())
    VE.build_multi_res_volumes([occ0, occ1], [cnt0, cnt1], 2, rate, 0)
    out.update(occ1=occ1.cpu().numpy(), cnt1=cnt1.cpu().numpy())
    tot = [int(cnt0.sum()), int(cnt1.sum())]
    octree = VE.MultiLayerOctree(2, B, rate, 0)
    octree.init_octree([occ0, occ1], tot, [cnt0, cnt1], [0, tot[0]], _t(sc["voxel_size"]), _t(sc["vol_bbox"]))
    octree.build_octree()
    out.update(occ0_post=occ0.cpu().numpy(), occ1_post=occ1.cpu().numpy(), counts=octree.get_num_nodes_valid())
    idx, t0, t1, vl = octree.voxel_traversal(_t(ori), _t(dirs), W, 0, th_early_stop, is_training, opt_num)
    si, sz = octree.ray_voxels_points_sampling_coarse(idx, t0, t1, _t(rands), vl, 0, S)
    srt, sidx = octree.sort_samplings(sz)
    torch.cuda.synchronize()
    out.update(idx=idx.cpu().numpy(), t0=t0.cpu().numpy(), t1=t1.cpu().numpy(), vl=vl.cpu().numpy(),
               si=si.cpu().numpy(), sz=sz.cpu().numpy(), srt=srt.cpu().numpy(), sidx=sidx.cpu().numpy(),
               octree=octree, nodes=octree.get_nodes_tensor().cpu().numpy())
    return out


CASES = [
    dict(name="r4_D128", seed=21, res=192, D=128, rate=4, S=48, tres=96, prims=12, rand=False),
    dict(name="r8_D128_rand", seed=22, res=192, D=128, rate=8, S=64, tres=96, prims=12, rand=True),
    dict(name="r2_D64_b2", seed=23, res=128, D=64, rate=2, S=32, tres=64, prims=8, rand=True, batch=2),
]


@pytest.fixture(scope="module", params=CASES, ids=[c["name"] for c in CASES])
def case(request):
    c = request.param
    B = c.get("batch", 1)
    sc = syn.make_scene(seed=c["seed"], n_views=4, res=c["res"], n_prims=c["prims"], D=c["D"], trunc=0.03,
                        batch=B)
    ori, dirs = syn.target_rays(seed=c["seed"], res=c["tres"], batch=B)
    rng = np.random.default_rng(c["seed"])
    R = ori.shape[1]
    rands = rng.random((B, R, c["S"]), dtype=np.float32) if c["rand"] else np.full((B, R, c["S"]), 0.5, np.float32)
    W = 1024
    g = gpu_chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, W)
    ref = orc.chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, W=W, trunc_weight=sc["trunc_weight"])
    return dict(c=c, sc=sc, ori=ori, dirs=dirs, rands=rands, g=g, ref=ref, W=W)


def test_fusion_bit_exact(case):
    g, f = case["g"], case["ref"]["fusion"]
    for k in ("tsdf", "weight", "color"):
        assert np.array_equal(g[k], f[k]), k
    assert np.array_equal(g["occ0"], f["occ"])
    assert np.array_equal(g["cnt0"].ravel(), f["count"].ravel())


def test_coarse_occupancy_exact(case):
    g, r = case["g"], case["ref"]
    assert np.array_equal(g["occ1"], r["top"])
    assert np.array_equal(g["cnt1"].ravel(), r["cnt_top"].ravel())


def test_tree_ids_exact(case):
    g, t = case["g"], case["ref"]["tree"]
    assert g["counts"] == [t["ntop"], t["nbot"]]
    assert np.array_equal(g["occ1_post"], t["occ_top"])
    assert np.array_equal(g["occ0_post"], t["occ_bot"])


def test_node_table(case):
    g, r = case["g"], case["ref"]
    t = r["tree"]
    nodes = g["nodes"]
    vs, bb = r["voxel_size"], r["vol_bbox"]
    for gid in list(range(min(50, t["nbot"]))) + list(range(t["base_top"], t["base_top"] + min(50, t["ntop"]))):
        lvl, b, x, y, z = orc.node_keys(t, np.array([gid]))[0]
        size = t["Db"] // t["Dt"] if lvl == 1 else 1
        c, nvs = orc.node_geometry(vs[b, 0], size, bb[b, :, 0], np.array([x, y, z]))
        assert np.array_equal(nodes[gid, :3], c) and nodes[gid, 3] == np.float32(nvs)
        assert nodes[gid, 4] == 1 and nodes[gid, 5] == b


def test_traversal(case):
    g, h = case["g"], case["ref"]["hits"]
    ok = h["flags"] == 0
    rows_eq = np.all(g["idx"] == h["idx"], axis=-1)
    assert rows_eq[ok].all(), f"{(~rows_eq[ok]).sum()} unflagged rays differ"
    # stated: flagged rays (near ties) may differ; report how many
    print(f"traversal: {int((~ok).sum())} of {ok.size} rays flagged, {int((~rows_eq).sum())} differ")
    m = (h["idx"] >= 0) & rows_eq[..., None]
    assert np.abs(g["t0"][m] - h["t0"][m]).max() <= ATOL
    assert np.abs(g["t1"][m] - h["t1"][m]).max() <= ATOL
    assert np.abs(g["vl"][..., 0][rows_eq] - h["valid_len"][..., 0][rows_eq]).max() <= 1e-4
    pad = (h["idx"] < 0) & rows_eq[..., None]
    assert (g["idx"][pad] == -1).all() and (g["t0"][pad] == -1).all() and (g["t1"][pad] == -1).all()


def test_axis_aligned_rays(case):
    """Rays along the axes and in the axis planes (direction components
    exactly 0, so the slab test's reciprocals are infinite), started outside
    the volume on the far side of a random inside point: traversal rows equal
    the oracle's on unflagged rays, and the samples given those rows too."""
    g, r = case["g"], case["ref"]
    bb = r["vol_bbox"]
    B = bb.shape[0]
    n = 3000
    rng = np.random.default_rng(11)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0.6, 0.8, 0], [0, -0.8, 0.6], [0.8, 0, -0.6]], np.float32)
    dirs = axes[rng.integers(0, len(axes), (B, n))]
    lo, hi = bb[:, None, :, 0], bb[:, None, :, 1]
    inside = lo + (hi - lo) * rng.random((B, n, 3))
    ori = (inside - dirs * (hi - lo).max() * 1.5).astype(np.float32)
    W = case["W"]
    octree = g["octree"]
    idx, t0, t1, vl = octree.voxel_traversal(_t(ori), _t(dirs), W, 0, -1, False, -1)
    h = orc.voxel_traversal(r["tree"], ori, dirs, r["voxel_size"], bb, W=W)
    idx, t0, t1 = idx.cpu().numpy(), t0.cpu().numpy(), t1.cpu().numpy()
    ok = h["flags"] == 0
    rows_eq = np.all(idx == h["idx"], axis=-1)
    assert rows_eq[ok].all(), f"{(~rows_eq[ok]).sum()} unflagged rays differ"
    assert ok.mean() > 0.9 and (h["idx"] >= 0).sum() > 100
    m = (h["idx"] >= 0) & rows_eq[..., None]
    assert np.abs(t0[m] - h["t0"][m]).max() <= ATOL and np.abs(t1[m] - h["t1"][m]).max() <= ATOL
    S = case["c"]["S"]
    rands = rng.random((B, n, S), dtype=np.float32)
    si, sz = octree.ray_voxels_points_sampling_coarse(_t(h["idx"], torch.int32), _t(h["t0"]), _t(h["t1"]),
                                                      _t(rands), _t(h["valid_len"]), 0, S)
    si2, sz2, _ = orc.sample_coarse(r["tree"], h, rands, r["voxel_size"], S)
    assert np.array_equal(si.cpu().numpy(), si2) and np.array_equal(sz.cpu().numpy(), sz2)


@pytest.mark.parametrize("mode", ["inference", "training", "early_stop", "opt_num"])
def test_intersection_variants_identical(case, mode):
    """The warp-cooperative intersection (a warp per hit brick's children)
    and the thread-per-ray one give the same rows, counts, t-intervals and
    valid lengths bit for bit, in every traversal mode, with padded rows and
    with rows too narrow for some rays."""
    from sailor_gb300 import autotune
    g = case["g"]
    octree = g["octree"]
    args = dict(inference=(-1, False, -1), training=(-1, True, -1), early_stop=(2, False, -1),
                opt_num=(-1, False, 3))[mode]
    saved = autotune.current()
    outs = []
    try:
        for wv in (0, 1):
            autotune.set_knob("isect_warp", wv)
            for W in (case["W"], 8):
                idx, t0, t1, vl = octree.voxel_traversal(_t(case["ori"]), _t(case["dirs"]), W, 0, args[0], args[1],
                                                         args[2])
                torch.cuda.synchronize()
                outs.append((idx.clone(), t0.clone(), t1.clone(), vl.clone(), octree._status.clone()))
    finally:
        for k, v in saved.items():
            autotune.set_knob(k, v)
    for a, b in zip(outs[:2], outs[2:]):
        for x, y in zip(a, b):
            assert torch.equal(x, y)
    assert (outs[0][0] >= 0).sum().item() > 100


@pytest.mark.parametrize("mode", ["inference", "training", "early_stop", "opt_num"])
def test_brick_box_exit_identical(case, mode):
    """The walk that stops once it has passed the frame's kept-brick bounds
    (SgTree.brick_box) gives the full walk's rows, counts, t-intervals,
    valid lengths and status bit for bit; the bounds are the kept bricks'
    coordinate extremes."""
    g = case["g"]
    octree = g["octree"]
    args = dict(inference=(-1, False, -1), training=(-1, True, -1), early_stop=(2, False, -1),
                opt_num=(-1, False, 3))[mode]
    box = octree.tree_arrays()["brick_box"].cpu().numpy().reshape(-1, 6)
    t = octree._tree
    Dt = t.Dt
    nt = octree.get_num_nodes_valid()[0]
    keys = octree.tree_arrays()["top_key"][:nt].cpu().numpy().astype(np.int64)
    fb, lin = keys // Dt ** 3, keys % Dt ** 3
    xyz = np.stack([lin // (Dt * Dt), (lin // Dt) % Dt, lin % Dt], 1)
    for b in range(box.shape[0]):
        m = fb == b
        assert np.array_equal(box[b, :3], xyz[m].min(0)) and np.array_equal(box[b, 3:], xyz[m].max(0))
    outs = []
    saved = t.brick_box
    try:
        for ptr in (saved, None):
            t.brick_box = ptr
            idx, t0, t1, vl = octree.voxel_traversal(_t(case["ori"]), _t(case["dirs"]), case["W"], 0, args[0],
                                                     args[1], args[2])
            torch.cuda.synchronize()
            outs.append((idx.clone(), t0.clone(), t1.clone(), vl.clone(), octree._status.clone()))
    finally:
        t.brick_box = saved
    for x, y in zip(*outs):
        assert torch.equal(x, y)
    assert (outs[0][0] >= 0).sum().item() > 100


def test_rays_starting_inside(case):
    """Rays whose origin lies inside the volume (the whole-grid slab test
    clamps the entry to t = 0, so the walk starts in the origin's brick):
    rows as the oracle's on unflagged rays (t-values and valid lengths within
    the traversal tolerances), and the samples given the oracle's rows bit
    for bit."""
    g, r = case["g"], case["ref"]
    bb = r["vol_bbox"]
    B = bb.shape[0]
    n = 2000
    rng = np.random.default_rng(12)
    lo, hi = bb[:, None, :, 0], bb[:, None, :, 1]
    ori = (lo + (hi - lo) * rng.uniform(0.05, 0.95, (B, n, 3))).astype(np.float32)
    d = rng.normal(size=(B, n, 3))
    dirs = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    octree = g["octree"]
    idx, t0, t1, vl = octree.voxel_traversal(_t(ori), _t(dirs), case["W"], 0, -1, False, -1)
    h = orc.voxel_traversal(r["tree"], ori, dirs, r["voxel_size"], bb, W=case["W"])
    ok = h["flags"] == 0
    idx = idx.cpu().numpy()
    assert np.array_equal(idx[ok], h["idx"][ok]) and ok.mean() > 0.9 and (h["idx"] >= 0).sum() > 100
    # t-values from the reference's approximate reciprocal: within ATOL
    m = (h["idx"] >= 0) & ok[..., None]
    assert np.abs(t0.cpu().numpy()[m] - h["t0"][m]).max() <= ATOL
    assert np.abs(vl.cpu().numpy()[..., 0][ok] - h["valid_len"][..., 0][ok]).max() <= 1e-4
    S = case["c"]["S"]
    rands = rng.random((B, n, S), dtype=np.float32)
    si, sz = octree.ray_voxels_points_sampling_coarse(_t(h["idx"], torch.int32), _t(h["t0"]), _t(h["t1"]),
                                                      _t(rands), _t(h["valid_len"]), 0, S)
    si2, sz2, _ = orc.sample_coarse(r["tree"], h, rands, r["voxel_size"], S)
    assert np.array_equal(si.cpu().numpy(), si2) and np.array_equal(sz.cpu().numpy(), sz2)


def test_empty_scene_chain():
    """Views with no valid depth: nothing is fused (TSDF 1, weight 0, no
    occupied voxel), the tree is empty, every ray misses, every sample slot
    is -1 and compositing gives zeros -- as the oracle."""
    sc = syn.make_scene(seed=41, n_views=4, res=96, n_prims=6, D=64, trunc=0.03)
    sc["depths"] = np.zeros_like(sc["depths"])
    ori, dirs = syn.target_rays(seed=41, res=32)
    S = 32
    rands = np.full((1, ori.shape[1], S), 0.5, np.float32)
    g = gpu_chain(sc, 64, 4, S, ori, dirs, rands, 256)
    ref = orc.chain(sc, 64, 4, S, ori, dirs, rands, W=256, trunc_weight=sc["trunc_weight"])
    assert (g["tsdf"] == 1).all() and (g["weight"] == 0).all() and (g["occ0"] == -1).all()
    assert int(g["cnt0"].sum()) == 0 and g["counts"] == [0, 0]
    for k in ("tsdf", "weight", "color"):
        assert np.array_equal(g[k], ref["fusion"][k])
    assert (g["idx"] == -1).all() and (g["si"] == -1).all() and (g["sz"] == -1).all()
    assert np.array_equal(g["srt"], ref["sorted_z"]) and np.array_equal(g["sidx"], ref["sort_idx"])
    R = ori.shape[1]
    from sailor_gb300.dist import VoxelEncoding as VE
    feats, d, ws, al = VE.volume_rendering_training_forward(_t(g["srt"]), _t(g["sidx"], torch.int32),
                                                            torch.ones((1, R, S, 1), device="cuda"),
                                                            torch.ones((1, R, S, 3), device="cuda"), 0, 1e-4, False)
    for t in (feats, d, ws, al):
        assert (t == 0).all()


def test_sampling_given_oracle_hits(case):
    """Same hit lists in -> bit-identical samples out (counts, ids, depths)."""
    from sailor_gb300.dist import VoxelEncoding as VE  # noqa: F401
    h, r = case["ref"]["hits"], case["ref"]
    octree = case["g"]["octree"]
    si, sz = octree.ray_voxels_points_sampling_coarse(_t(h["idx"], torch.int32), _t(h["t0"]), _t(h["t1"]),
                                                      _t(case["rands"]), _t(h["valid_len"]), 0, case["c"]["S"])
    si2, sz2, _ = orc.sample_coarse(r["tree"], h, case["rands"], r["voxel_size"], case["c"]["S"])
    assert np.array_equal(si.cpu().numpy(), si2)
    assert np.array_equal(sz.cpu().numpy(), sz2)


def test_sampling_chain(case):
    g, r = case["g"], case["ref"]
    ok = r["flags"] == 0
    assert np.array_equal(g["si"][ok], r["sampled_idx"][ok])
    assert np.abs(g["sz"][ok] - r["sampled_z"][ok]).max() <= ATOL


def test_sort_exact(case):
    octree = case["g"]["octree"]
    z = case["ref"]["sampled_z"]
    srt, idx = octree.sort_samplings(_t(z))
    s2, i2 = orc.sort(z)
    assert np.array_equal(srt.cpu().numpy(), s2)
    assert np.array_equal(idx.cpu().numpy(), i2)


@pytest.mark.parametrize("S", [1, 7, 31, 32, 33, 50, 64, 96, 100, 128, 132, 200, 256])
def test_sort_row_lengths(S):
    """sort_samplings over every network size (rows of up to 32, 64, 128,
    256), row lengths off the vector width, -1 padding and repeated depths:
    exactly the oracle's stable order; a view that starts 4 bytes
    past an allocation takes the scalar path with the same result."""
    rng = np.random.default_rng(S)
    R = 300
    z = rng.uniform(0.0, 4.0, (1, R, S)).astype(np.float32)
    z[0, ::3, S // 2:] = -1.0  # the sampler's padding
    z[0, 1::5, :] = -1.0  # rays with no sample
    z[0, 2::7, : max(1, S // 3)] = np.float32(1.25)  # repeated depths
    z[0, 4::11, ::2] = 0.0
    from sailor_gb300.dist import VoxelEncoding as VE
    octree = VE.MultiLayerOctree(2, 1, 4, 0)
    s2, i2 = orc.sort(z)
    srt, idx = octree.sort_samplings(_t(z))
    assert np.array_equal(srt.cpu().numpy().view(np.uint32), s2.view(np.uint32))
    assert np.array_equal(idx.cpu().numpy(), i2)
    buf = torch.empty(z.size + 1, device="cuda")
    view = buf[1:].view(z.shape)
    view.copy_(_t(z))
    srt, idx = octree.sort_samplings(view)
    assert np.array_equal(srt.cpu().numpy().view(np.uint32), s2.view(np.uint32))
    assert np.array_equal(idx.cpu().numpy(), i2)


def test_sort_empty_rows():
    """As torch.sort along the last axis: empty in, empty out."""
    from sailor_gb300.dist import VoxelEncoding as VE
    octree = VE.MultiLayerOctree(2, 1, 4, 0)
    for shape in ((1, 0, 16), (2, 5, 0)):
        srt, idx = octree.sort_samplings(torch.empty(shape, device="cuda"))
        assert srt.shape == shape and idx.shape == shape and idx.dtype == torch.int32


@pytest.mark.parametrize("S", [1, 200, 256])
def test_sampling_sizes_given_oracle_hits(case, S):
    """The smallest and the largest sample rows (one sample; 200 and 256:
    the 8-per-lane layout) give the oracle's samples bit for bit."""
    h, r = case["ref"]["hits"], case["ref"]
    octree = case["g"]["octree"]
    B, R = h["idx"].shape[:2]
    rands = np.random.default_rng(S).random((B, R, S), dtype=np.float32)
    si, sz = octree.ray_voxels_points_sampling_coarse(_t(h["idx"], torch.int32), _t(h["t0"]), _t(h["t1"]),
                                                      _t(rands), _t(h["valid_len"]), 0, S)
    si2, sz2, _ = orc.sample_coarse(r["tree"], h, rands, r["voxel_size"], S)
    assert np.array_equal(si.cpu().numpy(), si2)
    assert np.array_equal(sz.cpu().numpy(), sz2)
    assert (si2 >= 0).any()


def test_trilerp_nodes(case):
    g, r = case["g"], case["ref"]
    octree = g["octree"]
    B, R, S = r["sampled_idx"].shape
    Cf = 4
    rng = np.random.default_rng(1)
    feats = rng.normal(size=(B, Cf, R, S, 8)).astype(np.float32)
    gout = rng.normal(size=(B, Cf, R, S)).astype(np.float32)
    si, sz = _t(r["sampled_idx"], torch.int32), _t(r["sampled_z"])
    out = octree.trilinear_aggregate_features(_t(case["ori"]), _t(case["dirs"]), sz, si, _t(feats)).cpu().numpy()
    gin = octree.trilinear_aggregate_features_backward(_t(case["ori"]), _t(case["dirs"]), sz, si, _t(feats),
                                                       _t(gout)).cpu().numpy()
    # oracle: corners of each sample's node
    t = r["tree"]
    ids = r["sampled_idx"].reshape(-1)
    valid = (ids >= 0).astype(np.int32)
    keys = orc.node_keys(t, np.where(ids >= 0, ids, t["base_top"]))
    corners = np.zeros((ids.size, 8, 3), np.float32)
    pts = (case["ori"][:, :, None, :] + case["dirs"][:, :, None, :] * r["sampled_z"][..., None]).reshape(-1, 3)
    for k in np.nonzero(valid)[0]:
        lvl, b, x, y, z = keys[k]
        size = t["Db"] // t["Dt"] if lvl == 1 else 1
        c, nvs = orc.node_geometry(r["voxel_size"][b, 0], size, r["vol_bbox"][b, :, 0], np.array([x, y, z]))
        h = np.float32(nvs) / np.float32(2)
        corners[k] = [[c[0] + sx * h, c[1] + sy * h, c[2] + sz_ * h] for sx in (-1, 1) for sy in (-1, 1)
                      for sz_ in (-1, 1)]
    fo = feats.transpose(1, 0, 2, 3, 4).reshape(Cf, -1, 8)
    go = gout.transpose(1, 0, 2, 3).reshape(Cf, -1)
    ro, rg = orc.trilerp_nodes(pts, corners, valid, fo, go)
    ro = ro.reshape(Cf, B, R, S).transpose(1, 0, 2, 3)
    rg = rg.reshape(Cf, B, R, S, 8).transpose(1, 0, 2, 3, 4)
    assert np.abs(out - ro).max() <= 1e-4
    assert np.abs(gin - rg).max() <= 1e-4


# ---------------------------------------------------------------------------
# compositing
# ---------------------------------------------------------------------------
def _comp_inputs(seed, R=4096, S=48, C=3, presorted=False):
    rng = np.random.default_rng(seed)
    z = rng.uniform(1.5, 3.5, (1, R, S)).astype(np.float32)
    npad = rng.integers(0, S, R)
    npad[:32] = S
    npad[32:64] = 0
    for r in range(R):
        z[0, r, S - npad[r]:] = -1.0
    sigma = rng.gamma(0.8, 20.0, (1, R, S, 1)).astype(np.float32)
    occ = (1.0 / (1.0 + np.exp(-rng.normal(0, 3, (1, R, S, 1))))).astype(np.float32)
    feats = rng.random((1, R, S, C), dtype=np.float32)
    srt, idx = orc.sort(z)
    grads = [rng.normal(size=s).astype(np.float32) for s in ((1, R, C), (1, R, 1), (1, R, 1), (1, R, 1))]
    return z, idx, sigma, occ, feats, grads


@pytest.mark.parametrize("occ_mode", [False, True])
def test_composite_fwd(occ_mode):
    from sailor_gb300.dist import VoxelEncoding as VE
    z, idx, sigma, occ, feats, _ = _comp_inputs(3)
    sg = occ if occ_mode else sigma
    out = VE.volume_rendering_training_forward(_t(z), _t(idx, torch.int32), _t(sg), _t(feats), 0, 1e-4, occ_mode)
    rf, rd, rw, ra, fl = orc.composite_fwd(z, idx, sg, feats, 1e-4, occ_mode)
    ok = fl == 0
    for a, b in zip(out, (rf, rd, rw, ra)):
        err = np.abs(a.cpu().numpy() - b)[ok].max()
        assert err <= ATOL, err


def test_composite_presorted():
    from sailor_gb300.dist import VoxelEncoding as VE
    z, idx, sigma, occ, feats, _ = _comp_inputs(4)
    zs = np.take_along_axis(z, idx.astype(np.int64), 2)
    os_ = np.take_along_axis(occ[..., 0], idx.astype(np.int64), 2)[..., None]
    fs = np.take_along_axis(feats, idx.astype(np.int64)[..., None], 2)
    out = VE.volume_rendering_occ_forward(_t(zs), _t(os_), _t(fs), 0, 1e-4)
    rf, rd, rw, ra, fl = orc.composite_fwd(zs, None, os_, fs, 1e-4, True)
    ok = fl == 0
    for a, b in zip(out, (rf, rd, rw, ra)):
        assert np.abs(a.cpu().numpy() - b)[ok].max() <= ATOL


@pytest.mark.parametrize("alpha_lo,alpha_hi,t_thres", [(-0.3, 1.4, 1e-4), (0.0, 1.0, 1.5)])
def test_composite_alpha_outside_unit_interval(alpha_lo, alpha_hi, t_thres):
    """Occupancy compositing (alpha given) with alphas outside [0, 1], where
    the transmittance can rise or change sign, and a threshold above 1 (stop
    at the first sample): outputs, and so the early-termination positions,
    match the oracle."""
    from sailor_gb300.dist import VoxelEncoding as VE
    z, idx, _, _, feats, _ = _comp_inputs(5)
    a = np.random.default_rng(6).uniform(alpha_lo, alpha_hi, z.shape + (1,)).astype(np.float32)
    out = VE.volume_rendering_training_forward(_t(z), _t(idx, torch.int32), _t(a), _t(feats), 0, t_thres, True)
    rf, rd, rw, ra, fl = orc.composite_fwd(z, idx, a, feats, t_thres, True)
    ok = fl == 0
    assert ok.mean() > 0.9
    for x, y in zip(out, (rf, rd, rw, ra)):
        # relative to the largest output: the transmittance can grow past 1
        assert np.abs(x.cpu().numpy() - y)[ok].max() <= ATOL * max(1.0, np.abs(y).max())


@pytest.mark.parametrize("occ_mode", [False, True])
def test_composite_bwd_reference_formula(occ_mode):
    """The reference gradient formula (volume_rendering.cu:244-522).  The last
    valid sample of a density ray carries delta = 1e10, which multiplies a
    cancellation residue; those entries are compared relative to 1e10*ulp."""
    from sailor_gb300.dist import VoxelEncoding as VE
    z, idx, sigma, occ, feats, grads = _comp_inputs(5)
    sg = occ if occ_mode else sigma
    outs = VE.volume_rendering_training_forward(_t(z), _t(idx, torch.int32), _t(sg), _t(feats), 0, 1e-4, occ_mode)
    gf, gs = VE.volume_rendering_training_backward(*[_t(a) for a in grads], *outs, _t(z), _t(idx, torch.int32),
                                                   _t(sg), _t(feats), 0, 1e-4, occ_mode)
    o = [a.cpu().numpy() for a in outs]
    rgf, rgs = orc.composite_bwd_ref(*grads, *o, z, idx, sg, feats, 1e-4, occ_mode)
    _, _, _, _, fl = orc.composite_fwd(z, idx, sg, feats, 1e-4, occ_mode)
    ok = fl == 0
    assert np.abs(gf.cpu().numpy() - rgf)[0][ok[0]].max() <= ATOL
    gs, rgs = gs.cpu().numpy()[..., 0], rgs[..., 0]
    last = np.zeros_like(gs, bool)
    if not occ_mode:
        srt = np.take_along_axis(z, idx.astype(np.int64), 2)
        lastpos = np.where(srt[..., -1] >= 0, idx[..., -1], -1)
        for r in range(z.shape[1]):
            if lastpos[0, r] >= 0:
                last[0, r, lastpos[0, r]] = True
    tight = ok[..., None] & ~last
    assert np.abs(gs - rgs)[tight].max() <= 1e-4
    assert np.abs(gs - rgs)[last & ok[..., None]].max(initial=0) <= 1e10 * 1e-6


def _torch_composite(z, idx, sigma, feats, occ_mode):
    """Plain PyTorch float64 compositing with the kernel's semantics (sorted
    order, invalid samples skipped, last delta 1e10, no early termination)."""
    zz = torch.gather(z, 2, idx)
    sg = torch.gather(sigma[..., 0], 2, idx)
    ft = torch.gather(feats, 2, idx[..., None].expand(-1, -1, -1, feats.shape[-1]))
    valid = zz >= 0
    S = zz.shape[-1]
    if occ_mode:
        alpha = torch.where(valid, sg, torch.zeros_like(sg))
    else:
        nxt = torch.cat([zz[..., 1:], torch.full_like(zz[..., :1], 1e10)], -1)
        delta = torch.where(torch.arange(S) == S - 1, torch.full_like(zz, 1e10), nxt - zz)
        alpha = torch.where(valid, 1 - torch.exp(-sg * delta), torch.zeros_like(sg))
    T = torch.cumprod(torch.cat([torch.ones_like(alpha[..., :1]), 1 - alpha], -1), -1)[..., :-1]
    w = alpha * T
    return ((w[..., None] * ft).sum(-2), (w * zz).sum(-1, keepdim=True), w.sum(-1, keepdim=True),
            (w * alpha).sum(-1, keepdim=True))


@pytest.mark.parametrize("occ_mode", [False, True])
def test_exact_adjoint_vs_autograd_and_fd(occ_mode):
    """True adjoint vs float64 autograd of a plain PyTorch compositing and vs
    float64 central finite differences (h = 1e-4).  t_thres = 0 so no early
    termination, and all samples valid and ascending (no padding)."""
    from sailor_gb300.dist import VoxelEncoding as VE
    rng = np.random.default_rng(7)
    R, S, Cf = 256, 32, 3
    z = np.sort(rng.uniform(1.0, 2.0, (1, R, S)), -1).astype(np.float32)
    idx = np.tile(np.arange(S, dtype=np.int32), (1, R, 1))
    sg = (rng.random((1, R, S, 1)) * (0.9 if occ_mode else 30.0)).astype(np.float32)
    feats = rng.random((1, R, S, Cf), dtype=np.float32)
    grads = [rng.normal(size=s).astype(np.float32) for s in ((1, R, Cf), (1, R, 1), (1, R, 1), (1, R, 1))]
    gf, gs = VE.volume_rendering_training_backward(*[_t(a) for a in grads], *[_t(np.zeros(1))] * 4, _t(z),
                                                   _t(idx, torch.int32), _t(sg), _t(feats), 0, 0.0, occ_mode,
                                                   exact=True)
    zt = torch.tensor(z, dtype=torch.float64)
    it = torch.tensor(idx, dtype=torch.int64)
    st = torch.tensor(sg, dtype=torch.float64, requires_grad=True)
    ftt = torch.tensor(feats, dtype=torch.float64, requires_grad=True)
    outs = _torch_composite(zt, it, st, ftt, occ_mode)
    loss = sum((o * torch.tensor(g, dtype=torch.float64)).sum() for o, g in zip(outs, grads))
    loss.backward()
    assert np.abs(gs.cpu().numpy() - st.grad.numpy()).max() <= 1e-4 * max(1.0, np.abs(st.grad.numpy()).max())
    assert np.abs(gf.cpu().numpy() - ftt.grad.numpy()).max() <= ATOL
    # float64 central differences on 512 (ray, sample) entries
    h = 1e-4
    sel = rng.choice(R * S, 512, replace=False)
    with torch.no_grad():
        fd = np.zeros(512)
        for n, k in enumerate(sel):
            r, s = divmod(int(k), S)
            sp = st.detach().clone()
            sm = st.detach().clone()
            sp[0, r, s, 0] += h
            sm[0, r, s, 0] -= h
            lp = sum((o * torch.tensor(g, dtype=torch.float64)).sum()
                     for o, g in zip(_torch_composite(zt, it, sp, ftt, occ_mode), grads))
            lm = sum((o * torch.tensor(g, dtype=torch.float64)).sum()
                     for o, g in zip(_torch_composite(zt, it, sm, ftt, occ_mode), grads))
            fd[n] = (lp - lm) / (2 * h)
    got = gs.cpu().numpy().reshape(-1)[sel]
    assert np.abs(got - fd).max() <= 1e-3 * max(1.0, np.abs(fd).max())


# ---------------------------------------------------------------------------
# fast pipeline (compact hits, fused sample+sort, field gathers)
# ---------------------------------------------------------------------------
def test_pipeline_matches_oracle():
    from sailor_gb300.pipeline import FramePipeline
    D, rate, S = 128, 8, 64
    sc = syn.make_scene(seed=31, n_views=4, res=256, n_prims=12, D=D, trunc=0.03)
    ori, dirs = syn.target_rays(seed=31, res=96)
    R = ori.shape[1]
    rng = np.random.default_rng(31)
    Dc = 32
    cgrid = rng.random((1, Dc, Dc, Dc, 3), dtype=np.float32)
    cvs = np.full((1, 1), np.float32(2.0) / np.float32(Dc - 1), np.float32)
    cbb = np.array([[[-1.0, 1.0]] * 3], np.float32)
    pipe = FramePipeline(1, D, rate, R, S, W_hits=1024)
    pipe.build(_t(sc["K"]), _t(sc["RT"]), _t(sc["colors"]), _t(sc["depths"]), _t(sc["vol_bbox"]),
               _t(sc["voxel_size"]), sc["trunc_weight"])
    trunc_m = float(sc["voxel_size"][0, 0]) * sc["trunc_weight"]
    rgb, dep, ws, al = pipe.render(_t(ori), _t(dirs), _t(cgrid), _t(cbb), _t(cvs), trunc_m, fused=False)
    torch.cuda.synchronize()
    unfused = [a.clone() for a in (rgb, dep, ws, al, pipe.z, pipe.node)]
    assert pipe.status[0].item() == 0
    rands = np.full((1, R, S), 0.5, np.float32)
    ref = orc.chain(sc, D, rate, S, ori, dirs, rands, W=1024, trunc_weight=sc["trunc_weight"])
    ok = ref["flags"][0] == 0
    z = pipe.z.cpu().numpy()
    # depths: t-intervals differ by a few ulp (__fdividef), so within 1e-5
    assert np.abs(z[ok] - ref["sorted_z"][0][ok]).max() <= ATOL
    # node ids: the pipeline numbers top nodes from B*D^3; compare per-ray
    # multisets (equal depths within an ulp may swap sorted positions)
    node = pipe.node.cpu().numpy()
    t = ref["tree"]
    ref_nodes = np.take_along_axis(ref["sampled_idx"][0], ref["sort_idx"][0].astype(np.int64), 1)
    mine = np.where(node >= D ** 3, node - D ** 3 + t["base_top"], node)
    assert np.array_equal(np.sort(mine[ok], 1), np.sort(ref_nodes[ok], 1))
    # fields and compositing against the oracle on the same sorted samples
    # the sample points as the kernels form them (fused multiply-add)
    pts = orc.sample_points(ori[0], dirs[0], np.maximum(z, 0)).reshape(-1, 3)
    tsdf = orc.grid_gather(pts, ref["fusion"]["tsdf"][..., None], sc["vol_bbox"][:, :, 0], sc["voxel_size"][:, 0])
    sig = 1.0 / (1.0 + np.exp(tsdf[:, 0] * trunc_m / 0.005)) / 0.005
    sig = np.where(z.reshape(-1) >= 0, sig, 0).reshape(R, S)
    # sigma <= 200 and steep in the TSDF (slope up to 6 / 0.005^2 / 4 per unit
    # TSDF): float32 gather and exp against float64
    assert np.abs(pipe.sigma.cpu().numpy() - sig).max() <= 5e-3
    col = orc.grid_gather(pts, cgrid, cbb[:, :, 0], cvs[:, 0]).reshape(R, S, 3)
    col = np.where(z[..., None] >= 0, col, 0)
    assert np.abs(pipe.rgb.cpu().numpy() - col).max() <= 1e-5
    rf, rd, rw, ra, fl = orc.composite_fwd(z[None], None, pipe.sigma.cpu().numpy()[None, ..., None],
                                           pipe.rgb.cpu().numpy()[None], 1e-4, False)
    good = fl[0] == 0
    assert np.abs(rgb.cpu().numpy() - rf[0])[good].max() <= ATOL
    assert np.abs(dep.cpu().numpy() - rd[0, :, 0])[good].max() <= ATOL
    assert np.abs(ws.cpu().numpy() - rw[0, :, 0])[good].max() <= ATOL

    # the fused render kernel gives the unfused chain's results bit for bit
    pipe.render(_t(ori), _t(dirs), _t(cgrid), _t(cbb), _t(cvs), trunc_m, fused=True, keep_samples=True)
    torch.cuda.synchronize()
    for a, b in zip((pipe.out_rgb, pipe.out_depth, pipe.out_ws, pipe.out_alpha, pipe.z, pipe.node), unfused):
        assert torch.equal(a, b)


@pytest.mark.parametrize("obs,views,frac_colour", [(1.0, 12, False), (0.7, 4, False), (1.0, 4, True)])
def test_fusion_paths_bit_exact(obs, views, frac_colour):
    """The fused kernel's shortcuts (first observation, free space, integer
    colour channels, approximate pixel quotient with exact fall-back) and
    its general path all reproduce the reference arithmetic bit for bit."""
    from sailor_gb300.dist import VoxelEncoding as VE
    D = 96
    sc = syn.make_scene(seed=41, n_views=views, res=160, n_prims=10, D=D, trunc=0.03)
    colors = sc["colors"].copy()
    if frac_colour:
        colors = colors + np.float32(0.37)  # packed values that are not integers
    occ = torch.full((1, D, D, D), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros((1, 1), dtype=torch.int32, device="cuda")
    ts, w, c = VE.integrate_in_box(occ, cnt, _t(sc["K"]), _t(sc["RT"]), _t(colors), _t(sc["depths"]),
                                   _t(sc["vol_bbox"]), _t(sc["voxel_size"]), obs, sc["trunc_weight"], 13.5, 13.5, 0)
    ref = orc.integrate(sc["K"], sc["RT"], colors, sc["depths"], D, sc["vol_bbox"], sc["voxel_size"], obs,
                        sc["trunc_weight"], 13.5, 13.5)
    assert np.array_equal(ts.cpu().numpy(), ref["tsdf"])
    assert np.array_equal(w.cpu().numpy(), ref["weight"])
    assert np.array_equal(c.cpu().numpy(), ref["color"])
    assert np.array_equal(occ.cpu().numpy(), ref["occ"])


@pytest.mark.parametrize("seed,views,res", [(61, 4, 128), (62, 6, 96)])
def test_integrate_auto_bbox_bit_exact(seed, views, res):
    """integrate in the reference's own mode (the cubic box fitted to the
    back-projected depth points, fusion_kernel.cu:51-184): camera inverses,
    origin box, resized box, voxel size and the fused volumes, bit for bit
    against the oracle; get_origin_bbox gives the same origin box."""
    from sailor_gb300.dist import VoxelEncoding as VE
    D = 64
    sc = syn.make_scene(seed=seed, n_views=views, res=res, n_prims=8, D=D, trunc=0.03)
    K, RT = sc["K"], sc["RT"]
    R, T = RT[..., :3], RT[..., 3]
    B = K.shape[0]
    occ = torch.full((B, D, D, D), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros((B, 1), dtype=torch.int32, device="cuda")
    masks = torch.ones(sc["depths"].shape, dtype=torch.int32, device="cuda")
    ts, w, c, vo, vb, vs = VE.integrate(occ, cnt, _t(K), _t(RT), _t(R), _t(T), _t(sc["colors"]), _t(sc["depths"]),
                                        masks, 1.0, 0.025, sc["trunc_weight"], 13.5, 13.5, 0)
    rvo, rvb, rvs = orc.auto_bbox(sc["depths"], K, R, T, D, 0.025)
    assert np.array_equal(vo.cpu().numpy(), rvo)
    assert np.array_equal(vb.cpu().numpy(), rvb)
    assert np.array_equal(vs.cpu().numpy().reshape(-1), rvs.reshape(-1))
    ref = orc.integrate(K, RT, sc["colors"], sc["depths"], D, rvb, rvs, 1.0, sc["trunc_weight"], 13.5, 13.5)
    assert np.array_equal(ts.cpu().numpy(), ref["tsdf"]) and np.array_equal(w.cpu().numpy(), ref["weight"])
    assert np.array_equal(c.cpu().numpy(), ref["color"]) and np.array_equal(occ.cpu().numpy(), ref["occ"])
    org = VE.get_origin_bbox(_t(sc["depths"]), _t(K), _t(R), _t(T), 0.025, 0)
    assert torch.equal(org, vo)


@pytest.mark.parametrize("D", [64, 72])
def test_launch_shapes_do_not_change_results(D):
    """Every autotuner knob value gives bit-identical outputs (D = 72: the
    16^3 fusion tiles are partial at the grid's far faces)."""
    from sailor_gb300 import autotune
    from sailor_gb300.dist import VoxelEncoding as VE
    sc = syn.make_scene(seed=51, n_views=4, res=128, n_prims=8, D=D, trunc=0.03)
    saved = autotune.current()
    outs = []
    try:
        for tiled, vpt, blk in ((1, 4, 128), (0, 1, 64), (0, 2, 128), (0, 4, 256)):
            autotune.set_knob("fuse_tiled", tiled)
            autotune.set_knob("fuse_vpt", vpt)
            autotune.set_knob("fuse_block", blk)
            occ = torch.full((1, D, D, D), -1, dtype=torch.int32, device="cuda")
            cnt = torch.zeros((1, 1), dtype=torch.int32, device="cuda")
            r = VE.integrate_in_box(occ, cnt, _t(sc["K"]), _t(sc["RT"]), _t(sc["colors"]), _t(sc["depths"]),
                                    _t(sc["vol_bbox"]), _t(sc["voxel_size"]), 1.0, sc["trunc_weight"], 13.5, 13.5, 0)
            outs.append([t.clone() for t in r] + [occ, cnt])
    finally:
        for k, v in saved.items():
            autotune.set_knob(k, v)
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert torch.equal(a, b)
