"""Pin the CPU oracle against the reference's own outputs (CPU only).

The golden files were produced by running SAILOR's CUDA kernels, compiled
from its sources for sm_103a and launched from cubins
(tests/golden/make_golden.py).  The reference's node ids come from atomicAdd
queues, so nodes are compared through canonical (level, frame, x, y, z)
keys.  The oracle uses a correctly rounded reciprocal where the reference
uses __fdividef; rays the oracle flags as near-ties are excluded from the
bit-exact hit comparisons, and t-intervals are compared within 1e-5.
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CHAINS = ["explicit", "auto"]


@pytest.fixture(scope="module", params=CHAINS)
def chain(request, golden):
    g = golden(f"ref_chain_{request.param}.npz")
    D, rate = int(g["meta_D"]), int(g["meta_rate"])
    tw = float(g["meta_trunc_weight"])
    out = dict(g=g, D=D, rate=rate, S=int(g["meta_S"]), tw=tw, name=request.param)
    if request.param == "auto":
        R = np.ascontiguousarray(g["RT"][..., :3])
        T = np.ascontiguousarray(g["RT"][..., 3])
        out["auto"] = orc.auto_bbox(g["depths"], g["K"], R, T, D, 0.025)
    vb, vs = g["fusion_vol_bbox"], g["fusion_voxel_size"]
    fz = orc.integrate(g["K"], g["RT"], g["colors"], g["depths"], D, vb, vs, 1.0, tw, 13.5, 13.5)
    top, cnt = orc.merge(fz["occ"], rate)
    tree = orc.build_tree(top, fz["occ"])
    hits = orc.voxel_traversal(tree, g["ori"], g["dirs"], vs, vb, W=1024)
    out.update(fz=fz, top=top, cnt=cnt, tree=tree, hits=hits, vb=vb, vs=vs)
    return out


def test_camera_inverse_and_bbox(chain):
    if chain["name"] != "auto":
        pytest.skip("explicit box")
    g = chain["g"]
    R = np.ascontiguousarray(g["RT"][..., :3])
    assert np.array_equal(orc.inverse3x3(g["K"]), g["Kinv"])
    assert np.array_equal(orc.inverse3x3(R), g["Rinv"])
    vo, vb, vs = chain["auto"]
    assert np.array_equal(vo, g["fusion_vol_origin"])
    assert np.array_equal(vb, g["fusion_vol_bbox"])
    assert np.array_equal(vs, g["fusion_voxel_size"])


def test_fusion_bit_exact(chain):
    g, fz = chain["g"], chain["fz"]
    for k in ("tsdf", "weight", "color", "occ"):
        assert np.array_equal(fz[k], g["fusion_" + k]), k
    assert np.array_equal(fz["count"].ravel(), g["fusion_count"].ravel())


def test_merge_exact(chain):
    g = chain["g"]
    assert np.array_equal(chain["top"], g["merge_occ"])
    assert np.array_equal(chain["cnt"].ravel(), g["merge_count"].ravel())


def test_tree_node_sets(chain):
    g, t = chain["g"], chain["tree"]
    assert [t["ntop"], t["nbot"]] == g["tree_queue"].tolist()
    keys = g["tree_node_keys"]
    ref = {tuple(k) for k in keys[keys[:, 0] >= 0].tolist()}
    ids = list(range(t["base_top"], t["base_top"] + t["ntop"])) + list(range(t["nbot"]))
    mine = {tuple(k) for k in orc.node_keys(t, np.array(ids)).tolist()}
    assert ref == mine
    # node geometry (centre, edge) of every reference node
    cen, nvs, valid = g["tree_node_centre"], g["tree_node_vs"], g["tree_node_valid"]
    vs, vb = chain["vs"], chain["vb"]
    rate = chain["rate"]
    for n in np.nonzero(valid)[0][::7]:
        lvl, b, x, y, z = keys[n]
        c, v = orc.node_geometry(vs[b, 0], rate if lvl == 1 else 1, vb[b, :, 0], np.array([x, y, z]))
        assert np.array_equal(c, cen[n]) and np.float32(v) == nvs[n]
    # children lists: the reference's child order is its own atomic order;
    # the set of children per top node must match
    ch = g["tree_node_children"]
    for n in np.nonzero((keys[:, 0] == 1))[0][:200]:
        kids = {tuple(k) for k in ch[n].tolist() if k[0] >= 0}
        k = keys[n]
        mine_k = {(0, k[1], k[2] * rate + a, k[3] * rate + c, k[4] * rate + e)
                  for a in range(rate) for c in range(rate) for e in range(rate)}
        assert kids <= mine_k


def _canon_rows(tree, idx):
    k = orc.node_keys(tree, idx)
    k[idx < 0] = -1
    return k


def test_traversal_rows(chain):
    g, h, t = chain["g"], chain["hits"], chain["tree"]
    mh = int(g["trav_max_hits"])
    assert h["max_hits"] == mh
    mine = _canon_rows(t, h["idx"][..., :mh])
    rows = np.all(mine == g["trav_keys"], axis=(-1, -2))
    ok = h["flags"] == 0
    assert rows[ok].all()
    assert ok.mean() > 0.95
    m = (g["trav_keys"][..., 0] >= 0) & rows[..., None]
    assert np.abs(h["t0"][..., :mh][m] - g["trav_t0"][m]).max() <= 1e-5
    assert np.abs(h["t1"][..., :mh][m] - g["trav_t1"][m]).max() <= 1e-5
    assert np.array_equal(h["nhit"][ok], g["trav_count"][ok])


def test_traversal_training_and_early_stop(chain):
    g, t = chain["g"], chain["tree"]
    h = orc.voxel_traversal(t, g["ori"], g["dirs"], chain["vs"], chain["vb"], W=1024, is_training=True)
    w = g["trav_train_keys"].shape[-2]
    rows = np.all(_canon_rows(t, h["idx"][..., :w]) == g["trav_train_keys"], axis=(-1, -2))
    assert rows[h["flags"] == 0].all()
    h = orc.voxel_traversal(t, g["ori"], g["dirs"], chain["vs"], chain["vb"], W=1024, th_early_stop=3, opt_num=6)
    w = g["trav_stop_keys"].shape[-2]
    rows = np.all(_canon_rows(t, h["idx"][..., :w]) == g["trav_stop_keys"], axis=(-1, -2))
    assert rows[h["flags"] == 0].all()
    assert np.array_equal(h["nhit"][h["flags"] == 0], g["trav_stop_count"][h["flags"] == 0])


@pytest.mark.parametrize("j", [0, 1])
def test_sampling_bit_exact_given_reference_hits(chain, j):
    """Reference hit lists in -> the oracle's samples equal the reference's
    bit for bit (counts, node keys, depths), for inference (rand = 0.5) and
    random jitter (the reference's double-precision depth expression)."""
    g, t = chain["g"], chain["tree"]
    ids = list(range(t["base_top"], t["base_top"] + t["ntop"])) + list(range(t["nbot"]))
    kmap = {tuple(k): i for k, i in zip(orc.node_keys(t, np.array(ids)).tolist(), ids)}
    rk = g["trav_keys"]
    idx = np.full(rk.shape[:-1], -1, np.int32)
    m = rk[..., 0] >= 0
    idx[m] = [kmap[tuple(k)] for k in rk[m].tolist()]
    hits = dict(idx=idx, t0=g["trav_t0"], t1=g["trav_t1"], valid_len=g["trav_valid_len"],
                max_hits=int(g["trav_max_hits"]), flags=np.zeros(idx.shape[:2], np.int32))
    si, sz, _ = orc.sample_coarse(t, hits, g[f"rands{j}"], chain["vs"], chain["S"])
    assert np.array_equal(sz, g[f"samp{j}_z"])
    assert np.array_equal(_canon_rows(t, si), g[f"samp{j}_keys"])
    srt, sidx = orc.sort(sz)
    assert np.array_equal(srt, g[f"samp{j}_sorted"])
    # torch::sort's order of equal keys is unspecified: compare modulo ties
    assert np.array_equal(np.take_along_axis(sz, sidx.astype(np.int64), -1),
                          np.take_along_axis(sz, g[f"samp{j}_sort_idx"].astype(np.int64), -1))


@pytest.mark.parametrize("tag,occ", [("den", False), ("occ", True)])
def test_composite_fwd_bwd_vs_reference(golden, tag, occ):
    c = golden("ref_composite.npz")
    sg = c["occ"] if occ else c["sigma"]
    of, od, ow, oa, fl = orc.composite_fwd(c["z"], c["sort_idx"], sg, c["feats"], 1e-4, occ)
    ok = fl == 0
    for mine, k in ((of, "feat"), (od, "depth"), (ow, "ws"), (oa, "alpha")):
        assert np.abs(mine - c[f"{tag}_fwd_{k}"])[ok].max() <= 1e-5, k
    outs = [c[f"{tag}_fwd_{k}"] for k in ("feat", "depth", "ws", "alpha")]
    gf, gs = orc.composite_bwd_ref(c["g_feat"], c["g_depth"], c["g_ws"], c["g_alpha"], *outs, c["z"],
                                   c["sort_idx"], sg, c["feats"], 1e-4, occ)
    assert np.abs(gf - c[f"{tag}_bwd_feat"])[ok].max() <= 1e-5
    ref = c[f"{tag}_bwd_sigma"]
    big = np.abs(ref) > 1e3  # delta = 1e10 entries (last sample): cancellation noise
    d = np.abs(gs - ref)[ok]
    assert d[~big[ok]].max() <= 1e-4
    assert (d[big[ok]] <= 1e-3 * np.abs(ref[ok][big[ok]]) + 1e4).all()


def test_presorted_occupancy(golden):
    c = golden("ref_composite.npz")
    of, od, ow, oa, fl = orc.composite_fwd(c["sorted_z"], None, c["presorted_occ"], c["presorted_feats"], 1e-4,
                                           True)
    ok = fl == 0
    for mine, k in ((of, "feat"), (od, "depth"), (ow, "ws"), (oa, "alpha")):
        assert np.abs(mine - c[f"presorted_fwd_{k}"])[ok].max() <= 1e-5, k


def test_rays_bit_exact_vs_reference():
    """Ray generation (rays_calculating, sampling_kernel.cu:674-731) against
    the reference kernel's own output: origins, directions and the inverses,
    bit for bit (ring cameras and cameras with skew and an off-centre
    principal point)."""
    import os
    p = os.path.join(os.path.dirname(__file__), "golden", "ref_rays.npz")
    if not os.path.exists(p):
        pytest.skip("ref_rays.npz not generated")
    g = np.load(p)
    H = int(g["load_size"])
    out = orc.rays(g["K"], g["R"], g["T"], H)
    assert np.array_equal(out.view(np.uint32), g["rays"].view(np.uint32))
    assert np.array_equal(orc.inverse3x3(g["K"]).view(np.uint32), g["Kinv"].view(np.uint32))
    assert np.array_equal(orc.inverse3x3(g["R"]).view(np.uint32), g["Rinv"].view(np.uint32))


def test_project_xyz_bit_exact_vs_reference(golden):
    """Projection of sampled points (project_xyz, sampling_kernel.cu:55-159)
    against the reference kernel's own output, with node corners at 640 x 480
    (the double-precision normalisation with half sizes that are not powers
    of two) and without at 512 x 512: bit for bit, -1 fills included.  The
    corner table is the reference's node array (ids remapped)."""
    g = golden("ref_project.npz")
    for name, table in (("corners", g["node_corners"]), ("point", None)):
        w, h = (int(v) for v in g[f"{name}_size"])
        xy, pz = orc.project_xyz(g["ori"], g["dirs"], g["sampled_z"], g["sampled_idx"], g["K"], g["RT"], w, h,
                                 corners=table)
        assert np.array_equal(xy.reshape(-1).view(np.uint32), g[f"{name}_xy"].reshape(-1).view(np.uint32)), name
        assert np.array_equal(pz.reshape(-1).view(np.uint32), g[f"{name}_z"].reshape(-1).view(np.uint32)), name
    assert (g["sampled_idx"] == -1).any() and (g["corners_xy"] != -1).any()


def test_node_corners_bit_exact_vs_reference(golden):
    """The oracle's node geometry (centre plus or minus half the edge, the
    corner order of octree.h:120-129) gives the reference's corner table bit
    for bit, for top bricks and fine voxels."""
    g = golden("ref_project.npz")
    vs = float(np.asarray(g["voxel_size"]).reshape(-1)[0])
    bmin = np.ascontiguousarray(g["vol_bbox"][0, :, 0])
    rate = int(g["rate"])
    levels = set()
    for key, ref in zip(g["node_keys"], g["node_corners"]):
        lvl, b, x, y, z = (int(v) for v in key)
        levels.add(lvl)
        c, nvs = orc.node_geometry(vs, rate if lvl == 1 else 1, bmin, np.array([x, y, z], np.int32))
        hh = np.float32(nvs) / np.float32(2.0)
        for i in range(8):
            sgn = np.array([1 if i & 4 else -1, 1 if i & 2 else -1, 1 if i & 1 else -1], np.float32)
            assert np.array_equal((c + sgn * hh).view(np.uint32), ref[i].view(np.uint32))
    assert levels == {0, 1}


def test_grid_sample_restatement_vs_torch():
    """The oracle's float64 bilinear gather against torch's F.grid_sample
    (CPU, float64, align_corners=True, zero padding), edges and the -2
    invalid marker included."""
    import torch
    import torch.nn.functional as F
    rng = np.random.default_rng(1)
    img = rng.normal(size=(3, 5, 17, 23))
    grid = rng.uniform(-1.2, 1.2, (3, 400, 2))
    grid[:, :10] = -2.0
    grid[:, 10:20, 0] = 1.0
    grid[:, 20:30, 1] = -1.0
    ref = F.grid_sample(torch.tensor(img), torch.tensor(grid)[:, :, None, :], align_corners=True,
                        mode="bilinear")[..., 0].permute(0, 2, 1).numpy()
    assert np.abs(orc.grid_sample(img, grid) - ref).max() <= 1e-12


def test_trilerp_nodes_against_reference_golden():
    """Pin of the node-corner trilinear gather and its adjoint
    (trilinear_aggregate_features(_backward), sampling_kernel.cu:162-327):
    the reference's kernels, run on its own two-level tree and coarse samples
    (tests/golden/ref_trilerp.npz, inputs at the kernels' per-sample stride
    of 64 so that they stay in bounds), against the oracle's float64
    restatement on the same node corners and sample points (the kernels'
    fused multiply-add point): outputs and gradients within 1e-6 relative to
    the values' scale (the reference forms its fractions in float32; the
    measured gap is 1e-7 and 2e-7)."""
    path = os.path.join(GOLDEN, "ref_trilerp.npz")
    if not os.path.exists(path):
        pytest.skip("ref_trilerp.npz not generated (tests/golden/make_golden.py --only trilerp)")
    g = np.load(path)
    B, C, R, S, _ = g["feats"].shape
    pts = orc.sample_points(g["ori"][0], g["dirs"][0], g["sampled_z"][0]).reshape(-1, 3)
    valid = g["valid"].reshape(-1).astype(np.int32)
    assert valid.mean() > 0.5
    corners = g["corners"].reshape(-1, 8, 3)
    fo = g["feats"].transpose(1, 0, 2, 3, 4).reshape(C, -1, 8)
    go = g["gout"].transpose(1, 0, 2, 3).reshape(C, -1)
    ro, rg = orc.trilerp_nodes(pts, corners, valid, fo, go)
    ro = ro.reshape(C, B, R, S).transpose(1, 0, 2, 3)
    rg = rg.reshape(C, B, R, S, 8).transpose(1, 0, 2, 3, 4)
    scale_o = np.abs(g["out"]).max()
    scale_g = np.abs(g["grad"]).max()
    assert np.abs(ro - g["out"]).max() <= 1e-6 * scale_o
    assert np.abs(rg - g["grad"]).max() <= 1e-6 * scale_g
    # samples without a node: zeros in both
    inv = ~valid.astype(bool).reshape(B, R, S)
    assert np.all(g["out"][:, :, inv[0]] == 0) and np.all(ro[:, :, inv[0]] == 0)
