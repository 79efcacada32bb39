"""Multi-level tree, depth-first traversal and fine sampling on the GPU
(sg_octree_build, sg_octree_traversal, sg_sample_fine through the drop-in
MultiLayerOctree) against the oracle (oracle/octree_oracle.c):

* the build is bit-exact: node tables, the node ids written into every
  level's volume, the node table tensor's geometry;
* traversal rows: node ids bit-exact on every ray the oracle does not flag
  (coarse and fine rows, counts), depths within 1e-5 relative (the
  reference's __fdividef reciprocal), valid lengths within 1e-5 relative;
  early stop and the coarse-hit cap as the reference has them;
* fine sampling: bit-exact against the oracle run on the GPU's own rows
  (every ray: no approximate operation is involved);
* row overflow is reported (status flag and largest counts) and the
  sampling call then refuses to run;
* a 256^3 four-level tree with a 512^2 target (the headline grid size),
  checked on a subsample of rays.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

REL = 1e-5


def _cuda(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


def _scene(D, res, n_views, tres, seed, batch=1):
    sc = syn.make_scene(seed=seed, n_views=n_views, res=res, n_prims=10, D=D, trunc=0.03, batch=batch)
    fz = orc.integrate(sc["K"], sc["RT"], sc["colors"], sc["depths"], D, sc["vol_bbox"], sc["voxel_size"], 1.0,
                       sc["trunc_weight"], 13.5, 13.5)
    ori, dirs = syn.target_rays(seed=seed, res=tres, batch=batch)
    return dict(sc=sc, occ=fz["occ"], ori=ori, dirs=dirs, vs=sc["voxel_size"].reshape(-1).astype(np.float32),
                bbox=sc["vol_bbox"].astype(np.float32))


@pytest.fixture(scope="module")
def s64():
    return _scene(64, 128, 4, 64, 5)


def _trees(s, rate, L):
    from sailor_gb300.dist import VoxelEncoding as VE
    occ = s["occ"]
    vols, cnts = orc.merge_levels(occ, (occ > -1).reshape(occ.shape[0], -1).sum(1), rate, L)
    ref = orc.build_octree(vols, rate)
    totals = [int((v > -1).sum()) for v in vols]
    index = [sum(totals[:l]) for l in range(L)]
    gv = [_cuda(v, torch.int32) for v in vols]
    o = VE.MultiLayerOctree(L, occ.shape[0], rate, 0)
    o.init_octree(gv, totals, [_cuda(c, torch.int32) for c in cnts], index, _cuda(s["vs"]), _cuda(s["bbox"]))
    o.build_octree()
    o._levels()  # two levels: the multi-level tables are otherwise built on first use
    torch.cuda.synchronize()
    return o, gv, ref


def _close(a, b):
    return np.all(np.abs(a - b) <= REL * np.maximum(np.abs(a), np.abs(b)) + 1e-6)


@pytest.mark.parametrize("rate,L", [(4, 2), (2, 3), (2, 4)])
def test_build_matches_oracle(s64, rate, L):
    o, gv, ref = _trees(s64, rate, L)
    assert o._ostatus[0].item() == 0
    assert np.array_equal(o._obufs["counts"].cpu().numpy(), ref["counts"])
    for l in range(L):
        assert np.array_equal(gv[l].cpu().numpy(), ref["vols"][l]), l
        n = ref["counts"][l]
        coff = int(np.sum(ref["cap"][:l]))
        assert np.array_equal(o._obufs["key"][l][:n].cpu().numpy(), ref["key"][coff:coff + n])
        assert np.array_equal(o._obufs["parent"][l][:n].cpu().numpy(), ref["parent"][coff:coff + n])
        if l > 0:
            assert np.array_equal(o._obufs["nchild"][l][:n].cpu().numpy(), ref["nchild"][coff:coff + n])
            assert np.array_equal(o._obufs["child_base"][l][:n].cpu().numpy(), ref["child_base"][coff:coff + n])
    nodes = o.get_nodes_tensor().cpu().numpy()
    keys = orc.octree_node_keys(ref, np.arange(ref["n_nodes"]))
    lv = orc.octree_level_of(ref, np.arange(ref["n_nodes"]))
    built = np.zeros(ref["n_nodes"], bool)
    for l in range(L):
        built[ref["base"][l]:ref["base"][l] + ref["counts"][l]] = True
    assert np.all(nodes[~built] == 0) and np.all(nodes[built, 4] == 1)
    for g in np.flatnonzero(built)[::7]:
        c, nvs = orc.node_geometry(s64["vs"][keys[g, 1]], int(ref["dims"][0] // ref["dims"][lv[g]]),
                                   s64["bbox"][keys[g, 1], :, 0], keys[g, 2:])
        assert np.array_equal(nodes[g, :3], c) and nodes[g, 3] == np.float32(nvs)
    if L == 2:  # the same ids as the two-level tree
        assert np.array_equal(o.tree_arrays()["top_key"][:ref["counts"][1]].cpu().numpy(),
                              ref["key"][ref["cap"][0]:ref["cap"][0] + ref["counts"][1]])


def _compare_rows(ot, g, what, max_scale):
    """Rows of the rays the oracle does not flag: ids exact, depths within
    1e-5 relative, valid lengths within the depth error carried through
    (t1 - t0) x scale of every entry (see test_oracle_octree.vl_tol).  Deep
    descents flag more rays: a descendant's depths come within an ulp of an
    entry's far more often than the DDA's crossings do."""
    from test_oracle_octree import vl_tol
    ok = ot["flags"][0] == 0
    assert ok.mean() > 0.75 and ok.sum() > 500, what
    for name in ("idx_c", "idx"):
        a = g[name][0][ok]
        b = ot[name][0][ok]
        assert np.array_equal(a, b), (what, name, np.flatnonzero(ok)[np.any(a != b, 1)][:5])
    for name in ("t0_c", "t1_c", "t0", "t1"):
        assert _close(g[name][0][ok], ot[name][0][ok]), (what, name)
    vl = ot["valid_len"][0, :, 0]
    assert (np.abs(g["valid_len"][0, :, 0] - vl) <= vl_tol(ot, vl, max_scale))[ok].all(), what
    return ok


def _gpu_rows(o, s, start, Wc, Wf, th=-1, opt=-1, ori=None, dirs=None):
    ori = s["ori"] if ori is None else ori
    dirs = s["dirs"] if dirs is None else dirs
    idx, t0, t1, vl, idx_c, t0_c, t1_c = o.octree_traversal(_cuda(ori), _cuda(dirs), Wc, Wf, start, th, opt)
    torch.cuda.synchronize()
    return dict(idx=idx.cpu().numpy(), t0=t0.cpu().numpy(), t1=t1.cpu().numpy(), valid_len=vl.cpu().numpy(),
                idx_c=idx_c.cpu().numpy(), t0_c=t0_c.cpu().numpy(), t1_c=t1_c.cpu().numpy(),
                gpu=(idx, t0, t1, vl))


@pytest.mark.parametrize("rate,L,start", [(4, 2, 0), (2, 3, 0), (2, 3, 1), (2, 4, 0), (2, 4, 2)])
def test_traversal_matches_oracle(s64, rate, L, start):
    o, _, ref = _trees(s64, rate, L)
    s = L - 1 - start
    Wc, Wf = 4 * int(ref["dims"][s]), 2048
    g = _gpu_rows(o, s64, start, Wc, Wf)
    ot = orc.octree_traversal(ref, s64["ori"], s64["dirs"], s64["vs"], s64["bbox"], start, Wc, Wf)
    ok = _compare_rows(ot, g, (rate, L, start), rate ** s)
    assert ot["max_fine"] > ot["max_coarse"] > 2
    st = o._ostatus.cpu().numpy()
    assert st[0] == 0 and st[1] == (g["idx_c"] >= 0).sum(-1).max() and st[2] == (g["idx"] >= 0).sum(-1).max()
    assert ok.sum() > 800


def test_traversal_early_stop_and_cap(s64):
    o, _, ref = _trees(s64, 2, 3)
    Wc, Wf = 128, 1024
    for th, opt in ((3, -1), (-1, 4), (2, 6)):
        g = _gpu_rows(o, s64, 0, Wc, Wf, th, opt)
        ot = orc.octree_traversal(ref, s64["ori"], s64["dirs"], s64["vs"], s64["bbox"], 0, Wc, Wf, th, opt)
        _compare_rows(ot, g, (th, opt), 4)
        if opt > 0:
            assert ((g["idx_c"] >= 0).sum(-1) <= opt).all()


@pytest.mark.parametrize("rate,L,start,S", [(2, 3, 0, 32), (2, 3, 1, 96), (2, 4, 1, 64), (4, 2, 0, 48)])
def test_sample_fine_matches_oracle(s64, rate, L, start, S):
    o, _, ref = _trees(s64, rate, L)
    s = L - 1 - start
    g = _gpu_rows(o, s64, start, 4 * int(ref["dims"][s]), 2048)
    B, N = s64["ori"].shape[:2]
    rd = np.random.default_rng(11).random((B, N, S), dtype=np.float32)
    idx, t0, t1, vl = g["gpu"]
    si, sz = o.ray_voxels_points_sampling(idx, t0, t1, vl, _cuda(rd), start, S)
    torch.cuda.synchronize()
    ri, rz, fl = orc.sample_fine(ref, g["idx"], g["t0"], g["t1"], g["valid_len"], rd, s64["vs"], S, start)
    assert np.array_equal(si.cpu().numpy(), ri)
    assert np.array_equal(sz.cpu().numpy(), rz)
    hit = (g["idx"][0] >= 0).any(1)
    assert hit.sum() > 500 and ((ri[0][hit] >= 0).sum(1) == S).all() and (ri[0][~hit] == -1).all()


def test_row_overflow_reported(s64):
    from sailor_gb300 import _native as N
    o, _, ref = _trees(s64, 2, 3)
    ot = orc.octree_traversal(ref, s64["ori"], s64["dirs"], s64["vs"], s64["bbox"], 0, 128, 2048)
    Wf = 4
    assert ot["max_fine"] > Wf
    g = _gpu_rows(o, s64, 0, 128, Wf)
    st = o._ostatus.cpu().numpy()
    ok = ot["flags"][0] == 0
    assert st[0] & N.SG_FLAG_HIT_OVERFLOW and st[2] >= ot["cnt"][0][ok].max() > Wf
    # the first Wf entries are kept
    assert np.array_equal(g["idx"][0][ok], ot["idx"][0][ok][:, :Wf])
    idx, t0, t1, vl = g["gpu"]
    with pytest.raises(RuntimeError, match="overflow"):
        o.ray_voxels_points_sampling(idx, t0, t1, vl, torch.rand(1, s64["ori"].shape[1], 16, device="cuda"), 0, 16)


def test_headline_grid_four_levels():
    """256^3 fine grid, rate 2, four levels (256/128/64/32), 4 views of
    512^2 and a 512^2 target: GPU traversal and fine sampling over all
    262,144 rays; rows and samples checked against the oracle on 8,192 of
    them."""
    s = _scene(256, 512, 4, 512, 3)
    o, _, ref = _trees(s, 2, 4)
    N = s["ori"].shape[1]
    start, S = 1, 64
    g = _gpu_rows(o, s, start, 4 * 64, 2048)
    pick = np.random.default_rng(2).choice(N, 8192, replace=False)
    pick.sort()
    ot = orc.octree_traversal(ref, s["ori"][:, pick], s["dirs"][:, pick], s["vs"], s["bbox"], start, 256, 2048)
    sub = {k: v[:, pick] for k, v in g.items() if k != "gpu"}
    ok = _compare_rows(ot, sub, "headline", 4)
    assert (ot["cnt"][0] > 0).sum() > 1000
    rd = np.random.default_rng(4).random((1, N, S), dtype=np.float32)
    idx, t0, t1, vl = g["gpu"]
    si, sz = o.ray_voxels_points_sampling(idx, t0, t1, vl, _cuda(rd), start, S)
    ri, rz, _ = orc.sample_fine(ref, sub["idx"], sub["t0"], sub["t1"], sub["valid_len"], rd[:, pick], s["vs"], S,
                                start)
    assert np.array_equal(si.cpu().numpy()[:, pick], ri) and np.array_equal(sz.cpu().numpy()[:, pick], rz)
    del ok


def test_two_frames():
    """Two frames in one tree (node keys carry the frame): build, traversal
    from the top and from the middle level, and fine sampling against the
    oracle."""
    s = _scene(64, 128, 4, 48, 9, batch=2)
    o, gv, ref = _trees(s, 2, 3)
    for l in range(3):
        assert np.array_equal(gv[l].cpu().numpy(), ref["vols"][l])
    for start in (0, 1):
        sl = 2 - start
        Wc = 4 * int(ref["dims"][sl])
        g = _gpu_rows(o, s, start, Wc, 2048)
        ot = orc.octree_traversal(ref, s["ori"], s["dirs"], s["vs"], s["bbox"], start, Wc, 2048)
        for b in range(2):
            sub_g = {k: v[b:b + 1] for k, v in g.items() if k != "gpu"}
            sub_o = dict(ot, **{k: ot[k][b:b + 1] for k in ("idx", "t0", "t1", "idx_c", "t0_c", "t1_c", "valid_len",
                                                             "flags", "cnt")})
            _compare_rows(sub_o, sub_g, ("two frames", start, b), 2 ** sl)
        idx, t0, t1, vl = g["gpu"]
        S = 48
        rd = np.random.default_rng(3).random((2, s["ori"].shape[1], S), dtype=np.float32)
        si, sz = o.ray_voxels_points_sampling(idx, t0, t1, vl, _cuda(rd), start, S)
        ri, rz, _ = orc.sample_fine(ref, g["idx"], g["t0"], g["t1"], g["valid_len"], rd, s["vs"], S, start)
        assert np.array_equal(si.cpu().numpy(), ri) and np.array_equal(sz.cpu().numpy(), rz)
        assert (g["idx"][1] >= 0).sum() > 100  # the second frame's rays hit its own tree
