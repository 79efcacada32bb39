"""GPU parity at the headline sizes: the plain configuration (4 synthetic
RGBD views of 512^2 with 12 capsules/ellipsoids, a 256^3 TSDF grid over the
2 m cube (7.8 mm voxels), 3 cm truncation, 8^3 bricks, one 512^2 target view,
64 samples per ray at rand 0.5, density sigmoid(-sdf / 5 mm) / 5 mm from the
fused TSDF, colour trilinear from a seeded 256^3 x 3 grid), every stage
against the oracle through the C ABI:

* fusion (tsdf, weight, colour, occupancy, count) bit-exact;
* coarse occupancy, node ids and the rewritten volumes exact;
* traversal rows exact on unflagged rays, t-intervals within 1e-5;
* coarse sampling + sort: node ids exact and depths within 1e-5 from the
  oracle's own rows, bit-exact on every ray from the GPU's rows;
* end to end: the fused render (sampling, sort, field taps, compositing in
  one kernel) and the unfused four-kernel chain against the float64 render
  of those samples (float32 sample points as the kernels form them, then
  taps, density and compositing in float64): each composited output within
  ATOL of the FP64 oracle on every ray but early-termination ties; the
  errors are printed.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from sailor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

ATOL = 1e-5
CFG = dict(seed=7, views=4, res=512, prims=12, D=256, rate=8, trunc=0.03, target=512, S=64, W=256, Dc=256,
           sdf_s=0.005)


def _t(a, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")


@pytest.fixture(scope="module")
def headline():
    from test_gpu_parity import gpu_chain
    c = CFG
    sc = syn.make_scene(seed=c["seed"], n_views=c["views"], res=c["res"], n_prims=c["prims"], D=c["D"],
                        trunc=c["trunc"])
    ori, dirs = syn.target_rays(seed=c["seed"], res=c["target"])
    R = ori.shape[1]
    rands = np.full((1, R, c["S"]), 0.5, np.float32)
    g = gpu_chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, c["W"])
    ref = orc.chain(sc, c["D"], c["rate"], c["S"], ori, dirs, rands, W=c["W"], trunc_weight=sc["trunc_weight"])
    g.pop("octree")
    return dict(sc=sc, ori=ori, dirs=dirs, g=g, ref=ref)


def test_headline_fusion_and_tree_exact(headline):
    g, r = headline["g"], headline["ref"]
    f = r["fusion"]
    for k in ("tsdf", "weight", "color"):
        assert np.array_equal(g[k].view(np.uint32), f[k].view(np.uint32)), k
    assert np.array_equal(g["occ0"], f["occ"]) and np.array_equal(g["cnt0"].ravel(), f["count"].ravel())
    assert np.array_equal(g["occ1"], r["top"]) and np.array_equal(g["cnt1"].ravel(), r["cnt_top"].ravel())
    t = r["tree"]
    assert g["counts"] == [t["ntop"], t["nbot"]] and t["ntop"] > 500
    assert np.array_equal(g["occ1_post"], t["occ_top"]) and np.array_equal(g["occ0_post"], t["occ_bot"])
    print(f"headline fusion: {int(f['count'].sum())} occupied voxels, {t['ntop']} top nodes, "
          f"{t['nbot']} fine nodes")


def test_headline_traversal_and_samples_exact(headline):
    g, r = headline["g"], headline["ref"]
    h = r["hits"]
    assert h["max_hits"] <= CFG["W"], "rows too narrow for the scene"
    ok = (h["flags"] == 0) & (r["flags"] == 0)
    rows_eq = np.all(g["idx"] == h["idx"], axis=-1)
    assert rows_eq[h["flags"] == 0].all()
    m = (h["idx"] >= 0) & rows_eq[..., None]
    assert np.abs(g["t0"][m] - h["t0"][m]).max() <= ATOL and np.abs(g["t1"][m] - h["t1"][m]).max() <= ATOL
    # samples from the oracle's own rows: node ids exact, depths within 1e-5
    # (the rows' t-intervals differ by ulps: the GPU's approximate reciprocal)
    assert np.array_equal(g["si"][ok], r["sampled_idx"][ok])
    assert np.abs(g["sz"][ok] - r["sampled_z"][ok]).max() <= ATOL
    # sampling and sort of the GPU's own rows: bit for bit on every ray
    rows = dict(idx=g["idx"], t0=g["t0"], t1=g["t1"], valid_len=g["vl"], max_hits=int((g["idx"] >= 0).sum(-1).max()),
                flags=np.zeros(g["idx"].shape[:2], np.int32))
    si, sz, _ = orc.sample_coarse(r["tree"], rows, np.full(g["sz"].shape, 0.5, np.float32), r["voxel_size"],
                                  CFG["S"])
    srt, _ = orc.sort(sz)
    assert np.array_equal(g["si"], si) and np.array_equal(g["sz"].view(np.uint32), sz.view(np.uint32))
    assert np.array_equal(g["srt"].view(np.uint32), srt.view(np.uint32))
    hit = (h["idx"][..., 0] >= 0)
    print(f"headline traversal: {int(hit.sum())} of {hit.size} rays hit, {int((~ok).sum())} flagged, "
          f"max hits {h['max_hits']}")
    assert hit.sum() > 0.1 * hit.size and (~ok).mean() < 0.05


@pytest.mark.parametrize("fused", [True, False])
def test_headline_render_vs_fp64(headline, fused):
    from sailor_gb300.pipeline import FramePipeline
    c, sc, r = CFG, headline["sc"], headline["ref"]
    ori, dirs = headline["ori"], headline["dirs"]
    R, S, D = ori.shape[1], c["S"], c["D"]
    rng = np.random.default_rng(c["seed"])
    Dc = c["Dc"]
    cgrid = rng.random((1, Dc, Dc, Dc, 3), dtype=np.float32)
    cvs = np.full((1, 1), np.float32(2.0) / np.float32(Dc - 1), np.float32)
    cbb = np.array([[[-1.0, 1.0]] * 3], np.float32)
    pipe = FramePipeline(1, D, c["rate"], R, S, W_hits=c["W"])
    pipe.build(_t(sc["K"]), _t(sc["RT"]), _t(sc["colors"]), _t(sc["depths"]), _t(sc["vol_bbox"]),
               _t(sc["voxel_size"]), sc["trunc_weight"])
    trunc_m = float(sc["voxel_size"][0, 0]) * sc["trunc_weight"]
    out = pipe.render(_t(ori), _t(dirs), _t(cgrid), _t(cbb), _t(cvs), trunc_m, sdf_scale=c["sdf_s"], fused=fused,
                      keep_samples=True)
    torch.cuda.synchronize()
    assert pipe.status[0].item() == 0
    rgb, dep, ws, al = (o.cpu().numpy().reshape(R, -1) for o in out)
    z = pipe.z.cpu().numpy()
    # the pipeline's samples: the oracle's sampling of the GPU rows (checked
    # bit for bit above); here against the drop-in chain's sorted samples
    assert np.array_equal(z.view(np.uint32), headline["g"]["srt"][0].view(np.uint32))
    f64 = orc.render_fp64(ori[0], dirs[0], z, r["fusion"]["tsdf"], sc["vol_bbox"][:, :, 0],
                          sc["voxel_size"][:, 0], trunc_m, c["sdf_s"], cgrid, None, 1e-4,
                          feat_bbox_min=cbb[:, :, 0], feat_voxel_size=cvs[:, 0])
    ok = f64["flags"] == 0
    assert ok.mean() > 0.999
    errs = dict(rgb=np.abs(rgb - f64["rgb"])[ok].max(), depth=np.abs(dep[:, 0] - f64["depth"])[ok].max(),
                ws=np.abs(ws[:, 0] - f64["ws"])[ok].max(), alpha=np.abs(al[:, 0] - f64["alpha"])[ok].max())
    print(f"headline render ({'fused' if fused else 'unfused'}) vs FP64 on {int(ok.sum())} of {R} rays: "
          + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert f64["ws"].max() > 0.5
    for k, v in errs.items():
        assert v <= ATOL, (k, v)
