"""CPU checks of the oracle's float64 render of sorted samples
(oracle.composite_sorted_fp64, oracle.render_fp64): pinned to the
reference's compositing kernel through the golden vectors, and to the C
oracle's compositing and trilinear gather."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _sorted_golden():
    c = np.load(os.path.join(GOLDEN, "ref_composite.npz"))
    idx = c["sort_idx"][0].astype(np.int64)
    z = np.take_along_axis(c["z"][0], idx, 1)
    sig = np.take_along_axis(c["sigma"][0, ..., 0], idx, 1)
    feats = np.take_along_axis(c["feats"][0], idx[..., None], 1)
    return c, z, sig, feats


def test_composite_sorted_fp64_vs_reference_kernel():
    """The reference's compositing kernel's outputs (float32, golden) within
    1e-5 of the float64 restatement on the same sorted samples, and the C
    oracle's double-accumulated compositing within 1e-12."""
    c, z, sig, feats = _sorted_golden()
    assert np.array_equal(z, c["sorted_z"][0])
    rgb, d, ws, a, flags = orc.composite_sorted_fp64(z, sig.astype(np.float64), feats.astype(np.float64), 1e-4)
    ok = flags == 0
    assert ok.mean() > 0.99
    assert np.abs(rgb - c["den_fwd_feat"][0])[ok].max() <= 1e-5
    assert np.abs(d - c["den_fwd_depth"][0, :, 0])[ok].max() <= 1e-5
    assert np.abs(ws - c["den_fwd_ws"][0, :, 0])[ok].max() <= 1e-5
    assert np.abs(a - c["den_fwd_alpha"][0, :, 0])[ok].max() <= 1e-5
    of, od, ow, oa, fl = orc.composite_fwd(z[None], None, sig[None, ..., None], feats[None], 1e-4, False)
    assert np.array_equal(fl[0] != 0, flags != 0)
    for got, ref in ((rgb, of[0]), (d, od[0, :, 0]), (ws, ow[0, :, 0]), (a, oa[0, :, 0])):
        assert np.abs(got - ref).max() <= 1e-12


def test_render_fp64_matches_parts():
    """render_fp64 = the C oracle's trilinear gathers (TSDF and features at
    the float32 sample points) -> density, head -> float64 compositing."""
    rng = np.random.default_rng(3)
    B, D, C, R, S = 2, 12, 16, 64, 24
    tsdf = rng.uniform(-1, 1, (B, D, D, D)).astype(np.float32)
    feat = rng.normal(0, 0.1, (B, D, D, D, C)).astype(np.float32)
    head = rng.normal(0, 0.5, (3, C)).astype(np.float32)
    bmin = np.full((B, 3), -1.0, np.float32)
    vs = np.full(B, 2.0 / (D - 1), np.float32)
    ori = np.tile(np.array([[-1.6, 0.05, 0.1]], np.float32), (R, 1)) + rng.normal(0, 0.01, (R, 3)).astype(np.float32)
    dirs = rng.normal(0, 0.05, (R, 3)).astype(np.float32) + np.array([1.0, 0, 0], np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    z = np.sort(rng.uniform(0.7, 2.5, (R, S)), 1).astype(np.float32)
    z[:, :5] = -1.0  # padding first, as sorted rows hold it
    z[:4] = -1.0     # rays without samples
    batch = rng.integers(0, B, R).astype(np.int32)
    out = orc.render_fp64(ori, dirs, z, tsdf, bmin, vs, 0.03, 0.01, feat, head, 1e-4, batch=batch)
    pts = orc.sample_points(ori, dirs, z).reshape(-1, 3)
    bt = np.repeat(batch, S)
    t = orc.grid_gather(pts, tsdf[..., None], bmin, vs, batch=bt)[:, 0].reshape(R, S)
    sig = np.where(z >= 0, 1.0 / (1.0 + np.exp(t * 3.0)) / 0.01, 0.0)
    rgb = np.where((z >= 0)[..., None], (orc.grid_gather(pts, feat, bmin, vs, batch=bt) @ head.T.astype(
        np.float64)).reshape(R, S, 3), 0.0)
    assert np.abs(out["sigma"] - sig).max() <= 1e-9 * sig.max()
    assert np.abs(out["rgb_s"] - rgb).max() <= 1e-12
    ref = orc.composite_sorted_fp64(z, sig, rgb, 1e-4)
    assert np.abs(out["rgb"] - ref[0]).max() <= 1e-9
    assert (out["rgb"][:4] == 0).all() and (out["ws"][:4] == 0).all()
    assert out["ws"][4:].max() > 0.1
    # the float32 points are the kernels' fma(dir, z, ori)
    p = pts.reshape(R, S, 3)[7, 9]
    want = (dirs[7].astype(np.float64) * np.float64(z[7, 9]) + ori[7]).astype(np.float32)
    assert np.array_equal(p, want)


@pytest.mark.parametrize("t_thres", [1e-4, 0.0])
def test_composite_sorted_fp64_early_stop(t_thres):
    """The sample that takes T below t_thres is composited, the ones after it
    are not; t_thres = 0 composites every sample."""
    z = np.array([[-1.0, 0.5, 0.6, 0.7, 0.8]], np.float32)
    sig = np.array([[0.0, 50.0, 200.0, 1.0, 1.0]])
    rgb = np.ones((1, 5, 3))
    out = orc.composite_sorted_fp64(z, sig, rgb, t_thres)
    a1 = 1 - np.exp(-50.0 * np.float64(np.float32(0.6) - np.float32(0.5)))
    a2 = 1 - np.exp(-200.0 * np.float64(np.float32(0.7) - np.float32(0.6)))
    ws = a1 + (1 - a1) * a2
    if t_thres > 0:
        assert abs(out[2][0] - ws) <= 1e-15
    else:
        assert out[2][0] > ws
