"""FastNerf's occupancy network on the tensor cores (sg_nerf_density through
sailor_gb300.nerf.infer_density) against three CPU evaluations of the same
float16 network (oracle/fastnerf.py):

* the reference's arithmetic (float16 __hfma chains, infer_mlp.cu:80-240);
* float32 layer sums with float16 layer outputs -- the kernel's own
  arithmetic up to the order of the tensor cores' float32 additions: most
  densities are bit-equal, the rest within a float16 rounding carried
  through the layers;
* the float64 network: the kernel is at least as close to it as the
  reference (max and mean error), both in densities and geometry features.

Shapes: one, three and five views (tiles of floor(128 / V) points), two
frames, point counts that do not fill the last tile; a 2^18-point case;
argument errors raised on the host.
"""
import numpy as np
import pytest
import torch

from oracle import fastnerf as fn

pytestmark = pytest.mark.gpu


def _inputs(seed, B, V, N, scale):
    rng = np.random.default_rng(seed)
    params = (rng.normal(0, 1, fn.PARAM_COUNT) * scale).astype(np.float16)
    z = rng.uniform(0.5, 3.0, (B, V, N, 1)).astype(np.float32)
    tp = rng.uniform(-1.0, 1.0, (B, V, N, 1)).astype(np.float32)
    g = rng.normal(0, 0.5, (B, V, N, 16)).astype(np.float32)
    return params, z, tp, g


def _gpu(params, z, tp, g, B, N, V):
    from sailor_gb300.nerf import infer_density
    c = lambda a, dt=torch.float32: torch.as_tensor(a, dtype=dt, device="cuda")  # noqa: E731
    d, geo = infer_density(c(z), c(tp), c(g), c(params, torch.float16), B, N, V, 0, return_geo=True)
    torch.cuda.synchronize()
    return d.cpu().numpy().astype(np.float64), geo.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("V,scale", [(1, 0.15), (3, 0.15), (3, 0.3), (5, 0.3)])
def test_density_matches_cpu_evaluations(V, scale):
    B, N = 2, 1000
    params, z, tp, g = _inputs(23 + V, B, V, N, scale)
    d, geo = _gpu(params, z, tp, g, B, N, V)
    do, go = fn.infer_density(z, tp, g, params, B, N, V)
    d32, g32 = fn.infer_density_acc(z, tp, g, params, B, N, V, np.float32)
    d64, g64 = fn.infer_density_acc(z, tp, g, params, B, N, V, np.float64)
    assert d.shape == (B, 1, N) and geo.shape == (B, V, N, 8)
    # the kernel's own arithmetic
    assert (d == d32).mean() > 0.9 and (geo == g32).mean() > 0.9
    assert np.abs(d - d32).max() <= (2e-3 if scale < 0.2 else 1e-2)
    assert np.abs(geo - g32).max() <= 2.0 ** -8 * max(1.0, np.abs(g32).max())
    # at least as close to the float64 network as the reference's float16 chains
    for mine, ref, exact in ((d, do, d64), (geo, go, g64)):
        e_mine, e_ref = np.abs(mine - exact), np.abs(ref.astype(np.float64) - exact)
        assert e_mine.max() <= e_ref.max() and e_mine.mean() <= e_ref.mean()


def test_density_large():
    B, V, N = 1, 3, 1 << 18
    params, z, tp, g = _inputs(5, B, V, N, 0.3)
    d, geo = _gpu(params, z, tp, g, B, N, V)
    pick = np.random.default_rng(1).choice(N, 4096, replace=False)
    sub = lambda a: np.ascontiguousarray(a[:, :, pick])  # noqa: E731
    d32, _ = fn.infer_density_acc(sub(z), sub(tp), sub(g), params, B, 4096, V, np.float32)
    d64, _ = fn.infer_density_acc(sub(z), sub(tp), sub(g), params, B, 4096, V, np.float64)
    do, _ = fn.infer_density(sub(z), sub(tp), sub(g), params, B, 4096, V)
    mine = d[:, :, pick]
    assert (mine == d32).mean() > 0.9
    assert np.abs(mine - d64).mean() <= np.abs(do - d64).mean()
    assert np.isfinite(d).all() and (d >= 0).all() and (d <= 1).all()


def test_argument_errors():
    from sailor_gb300.nerf import infer_density
    params, z, tp, g = _inputs(1, 1, 2, 64, 0.1)
    c = lambda a, dt=torch.float32: torch.as_tensor(a, dtype=dt, device="cuda")  # noqa: E731
    with pytest.raises(RuntimeError, match="net_params_density"):
        infer_density(c(z), c(tp), c(g), c(params[:-1], torch.float16), 1, 64, 2, 0)
    with pytest.raises(RuntimeError, match="points"):
        infer_density(c(z), c(tp), c(g), c(params, torch.float16), 1, 65, 2, 0)
    z2 = np.zeros((1, 129, 1, 1), np.float32)
    g2 = np.zeros((1, 129, 1, 16), np.float32)
    with pytest.raises(RuntimeError, match="invalid"):
        infer_density(c(z2), c(z2), c(g2), c(params, torch.float16), 1, 1, 129, 0)


def test_occupancy_compositing_30_channels():
    """FastNerf's compositing of 30-channel features by occupancies, against
    the float64 oracle (<= 1e-5; rays within 1e-4 of the termination
    threshold are flagged by the oracle and left out)."""
    from oracle import oracle as orc
    from sailor_gb300.nerf import occupancy_compositing
    rng = np.random.default_rng(9)
    B, R, S, C = 2, 700, 96, 30
    z = np.sort(rng.uniform(1.0, 3.0, (B, R, S)), -1).astype(np.float32)
    z[:, :40, :10] = -1.0          # padding first, as sorted rows hold it
    z[:, 40:50, :] = -1.0          # rays without samples
    occ = rng.uniform(0.0, 0.2, (B, R, S)).astype(np.float32)
    feats = rng.random((B, R, S, C), dtype=np.float32)
    c = lambda a: torch.as_tensor(a, device="cuda")  # noqa: E731
    f, d = occupancy_compositing(c(z), c(occ), c(feats), 1e-4, 0)
    torch.cuda.synchronize()
    of, od, _, _, fl = orc.composite_fwd(z, None, occ[..., None], feats, 1e-4, True)
    ok = fl == 0
    assert ok.mean() > 0.95
    assert np.abs(f.cpu().numpy() - of)[ok].max() <= 1e-5
    assert np.abs(d.cpu().numpy() - od)[ok].max() <= 1e-5 * 3.0
    assert (f.cpu().numpy()[:, 40:50] == 0).all() and (d.cpu().numpy()[:, 40:50] == 0).all()
