"""GPU checks of the dense-grid gathers and their adjoint (sg_grid_scatter)
through the autograd Functions of sailor_gb300.fields.

References: the oracle's float64 scatter, float64 autograd of a plain
PyTorch trilinear interpolation (and of a plain PyTorch compositing for the
whole chain), and float64 central finite differences (h = 1e-4) for the
nonlinear density gather.  Tolerances are stated per check, relative to the
largest reference magnitude.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _rays(rng, B, R, S, pad=0.2):
    """Rays from a 1.6 m sphere through the [-1, 1]^3 box; sorted depths with
    some -1 (invalid) samples at random positions."""
    c = rng.normal(size=(B, R, 3))
    ori = 1.6 * c / np.linalg.norm(c, axis=-1, keepdims=True)
    tgt = rng.uniform(-0.8, 0.8, (B, R, 3))
    d = tgt - ori
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    z = np.sort(rng.uniform(0.3, 2.9, (B, R, S)), -1)
    z[rng.random((B, R, S)) < pad] = -1.0
    return ori.astype(np.float32), d.astype(np.float32), z.astype(np.float32)


def _torch_trilinear(grid, ori, dirs, z, bmin, vs):
    """float64 trilinear gather with the kernel's conventions: voxel (x, y, z)
    at bmin + (x, y, z) * vs, corners outside the grid contribute 0, samples
    with z < 0 give 0.  grid [B, D, D, D, C]; returns [B, N, S, C]."""
    B, D, C = grid.shape[0], grid.shape[1], grid.shape[-1]
    pts = ori[:, :, None, :] + z[..., None] * dirs[:, :, None, :]
    u = (pts - bmin[:, None, None, :]) / vs[:, None, None, None]
    i0 = torch.floor(u)
    f = u - i0
    i0 = i0.long()
    bidx = torch.arange(B)[:, None, None].expand(z.shape)
    out = torch.zeros(z.shape + (C,), dtype=grid.dtype)
    for cr in range(8):
        d = ((cr >> 2) & 1, (cr >> 1) & 1, cr & 1)
        idx = [i0[..., a] + d[a] for a in range(3)]
        inside = (idx[0] >= 0) & (idx[0] < D) & (idx[1] >= 0) & (idx[1] < D) & (idx[2] >= 0) & (idx[2] < D)
        w = torch.ones_like(z)
        for a in range(3):
            w = w * (f[..., a] if d[a] else 1 - f[..., a])
        g = grid[bidx, idx[0].clamp(0, D - 1), idx[1].clamp(0, D - 1), idx[2].clamp(0, D - 1)]
        out = out + (w * inside)[..., None] * g
    return torch.where((z >= 0)[..., None], out, torch.zeros_like(out))


def _setup(rng, B, D, C, R, S):
    ori, dirs, z = _rays(rng, B, R, S)
    bbox = np.tile(np.array([[-1.0, 1.0]] * 3, np.float32), (B, 1, 1))
    vs = np.full((B,), 2.0 / (D - 1), np.float32)
    grid = rng.normal(0, 0.1, (B, D, D, D, C)).astype(np.float32)
    return ori, dirs, z, bbox, vs, grid


def _cuda(a):
    return torch.as_tensor(a, device="cuda").contiguous()


def _f64(a, grad=False):
    return torch.tensor(np.asarray(a, np.float64), requires_grad=grad)


@pytest.mark.parametrize("C", [1, 3, 16])
def test_grid_gather_and_adjoint_vs_torch_fp64(C):
    from sailor_gb300.fields import grid_gather
    rng = np.random.default_rng(10 + C)
    B, D, R, S = 2, 32, 384, 64
    ori, dirs, z, bbox, vs, grid = _setup(rng, B, D, C, R, S)
    gout = rng.normal(size=(B, R, S, C)).astype(np.float32)
    gg = _cuda(grid).requires_grad_(True)
    out = grid_gather(gg, _cuda(ori), _cuda(dirs), _cuda(z), _cuda(bbox), _cuda(vs))
    out.backward(_cuda(gout))
    gt = _f64(grid, True)
    ref = _torch_trilinear(gt, _f64(ori), _f64(dirs), _f64(z), _f64(bbox[:, :, 0]), _f64(vs))
    (ref * _f64(gout)).sum().backward()
    # forward within 1e-5 of float64; adjoint within 1e-5 of the largest gradient
    assert np.abs(out.detach().cpu().numpy() - ref.detach().numpy()).max() <= 1e-5
    rg = gt.grad.numpy()
    assert np.abs(gg.grad.cpu().numpy() - rg).max() <= 1e-5 * max(1.0, np.abs(rg).max())
    assert np.abs(rg).max() > 0.5  # the check is not vacuous


def test_grid_scatter_vs_oracle():
    """sg_grid_scatter against the oracle's sequential float64 scatter at
    the same float32 sample points."""
    from sailor_gb300 import _native as N
    rng = np.random.default_rng(3)
    B, D, C, R, S = 2, 24, 4, 256, 48
    ori, dirs, z, bbox, vs, grid = _setup(rng, B, D, C, R, S)
    gout = rng.normal(size=(B, R, S, C)).astype(np.float32)
    ggrid = torch.zeros((B, D, D, D, C), dtype=torch.float32, device="cuda")
    t = [_cuda(a) for a in (ori, dirs, z, gout, bbox, vs)]
    N.check(N.lib.sg_grid_scatter(N.ptr(t[0]), N.ptr(t[1]), N.ptr(t[2]), B, R, S, N.ptr(t[3]), None, D, C,
                                  N.ptr(t[4]), N.ptr(t[5]), 0, 1.0, 1.0, N.ptr(ggrid), N.stream()), "scatter")
    # sample points exactly as the kernel forms them: fma(dir, z, ori) in float32
    pts = (dirs[:, :, None, :].astype(np.float64) * z[..., None] + ori[:, :, None, :]).astype(np.float32)
    valid = (z >= 0).reshape(-1)
    batch = np.repeat(np.arange(B, dtype=np.int32), R * S)[valid]
    ref = orc.grid_scatter(pts.reshape(-1, 3)[valid], gout.reshape(-1, C)[valid], B, D,
                           bbox[:, :, 0], vs, batch=batch)
    ref = ref.reshape(B, D, D, D, C)
    got = ggrid.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def _density_f64(tsdf, ori, dirs, z, bbox, vs, scale, s):
    t = _torch_trilinear(tsdf[..., None], ori, dirs, z, bbox[:, :, 0], vs)[..., 0]
    sig = torch.sigmoid(-t * scale / s) / s
    return torch.where(z >= 0, sig, torch.zeros_like(sig))


def test_tsdf_density_adjoint_vs_autograd_and_fd():
    from sailor_gb300.fields import tsdf_density
    rng = np.random.default_rng(5)
    B, D, R, S = 1, 32, 512, 64
    scale, s = 0.02, 0.005
    ori, dirs, z, bbox, vs, _ = _setup(rng, B, D, 1, R, S)
    tsdf = rng.uniform(-1.0, 1.0, (B, D, D, D)).astype(np.float32)
    gout = rng.normal(size=(B, R, S)).astype(np.float32)
    tg = _cuda(tsdf).requires_grad_(True)
    sig = tsdf_density(tg, _cuda(ori), _cuda(dirs), _cuda(z), _cuda(bbox), _cuda(vs), scale, s)
    sig.backward(_cuda(gout))
    got = tg.grad.cpu().numpy()
    tt = _f64(tsdf, True)
    args = (_f64(ori), _f64(dirs), _f64(z), _f64(bbox), _f64(vs), scale, s)
    ref = _density_f64(tt, *args)
    assert np.abs(sig.detach().cpu().numpy() - ref.detach().numpy()).max() <= 1e-5 * max(1.0, float(ref.detach().max()))
    (ref * _f64(gout)).sum().backward()
    rg = tt.grad.numpy()
    assert np.abs(got - rg).max() <= 1e-5 * np.abs(rg).max()
    # float64 central differences on the 16 voxels with the largest gradients
    h = 1e-4
    flat = np.argsort(-np.abs(rg).reshape(-1))[:16]
    with torch.no_grad():
        for k in flat:
            idx = np.unravel_index(k, rg.shape)
            tp, tm = tt.detach().clone(), tt.detach().clone()
            tp[idx] += h
            tm[idx] -= h
            fd = ((_density_f64(tp, *args) - _density_f64(tm, *args)) * _f64(gout)).sum().item() / (2 * h)
            assert abs(got[idx] - fd) <= 1e-4 * np.abs(rg).max()


def test_render_chain_grid_gradients_vs_torch_fp64():
    """Compositing (exact adjoint) of sigma = tsdf_density(tsdf grid) and
    rgb = grid_gather(colour grid): gradients of both grids against float64
    autograd of the same chain in plain PyTorch (t_thres = 0, so no early
    termination; all samples valid)."""
    from sailor_gb300.fields import grid_gather, tsdf_density
    from sailor_gb300.voxel_encoding_helper import volume_render_exact
    from test_gpu_parity import _torch_composite
    rng = np.random.default_rng(9)
    B, D, R, S = 1, 32, 256, 32
    scale, s = 0.02, 0.005
    ori, dirs, z, bbox, vs, col = _setup(rng, B, D, 3, R, S)
    z = np.sort(rng.uniform(0.3, 2.9, (B, R, S)), -1).astype(np.float32)
    tsdf = rng.uniform(-1.0, 1.0, (B, D, D, D)).astype(np.float32)
    grads = [rng.normal(size=sh).astype(np.float32) for sh in ((B, R, 3), (B, R, 1), (B, R, 1), (B, R, 1))]
    idx = np.tile(np.arange(S, dtype=np.int32), (B, R, 1))
    tg, cg = _cuda(tsdf).requires_grad_(True), _cuda(col).requires_grad_(True)
    rays = [_cuda(a) for a in (ori, dirs, z, bbox, vs)]
    sigma = tsdf_density(tg, *rays, scale, s)
    rgb = grid_gather(cg, *rays)
    outs = volume_render_exact(rays[2], _cuda(idx), sigma[..., None], rgb, 0.0, False)
    sum((o * _cuda(g)).sum() for o, g in zip(outs, grads)).backward()
    tt, ct = _f64(tsdf, True), _f64(col, True)
    args = (_f64(ori), _f64(dirs), _f64(z), _f64(bbox), _f64(vs))
    sg64 = _density_f64(tt, *args, scale, s)
    rgb64 = _torch_trilinear(ct, args[0], args[1], args[2], args[3][:, :, 0], args[4])
    outs64 = _torch_composite(args[2], torch.tensor(idx, dtype=torch.int64), sg64[..., None], rgb64, False)
    sum((o * _f64(g)).sum() for o, g in zip(outs64, grads)).backward()
    for got, ref in ((tg.grad, tt.grad), (cg.grad, ct.grad)):
        ref = ref.numpy()
        assert np.abs(got.cpu().numpy() - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
