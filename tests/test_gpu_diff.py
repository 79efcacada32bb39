"""The differentiation workload at its stated size: 2^20 seeded random rays
(origins on a 3 m sphere, aimed at uniform points of the 2 m cube) through
the fused 256^3 volume of the plain small scene (8^3 bricks), 96 samples
per ray, a 256^3 x 16 feature grid ~ N(0, 0.1) with a linear colour head,
upstream gradients ~ N(0, 1) on colour, depth and alpha.  One step =
intersection, fused forward, fused exact adjoint (per-sample sigma and colour
gradients, feature- and TSDF-grid gradients).

Bars (bench.parity_diff): fusion bit-exact; on 512 rays with hits,
traversal rows equal the oracle's (unflagged rays), samples equal the
oracle's sampling of those rows bit for bit, forward outputs within 1e-5 of
the float64 oracle render; per-sample sigma gradients within a
relative 1e-4 (of the largest) and colour gradients within 1e-5 of float64
central differences (h = 1e-4) on those rays, and of float64 autograd of a
plain PyTorch compositing on every ray; grid gradients within a relative
1e-4 of float64 central differences over every ray that reaches the entry.
"""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_diff_workload_full_size():
    import bench
    cfg = dict(bench.DIFF)
    d = bench.diff_setup(cfg, torch.device("cuda", 0))
    d["bp"].build()
    bench.diff_step(d)
    torch.cuda.synchronize()
    assert not (d["bp"].status[0].item() & 1)
    par = bench.parity_diff(d, cfg)
    print(par)
    assert par["fusion_bit_exact"]
    tr = par["traversal"]
    assert tr["unflagged_row_mismatches"] == 0 and tr["t_max_abs_err"] <= 1e-5
    assert par["sample_mismatches"] == 0 and par["composite_rays_flagged"] <= 5
    for k, v in par["forward_max_abs_err"].items():
        assert v <= 1e-5, (k, v)
    for name in ("sample_grad_fd", "sample_grad_autograd"):
        r = par[name]
        assert r["sigma_max_abs_err"] <= 1e-4 * max(1.0, r["sigma_max_abs"]), (name, r)
        assert r["rgb_max_abs_err"] <= 1e-5, (name, r)
    assert par["sample_grad_autograd"]["rays"] > 0.99 * (1 << 20)
    for grid, r in par["grid_grad_fd"].items():
        assert r["max_abs_fd"] > 0 and r["max_abs_err"] <= 1e-4 * r["max_abs_fd"], (grid, r)
