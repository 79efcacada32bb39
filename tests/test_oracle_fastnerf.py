"""CPU checks of the float16 restatement of FastNerf's occupancy MLP
(oracle/fastnerf.py): __hfma's single rounding against exact rational
arithmetic, the parameter layout, and the network against a float64
evaluation of the same weights."""
import os
from fractions import Fraction

import numpy as np
import pytest

from oracle import fastnerf as fn

F16 = np.float16


def _round_half_exact(q):
    """The float16 nearest to the rational q (ties to even), by search;
    magnitudes from 65520 (the largest float16 plus half its ulp) round to
    infinity."""
    if abs(q) >= 65520:
        return F16(np.inf) if q > 0 else F16(-np.inf)
    x = F16(float(q))
    best = None
    for cand in (np.nextafter(np.nextafter(x, F16(-np.inf)), F16(-np.inf)), np.nextafter(x, F16(-np.inf)), x,
                 np.nextafter(x, F16(np.inf)), np.nextafter(np.nextafter(x, F16(np.inf)), F16(np.inf))):
        if not np.isfinite(cand):
            continue
        d = abs(Fraction(float(cand)) - q)
        even = (int(cand.view(np.uint16)) & 1) == 0
        key = (d, not even)
        if best is None or key < best[0]:
            best = (key, cand)
    return best[1]


def test_hfma_single_rounding():
    rng = np.random.default_rng(0)
    n = 4000
    a = rng.normal(0, 1, n).astype(F16)
    b = rng.normal(0, 1, n).astype(F16)
    c = rng.normal(0, 1, n).astype(F16)
    # half-way cases: c chosen so that a*b + c sits on a float16 midpoint
    # before a tiny extra term, and tiny or huge magnitude differences
    c[:500] = (-(a[:500].astype(np.float64) * b[:500])).astype(F16)
    a[500:1000] = F16(1.0) + F16(2.0 ** -10)
    b[500:1000] = F16(1.0) + F16(2.0 ** -10)
    c[1000:1200] = F16(2.0 ** -24)  # the smallest subnormal
    a[1200:1400] *= F16(200.0)
    b[1200:1400] *= F16(200.0)
    got = fn.hfma(a, b, c)
    for i in range(n):
        q = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        want = _round_half_exact(q)
        assert got[i] == want or (got[i] == 0 and want == 0), (i, a[i], b[i], c[i], got[i], want)


def test_hfma_subnormal_operands():
    """Products of float16 subnormals reach 2^-48, so the float64 sum with a
    large addend is inexact; the float16 result must still equal the single
    rounding of the exact rational value."""
    rng = np.random.default_rng(1)
    n = 3000
    sub = lambda k: (rng.integers(1, 1024, k) * 2.0 ** -24 * rng.choice([-1.0, 1.0], k)).astype(F16)  # noqa: E731
    a, b = sub(n), rng.normal(0, 1, n).astype(F16)
    b[:1000] = sub(1000)                                        # subnormal x subnormal
    c = (rng.uniform(64.0, 60000.0, n) * rng.choice([-1.0, 1.0], n)).astype(F16)
    c[1000:1500] = (F16(1.0) + F16(2.0 ** -10)) * F16(2.0 ** 10)  # c on a float16 value next to a midpoint
    c[1500:2000] = sub(500)                                     # small addends, exact sums
    c[2000:2500] = F16(65504.0)                                 # the largest finite value
    got = fn.hfma(a, b, c)
    for i in range(n):
        q = Fraction(float(a[i])) * Fraction(float(b[i])) + Fraction(float(c[i]))
        want = _round_half_exact(q)
        assert got[i] == want or (got[i] == 0 and want == 0), (i, a[i], b[i], c[i], got[i], want)
    assert np.any(np.abs(a.astype(np.float64) * b) < 2.0 ** -40)  # inexact float64 sums occur


def test_hfma_rounds_once():
    # (1 + 2^-10)^2 = 1 + 2^-9 + 2^-20; with c = -2^-9 the exact 1 + 2^-20
    # lies below the midpoint 1 + 2^-11 (rounds to 1), with
    # c = -2^-9 + 2^-11 it lies just above it (rounds to 1 + 2^-10); with
    # the product rounded first (to 1 + 2^-9) both would give 1
    a = np.array([1.0 + 2.0 ** -10], F16)
    assert fn.hfma(a, a, np.array([-2.0 ** -9], F16))[0] == F16(1.0)
    assert fn.hfma(a, a, np.array([-2.0 ** -9 + 2.0 ** -11], F16))[0] == F16(1.0 + 2.0 ** -10)


def test_parameter_layout_and_relu():
    assert fn.layer_sizes(fn.FEAT_LAYERS) == fn.SIGMA_OFFSET
    assert fn.SIGMA_OFFSET + fn.layer_sizes(fn.SIGMA_LAYERS) == fn.GEO_OFFSET
    assert fn.layer_sizes(fn.GEO_LAYERS) == fn.PARAM_COUNT - fn.GEO_OFFSET == 440
    # one layer with W = [I | 0] and bias b: out = relu(x[:n_out] + b)
    n_in, n_out = 18, 16
    params = np.zeros(n_in * n_out + n_out, F16)
    W = params[:n_in * n_out].reshape(n_out, n_in)
    W[np.arange(n_out), np.arange(n_out)] = 1.0
    params[n_in * n_out:] = np.arange(n_out, dtype=F16) * F16(0.25) - F16(1.0)
    x = np.random.default_rng(1).normal(0, 1, (7, n_in)).astype(F16)
    out = fn.relu16(fn.fc16(x, params, 0, n_in, n_out))
    want = fn.relu16(fn.hfma(F16(1.0), x[:, :n_out], params[n_in * n_out:]))
    assert np.array_equal(out, want) and (out >= 0).all()
    assert fn.relu16(np.array([np.nan, -3.0, 2.5], F16)).tolist() == [0.0, 0.0, 2.5]


def test_density_network_against_float64():
    rng = np.random.default_rng(2)
    params = (rng.normal(0, 1, fn.PARAM_COUNT) * 0.15).astype(F16)
    B, V, N = 1, 3, 64
    z = rng.uniform(0.5, 3.0, (B, V, N, 1)).astype(np.float32)
    tp = rng.uniform(-1, 1, (B, V, N, 1)).astype(np.float32)
    g = rng.normal(0, 0.5, (B, V, N, 16)).astype(np.float32)
    dens, geo = fn.infer_density(z, tp, g, params, B, N, V)
    assert dens.shape == (B, 1, N) and geo.shape == (B, V, N, 8)
    # float64 evaluation of the same (float16) weights and inputs
    P = params.astype(np.float64)

    def mlp64(x, off, layers, last_relu=True):
        for k, (i, o) in enumerate(layers):
            W = P[off:off + i * o].reshape(o, i)
            x = x @ W.T + P[off + i * o:off + i * o + o]
            off += i * o + o
            if last_relu or k + 1 < len(layers):
                x = np.maximum(x, 0)
        return x
    x = np.concatenate([z, tp, g], axis=-1).reshape(-1, 18).astype(F16).astype(np.float64)
    d64 = mlp64(x, 0, fn.FEAT_LAYERS).reshape(B, V, N, 64).mean(axis=1).reshape(-1, 64)
    s64 = 1.0 / (1.0 + np.exp(-mlp64(d64.astype(F16).astype(np.float64), fn.SIGMA_OFFSET, fn.SIGMA_LAYERS,
                                     last_relu=False)[:, 0]))
    g64 = mlp64(x, fn.GEO_OFFSET, fn.GEO_LAYERS).reshape(B, V, N, 8)
    # float16 accumulation over up to 64 terms per layer: a few float16 ulps
    assert np.abs(dens.reshape(-1) - s64).max() < 2e-2
    assert np.abs(geo - g64).max() < 5e-2 * max(1.0, np.abs(g64).max())
    assert dens.std() > 1e-3  # the densities are not constant


def test_occupancy_compositing_against_loop():
    """The compositing restatement against a direct loop of the kernel's
    steps, 30 channels, with padded, invalid and early-terminating rays."""
    rng = np.random.default_rng(3)
    R, S, C = 64, 24, 30
    z = np.sort(rng.uniform(0.5, 3.0, (R, S)), axis=1).astype(np.float32)
    z[:8, :5] = -1.0  # leading padding
    z[8:12, -1] = -1.0  # last raw depth negative: an invalid ray
    occ = rng.uniform(0.0, 0.6, (R, S)).astype(np.float32)
    occ[12:16] = 0.999  # transmittance falls under the threshold early
    feats = rng.normal(0, 1, (R, S, C)).astype(np.float32)
    of, od = fn.composite_occ(z, occ, feats)
    for r in range(R):
        f = np.zeros(C)
        d = 0.0
        if z[r, -1] >= 0:
            T = 1.0
            for i in range(S):
                if z[r, i] < 0:
                    continue
                w = float(occ[r, i]) * T
                f += w * feats[r, i].astype(np.float64)
                d += w * float(z[r, i])
                T *= 1.0 - float(occ[r, i])
                if T < 1e-4:
                    break
        assert np.abs(of[r] - f).max() <= 1e-5 and abs(od[r, 0] - d) <= 1e-5, r


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_density_mlp.npz")


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="no golden vectors of the reference MLP yet")
def test_density_mlp_against_reference_golden():
    """Pin: the restatement against the reference kernels' outputs
    (tests/golden/ref_density_mlp.npz, made by make_golden.py --only
    density_mlp on a GPU from the reference's own infer_mlp.cu): the
    geometry features and the densities bit for bit (the float32 view mean
    in view order times 1/V equals torch's mean here)."""
    g = np.load(GOLDEN)
    B, V, N = (int(x) for x in g["shape"])
    dens, geo = fn.infer_density(g["points_z"], g["points_tpsdf"], g["feats_geo"], g["params"], B, N, V)
    assert np.array_equal(geo, g["geo_feats"])
    assert np.array_equal(dens, g["density"])
