"""Host check of the exact-rounding shortcuts the fusion kernel uses
(sailor_gb300/csrc/fusion.cu: round_div, div_weight).

round_div decides roundf(a / b) from q = a * r, where r is the hardware's
approximate reciprocal of b (at most 1 ulp off), and falls back to the IEEE
quotient only near a rounding tie.  Here r is taken 1 ulp below, at, and 1
ulp above the correctly rounded 1/b (the worst cases of the documented
bound), q is the correctly rounded float32 product, and the fast-path result
must equal roundf of the correctly rounded quotient for every input that does
not fall back -- on random quotients and on quotients within a few ulps of
half-integers.  div_weight's power-of-two product must equal the quotient.
"""
import numpy as np

f32 = np.float32


def roundf(x):
    """C roundf (half away from zero) on float32 values, computed exactly."""
    x = np.asarray(x, np.float64)
    return np.copysign(np.floor(np.abs(x) + 0.5), x).astype(np.float32)


def round_div_fast(a, b, r):
    """The kernel's fast path: (value, taken) per element."""
    q = (a * r).astype(f32)
    aq, ab = np.abs(q), np.abs(b)
    fl = np.floor(q).astype(f32)
    d = (q - fl).astype(f32)
    margin = (aq.astype(np.float64) * f32(4.8e-7) + f32(6.0e-8)).astype(f32)
    taken = (aq < 1048576.0) & (ab >= f32(1e-30)) & (ab <= f32(1e30)) & (np.abs(d - f32(0.5)) > margin)
    val = np.where(d > 0.5, fl + f32(1.0), fl).astype(f32)
    val = np.copysign(val, q).astype(f32)
    return val, taken


def _check(a, b):
    a, b = a.astype(f32), b.astype(f32)
    exact = roundf((a / b).astype(f32))
    r0 = (f32(1.0) / b).astype(f32)
    n_fast = 0
    for r in (np.nextafter(r0, f32(-np.inf)), r0, np.nextafter(r0, f32(np.inf))):
        val, taken = round_div_fast(a, b, r.astype(f32))
        bad = taken & (val.view(np.uint32) != exact.view(np.uint32))
        assert not bad.any(), (a[bad][:5], b[bad][:5], val[bad][:5], exact[bad][:5])
        n_fast += int(taken.sum())
    return n_fast


def test_round_div_random_quotients():
    rng = np.random.default_rng(0)
    n = 400_000
    b = (rng.uniform(0.5, 4.0, n) * 10.0 ** rng.integers(-3, 4, n)).astype(f32)
    b *= np.where(rng.random(n) < 0.2, -1, 1).astype(f32)
    q = rng.uniform(-2000, 2000, n)
    a = (q * b).astype(f32)
    assert _check(a, b) > 0.99 * 3 * n


def test_round_div_near_ties():
    rng = np.random.default_rng(1)
    n = 400_000
    b = (rng.uniform(0.5, 4.0, n) * 10.0 ** rng.integers(-2, 3, n)).astype(f32)
    k = rng.integers(-1500, 1500, n).astype(np.float64)
    a = ((k + 0.5) * b.astype(np.float64)).astype(f32)
    steps = rng.integers(-12, 13, n)
    for s in range(1, 13):  # nudge a by up to 12 ulps either way
        up, dn = steps >= s, steps <= -s
        a = np.where(up, np.nextafter(a, f32(np.inf)), a)
        a = np.where(dn, np.nextafter(a, f32(-np.inf)), a).astype(f32)
    _check(a, b)


def test_round_div_small_and_signed_zero():
    b = np.array([3.0, -3.0, 7.0, 1.0, 2.0, 1e-3], f32)
    a = np.array([-0.0, 0.0, -1e-7, -1.0, 1.0, -1.5e-3], f32)
    _check(a, b)
    val, taken = round_div_fast(np.array([-0.3], f32), np.array([1.0], f32), np.array([1.0], f32))
    assert taken[0] and val[0] == 0 and np.signbit(val[0])  # roundf(-0.3) == -0.0


def test_div_weight_power_of_two():
    rng = np.random.default_rng(2)
    x = rng.normal(0, 100, 100_000).astype(f32)
    for e in (-20, -3, 0, 1, 2, 5, 40):
        w = f32(2.0 ** e)
        wb = np.array([w], f32).view(np.uint32)[0]
        rw = np.array([0x7F000000 - int(wb)], np.uint32).view(f32)[0]
        assert rw == f32(2.0 ** -e)
        assert np.array_equal((x * rw).astype(f32).view(np.uint32), (x / w).astype(f32).view(np.uint32))
