"""The device square root of the strain magnitudes (chl_sqrt: two Newton
steps from the GPU's approximate reciprocal square root) against correctly
rounded roots (numpy's sqrt, which is IEEE's, as CUDA's sqrt() is).

Tolerance: within 1 ulp on every positive normal argument; bit for bit
IEEE on zero, subnormal, negative, infinite and NaN arguments."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    return np.abs(a.view(np.int64) - b.view(np.int64))


def test_newton_root_is_within_one_ulp():
    from channel_rl_gb300.host import sqrt_selftest
    rng = np.random.default_rng(5)
    fin = np.finfo(np.float64)
    wide = np.ldexp(rng.uniform(1.0, 2.0, 1 << 20), rng.integers(-1022, 1024, 1 << 20))
    strain_like = rng.lognormal(0.0, 6.0, 1 << 20)          # the magnitudes a step sees
    q = rng.integers(1, 1 << 26, 1 << 16).astype(np.float64)
    edges = np.array([fin.tiny, np.nextafter(fin.tiny, 1.0), fin.max, np.nextafter(fin.max, 0.0),
                      1.0, 2.0, 4.0, 0.5, 0.25, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])
    a = np.concatenate([wide, strain_like, q * q, edges])
    assert np.all(np.isfinite(a) & (a >= fin.tiny))
    y = sqrt_selftest(a)
    u = _ulps(y, np.sqrt(a))
    assert u.max() <= 1, (a[u.argmax()], y[u.argmax()], np.sqrt(a[u.argmax()]))
    assert np.mean(u == 0) > 0.99


def test_special_arguments_are_ieee():
    from channel_rl_gb300.host import sqrt_selftest
    fin = np.finfo(np.float64)
    a = np.array([0.0, -0.0, 5e-324, fin.tiny / 2, np.nextafter(fin.tiny, 0.0), -1.0, -fin.tiny, -5e-324,
                  np.inf, -np.inf, np.nan, -1e300])
    with np.errstate(invalid="ignore"):
        want = np.sqrt(a)
    y = sqrt_selftest(a)
    same = (y.view(np.int64) == want.view(np.int64)) | (np.isnan(y) & np.isnan(want))
    assert same.all(), list(zip(a[~same], y[~same], want[~same]))
    assert np.array_equal(sqrt_selftest(np.zeros(0)), np.zeros(0))
