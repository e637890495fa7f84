"""Accuracy of the library's own elementary functions (host build) against
float64 numpy, and of its binary16 / bfloat16 storage rounding against IEEE
round-to-nearest-even.  The device build is checked bit for bit against
this host build in the GPU suite."""
import numpy as np
import pytest


def ulp32(x):
    x = np.abs(np.asarray(x, np.float64)).astype(np.float32)
    return (np.nextafter(x, np.float32(np.inf)) - x).astype(np.float64)


@pytest.fixture(scope="module")
def om(oracle_mod):
    return oracle_mod


def test_sin_cos(om):
    x = np.random.default_rng(0).uniform(-300, 300, 200000).astype(np.float32)
    for fn, ref in ((0, np.sin), (1, np.cos)):
        err = np.abs(om.eval_math(fn, x).astype(np.float64) - ref(x.astype(np.float64)))
        assert err.max() < 4e-7, (fn, err.max())


def test_exp(om):
    x = np.random.default_rng(1).uniform(-87, 88, 200000).astype(np.float32)
    y = om.eval_math(2, x).astype(np.float64)
    r = np.exp(x.astype(np.float64))
    assert (np.abs(y - r) / r).max() < 3e-7


def test_log_pow(om):
    rng = np.random.default_rng(2)
    x = np.exp(rng.uniform(-85, 85, 200000)).astype(np.float32)
    y = om.eval_math(3, x).astype(np.float64)
    r = np.log(x.astype(np.float64))
    assert np.abs(y - r).max() < 1e-5 and (np.abs(y - r) / np.maximum(np.abs(r), 1.0)).max() < 3e-7
    a = rng.uniform(1e-4, 3, 100000).astype(np.float32)
    b = rng.uniform(0, 2, 100000).astype(np.float32)
    p = om.eval_math(4, a, b).astype(np.float64)
    pr = np.power(a.astype(np.float64), b.astype(np.float64))
    assert (np.abs(p - pr) / pr).max() < 2e-6
    assert om.eval_math(4, np.float32([0.0]), np.float32([0.66]))[0] == 0.0


def test_atan2(om):
    rng = np.random.default_rng(3)
    y = rng.normal(0, 1, 200000).astype(np.float32)
    x = rng.normal(0, 1, 200000).astype(np.float32)
    a = om.eval_math(5, y, x).astype(np.float64)
    r = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.abs(a - r).max() < 5e-7
    assert om.eval_math(5, np.float32([0.0]), np.float32([0.0]))[0] == 0.0


def test_tanh(om):
    x = np.random.default_rng(4).uniform(-12, 12, 200000).astype(np.float32)
    t = om.eval_math(6, x).astype(np.float64)
    r = np.tanh(x.astype(np.float64))
    assert np.abs(t - r).max() < 3e-7
    small = np.float32([1e-4, 6.5e-4, 1e-2])
    ts = om.eval_math(6, small).astype(np.float64)
    assert (np.abs(ts - np.tanh(small.astype(np.float64))) / small).max() < 1e-6


def test_binary16_rounding_matches_ieee(om):
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.normal(0, s, 50000) for s in (1e-7, 1e-5, 1e-3, 1, 1e3, 6e4)]).astype(np.float32)
    # exact ties between neighbouring binary16 values
    h = rng.integers(0, 0x7BFF, 20000).astype(np.uint16).view(np.float16).astype(np.float64)
    h2 = np.nextafter(h.astype(np.float16), np.float16(np.inf)).astype(np.float64)
    x = np.concatenate([x, ((h + h2) / 2).astype(np.float32), np.float32([65504, 65519.99, 65520, 1e9, 2.9802322e-8])])
    np.testing.assert_array_equal(om.eval_math(7, x), x.astype(np.float16).astype(np.float32))


def test_bfloat16_rounding_matches_ieee(om):
    rng = np.random.default_rng(6)
    x = np.concatenate([rng.normal(0, s, 50000) for s in (1e-30, 1e-3, 1, 1e20)]).astype(np.float32)
    bits = x.view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16) << 16
    ref = rounded.astype(np.uint32).view(np.float32)
    np.testing.assert_array_equal(om.eval_math(8, x), ref)
