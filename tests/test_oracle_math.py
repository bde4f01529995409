"""The deterministic math shared (as the same algorithm) by the oracle and
libvpt: error bounds against float64, and bit-identity between the oracle's
copy and libvpt's host build of it."""
import numpy as np
import pytest


def ulp_err(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    spacing = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    spacing = np.maximum(spacing, np.finfo(np.float32).tiny)
    return np.abs(got - ref) / spacing


def oracle_vec(fn, xs, ys=None):
    if ys is None:
        return np.array([fn(float(x)) for x in xs], np.float32)
    return np.array([fn(float(x), float(y)) for x, y in zip(xs, ys)], np.float32)


@pytest.fixture(scope="module")
def L(oracle):
    return oracle.lib()


def test_exp_bounds(L):
    x = np.random.default_rng(0).uniform(-87, 88.5, 4000).astype(np.float32)
    got = oracle_vec(L.vpto_exp, x)
    assert ulp_err(got, np.exp(x.astype(np.float64))).max() <= 4


def test_exp2_log2_bounds(L):
    rng = np.random.default_rng(1)
    x = rng.uniform(-125, 127, 4000).astype(np.float32)
    assert ulp_err(oracle_vec(L.vpto_exp2, x), np.exp2(x.astype(np.float64))).max() <= 4
    y = np.exp(rng.uniform(-80, 80, 4000)).astype(np.float32)
    got = oracle_vec(L.vpto_log2, y)
    ref = np.log2(y.astype(np.float64))
    assert np.abs(got - ref).max() <= 4e-6 * np.maximum(1.0, np.abs(ref)).max()


def test_sin_cos_bounds(L):
    x = np.random.default_rng(2).uniform(0, 2 * np.pi, 4000).astype(np.float32)
    for fn, ref in ((L.vpto_sin, np.sin), (L.vpto_cos, np.cos)):
        got = oracle_vec(fn, x)
        assert np.abs(got - ref(x.astype(np.float64))).max() < 3e-7


def test_pow_integer_and_fractional(L):
    rng = np.random.default_rng(3)
    x = rng.uniform(0.01, 2.0, 2000).astype(np.float32)
    for y in (2.0, 5.0, 16.0, 32.0, 134.0, 2.2, 1.5, 2.9, 1.25):
        got = oracle_vec(L.vpto_pow, x, np.full_like(x, y))
        ref = np.power(x.astype(np.float64), y)
        rel = np.abs(got - ref) / np.maximum(ref, 1e-30)
        assert rel[np.isfinite(ref) & (ref > 1e-30) & (ref < 1e30)].max() < 4e-5, y
    # GLSL-defined cases
    assert L.vpto_pow(0.0, 3.0) == 0.0
    assert L.vpto_pow(1.0, 1e9) == 1.0
    assert L.vpto_pow(5.0, 0.0) == 1.0
    assert L.vpto_pow(2.0, 3.0) == 8.0
    assert np.isnan(L.vpto_pow(-1.0, 2.0))


def test_half_round_matches_ieee(L):
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.normal(0, 1, 3000), rng.normal(0, 3000, 3000), rng.uniform(-7e4, 7e4, 2000),
                        np.exp(rng.uniform(-20, 0, 2000)) * rng.choice([-1, 1], 2000),
                        [65504.0, 65519.0, 65520.0, 1e-8, 2.0 ** -25, 2.0 ** -24, 3 * 2.0 ** -26]]).astype(np.float32)
    got = oracle_vec(L.vpto_half_round, x)
    ref = x.astype(np.float16).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_libvpt_host_math_is_bit_identical_to_oracle(vpt, L):
    rng = np.random.default_rng(6)
    cases = {
        0: (vpt.detmath, L.vpto_exp, rng.uniform(-110, 90, 3000)),
        1: (vpt.detmath, L.vpto_exp2, rng.uniform(-160, 130, 3000)),
        2: (vpt.detmath, L.vpto_log2, np.exp(rng.uniform(-100, 80, 3000))),
        4: (vpt.detmath, L.vpto_sin, rng.uniform(-50, 50, 3000)),
        5: (vpt.detmath, L.vpto_cos, rng.uniform(-50, 50, 3000)),
    }
    for op, (dev, ofn, x) in cases.items():
        x = x.astype(np.float32)
        a = dev(op, x, on_device=False)
        b = oracle_vec(ofn, x)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), op
    x = rng.uniform(0, 3, 3000).astype(np.float32)
    y = np.concatenate([rng.integers(1, 140, 1500), rng.uniform(-4, 140, 1500)]).astype(np.float32)
    a = vpt.detmath(3, x, y, on_device=False)
    b = oracle_vec(L.vpto_pow, x, y)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_division_by_five_in_three_operations_is_exact(L):
    """The device's x / 5 (one product, one remainder correction) equals
    IEEE division for every non-negative finite float; the form is odd in
    x, so for every finite float."""
    assert L.vpto_check_div_const(5.0, 0, 0x7F800000) == 0
    # the check does see a difference: infinity, which the form turns into NaN
    assert L.vpto_check_div_const(5.0, 0x7F800000, 0x7F800001) == 1


def test_libvpt_host_references_of_the_packed_checks(vpt):
    """The host side of detmath's packed-pair checks (ops 6..17), the values
    the device's packed forms are compared with: IEEE products, sums, x + y x,
    the two-row bilinear blend and x / 5, as numpy's float32 gives them."""
    rng = np.random.default_rng(12)
    n = 4000
    x = (rng.uniform(-1, 1, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    y = (rng.uniform(-1, 1, n) * np.exp2(rng.integers(-20, 20, n))).astype(np.float32)
    with np.errstate(over="ignore", invalid="ignore"):
        for op, want in ((6, x * y), (7, x * y), (8, x + y), (9, x + y), (12, x + y * x), (15, x / np.float32(5))):
            got = vpt.detmath(op, x, y, on_device=False)
            assert np.array_equal(got.view(np.uint32), want.astype(np.float32).view(np.uint32)), op
        w = rng.uniform(0, 8, n).astype(np.float32)
        ax = w - np.floor(w)
        ay = np.float32(2) * w - np.floor(np.float32(2) * w)
        bx, by = np.float32(1) - ax, np.float32(1) - ay
        lo = x * bx + (np.float32(2) * x) * ax
        hi = (-x) * bx + w * ax
        want = lo * by + hi * ay
        for op in (13, 14):
            got = vpt.detmath(op, x, w, on_device=False)
            assert np.array_equal(got.view(np.uint32), want.astype(np.float32).view(np.uint32)), op
        # ops 16 and 17 (the packed exponential for non-positive arguments): exp(x) itself
        xn = -np.abs(x)
        for op in (16, 17):
            got = vpt.detmath(op, xn, -np.abs(y), on_device=False)
            assert np.array_equal(got.view(np.uint32), vpt.detmath(0, xn, on_device=False).view(np.uint32)), op
