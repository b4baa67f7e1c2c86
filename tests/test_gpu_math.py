"""The stage kernels' reciprocal, quotient and Roe square-root product
(Num<R>::rcp/div/geo_mean) against correctly rounded NumPy arithmetic.

The float64 reciprocal and square root are third-order refinements of the
special-function unit's seeds and must stay within 1 ulp of the correctly
rounded results over the whole seeded range, with IEEE results (inf, NaN,
subnormal handling) outside it; the float64 quotient of the limiter/HLLE
weights multiplies by that reciprocal and must stay within 2 ulp (IEEE
outside the range); float32 uses the unit's approximations and must stay
within 2-3 ulp.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def probe(a, b):
    import torch
    from jathenax_gb300 import _lib
    dtype = _lib.JX_F64 if a.dtype == np.float64 else _lib.JX_F32
    A, B = torch.as_tensor(a, device="cuda"), torch.as_tensor(b, device="cuda")
    out = [torch.empty_like(A) for _ in range(3)]
    _lib.call("jx_probe_math", dtype, a.size, _lib.ptr(A), _lib.ptr(B), *(_lib.ptr(o) for o in out),
              _lib.stream_handle())
    return [o.cpu().numpy() for o in out]


def ulps(x, ref):
    return np.abs(x - ref) / np.spacing(np.abs(ref).astype(ref.dtype))


def wide(rng, n, dtype, lo, hi):
    e = rng.uniform(lo, hi, n)
    return (rng.choice([-1.0, 1.0], n) * rng.uniform(1.0, 2.0, n) * 2.0**np.floor(e)).astype(dtype)


def test_float64_reciprocal_within_one_ulp_and_quotient_within_two():
    rng = np.random.default_rng(1)
    b = np.concatenate([wide(rng, 400000, np.float64, -990, 970), rng.uniform(0.5, 2.0, 100000),
                        2.0 ** np.arange(-990, 970, dtype=np.float64)])
    a = wide(rng, b.size, np.float64, -300, 300)
    rcp, div, geo = probe(a, b)
    with np.errstate(over="ignore", under="ignore"):
        assert ulps(rcp, 1.0 / b).max() <= 1.0
        q = a / b
        ok = np.isfinite(q) & (np.abs(q) > np.finfo(np.float64).tiny)
        assert ulps(div[ok], q[ok]).max() <= 2.0
    ref = np.sqrt(np.abs(a)) * np.sqrt(np.abs(b))
    assert ulps(geo, ref).max() <= 2.0


def test_float64_square_root_within_one_ulp():
    # geo_mean(p, 1) is the refined square root of p inside the seed's range
    # and the correctly rounded one outside it.
    rng = np.random.default_rng(3)
    p = np.concatenate([np.abs(wide(rng, 400000, np.float64, -990, 970)), rng.uniform(0.25, 4.0, 100000),
                        2.0 ** np.arange(-1020, 1020, dtype=np.float64), [0.0, np.inf, np.finfo(np.float64).tiny]])
    _, _, geo = probe(p, np.ones_like(p))
    finite = np.isfinite(p) & (p > 0)
    assert ulps(geo[finite], np.sqrt(p[finite])).max() <= 1.0
    np.testing.assert_array_equal(geo[~finite], np.sqrt(p[~finite]))


def test_float64_edges_take_ieee_arithmetic():
    # Outside the seed's range (zero, subnormal, |b| < 2^-999 or > 2^977,
    # non-finite) the reciprocal is the correctly rounded IEEE one.
    tiny = np.finfo(np.float64).tiny
    b = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, tiny, tiny / 8, 2.0**-1000, 2.0**1000, 1e308, 1.0, 1e-200])
    a = np.array([1.0, 1.0, 2.0, 2.0, 1.0, 1.0, 1.0, 3.0, 3.0, 1.0, np.inf, 1e200])
    rcp, div, _ = probe(a, b)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        np.testing.assert_array_equal(rcp[:10], 1.0 / b[:10])
        np.testing.assert_array_equal(div, a / b)
    assert np.isinf(div[-1]) and div[-2] == np.inf


def test_float32_reciprocal_and_quotient_within_two_ulp():
    rng = np.random.default_rng(2)
    b = wide(rng, 300000, np.float32, -120, 120)
    a = wide(rng, b.size, np.float32, -30, 30)
    rcp, div, geo = probe(a, b)
    with np.errstate(over="ignore", under="ignore"):
        assert ulps(rcp, (1.0 / b.astype(np.float64)).astype(np.float32)).max() <= 2.0
        q = (a.astype(np.float64) / b).astype(np.float32)
        ok = np.isfinite(q) & (np.abs(q) > np.finfo(np.float32).tiny)
        assert ulps(div[ok], q[ok]).max() <= 3.0
    ref = (np.sqrt(np.abs(a.astype(np.float64))) * np.sqrt(np.abs(b.astype(np.float64)))).astype(np.float32)
    assert ulps(geo, ref).max() <= 3.0
