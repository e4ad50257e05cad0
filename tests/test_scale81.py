"""The FP32 evaluation of (float)((double)v * (1./81.)) used by the
extrapolation sweep (mul_inv81 in ofblend_gb300/csrc/flof_common.cuh),
modelled in numpy: every step of the device function is reproduced with
exactly rounded float32 operations (float64 holds each intermediate exactly
here), and the result must equal the reference's double-then-float rounding
for every input, including products constructed next to float rounding
midpoints, where the device function takes its double path."""
import numpy as np

C = 1.0 / 81.0
C_HI = np.float32(C)
C_LO = np.float32(C - np.float64(C_HI))


def model(v):
    v = np.asarray(v, np.float32)
    v64 = v.astype(np.float64)
    p = (v64 * np.float64(C_HI)).astype(np.float32)                      # v*c_hi, rounded
    pe = (v64 * np.float64(C_HI) - p.astype(np.float64)).astype(np.float32)  # exact error
    lo = (v64 * np.float64(C_LO) + pe.astype(np.float64)).astype(np.float32)  # fma
    f = (p.astype(np.float64) + lo.astype(np.float64)).astype(np.float32)
    bits = f.view(np.uint32)
    E = (bits >> 23) & 0xFF
    rem = ((p.astype(np.float64) - f.astype(np.float64)).astype(np.float32).astype(np.float64)
           + lo.astype(np.float64)).astype(np.float32)
    with np.errstate(over="ignore"):
        half_ulp = ((E.astype(np.int64) - 24).clip(0) << 23).astype(np.uint32).view(np.float32)
        margin = ((E.astype(np.int64) - 40).clip(0) << 23).astype(np.uint32).view(np.float32)
    fast = (E > 41) & (E < 255) & (np.abs(np.abs(rem) - half_ulp) > margin)
    fast |= v == 0
    slow = (v64 * C).astype(np.float32)
    return np.where(fast, f, slow), fast


def reference(v):
    return (np.asarray(v, np.float32).astype(np.float64) * C).astype(np.float32)


def test_random_magnitudes():
    rng = np.random.default_rng(0)
    for scale in (1e-30, 1e-6, 1e-3, 1.0, 1e3, 1e20):
        v = (rng.standard_normal(2_000_000) * scale).astype(np.float32)
        got, fast = model(v)
        assert np.array_equal(got.view(np.uint32), reference(v).view(np.uint32))
        assert fast.mean() > 0.999 or scale < 1e-20


def test_all_mantissas_of_two_binades():
    # every float in [1, 4): the exhaustive check of the significand range
    v = np.arange(0x3F800000, 0x40800000, dtype=np.uint32).view(np.float32)
    got, fast = model(v)
    assert np.array_equal(got.view(np.uint32), reference(v).view(np.uint32))
    assert fast.all()  # no normal input takes the double path


def test_products_stay_far_from_midpoints():
    # For v = m 2^-23 the product v/81 lies k/81 of a float ulp away from the
    # float grid (k an integer, 81 odd), so it is never closer than 1/162 ulp
    # to a rounding midpoint: the FP32 path is exact for every normal input
    # and the double path only serves tiny and non-finite values.
    v = np.arange(0x3F800000, 0x40000000, 97, dtype=np.uint32).view(np.float32)
    prod = v.astype(np.float64) * C
    f = prod.astype(np.float32)
    ulp = np.spacing(f).astype(np.float64)
    dist = np.abs(np.abs(prod - f.astype(np.float64)) - ulp / 2) / ulp
    assert dist.min() > 1.0 / 200
    got, fast = model(v)
    assert fast.all()
    tiny = np.array([1e-40, -3e-39, 1e-45, np.inf, -np.inf], np.float32)
    got, fast = model(tiny)
    assert not fast.any()
    assert np.array_equal(got.view(np.uint32), reference(tiny).view(np.uint32))
