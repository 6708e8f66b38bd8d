"""The kernels' own arithmetic (hf_device.cuh / hf_intdiv.cuh, compiled for the host) against
IEEE division and square root and against the reference's HLLC and limiter fixtures -- on the
CPU, bit for bit.  The GPU build of the same source is checked by tests/test_intdiv.py and the
parity tests."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

LIB = os.path.join(ROOT, "hyperflow_gb300", "libhf_hostmath.so")


@pytest.fixture(scope="module")
def hm():
    if not os.path.exists(LIB):
        from hyperflow_gb300 import _build
        _build.build()
    L = C.CDLL(LIB)
    p, d, i, i64 = C.c_void_p, C.c_double, C.c_int, C.c_int64
    L.hm_div.argtypes = [p, p, p, i64]
    L.hm_sqrt.argtypes = [p, p, i64]
    L.hm_half.argtypes = [p, p, i64]
    L.hm_hllc.argtypes = [d, p, p, i, p]
    L.hm_hllc.restype = i
    L.hm_limiter.argtypes = [i, d]
    L.hm_limiter.restype = d
    L.hm_slope.argtypes = [i, d, d, d]
    L.hm_slope.restype = d
    L.hm_wave_terms.argtypes = [d, p, p]
    L.hm_compare.argtypes = [d, d, p]
    L.hm_compare.restype = i
    return L


def _same(a, b):
    return np.array_equal(a.view(np.uint64), b.view(np.uint64)) or \
        np.array_equal(np.where(np.isnan(a), 0, a.view(np.uint64)), np.where(np.isnan(b), 0, b.view(np.uint64)))


def _operands(rng, n):
    raw = rng.integers(0, 2**64, size=(2, n), dtype=np.uint64).view(np.float64)
    norm_e = rng.integers(1023 - 300, 1023 + 300, size=(2, n), dtype=np.uint64)
    mant = rng.integers(0, 2**52, size=(2, n), dtype=np.uint64)
    norm = ((norm_e << np.uint64(52)) | mant).view(np.float64) * np.where(rng.random((2, n)) < 0.5, -1, 1)
    return np.concatenate([raw, norm], axis=1)


def test_division_equals_ieee(hm):
    rng = np.random.default_rng(0)
    a, b = _operands(rng, 1_000_000)
    out = np.empty_like(a)
    hm.hm_div(a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size)
    with np.errstate(all="ignore"):
        want = a / b
    bad = ~((out.view(np.uint64) == want.view(np.uint64)) | (np.isnan(out) & np.isnan(want)))
    assert not bad.any(), (a[bad][:3], b[bad][:3])


def test_sqrt_equals_ieee(hm):
    rng = np.random.default_rng(1)
    x = np.abs(_operands(rng, 1_000_000)[0])
    x[:1000] = -x[:1000]
    out = np.empty_like(x)
    hm.hm_sqrt(x.ctypes.data, out.ctypes.data, x.size)
    with np.errstate(all="ignore"):
        want = np.sqrt(x)
    bad = ~((out.view(np.uint64) == want.view(np.uint64)) | (np.isnan(out) & np.isnan(want)))
    assert not bad.any(), x[bad][:3]


def test_hllc_and_limiters_equal_reference_fixture(hm):
    d = np.load(f"{GOLDEN}/unit_hllc_limiter.npz")
    UL, UR, F, r, lim = d["UL"], d["UR"], d["F"], d["r"], d["lim"]
    out = np.zeros(4)
    for dirn in range(2):
        for k in range(len(UL)):
            a = np.ascontiguousarray(UL[k]); b = np.ascontiguousarray(UR[k])
            hm.hm_hllc(1.4, a.ctypes.data, b.ctypes.data, dirn, out.ctypes.data)
            np.testing.assert_array_equal(out, F[dirn, k])
    for kind in range(2):
        got = np.array([hm.hm_limiter(kind, float(x)) for x in r])
        np.testing.assert_array_equal(got, lim[kind])


def test_slopes_equal_oracle(hm, port_lib):
    """Limited slopes on differences straddling the 1e-6 clamp, sign changes and zeros."""
    rng = np.random.default_rng(2)
    vals = np.concatenate([rng.normal(0, 1, 3000), rng.normal(0, 1e-6, 3000), np.zeros(50),
                           rng.choice([1e-6, -1e-6, 2e-6], 100)])
    from oracle.oracle import Oracle  # noqa: F401 (ensures the oracle library is built)
    import ctypes
    port_lib.hfo_limiter.restype = ctypes.c_double
    for kind in range(2):
        for k in range(0, len(vals) - 2, 3):
            um, u0, up = 1.0 + vals[k], 1.0 + vals[k] + vals[k + 1], 1.0 + vals[k] + vals[k + 1] + vals[k + 2]
            dl, dr = u0 - um, up - u0
            dlc = dl if abs(dl) > 1e-6 else (1e-6 if dl == 0 else 1e-6 * np.sign(dl))
            drc = dr if abs(dr) > 1e-6 else (1e-6 if dr == 0 else 1e-6 * np.sign(dr))
            xi = port_lib.hfo_limiter(kind, dlc / drc)
            want = xi * (0.5 * dl + 0.5 * dr)
            got = hm.hm_slope(kind, um, u0, up)
            assert got == want or (np.isnan(got) and np.isnan(want)), (kind, um, u0, up, got, want)


def _specials():
    tiny = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1e-6, -1e-6,
                     np.nextafter(1e-6, 1), np.nextafter(1e-6, 0), -np.nextafter(1e-6, 1),
                     1.0, np.nextafter(1.0, 2), np.nextafter(1.0, 0), -1.0, 2.0, 1e300, -1e300,
                     np.inf, -np.inf, np.nan, -np.nan])
    return tiny


def test_integer_compares_follow_ieee(hm):
    """lt/le0/ge0/abs_le, smin/smax ((b<a)?b:a, (a<b)?b:a) and the wave-speed max on signed
    zeros, subnormals, infinities, NaN and values next to the 1e-6 clamp."""
    rng = np.random.default_rng(3)
    vals = np.concatenate([_specials(), rng.normal(0, 1, 200), rng.normal(0, 1e-6, 50)])
    out = np.zeros(3)
    with np.errstate(all="ignore"):
        for a in vals:
            for b in vals:
                bits = hm.hm_compare(float(a), float(b), out.ctypes.data)
                want = (int(a < b)) | (int(a <= 0.0) << 1) | (int(0.0 <= a) << 2) | (int(abs(a) <= 1e-6) << 3)
                assert bits == want, (a, b, bits, want)
                m = abs(b)
                exp = np.array([b if b < a else a, b if a < b else a, a if a > m else m])
                assert np.array_equal(out.view(np.uint64), exp.view(np.uint64)) or \
                    all((x == y and np.signbit(x) == np.signbit(y)) or (np.isnan(x) and np.isnan(y))
                        for x, y in zip(out, exp)), (a, b, out, exp)


def test_limiters_on_special_ratios(hm, port_lib):
    import ctypes
    port_lib.hfo_limiter.restype = ctypes.c_double
    port_lib.hfo_limiter.argtypes = [ctypes.c_int, ctypes.c_double]
    rng = np.random.default_rng(4)
    near_one = 1.0 + np.concatenate([np.arange(-64, 65) * np.finfo(float).eps, rng.uniform(-1e-3, 1e-3, 200)])
    tiny = np.array([5e-324, 1e-320, 2.2250738585072014e-308, 1e-300, 1e-200, 1e-20])
    huge = np.array([1e20, 1e200, 1e300, 1.7976931348623157e308])
    rs = np.concatenate([_specials(), rng.lognormal(0, 2, 20000), -rng.lognormal(0, 2, 50), near_one, tiny, huge])
    for kind in range(2):
        for r in rs:
            got, want = hm.hm_limiter(kind, float(r)), port_lib.hfo_limiter(kind, float(r))
            assert (np.isnan(got) and np.isnan(want)) or \
                np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64), (kind, r, got, want)


def test_half_equals_multiplication(hm):
    rng = np.random.default_rng(5)
    x = np.concatenate([_specials(), _operands(rng, 500_000)[0],
                        np.array([2.2250738585072014e-308 * k for k in (1.0, 1.5, 2.0, 3.0, 4.0)]),
                        -np.array([2.2250738585072014e-308 * k for k in (1.0, 1.5, 2.0, 3.0, 4.0)]),
                        np.array([5e-324 * k for k in range(1, 40)])])
    out = np.empty_like(x)
    hm.hm_half(x.ctypes.data, out.ctypes.data, x.size)
    with np.errstate(invalid="ignore"):   # signalling NaNs among the operands
        want = 0.5 * x
    same = (out.view(np.uint64) == want.view(np.uint64)) | (np.isnan(out) & np.isnan(want))
    assert same.all(), x[~same][:5]


