"""The exact %.12g formatter of the device MIE writer (pg_fmt.h, exported as
pg_format_g12) against the C library's printf("%.12g"), on the CPU: random
doubles over the whole exponent range, values one ulp either side of
12-digit rounding ties and of powers of ten, and the special values."""
from __future__ import annotations

import ctypes as C
import ctypes.util

import numpy as np
import pytest

import parent_gb300 as pg

_libc = C.CDLL(ctypes.util.find_library("c"))
_libc.snprintf.restype = C.c_int


def _c(v: float) -> bytes:
    buf = C.create_string_buffer(64)
    _libc.snprintf(buf, 64, b"%.12g", C.c_double(v))
    return buf.value


def _ours(v: float) -> bytes:
    buf = C.create_string_buffer(64)
    n = pg.lib().pg_format_g12(C.c_double(v), buf)
    assert n == len(buf.value)
    return buf.value


def _check(values):
    bad = [(float(v), _ours(float(v)), _c(float(v))) for v in values if _ours(float(v)) != _c(float(v))]
    assert not bad, bad[:5]


def test_random_magnitudes():
    rng = np.random.default_rng(1)
    exps = rng.uniform(-30, 60, 40000)
    vals = np.sign(rng.uniform(-1, 1, exps.size)) * 10.0 ** exps
    _check(vals)
    raw = rng.integers(0, 2**63, 20000, dtype=np.uint64) | (rng.integers(0, 2, 20000, dtype=np.uint64) << 63)
    _check(raw.view(np.float64)[np.isfinite(raw.view(np.float64))])


def test_near_rounding_ties():
    rng = np.random.default_rng(2)
    vals = []
    for _ in range(8000):
        d = int(rng.integers(10**11, 10**12))
        k = int(rng.integers(-22, 48))
        t = float(f"{d}5e{k - 12}")  # a 13th digit of 5: a tie in decimal
        vals += [t, np.nextafter(t, 0), np.nextafter(t, np.inf), -t]
    _check(vals)


def test_powers_of_ten_and_specials():
    vals = [0.0, -0.0, 1.0, -1.0, 0.5, 1e-5, 1e-4, 9.99999999999e-5, 1e-21, 1e-22, 1e46, 1e47, 1e300, 5e-324,
            2.2250738585072014e-308, float("inf"), float("-inf"), 999999999999.5, 9.9999999999995, 99999999999.95,
            123456789012.0, 1234567890123.0, 0.1, 0.2, 0.3, 1 / 3, 2 / 3, np.pi, -np.e * 1e10, 2.0 ** 52, 2.0 ** 53 + 2]
    for k in range(-25, 50):
        p = 10.0 ** k
        vals += [p, np.nextafter(p, 0), np.nextafter(p, np.inf)]
    _check(vals)
    assert _ours(float("nan")).lstrip(b"-") == b"nan"


@pytest.mark.parametrize("scale", [1e-3, 1.0, 1e3])
def test_entropy_like_values(scale):
    rng = np.random.default_rng(3)
    _check(rng.normal(0, scale, 20000))
    _check(rng.normal(0, 1, 5000) * 1e-15)  # MI rounding noise around zero
