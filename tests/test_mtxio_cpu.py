"""vecjac_gb300.mtxio: the raw matrix files and the `wide` singular-value files of the
command-line drivers -- round trips, size checks, and the special values of both wide
formats (zero, subnormal, infinity, NaN) against this host's long double where it is the
x87 format."""
from fractions import Fraction
import math

import numpy as np
import pytest

from vecjac_gb300 import mtxio


@pytest.mark.parametrize("dt", [np.float64, np.float32, np.complex128, np.complex64])
def test_matrix_round_trip(tmp_path, dt):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((7, 5))
    if np.dtype(dt).kind == "c":
        A = A + 1j * rng.standard_normal((7, 5))
    A = A.astype(dt)
    p = str(tmp_path / "a.G")
    mtxio.write_matrix(p, A)
    raw = np.fromfile(p, dtype=dt)
    assert np.array_equal(raw, A.T.reshape(-1))          # column-major
    assert np.array_equal(mtxio.read_matrix(p, 7, 5, dt), A)
    with pytest.raises(ValueError):
        mtxio.read_matrix(p, 8, 5, dt)


@pytest.mark.parametrize("fmt", ["q", "l"])
def test_wide_special_values(tmp_path, fmt):
    vals = [0.0, -0.0, 1.0, -2.5, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, Fraction(1, 3) ** 0]
    p = str(tmp_path / "s.S2")
    mtxio.write_wide(p, vals, fmt)
    got = mtxio.read_wide(p, len(vals), fmt)
    assert np.array_equal(got, np.array([float(v) for v in vals]))
    assert math.copysign(1.0, got[1]) == -1.0
    with pytest.raises(ValueError):
        mtxio.read_wide(p, len(vals) + 1, fmt)
    inf = (0x7FFF << 112).to_bytes(16, "little") if fmt == "q" else ((1 << 63) | (0x7FFF << 64)).to_bytes(16, "little")
    nan = ((0x7FFF << 112) | (1 << 111)).to_bytes(16, "little") if fmt == "q" else \
        ((3 << 62) | (0x7FFF << 64)).to_bytes(16, "little")
    assert mtxio.wide_to_float(inf, fmt) == math.inf and math.isnan(mtxio.wide_to_float(nan, fmt))


def test_wide_x87_against_long_double():
    if np.finfo(np.longdouble).nmant != 63:
        pytest.skip("this host's long double is not the x87 format")
    for v in [1.0, -3.0, 5e-324, 1e-310, 1.5e300, 2.0 ** -1074]:
        assert mtxio.encode_wide(v, "l")[:10] == np.longdouble(v).tobytes()[:10], v
    # a value between double's and x87's ranges, rounded to 64 significant bits
    x = Fraction(1, 3)
    assert mtxio.encode_wide(x, "l")[:10] == (np.longdouble(1) / np.longdouble(3)).tobytes()[:10]


def test_wide_rejects_overflow():
    with pytest.raises(OverflowError):
        mtxio.encode_wide(Fraction(2) ** 20000, "q")
