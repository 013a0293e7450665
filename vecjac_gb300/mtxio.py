"""The raw matrix files of the command-line drivers (t?vjsvd.exe), as the reference's
src/mtxio.c reads and writes them: no header, column-major, complex entries interleaved
(re, im), and singular values in the reference's `wide` type -- IEEE binary128 ("q",
its default build) or x87 80-bit extended in 16-byte slots ("l", WP=l).
"""
import numpy as np


def write_matrix(path, A):
    """Write the (m, n) array A column-major to path (its dtype as it is)."""
    np.asarray(A).T.tofile(path)  # tofile writes C order: the rows of A^T, i.e. A's columns


def read_matrix(path, m, n, dtype):
    """The (m, n) column-major matrix in path; the file must hold exactly m n entries."""
    a = np.fromfile(path, dtype=dtype)
    if a.size != m * n:
        raise ValueError("%s holds %d entries, not %d x %d" % (path, a.size, m, n))
    return a.reshape((n, m)).T


def wide_to_float(b, fmt="q"):
    """Value of one 16-byte `wide` (little-endian) as a Python float; exact when the value
    fits a double (always so for singular values written from (eS, fS) pairs)."""
    import math
    x = int.from_bytes(bytes(b[:16]), "little")
    if fmt == "q":
        s, e, f = x >> 127, (x >> 112) & 0x7FFF, x & ((1 << 112) - 1)
        if e == 0x7FFF:
            v = math.nan if f else math.inf
        elif e == 0:
            v = math.ldexp(float(f), -16382 - 112)
        else:
            v = math.ldexp(float((1 << 112) | f), e - 16383 - 112)
    elif fmt == "l":
        sig, se = x & ((1 << 64) - 1), (x >> 64) & 0xFFFF
        s, e = se >> 15, se & 0x7FFF
        if e == 0x7FFF:
            v = math.nan if (sig << 1) & ((1 << 64) - 1) else math.inf
        else:
            v = math.ldexp(float(sig), max(e, 1) - 16383 - 63)
    else:
        raise ValueError("fmt is 'q' or 'l'")
    return -v if s else v


def read_wide(path, n, fmt="q"):
    """The n singular values of a BaseName.S? file as float64."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size != 16 * n:
        raise ValueError("%s holds %d bytes, not 16 x %d" % (path, raw.size, n))
    return np.array([wide_to_float(raw[16 * i:16 * i + 16], fmt) for i in range(n)])


def encode_wide(x, fmt="q"):
    """16 little-endian bytes of the finite value x (a float, int or Fraction) in the wide
    type, rounded to nearest even: binary128 ("q") or x87 extended ("l", 6 zero padding
    bytes). Exact for the product of two doubles in binary128."""
    import math
    from fractions import Fraction
    # the sign of a float zero is kept (a Fraction has none)
    sign = 1 if (x < 0 or (isinstance(x, float) and math.copysign(1.0, x) < 0)) else 0
    x = abs(Fraction(x))
    P, EMIN = (113, -16382) if fmt == "q" else (64, -16382)
    if x == 0:
        sig, e = 0, None
    else:
        e = x.numerator.bit_length() - x.denominator.bit_length()
        if Fraction(2) ** e > x:
            e -= 1                                  # 2^e <= x < 2^(e+1)
        e = max(e, EMIN)
        q = x / Fraction(2) ** (e - P + 1)          # the significand scaled to P bits
        sig = q.numerator // q.denominator
        rem = q - sig
        if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and sig & 1):
            sig += 1
        if sig >> P:
            sig >>= 1
            e += 1
        if e > 16383:
            raise OverflowError("outside the wide type's range")
    if fmt == "q":
        if sig == 0:
            bits = 0
        elif sig >> (P - 1):
            bits = ((e + 16383) << 112) | (sig & ((1 << 112) - 1))
        else:
            bits = sig                              # subnormal
        return ((sign << 127) | bits).to_bytes(16, "little")
    if fmt != "l":
        raise ValueError("fmt is 'q' or 'l'")
    if sig == 0:
        se = 0
    else:
        se = (e + 16383) if sig >> (P - 1) else 0
    return (sig | (((sign << 15) | se) << 64)).to_bytes(16, "little")


def write_wide(path, values, fmt="q"):
    """Write the values (floats or Fractions) as a BaseName.S? file."""
    with open(path, "wb") as f:
        for v in values:
            f.write(encode_wide(v, fmt))
