"""CPU model of the tensor-core complex128 pass arithmetic (csrc/tcfx.cu).

Test infrastructure: it reproduces, step by step and exactly, what the
kernel computes for one pass -- the row exponent, the 60-bit fixed-point
integers, their balanced base-256 digits, the 36 digit products summed per
weight, the combination into one int64 and its FP64 rounding -- so a GPU
result can be compared with it bit for bit, and its error measured against
exact rational arithmetic on the CPU.

Rows are the 16 amplitudes that differ only in the four window bits; a
pass is y = U x per row, U a 16 x 16 unitary given as the integers
round(U * 2^62) (real and imaginary parts); the result is
Z = A.G / 2^63 over the kept digit products, times 2^(E - 1082).
"""
from fractions import Fraction

import numpy as np

MB = 61                    # |A| < 2^61
BIAS = 0x8080808080808080  # 128 in every byte
EMIN = 64                  # groups below 2^-959 are all zero


def _bits(v):
    return int(np.array(v, dtype=np.float64).view(np.uint64))


def row_exponent(parts):
    """Largest FP64 exponent field among the parts (4095 for tiny rows)."""
    e = max((_bits(v) >> 52) & 0x7FF for v in parts)
    return 4095 if e < EMIN else e


def fixed(v, E):
    """A = v * 2^(1022 + 61 - E) truncated toward zero, as the kernel forms it."""
    b = _bits(v)
    e = (b >> 52) & 0x7FF
    m = ((b & ((1 << 52) - 1)) | (1 << 52)) << 11  # hidden bit at bit 63 (zeros shift out)
    s = E - e + 64 - MB
    q = m >> s if s < 64 else 0
    return -q if b >> 63 else q


def digits(X):
    """Balanced base-256 digits (most significant first) of an integer |X| <= 2^62."""
    U = (X + BIAS) & ((1 << 64) - 1)
    return [((U >> (8 * (7 - t))) & 0xFF) - 128 for t in range(8)]


def real_form(g):
    """32 x 32 integer real form of the 16 x 16 complex integer matrix g[r][c] = (re, im):
    output real 2r+p, input real 2c+q."""
    G = np.zeros((32, 32), dtype=object)
    for r in range(16):
        for c in range(16):
            gr, gi = int(g[r][c][0]), int(g[r][c][1])
            G[2 * r, 2 * c], G[2 * r, 2 * c + 1] = gr, -gi
            G[2 * r + 1, 2 * c], G[2 * r + 1, 2 * c + 1] = gi, gr
    return G


def gate_digits(g):
    """Digits of U's real form: int64 array [output real, input real, digit]."""
    G = real_form(g)
    return np.array([[digits(int(G[o, k])) for k in range(32)] for o in range(32)], dtype=np.int64)


def pass_row_z(g, amps, gd=None):
    """The kernel's integers for one row before the FP64 conversion: (Z for
    the 32 output reals, the row exponent E); the output is Z * 2^(E - 1082).
    amps = 16 complex128 values (window index order), g = 16 x 16 x 2
    integers (gd: their gate_digits, if already formed)."""
    parts = [p for a in amps for p in (float(a.real), float(a.imag))]
    E = row_exponent(parts)
    Ad = np.array([digits(fixed(p, E)) for p in parts], dtype=np.int64)  # 32 x 8
    if gd is None:
        gd = gate_digits(g)
    prod = np.einsum("kt,oku->otu", Ad, gd)                                # exact: |entries| < 2^22
    zs = []
    for o in range(32):
        acc = [int(sum(prod[o, t, d - t] for t in range(d + 1))) for d in range(8)]
        assert all(abs(a) < (1 << 22) for a in acc), acc
        p = [acc[2 * j] * 256 + acc[2 * j + 1] for j in range(4)]
        Z = (p[0] << 41) + (p[1] << 25) + (p[2] << 9) + (p[3] >> 7)
        assert abs(Z) < (1 << 63)
        zs.append(Z)
    return zs, E


def pass_row(g, amps, gd=None):
    """The kernel's output for one row (16 complex128 values)."""
    zs, E = pass_row_z(g, amps, gd)
    out = [np.ldexp(float(Z), E - 1082) if Z else 0.0 for Z in zs]
    return np.array([complex(out[2 * c], out[2 * c + 1]) for c in range(16)])


def _round_half_away(f):
    n = abs(f.numerator) * 2 + f.denominator
    q = n // (2 * f.denominator)
    return q if f >= 0 else -q


def gate_integers(U):
    """round(U * 2^62) (half away from zero) of a complex 16 x 16 matrix of
    float64 entries, as the host forms them for a pass whose U needs no
    products of gates."""
    g = np.zeros((16, 16, 2), dtype=object)
    for r in range(16):
        for c in range(16):
            g[r][c][0] = _round_half_away(Fraction(float(U[r, c].real)) * 2 ** 62)
            g[r][c][1] = _round_half_away(Fraction(float(U[r, c].imag)) * 2 ** 62)
    return g
