"""The digit arithmetic of the tensor-core complex128 passes, on the CPU
(tests/txarith.py models the kernel step by step): its error against exact
rational arithmetic, the bound that keeps every FP32 accumulator exact
(below 2^22) on adversarial rows, and the digit and fixed-point forms
themselves.  The GPU tests compare the kernel with this model bit for bit."""
from fractions import Fraction

import numpy as np
import pytest

import txarith as tx


def _unitary(n, rng):
    q, r = np.linalg.qr(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_digits_and_fixed_point_forms():
    rng = np.random.default_rng(0)
    for x in [0, 1, -1, 2 ** 61 - 1, -(2 ** 61 - 1), 2 ** 62, -(2 ** 62)] + \
             [int(v) for v in rng.integers(-2 ** 62, 2 ** 62, 200)]:
        d = tx.digits(x)
        assert all(-128 <= v <= 127 for v in d)
        assert sum(v * 256 ** (7 - t) for t, v in enumerate(d)) == x
    # truncation toward zero at 2^-61 of the row's largest part
    for v in [1.0, -0.7, 3.5e-9, -2.2e-300, 0.0]:
        E = tx.row_exponent([v, 0.5 * v])
        A = tx.fixed(v, E)
        exact = Fraction(v) * 2 ** (1022 + 61 - E) if E != 4095 else Fraction(0)
        assert abs(Fraction(A)) <= abs(exact) < abs(Fraction(A)) + 1


@pytest.mark.parametrize("case", range(6))
def test_error_against_exact_arithmetic(case):
    """Per output: |Z 2^(E-1082) - (U x)| below 2^-55 of the row's largest
    part before the one FP64 rounding (the truncation of the 32 input parts,
    each below 2^-59 of it, summed through a unit row of U: at most
    sqrt(32) 2^-59 = 2^-56.5; the dropped digit products add less), and the
    stored FP64 value within one more rounding."""
    rng = np.random.default_rng(40 + case)
    U = _unitary(16, rng)
    g = tx.gate_integers(U)
    gd = tx.gate_digits(g)
    worst_z = worst_out = 0.0
    for trial in range(12):
        amps = (rng.normal(size=16) + 1j * rng.normal(size=16)) * 10.0 ** rng.uniform(-200, 50)
        if trial % 3 == 1:
            amps[rng.integers(0, 16, 6)] *= 10.0 ** rng.uniform(-30, -3)
        if trial % 3 == 2:
            amps[rng.integers(0, 16, 5)] = 0
        zs, E = tx.pass_row_z(g, amps, gd)
        out = tx.pass_row(g, amps, gd)
        mx = max(max(abs(a.real), abs(a.imag)) for a in amps)
        for r in range(16):
            ex_re = sum(Fraction(int(g[r][c][0])) * Fraction(float(amps[c].real)) -
                        Fraction(int(g[r][c][1])) * Fraction(float(amps[c].imag)) for c in range(16)) / 2 ** 62
            ex_im = sum(Fraction(int(g[r][c][0])) * Fraction(float(amps[c].imag)) +
                        Fraction(int(g[r][c][1])) * Fraction(float(amps[c].real)) for c in range(16)) / 2 ** 62
            scale = Fraction(2) ** (E - 1082)
            for z, ex, o in ((zs[2 * r], ex_re, out[r].real), (zs[2 * r + 1], ex_im, out[r].imag)):
                worst_z = max(worst_z, float(abs(z * scale - ex)) / mx)
                worst_out = max(worst_out, float(abs(Fraction(float(o)) - ex)) / mx)
    assert worst_z < 2.0 ** -55, worst_z
    assert worst_out < 2.0 ** -51, worst_out


def test_accumulators_stay_exact_on_extreme_rows():
    """Rows whose parts sit at the top of the fixed-point range with signs
    chosen to align every digit product: the eight accumulators stay below
    2^22 (pass_row_z asserts it) and the result still matches exactly."""
    rng = np.random.default_rng(3)
    for _ in range(4):
        U = _unitary(16, rng)
        g = tx.gate_integers(U)
        gd = tx.gate_digits(g)
        for sign_of in (lambda r: np.sign(U[r].real + 1e-300), lambda r: -np.ones(16)):
            for r in range(0, 16, 5):
                s = sign_of(r)
                amps = (np.where(s >= 0, 1.0, -1.0) * (1 - 2 ** -52)) * (1 + 1j)
                zs, E = tx.pass_row_z(g, amps.astype(np.complex128), gd)
                assert all(abs(z) < 2 ** 63 for z in zs)
