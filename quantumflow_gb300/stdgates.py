"""Standard gates (quantumflow/stdgates.py).

Each gate is its published matrix built on the host in complex128 (the
reference builds the same matrices with backend math, e.g. RX
stdgates.py:179-205, RZ :236-262, ZZ :944-968).  Parameterised gates keep
their parameters so ``.H`` returns the typed inverse (RX(-theta) ...), which
the adjoint-gradient path uses to identify differentiable angles.
"""
import copy
from math import pi, sqrt

import numpy as np

from .ops import Gate
from .qubits import Qubit

__all__ = ["I", "X", "Y", "Z", "H", "S", "T", "PHASE", "RX", "RY", "RZ", "CZ", "CNOT", "SWAP",
           "ISWAP", "CPHASE00", "CPHASE01", "CPHASE10", "CPHASE", "PSWAP", "CCNOT", "CSWAP",
           "RN", "TX", "TY", "TZ", "TH", "ZYZ", "CAN", "XX", "YY", "ZZ", "PISWAP", "EXCH",
           "CANONICAL", "S_H", "T_H", "STDGATES", "GATESET"]


def _cis(x):
    return np.exp(1j * x)


class I(Gate):
    """Identity on any number of qubits (quantumflow/gates.py:34-54)."""

    def __init__(self, *qubits: Qubit) -> None:
        if not qubits:
            qubits = (0,)
        super().__init__(np.eye(2 ** len(qubits)), qubits)

    @property
    def H(self) -> Gate:
        return self

    def __pow__(self, t: float) -> Gate:
        return self


class _Hermitian(Gate):
    @property
    def H(self) -> Gate:
        return copy.copy(self)


class X(_Hermitian):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[0, 1], [1, 0]], [q0])

    def __pow__(self, t):
        return TX(t, *self.qubits)


class Y(_Hermitian):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[0, -1j], [1j, 0]], [q0])

    def __pow__(self, t):
        return TY(t, *self.qubits)


class Z(_Hermitian):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1, 0], [0, -1.0]], [q0])

    def __pow__(self, t):
        return TZ(t, *self.qubits)


class H(_Hermitian):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__(np.array([[1, 1], [1, -1]]) / sqrt(2), [q0])

    def __pow__(self, t):
        return TH(t, *self.qubits)


class S(Gate):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1.0, 0.0], [0.0, 1.0j]], [q0])

    @property
    def H(self):
        return S_H(*self.qubits)

    def __pow__(self, t):
        return PHASE(pi / 2 * t, *self.qubits)


class T(Gate):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1.0, 0.0], [0.0, _cis(pi / 4.0)]], [q0])

    @property
    def H(self):
        return T_H(*self.qubits)

    def __pow__(self, t):
        return PHASE(pi / 4 * t, *self.qubits)


class S_H(Gate):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1.0, 0.0], [0.0, -1.0j]], [q0])

    @property
    def H(self):
        return S(*self.qubits)

    def __pow__(self, t):
        return PHASE(-pi / 2 * t, *self.qubits)


class T_H(Gate):
    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1.0, 0.0], [0.0, _cis(-pi / 4.0)]], [q0])

    @property
    def H(self):
        return T(*self.qubits)

    def __pow__(self, t):
        return PHASE(-pi / 4 * t, *self.qubits)


class PHASE(Gate):
    def __init__(self, theta: float, q0: Qubit = 0) -> None:
        super().__init__([[1.0, 0.0], [0.0, _cis(theta)]], [q0], dict(theta=theta))

    @property
    def H(self):
        theta = self.params["theta"]
        return PHASE(2.0 * pi - theta % (2.0 * pi), *self.qubits)

    def __pow__(self, t):
        return PHASE(self.params["theta"] * t, *self.qubits)


class RX(Gate):
    """exp(-i theta X / 2)."""

    def __init__(self, theta: float, q0: Qubit = 0) -> None:
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        super().__init__([[c, -1j * s], [-1j * s, c]], [q0], dict(theta=theta))

    @property
    def H(self):
        return RX(-self.params["theta"], *self.qubits)

    def __pow__(self, t):
        return RX(self.params["theta"] * t, *self.qubits)


class RY(Gate):
    """exp(-i theta Y / 2)."""

    def __init__(self, theta: float, q0: Qubit = 0) -> None:
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        super().__init__([[c, -s], [s, c]], [q0], dict(theta=theta))

    @property
    def H(self):
        return RY(-self.params["theta"], *self.qubits)

    def __pow__(self, t):
        return RY(self.params["theta"] * t, *self.qubits)


class RZ(Gate):
    """exp(-i theta Z / 2)."""

    def __init__(self, theta: float, q0: Qubit = 0) -> None:
        super().__init__([[_cis(-0.5 * theta), 0], [0, _cis(0.5 * theta)]], [q0], dict(theta=theta))

    @property
    def H(self):
        return RZ(-self.params["theta"], *self.qubits)

    def __pow__(self, t):
        return RZ(self.params["theta"] * t, *self.qubits)


class RN(Gate):
    """Rotation by theta about the unit axis (nx, ny, nz)."""

    def __init__(self, theta, nx, ny, nz, q0: Qubit = 0) -> None:
        c, s = np.cos(theta / 2), np.sin(theta / 2)
        m = [[c - 1j * s * nz, -1j * s * nx - s * ny],
             [-1j * s * nx + s * ny, c + 1j * s * nz]]
        super().__init__(m, [q0], dict(theta=theta, nx=nx, ny=ny, nz=nz))

    @property
    def H(self):
        p = self.params
        return RN(-p["theta"], p["nx"], p["ny"], p["nz"], *self.qubits)

    def __pow__(self, t):
        p = self.params
        return RN(t * p["theta"], p["nx"], p["ny"], p["nz"], *self.qubits)


def _turn(t, rot):
    """e^{i pi t/2} times the rotation by pi*t (powers of Paulis and H)."""
    th = pi * t
    return _cis(0.5 * th) * rot(th)


class TX(Gate):
    """X**t = e^{i pi t/2} RX(pi t)."""

    def __init__(self, t: float, q0: Qubit = 0) -> None:
        t = t % 2
        m = _turn(t, lambda th: np.array([[np.cos(th / 2), -1j * np.sin(th / 2)],
                                          [-1j * np.sin(th / 2), np.cos(th / 2)]]))
        super().__init__(m, [q0], dict(t=t))

    @property
    def H(self):
        return TX(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return TX(self.params["t"] * t, *self.qubits)


class TY(Gate):
    """Y**t = e^{i pi t/2} RY(pi t)."""

    def __init__(self, t: float, q0: Qubit = 0) -> None:
        t = t % 2
        m = _turn(t, lambda th: np.array([[np.cos(th / 2), -np.sin(th / 2)],
                                          [np.sin(th / 2), np.cos(th / 2)]]))
        super().__init__(m, [q0], dict(t=t))

    @property
    def H(self):
        return TY(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return TY(self.params["t"] * t, *self.qubits)


class TZ(Gate):
    """Z**t = e^{i pi t/2} RZ(pi t)."""

    def __init__(self, t: float, q0: Qubit = 0) -> None:
        t = t % 2
        m = _turn(t, lambda th: np.array([[_cis(-th / 2), 0], [0, _cis(th / 2)]]))
        super().__init__(m, [q0], dict(t=t))

    @property
    def H(self):
        return TZ(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return TZ(self.params["t"] * t, *self.qubits)


class TH(Gate):
    """H**t: rotation by pi*t about (X + Z)/sqrt(2), times e^{i pi t/2}."""

    def __init__(self, t: float, q0: Qubit = 0) -> None:
        th = pi * t
        ph = _cis(0.5 * th)
        c, s = np.cos(th / 2), np.sin(th / 2)
        m = [[ph * c - ph * 1j * s / sqrt(2), -(ph * 1j * s) / sqrt(2)],
             [-(ph * 1j * s) / sqrt(2), ph * c + ph * 1j * s / sqrt(2)]]
        super().__init__(m, [q0], dict(t=t))

    @property
    def H(self):
        return TH(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return TH(self.params["t"] * t, *self.qubits)


class ZYZ(Gate):
    """Z^t0 Y^t1 Z^t2 Euler decomposition (up to phase) in SU(2)."""

    def __init__(self, t0: float, t1: float, t2: float, q0: Qubit = 0) -> None:
        a0, a1, a2 = pi * t0, pi * t1, pi * t2
        m = [[_cis(-0.5 * a2 - 0.5 * a0) * np.cos(0.5 * a1), -_cis(-0.5 * a2 + 0.5 * a0) * np.sin(0.5 * a1)],
             [_cis(0.5 * a2 - 0.5 * a0) * np.sin(0.5 * a1), _cis(0.5 * a2 + 0.5 * a0) * np.cos(0.5 * a1)]]
        super().__init__(m, [q0], dict(t0=t0, t1=t1, t2=t2))

    @property
    def H(self):
        p = self.params
        return ZYZ(-p["t2"], -p["t1"], -p["t0"], *self.qubits)


class CZ(_Hermitian):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1) -> None:
        super().__init__(np.diag([1, 1, 1, -1]), [q0, q1])


class CNOT(_Hermitian):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1) -> None:
        super().__init__([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], [q0, q1])


class SWAP(_Hermitian):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1) -> None:
        super().__init__([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], [q0, q1])


class ISWAP(Gate):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1) -> None:
        super().__init__([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]], [q0, q1])


class _CPhaseBase(Gate):
    _slot = 3

    def __init__(self, theta: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        d = np.ones(4, dtype=complex)
        d[self._slot] = _cis(theta)
        super().__init__(np.diag(d), [q0, q1], dict(theta=theta))

    @property
    def H(self):
        return type(self)(-self.params["theta"], *self.qubits)

    def __pow__(self, t):
        return type(self)(self.params["theta"] * t, *self.qubits)


class CPHASE00(_CPhaseBase):
    _slot = 0


class CPHASE01(_CPhaseBase):
    _slot = 1


class CPHASE10(_CPhaseBase):
    _slot = 2


class CPHASE(_CPhaseBase):
    _slot = 3


class PSWAP(Gate):
    def __init__(self, theta: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        e = _cis(theta)
        super().__init__([[1, 0, 0, 0], [0, 0, e, 0], [0, e, 0, 0], [0, 0, 0, 1]], [q0, q1],
                         dict(theta=theta))

    @property
    def H(self):
        theta = self.params["theta"]
        return PSWAP(2.0 * pi - theta % (2.0 * pi), *self.qubits)


class PISWAP(Gate):
    def __init__(self, theta: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        c, s = np.cos(2 * theta), np.sin(2 * theta)
        super().__init__([[1, 0, 0, 0], [0, c, 1j * s, 0], [0, 1j * s, c, 0], [0, 0, 0, 1]], [q0, q1],
                         dict(theta=theta))

    @property
    def H(self):
        return PISWAP(-self.params["theta"], *self.qubits)

    def __pow__(self, t):
        return PISWAP(self.params["theta"] * t, *self.qubits)


class XX(Gate):
    """exp(-i pi t/2 X(x)X)."""

    def __init__(self, t: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        c, s = np.cos(pi * t / 2), np.sin(pi * t / 2)
        m = [[c, 0, 0, -1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [-1j * s, 0, 0, c]]
        super().__init__(m, [q0, q1], dict(t=t))

    @property
    def H(self):
        return XX(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return XX(self.params["t"] * t, *self.qubits)


class YY(Gate):
    """exp(-i pi t/2 Y(x)Y)."""

    def __init__(self, t: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        c, s = np.cos(pi * t / 2), np.sin(pi * t / 2)
        m = [[c, 0, 0, 1j * s], [0, c, -1j * s, 0], [0, -1j * s, c, 0], [1j * s, 0, 0, c]]
        super().__init__(m, [q0, q1], dict(t=t))

    @property
    def H(self):
        return YY(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return YY(self.params["t"] * t, *self.qubits)


class ZZ(Gate):
    """exp(-i pi t/2 Z(x)Z) = diag(e^{-i pi t/2}, e^{i pi t/2}, e^{i pi t/2}, e^{-i pi t/2})."""

    def __init__(self, t: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        th = pi * t
        super().__init__(np.diag([_cis(-th / 2), _cis(th / 2), _cis(th / 2), _cis(-th / 2)]),
                         [q0, q1], dict(t=t))

    @property
    def H(self):
        return ZZ(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return ZZ(self.params["t"] * t, *self.qubits)


class CAN(Gate):
    """Canonical gate exp(-i pi/2 (tx XX + ty YY + tz ZZ)) = ZZ(tz) YY(ty) XX(tx)."""

    def __init__(self, tx: float, ty: float, tz: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        m = ZZ(tz).asoperator() @ YY(ty).asoperator() @ XX(tx).asoperator()
        super().__init__(m, [q0, q1], dict(tx=tx, ty=ty, tz=tz))

    @property
    def H(self):
        p = self.params
        return CAN(-p["tx"], -p["ty"], -p["tz"], *self.qubits)

    def __pow__(self, t):
        p = self.params
        return CAN(p["tx"] * t, p["ty"] * t, p["tz"] * t, *self.qubits)


CANONICAL = CAN


class EXCH(Gate):
    """CAN(t, t, t)."""

    def __init__(self, t: float, q0: Qubit = 0, q1: Qubit = 1) -> None:
        super().__init__(CAN(t, t, t).tensor, [q0, q1], dict(t=t))

    @property
    def H(self):
        return EXCH(-self.params["t"], *self.qubits)

    def __pow__(self, t):
        return EXCH(self.params["t"] * t, *self.qubits)


class CCNOT(_Hermitian):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1, q2: Qubit = 2) -> None:
        m = np.eye(8)
        m[[6, 7]] = m[[7, 6]]
        super().__init__(m, [q0, q1, q2])


class CSWAP(_Hermitian):
    def __init__(self, q0: Qubit = 0, q1: Qubit = 1, q2: Qubit = 2) -> None:
        m = np.eye(8)
        m[[5, 6]] = m[[6, 5]]
        super().__init__(m, [q0, q1, q2])


GATESET = frozenset([I, X, Y, Z, H, S, T, PHASE, RX, RY, RZ, CZ, CNOT, SWAP, ISWAP, CPHASE00,
                     CPHASE01, CPHASE10, CPHASE, PSWAP, CCNOT, CSWAP, PISWAP, RN, TX, TY, TZ, TH,
                     ZYZ, CAN, XX, YY, ZZ, EXCH, S_H, T_H])
STDGATES = {cls.__name__: cls for cls in GATESET}
