"""Quantum channels (quantumflow/ops.py:265-420 ``Channel``,
quantumflow/channels.py:37-223 Kraus and the standard noise channels).

A channel is held on the host as its superoperator tensor in the
reference's format (``[2] * 4k``: ket-out, bra-out, ket-in, bra-in index
groups); channels are small (k <= 2 on the GPU engine), so algebra on them
(composition, sums, Kraus <-> superoperator conversion) stays in numpy.
Their action on a density matrix runs on the GPU: ``evolve`` applies the
superoperator as one 2k-qubit gate to the density's 2N-qubit buffer.
"""
from functools import reduce
from operator import add
from typing import Any, Dict, Sequence, Union

import numpy as np

from .densities import Density, evolve_superop
from .ops import Gate, Operation
from .qubits import Qubit, Qubits, QubitVector, asarray, outer_product, qubits_count_tuple
from .states import State
from .stdgates import I, X, Y, Z

__all__ = ["Channel", "Kraus", "UnitaryMixture", "Depolarizing", "Damping", "Dephasing",
           "join_channels", "channel_to_kraus", "kraus_iscomplete"]


def _host_tensormul(tensor0: np.ndarray, tensor1: np.ndarray, indices: Sequence[int]) -> np.ndarray:
    """The gate-contraction of quantumflow/backend/numpybk.py:159-214 on host
    arrays: tensor0 is a K-axis-pair operator applied to the given axes of
    tensor1 (used for channel algebra only, never for states)."""
    K = len(indices)
    N = tensor1.ndim
    g = np.asarray(tensor0).reshape([2] * (2 * K))
    letters = [chr(ord("a") + i) for i in range(N)]
    outs = [chr(ord("A") + i) for i in range(K)]
    gate_sub = "".join(outs) + "".join(letters[i] for i in indices)
    res = list(letters)
    for k, i in enumerate(indices):
        res[i] = outs[k]
    return np.einsum(f"{gate_sub},{''.join(letters)}->{''.join(res)}", g, tensor1)


class Channel(Operation):
    """A channel as its superoperator (quantumflow/ops.py:265-420)."""

    def __init__(self, tensor: Any, qubits: Union[int, Qubits], params: Dict[str, Any] = None,
                 name: str = None) -> None:
        _, qubits = qubits_count_tuple(qubits)
        self.vec = QubitVector(tensor, qubits, 4)
        self.params = params
        self._name = name if name is not None else self.__class__.__name__

    @property
    def name(self) -> str:
        return self._name

    @property
    def tensor(self) -> np.ndarray:
        return self.vec.tensor

    @property
    def qubits(self) -> Qubits:
        return self.vec.qubits

    @property
    def qubit_nb(self) -> int:
        return self.vec.qubit_nb

    def relabel(self, qubits: Qubits) -> "Channel":
        return Channel(self.tensor, qubits, self.params, self._name)

    def permute(self, qubits: Qubits) -> "Channel":
        vec = self.vec.permute(qubits)
        return Channel(vec.tensor, vec.qubits)

    @property
    def H(self) -> "Channel":
        return Channel(self.vec.H.tensor, self.qubits)

    @property
    def sharp(self) -> "Channel":
        """Swap the two bra-side super-indices (quantumflow/ops.py:310-332)."""
        N = self.qubit_nb
        t = self.tensor.reshape([2 ** N] * 4).transpose(0, 2, 1, 3)
        return Channel(t.reshape([2] * 4 * N), self.qubits)

    def choi(self) -> np.ndarray:
        """Choi matrix (quantumflow/ops.py:334-339)."""
        N = self.qubit_nb
        return self.sharp.tensor.reshape([2 ** (N * 2)] * 2)

    def chi(self) -> np.ndarray:
        N = self.qubit_nb
        return self.sharp.tensor.reshape([2 ** (N * 2)] * 2)

    def run(self, ket: State) -> State:
        raise TypeError()  # not possible in general

    def evolve(self, rho: Density) -> Density:
        """Apply to a density matrix (quantumflow/ops.py:354-363): one
        2k-qubit gate on the ket and bra axes of the channel's qubits."""
        k = self.qubit_nb
        return evolve_superop(rho, self.tensor.reshape(4 ** k, 4 ** k), self.qubits)

    def asgate(self) -> Gate:
        raise TypeError()  # not possible in general

    def aschannel(self) -> "Channel":
        return self

    def __add__(self, other: Any) -> "Channel":
        if isinstance(other, Channel):
            if not self.qubits == other.qubits:
                raise ValueError("Qubits must be identical")
            return Channel(self.tensor + other.tensor, self.qubits)
        raise NotImplementedError()

    def __mul__(self, other: Any) -> "Channel":
        return Channel(self.tensor * other, self.qubits)

    def __matmul__(self, other: "Channel") -> "Channel":
        """Compose: apply ``other`` then ``self`` (quantumflow/ops.py:383-397)."""
        if not isinstance(other, Channel):
            raise NotImplementedError()
        N = other.qubit_nb
        indices = [other.qubits.index(q) for q in self.qubits] + [other.qubits.index(q) + N for q in self.qubits]
        return Channel(_host_tensormul(self.tensor, other.tensor, indices), other.qubits)

    def trace(self) -> complex:
        return self.vec.trace()

    def partial_trace(self, qubits: Qubits) -> "Channel":
        vec = self.vec.partial_trace(qubits)
        return Channel(vec.tensor, vec.qubits)


def gate_aschannel(gate: Gate) -> Channel:
    """Superoperator of U: outer(U, U^dagger) with its index groups
    reordered to (ket-out, bra-out, ket-in, bra-in) (quantumflow/ops.py:244-253)."""
    N = gate.qubit_nb
    u = gate.asoperator()
    t = np.multiply.outer(u, np.conj(u).T).reshape([2 ** N] * 4).transpose(0, 3, 1, 2)
    return Channel(t.reshape([2] * 4 * N), gate.qubits)


class Kraus(Operation):
    """Operator-sum representation (quantumflow/channels.py:37-107)."""

    def __init__(self, operators: Sequence[Gate], weights: Sequence[float] = None) -> None:
        self.operators = list(operators)
        self.weights = tuple(weights) if weights is not None else tuple([1.0] * len(self.operators))

    def asgate(self) -> Gate:
        raise TypeError("Not possible in general")

    def aschannel(self) -> Channel:
        """sum_k w_k K_k (.) K_k^dagger as one superoperator."""
        qubits = self.qubits
        N = len(qubits)
        ident = gate_aschannel(Gate(np.eye(2 ** N), qubits=qubits))
        chans = [gate_aschannel(op) @ ident for op in self.operators]
        chans = [c * w for c, w in zip(chans, self.weights)]
        return reduce(add, chans)

    def run(self, ket: State) -> State:
        """One Kraus operator at random, weighted by w_k |K_k psi|^2, then
        normalised (quantumflow/channels.py:70-77)."""
        res = [op.run(ket) for op in self.operators]
        probs = np.asarray([r.norm() * w for r, w in zip(res, self.weights)])
        probs /= np.sum(probs)
        pick = np.random.choice(len(res), p=probs)
        return res[pick].normalize()

    def evolve(self, rho: Density) -> Density:
        """On the GPU as one superoperator pass (equal to the reference's
        sum of per-operator evolutions, quantumflow/channels.py:79-85)."""
        return self.aschannel().evolve(rho)

    @property
    def qubits(self) -> Qubits:
        qbs = sorted({q for op in self.operators for q in op.qubits})
        return tuple(qbs)

    @property
    def H(self) -> "Kraus":
        return Kraus([op.H for op in self.operators], self.weights)


class UnitaryMixture(Kraus):
    """A convex mixture of unitaries (quantumflow/channels.py:111-125)."""

    def asgate(self) -> Gate:
        return self.operators[np.random.choice(len(self.operators), p=self.weights)]

    def run(self, ket: State) -> State:
        return self.asgate().run(ket)


class Depolarizing(UnitaryMixture):
    """One-qubit depolarizing channel (quantumflow/channels.py:128-138)."""

    def __init__(self, prob: float, q0: Qubit) -> None:
        super().__init__([I(q0), X(q0), Y(q0), Z(q0)], [1 - prob, prob / 3.0, prob / 3.0, prob / 3.0])


class Damping(Kraus):
    """Amplitude damping on one qubit (quantumflow/channels.py:141-153)."""

    def __init__(self, prob: float, q0: Qubit) -> None:
        k0 = Gate([[1.0, 0.0], [0.0, np.sqrt(1 - prob)]], qubits=[q0])
        k1 = Gate([[0.0, np.sqrt(prob)], [0.0, 0.0]], qubits=[q0])
        super().__init__([k0, k1])


class Dephasing(UnitaryMixture):
    """Phase damping on one qubit (quantumflow/channels.py:156-166)."""

    def __init__(self, prob: float, q0: Qubit) -> None:
        super().__init__([I(q0), Z(q0)], [1 - prob / 2, prob / 2])


def join_channels(*channels: Channel) -> Channel:
    """Tensor product of channels on disjoint qubits (quantumflow/channels.py:170-175)."""
    vec = reduce(outer_product, [c.vec for c in channels])
    return Channel(vec.tensor, vec.qubits)


def channel_to_kraus(chan: Channel) -> Kraus:
    """Kraus operators from the Choi matrix's eigen-decomposition
    (quantumflow/channels.py:181-203)."""
    qubits = chan.qubits
    N = chan.qubit_nb
    evals, evecs = np.linalg.eig(asarray(chan.choi()))
    evecs = np.transpose(evecs)
    if not np.allclose(evals.imag, 0.0) or not np.all(evals.real >= -1e-12):
        raise ValueError("not a completely positive map")
    values = np.sqrt(np.maximum(evals.real, 0.0))
    ops = [Gate(np.reshape(evecs[i], (2 ** N, 2 ** N)) * values[i], qubits)
           for i in range(2 ** (2 * N)) if not np.isclose(values[i], 0.0)]
    return Kraus(ops)


def kraus_iscomplete(kraus: Kraus) -> bool:
    """sum_k w_k K_k^dagger K_k == I (quantumflow/channels.py:207-222)."""
    qubits = kraus.qubits
    N = len(qubits)
    total = np.zeros((2 ** N, 2 ** N), dtype=np.complex128)
    for op, w in zip(kraus.operators, kraus.weights):
        full = Gate(np.eye(2 ** N), qubits=qubits)
        m = (op.H @ (op @ full)).asoperator()
        total += w * m
    return bool(np.allclose(total, np.eye(2 ** N)))
