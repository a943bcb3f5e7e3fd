"""Gate utilities (quantumflow/gates.py): identity, join, control, random."""
from typing import Union

import numpy as np
import scipy.stats

from .config import TOLERANCE
from .ops import Gate
from .qubits import Qubit, Qubits, outer_product, qubits_count_tuple
from .stdgates import I

__all__ = ["identity_gate", "random_gate", "join_gates", "control_gate", "conditional_gate",
           "almost_unitary", "almost_identity", "almost_hermitian", "print_gate", "P0", "P1"]


def identity_gate(qubits: Union[int, Qubits]) -> Gate:
    """quantumflow/gates.py:57-60."""
    _, qubits = qubits_count_tuple(qubits)
    return I(*qubits)


def join_gates(*gates: Gate) -> Gate:
    """Direct product of gates on disjoint qubits (quantumflow/gates.py:63-68)."""
    vec = gates[0].vec
    for g in gates[1:]:
        vec = outer_product(vec, g.vec)
    return Gate(vec.tensor, vec.qubits)


class P0(Gate):
    """Projector onto |0> (quantumflow/gates.py:131-137)."""

    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[1, 0], [0, 0]], qubits=[q0])


class P1(Gate):
    """Projector onto |1> (quantumflow/gates.py:140-147)."""

    def __init__(self, q0: Qubit = 0) -> None:
        super().__init__([[0, 0], [0, 1]], qubits=[q0])


def control_gate(control: Qubit, gate: Gate) -> Gate:
    """Controlled version of a gate (quantumflow/gates.py:71-83)."""
    if control in gate.qubits:
        raise ValueError("Gate and control qubits overlap")
    t = join_gates(P0(control), identity_gate(gate.qubits)).tensor + join_gates(P1(control), gate).tensor
    return Gate(t, qubits=[control, *gate.qubits])


def conditional_gate(control: Qubit, gate0: Gate, gate1: Gate) -> Gate:
    """quantumflow/gates.py:86-94."""
    t = join_gates(P0(control), gate0).tensor + join_gates(P1(control), gate1).tensor
    return Gate(t, qubits=[control, *gate0.qubits])


def almost_unitary(gate: Gate) -> bool:
    N = gate.qubit_nb
    m = gate.asoperator()
    return np.allclose(m @ m.conj().T, np.eye(2 ** N), atol=TOLERANCE)


def almost_identity(gate: Gate) -> bool:
    return np.allclose(gate.asoperator(), np.eye(2 ** gate.qubit_nb))


def almost_hermitian(gate: Gate) -> bool:
    m = gate.asoperator()
    return np.allclose(m, m.conj().T)


def print_gate(gate: Gate, ndigits: int = 2, file=None) -> None:
    for index, amplitude in np.ndenumerate(gate.tensor):
        ket = "".join(str(n) for n in index[0:gate.qubit_nb])
        bra = "".join(str(index[n]) for n in range(gate.qubit_nb, 2 * gate.qubit_nb))
        if round(abs(amplitude) ** 2, ndigits) > 0.0:
            print(ket, "->", bra, " : ", round(amplitude.real, ndigits) + round(amplitude.imag, ndigits) * 1j,
                  file=file)


def random_gate(qubits: Union[int, Qubits], random_state=None) -> Gate:
    """Haar-random unitary on K qubits (quantumflow/gates.py:159-168)."""
    N, qubits = qubits_count_tuple(qubits)
    unitary = scipy.stats.unitary_group.rvs(2 ** N, random_state=random_state)
    return Gate(unitary, qubits=qubits, name="RAND{}".format(N))
