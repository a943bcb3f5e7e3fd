"""Measures on states and gates (quantumflow/measures.py:32-53 and the gate
measures it defines).  State measures reduce on the GPU (qf_inner)."""
import numpy as np

from .config import TOLERANCE
from .ops import Gate
from .qubits import fubini_study_angle, vectors_close
from .states import State, inner

__all__ = ["state_fidelity", "state_angle", "states_close", "gate_angle", "gates_close",
           "max_amplitude_error"]


def state_fidelity(state0: State, state1: State) -> float:
    """|<psi0|psi1>|^2 (quantumflow/measures.py:32-36)."""
    assert state0.qubits == state1.qubits
    return abs(inner(state0, state1)) ** 2


def state_angle(ket0: State, ket1: State) -> float:
    """Fubini-Study angle between states (quantumflow/measures.py:39-44)."""
    if ket0.qubit_nb != ket1.qubit_nb or set(ket0.qubits) ^ set(ket1.qubits):
        raise ValueError("Incompatibly vectors. Qubits and rank must match")
    ket1 = ket1.permute(ket0.qubits)
    h01 = inner(ket0, ket1)
    h00 = ket0.norm()
    h11 = ket1.norm()
    ratio = min(abs(h01) / np.sqrt(abs(h00 * h11)), 1.0)
    return float(np.arccos(ratio))


def states_close(state0: State, state1: State, tolerance: float = TOLERANCE) -> bool:
    """quantumflow/measures.py:47-53."""
    if state0.qubit_nb != state1.qubit_nb or set(state0.qubits) ^ set(state1.qubits):
        return False
    return state_angle(state0, state1) <= tolerance


def max_amplitude_error(state: State, reference) -> float:
    """max_x |psi_x - ref_x| against a host array in the same qubit order."""
    ref = np.asarray(reference).reshape(-1)
    return float(np.max(np.abs(state.asarray().reshape(-1) - ref)))


def gate_angle(gate0: Gate, gate1: Gate) -> float:
    """Fubini-Study angle between gates (quantumflow/measures.py gate_angle)."""
    return fubini_study_angle(gate0.vec, gate1.vec)


def gates_close(gate0: Gate, gate1: Gate, tolerance: float = TOLERANCE) -> bool:
    """quantumflow/measures.py gates_close."""
    return vectors_close(gate0.vec, gate1.vec, tolerance)
