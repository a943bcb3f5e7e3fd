"""Measures on states, densities, gates and channels
(quantumflow/measures.py:32-213).  State measures reduce on the GPU
(qf_inner); density purity is a GPU norm of the 2N-qubit buffer; the
spectral measures (fidelity, entropy) diagonalise small host matrices as
the reference does."""
import numpy as np
import scipy.linalg
import scipy.stats

from .config import TOLERANCE
from .ops import Gate
from .qubits import fubini_study_angle, vectors_close
from .states import State, inner

__all__ = ["state_fidelity", "state_angle", "states_close", "gate_angle", "gates_close",
           "max_amplitude_error", "purity", "fidelity", "bures_distance", "bures_angle", "density_angle",
           "densities_close", "entropy", "mutual_info", "channel_angle", "channels_close", "diamond_norm"]


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


# ----------------------------------------------------- density matrices ----
def purity(rho) -> float:
    """tr(rho^2) (quantumflow/measures.py:59-73); for Hermitian rho this is
    sum |rho_ij|^2, one reduction over the density's buffer."""
    return float(rho.norm())


def fidelity(rho0, rho1) -> float:
    """(tr sqrt(sqrt(rho0) rho1 sqrt(rho0)))^2, clipped to [0, 1]
    (quantumflow/measures.py:76-92)."""
    assert rho0.qubit_nb == rho1.qubit_nb
    rho1 = rho1.permute(rho0.qubits)
    op0 = rho0.asoperator().cpu().numpy()
    op1 = rho1.asoperator().cpu().numpy()
    s0 = scipy.linalg.sqrtm(op0)
    fid = np.real(np.trace(scipy.linalg.sqrtm(s0 @ op1 @ s0)) ** 2)
    return float(min(max(fid, 0.0), 1.0))


def bures_distance(rho0, rho1) -> float:
    """quantumflow/measures.py:95-107."""
    fid = fidelity(rho0, rho1)
    tr0 = np.trace(rho0.asoperator().cpu().numpy())
    tr1 = np.trace(rho1.asoperator().cpu().numpy())
    return np.sqrt(tr0 + tr1 - 2.0 * np.sqrt(fid))


def bures_angle(rho0, rho1) -> float:
    """quantumflow/measures.py:110-115."""
    return float(np.arccos(np.sqrt(fidelity(rho0, rho1))))


def density_angle(rho0, rho1) -> float:
    """Fubini-Study angle between densities (quantumflow/measures.py:118-120)."""
    return fubini_study_angle(rho0.vec, rho1.vec)


def densities_close(rho0, rho1, tolerance: float = TOLERANCE) -> bool:
    """quantumflow/measures.py:123-130."""
    return vectors_close(rho0.vec, rho1.vec, tolerance)


def entropy(rho, base: float = None) -> float:
    """von Neumann entropy from the eigenvalues (quantumflow/measures.py:133-149)."""
    probs = np.maximum(np.linalg.eigvalsh(rho.asoperator().cpu().numpy()), 0.0)
    return float(scipy.stats.entropy(probs, base=base))


def mutual_info(rho, qubits0, qubits1=None, base: float = None) -> float:
    """Bipartite mutual information (quantumflow/measures.py:152-180)."""
    if qubits1 is None:
        qubits1 = tuple(set(rho.qubits) - set(qubits0))
    rho0 = rho.partial_trace(qubits1)
    rho1 = rho.partial_trace(qubits0)
    return entropy(rho0, base) + entropy(rho1, base) - entropy(rho, base)


# -------------------------------------------------------------- channels ----
def channel_angle(chan0, chan1) -> float:
    """quantumflow/measures.py:199-201."""
    return fubini_study_angle(chan0.vec, chan1.vec)


def channels_close(chan0, chan1, tolerance: float = TOLERANCE) -> bool:
    """quantumflow/measures.py:204-210."""
    return vectors_close(chan0.vec, chan1.vec, tolerance)


def diamond_norm(chan0, chan1) -> float:
    """The reference solves a semidefinite program with cvxpy
    (quantumflow/measures.py:213-264); cvxpy is not available here."""
    raise NotImplementedError("diamond_norm needs a semidefinite-program solver (cvxpy), not installed")
