"""Qubit labels and the QubitVector container.

Mirrors quantumflow/qubits.py: a tensor plus qubit labels and a rank
(1 = vector, 2 = operator).  In this backend state vectors live on the GPU
(see states.py) and operator tensors (gates) are small host arrays, so
QubitVector here holds numpy arrays for operators; states wrap it with their
own device buffer.
"""
from typing import Any, Hashable, Sequence, Tuple, Union

import numpy as np

from .config import TOLERANCE

Qubit = Hashable
Qubits = Sequence[Qubit]

__all__ = ["Qubit", "Qubits", "asarray", "QubitVector", "inner_product",
           "outer_product", "fubini_study_angle", "vectors_close", "qubits_count_tuple"]


def asarray(tensor) -> np.ndarray:
    """Backend tensor -> numpy array (quantumflow/qubits.py:39-41)."""
    if hasattr(tensor, "detach"):
        return tensor.detach().cpu().numpy()
    return np.asarray(tensor)


def qubits_count_tuple(qubits: Union[int, Qubits]) -> Tuple[int, Qubits]:
    """Unravel 'qubits: Union[int, Qubits]' (quantumflow/qubits.py:328-333)."""
    if isinstance(qubits, int):
        return qubits, tuple(range(qubits))
    return len(qubits), tuple(qubits)


class QubitVector:
    """Host tensor in product form [2]*(N*rank) with qubit labels
    (quantumflow/qubits.py:97-121)."""

    def __init__(self, tensor: Any, qubits: Qubits, rank: int = None) -> None:
        arr = np.asarray(asarray(tensor), dtype=np.complex128)
        size = arr.size
        nbits = int(round(np.log2(size))) if size > 0 else 0
        if 2 ** nbits != size:
            raise ValueError("Incompatibility between tensor and qubits")
        arr = arr.reshape([2] * nbits)
        N = len(qubits)
        if rank is None:
            rank = 1 if N == 0 else nbits // N
        if rank not in (1, 2, 4, 8) or rank * N != nbits:
            raise ValueError("Incompatibility between tensor and qubits")
        self.tensor = arr
        self.qubits = tuple(qubits)
        self.qubit_nb = N
        self.rank = rank

    def asarray(self) -> np.ndarray:
        return self.tensor

    def flatten(self) -> np.ndarray:
        """Tensor with qubit indices flattened (quantumflow/qubits.py:130-134)."""
        return self.tensor.reshape([2 ** self.qubit_nb] * self.rank)

    def relabel(self, qubits: Qubits) -> "QubitVector":
        qubits = tuple(qubits)
        assert len(qubits) == self.qubit_nb
        return QubitVector(self.tensor, qubits, self.rank)

    def permute(self, qubits: Qubits) -> "QubitVector":
        """Permute the qubit order (quantumflow/qubits.py:144-160)."""
        qubits = tuple(qubits)
        if qubits == self.qubits:
            return self
        N = self.qubit_nb
        assert len(qubits) == N
        indices = [self.qubits.index(q) for q in qubits]
        perm = []
        for rr in range(self.rank):
            perm += [rr * N + idx for idx in indices]
        return QubitVector(np.transpose(self.tensor, perm), qubits, self.rank)

    @property
    def H(self) -> "QubitVector":
        """Conjugate transpose (quantumflow/qubits.py:162-177)."""
        N, R = self.qubit_nb, self.rank
        t = self.tensor.reshape([2 ** (N * R // 2)] * 2).T.conj()
        return QubitVector(t.reshape([2] * (R * N)), self.qubits, R)

    def norm(self) -> float:
        return float(np.abs(np.vdot(self.tensor, self.tensor)))

    def trace(self) -> complex:
        """Sum of the diagonal of the (super)operator (quantumflow/qubits.py:185-197)."""
        if self.rank == 1:
            raise ValueError("Cannot take trace of vector")
        N, R = self.qubit_nb, self.rank
        return complex(np.trace(self.tensor.reshape([2 ** (N * R // 2)] * 2)))

    def partial_trace(self, qubits: Qubits) -> "QubitVector":
        """Trace over some of the qubits (quantumflow/qubits.py:201-225): the
        remaining qubits keep their order."""
        if self.rank == 1:
            raise ValueError("Cannot take trace of vector")
        N, R = self.qubit_nb, self.rank
        keep = [q for q in self.qubits if q not in set(qubits)]
        if not keep:
            raise ValueError("Cannot remove all qubits with partial_trace.")
        t = self.tensor
        # contract each traced qubit's index in every rank group with the first
        idx = [self.qubits.index(q) for q in qubits]
        letters = [chr(ord("a") + i) if i < 26 else chr(ord("A") + i - 26) for i in range(N * R)]
        for i in idx:
            for r in range(1, R):
                letters[r * N + i] = letters[i]
        out = [letters[r * N + self.qubits.index(q)] for r in range(R) for q in keep]
        res = np.einsum("".join(letters) + "->" + "".join(out), t)
        return QubitVector(res, tuple(keep), R)


def inner_product(vec0, vec1):
    """Hilbert-Schmidt inner product (quantumflow/qubits.py:227-238)."""
    if vec0.rank != vec1.rank or vec0.qubit_nb != vec1.qubit_nb:
        raise ValueError("Incompatibly vectors. Qubits and rank must match")
    vec1 = vec1.permute(vec0.qubits)
    return np.vdot(vec0.tensor, vec1.tensor)


def outer_product(vec0, vec1):
    """Direct product of operator vectors (quantumflow/qubits.py:245-277)."""
    R, N0, N1 = vec0.rank, vec0.qubit_nb, vec1.qubit_nb
    if R != vec1.rank:
        raise ValueError("Incompatibly vectors. Rank must match")
    if not set(vec0.qubits).isdisjoint(vec1.qubits):
        raise ValueError("Overlapping qubits")
    t = np.multiply.outer(vec0.tensor, vec1.tensor)
    t = t.reshape([2 ** N0] * R + [2 ** N1] * R)
    perm = [idx for ij in zip(range(R), range(R, 2 * R)) for idx in ij]
    t = np.transpose(t, perm)
    return QubitVector(t.reshape([2] * ((N0 + N1) * R)), tuple(vec0.qubits) + tuple(vec1.qubits), R)


def fubini_study_angle(vec0, vec1) -> float:
    """Fubini-Study angle (quantumflow/qubits.py:282-306)."""
    if vec0.rank != vec1.rank or vec0.qubit_nb != vec1.qubit_nb:
        raise ValueError("Incompatibly vectors. Qubits and rank must match")
    vec1 = vec1.permute(vec0.qubits)
    t0, t1 = vec0.tensor, vec1.tensor
    hs01 = np.vdot(t0, t1)
    hs00 = np.vdot(t0, t0)
    hs11 = np.vdot(t1, t1)
    ratio = np.abs(hs01) / np.sqrt(np.abs(hs00 * hs11))
    return float(np.arccos(min(ratio, 1.0)))


def vectors_close(vec0, vec1, tolerance: float = TOLERANCE) -> bool:
    """quantumflow/qubits.py:310-325."""
    if vec0.rank != vec1.rank or vec0.qubit_nb != vec1.qubit_nb:
        return False
    if set(vec0.qubits) ^ set(vec1.qubits):
        return False
    return fubini_study_angle(vec0, vec1) <= tolerance
