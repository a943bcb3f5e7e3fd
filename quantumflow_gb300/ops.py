"""Operations on states: Operation and Gate (quantumflow/ops.py:35-262).

A Gate holds its matrix on the host (a [2]*2K complex128 numpy tensor: at
most a few KiB).  ``Gate.run`` applies it to a device State through
``qf_apply_gate`` -- the GPU replacement of the reference's
``bk.tensormul`` call at quantumflow/ops.py:161-166.
"""
import copy
from abc import ABC
from typing import Any, Dict

import numpy as np
import torch

from . import _native as nat
from .qubits import Qubits, QubitVector, asarray
from .states import State, gate_layout

__all__ = ["Operation", "Gate"]


class Operation(ABC):
    """An operation on a qubit state (quantumflow/ops.py:35-88)."""

    _qubits: Qubits = ()

    @property
    def qubits(self) -> Qubits:
        return self._qubits

    @property
    def qubit_nb(self) -> int:
        return len(self.qubits)

    @property
    def name(self) -> str:
        return self.__class__.__name__.upper()

    def run(self, ket: State) -> State:
        raise NotImplementedError()

    def evolve(self, rho):
        """Apply this operation to a density matrix (quantumflow/ops.py:62-64)."""
        raise NotImplementedError()

    def asgate(self) -> "Gate":
        raise NotImplementedError()

    def aschannel(self):
        raise NotImplementedError()

    @property
    def H(self) -> "Operation":
        raise NotImplementedError()

    def quil(self) -> str:
        return self.name

    def __str__(self) -> str:
        return self.quil()


class Gate(Operation):
    """A quantum logic gate (quantumflow/ops.py:91-262)."""

    def __init__(self, tensor: Any, qubits: Qubits = None, params: Dict[str, float] = None,
                 name: str = None) -> None:
        arr = np.asarray(asarray(tensor), dtype=np.complex128)
        if qubits is None:
            nbits = int(round(np.log2(arr.size)))
            qubits = range(nbits // 2)
        self.vec = QubitVector(arr, qubits)
        if self.vec.rank != 2:
            raise ValueError("Incompatibility between tensor and qubits")
        self.params = params if params is not None else {}
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

    def relabel(self, qubits: Qubits) -> "Gate":
        gate = copy.copy(self)
        gate.vec = gate.vec.relabel(qubits)
        return gate

    def permute(self, qubits: Qubits) -> "Gate":
        vec = self.vec.permute(qubits)
        return Gate(vec.tensor, qubits=vec.qubits)

    @property
    def H(self) -> "Gate":
        return Gate(tensor=self.vec.H.tensor, qubits=self.qubits)

    def asoperator(self) -> np.ndarray:
        """The gate as a (2^K, 2^K) matrix."""
        return self.vec.flatten()

    def matrix_doubles(self) -> np.ndarray:
        """Row-major interleaved (re, im) doubles of the operator (the C ABI
        gate-matrix format)."""
        m = np.ascontiguousarray(self.asoperator(), dtype=np.complex128)
        return m.view(np.float64).reshape(-1)

    def run(self, ket: State) -> State:
        """Apply this gate to a state (quantumflow/ops.py:161-166)."""
        indices = [ket.qubits.index(q) for q in self.qubits]
        src = ket.buffer.compute()
        out = src.empty_like()
        k = len(indices)
        if k > nat.MAX_GATE_QUBITS:
            # wide dense gate: the matrix goes to the device (it does not fit
            # the kernel parameters of qf_apply_gate)
            dmat = torch.from_numpy(np.ascontiguousarray(self.asoperator(), dtype=np.complex128)).to(src.device)
            nat.call("qf_apply_dense_gate", nat.ptr(src.data), nat.ptr(out.data), src.n, gate_layout(src), k,
                     nat.int_array(indices), nat.ptr(dmat), nat.stream_handle(src.device))
            return State(out, ket.qubits, ket._memory)
        mat = np.ascontiguousarray(self.matrix_doubles())
        nat.call("qf_apply_gate", nat.ptr(src.data), nat.ptr(out.data), src.n, gate_layout(src), k,
                 nat.int_array(indices), mat.ctypes.data_as(nat._dp), nat.stream_handle(src.device))
        return State(out, ket.qubits, ket._memory)

    def __pow__(self, t: float) -> "Gate":
        """Matrix power (quantumflow/ops.py:175-184)."""
        from scipy.linalg import fractional_matrix_power
        N = self.qubit_nb
        m = fractional_matrix_power(self.asoperator(), t)
        return Gate(np.reshape(m, [2] * (2 * N)), self.qubits)

    def __matmul__(self, other: "Gate") -> "Gate":
        """Apply this gate to another gate (quantumflow/ops.py:187-198); the
        other gate's qubits must contain this gate's."""
        if not isinstance(other, Gate):
            raise NotImplementedError()
        indices = [other.qubits.index(q) for q in self.qubits]
        K = self.qubit_nb
        N = 2 * other.qubit_nb
        A = self.tensor
        B = other.tensor
        # contract A's bra axes with B's axes `indices`; write ket axes back
        Bm = np.moveaxis(B, indices, list(range(K))).reshape(2 ** K, -1)
        Cm = A.reshape(2 ** K, 2 ** K) @ Bm
        C = np.moveaxis(Cm.reshape([2] * N), list(range(K)), indices)
        return Gate(tensor=C, qubits=other.qubits)

    def asgate(self) -> "Gate":
        return self

    def evolve(self, rho):
        """Apply to a density matrix (quantumflow/ops.py:168-172): U on the
        ket axes and conj(U) on the bra axes, one fused launch."""
        from .densities import evolve_gates
        return evolve_gates(rho, [self])

    def aschannel(self):
        """The gate's superoperator (quantumflow/ops.py:244-253)."""
        from .channels import gate_aschannel
        return gate_aschannel(self)

    def su(self) -> "Gate":
        rank = 2 ** self.qubit_nb
        U = self.asoperator().copy()
        U /= np.linalg.det(U) ** (1 / rank)
        return Gate(tensor=U, qubits=self.qubits)

    def quil(self) -> str:
        if self.name == "Gate":
            return super().__repr__()
        fqubits = " " + " ".join(str(q) for q in self.qubits)
        fparams = ""
        if self.params:
            fparams = "(" + ", ".join(str(p) for p in self.params.values()) + ")"
        return f"{self.name}{fparams}{fqubits}"

    def __str__(self) -> str:
        return self.quil()
