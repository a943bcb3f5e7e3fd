"""Density matrices on the GPU (quantumflow/states.py:264-357).

A :class:`Density` on N qubits is held as a 2N-qubit amplitude buffer in the
same element layouts as state vectors: axes 0..N-1 are the ket (row) indices
and axes N..2N-1 the bra (column) indices of rho, the reference's
``[2] * 2N`` tensor format.  Evolution therefore runs on the state-vector
kernels: a gate U is U on the ket axes and conj(U) on the bra axes (one
fused circuit launch), and a k-qubit channel is its superoperator applied as
one 2k-qubit gate on the ket and bra axes of its qubits (``qf_apply_gate``).
"""
import math
from collections import ChainMap
from functools import reduce
from typing import Any, Dict, Sequence, Union

import numpy as np
import torch

from . import _native as nat
from .qubits import Qubits, outer_product, qubits_count_tuple, QubitVector
from .states import Buffer, State, _DTYPES, _as_complex_tensor, _device, compute_layout, gate_layout

__all__ = ["Density", "mixed_density", "random_density", "join_densities"]


class Density(State):
    """A mixed state (quantumflow/states.py:264-319)."""

    def __init__(self, tensor: Any, qubits: Qubits = None, memory: Dict = None, *, dtype=None) -> None:
        if isinstance(tensor, Buffer):
            buf = tensor
        else:
            buf = Buffer.from_complex(_as_complex_tensor(tensor, dtype))
        if buf.n % 2:
            raise ValueError("Incompatibility between tensor and qubits")
        N = buf.n // 2
        qubits = tuple(range(N)) if qubits is None else tuple(qubits)
        if len(qubits) != N:
            raise ValueError("Incompatibility between tensor and qubits")
        self._buf = buf
        self._qubits = qubits
        self._memory = memory if memory is not None else {}

    # -- reference API ---------------------------------------------------
    @property
    def tensor(self) -> torch.Tensor:
        return self._buf.complex().reshape([2] * self._buf.n)

    @property
    def vec(self) -> QubitVector:
        return QubitVector(self.asarray(), self.qubits, 2)

    def matrix(self) -> torch.Tensor:
        M = 2 ** self.qubit_nb
        return self._buf.complex().reshape(M, M)

    def trace(self) -> complex:
        """Sum of the diagonal (quantumflow/states.py:277-279)."""
        return complex(torch.diagonal(self.matrix()).sum().item())

    def partial_trace(self, qubits: Qubits) -> "Density":
        """Trace out ``qubits`` (quantumflow/states.py:282-286)."""
        N = self.qubit_nb
        traced = set(qubits)
        keep = [q for q in self.qubits if q not in traced]
        if not keep:
            raise ValueError("Cannot remove all qubits with partial_trace.")
        letters = [chr(ord("a") + i) for i in range(2 * N)]
        for q in qubits:
            i = self.qubits.index(q)
            letters[N + i] = letters[i]
        out = [letters[self.qubits.index(q)] for q in keep] + [letters[N + self.qubits.index(q)] for q in keep]
        t = torch.einsum("".join(letters) + "->" + "".join(out), self.tensor)
        return Density(t.contiguous(), keep, self._memory)

    def relabel(self, qubits: Qubits) -> "Density":
        return Density(self._buf, qubits, self._memory)

    def permute(self, qubits: Qubits) -> "Density":
        qubits = tuple(qubits)
        if qubits == self.qubits:
            return self
        N = self.qubit_nb
        idx = [self.qubits.index(q) for q in qubits]
        t = self.tensor.permute(idx + [N + i for i in idx]).contiguous()
        return Density(t, qubits, self._memory)

    def normalize(self) -> "Density":
        """rho / trace(rho) (quantumflow/states.py:294-297)."""
        src = self._buf.compute()
        out = src.empty_like()
        out.data.copy_(src.data)
        nat.call("qf_scale", nat.ptr(out.data), out.n, out.layout, 1.0 / self.trace().real,
                 nat.stream_handle(out.device))
        return Density(out, self.qubits, self._memory)

    def probabilities(self) -> torch.Tensor:
        """Diagonal of rho as a [2]*N float64 tensor (quantumflow/states.py:300-304)."""
        return torch.diagonal(self.matrix()).real.to(torch.float64).reshape([2] * self.qubit_nb)

    def asoperator(self) -> torch.Tensor:
        return self.matrix()

    def asdensity(self) -> "Density":
        return self

    def update(self, memory: Dict) -> "Density":
        mem = self.memory
        mem.update(memory)
        return Density(self._buf, self.qubits, mem)

    def expectation(self, diag_hermitian: Any, trials: int = None) -> float:
        """sum_x h_x rho_xx."""
        h = torch.as_tensor(np.real(np.asarray(diag_hermitian)), dtype=torch.float64,
                            device=self._buf.device).reshape(-1)
        return float((self.probabilities().reshape(-1) * h).sum().item())


# -------------------------------------------------------------- evolution --
def evolve_gates(rho: Density, gates) -> Density:
    """Apply gates to rho: U on the ket axes and conj(U) on the bra axes of
    every gate, as one fused circuit launch on the 2N-qubit buffer."""
    N = rho.qubit_nb
    ks, axes, mats = [], [], []
    for g in gates:
        idx = [rho.qubits.index(q) for q in g.qubits]
        u = np.ascontiguousarray(g.asoperator(), dtype=np.complex128)
        ks += [len(idx), len(idx)]
        axes += idx + [N + i for i in idx]
        mats += [u.view(np.float64).reshape(-1), np.conj(u).view(np.float64).reshape(-1)]
    if not ks:
        return rho
    src = rho.buffer.compute()
    out = src.empty_like()
    op_k = np.asarray(ks, dtype=np.int32)
    op_axes = np.asarray(axes, dtype=np.int32)
    op_mats = np.ascontiguousarray(np.concatenate(mats))
    passes = (nat.ctypes.c_int * 1)()
    nat.call("qf_run_circuit", nat.ptr(src.data), nat.ptr(out.data), src.n, gate_layout(src), len(ks),
             op_k.ctypes.data_as(nat._ip), op_axes.ctypes.data_as(nat._ip), op_mats.ctypes.data_as(nat._dp),
             0, passes, nat.stream_handle(src.device))
    return Density(out, rho.qubits, rho._memory)


def evolve_superop(rho: Density, superop: np.ndarray, qubits: Qubits) -> Density:
    """Apply a k-qubit superoperator (a (4^k, 4^k) matrix: rows ket-out then
    bra-out bits, columns ket-in then bra-in) as one 2k-qubit gate."""
    k = len(qubits)
    if 2 * k > 5:
        return _evolve_by_choi(rho, superop, qubits)
    N = rho.qubit_nb
    idx = [rho.qubits.index(q) for q in qubits]
    axes = idx + [N + i for i in idx]
    m = np.ascontiguousarray(np.asarray(superop, dtype=np.complex128).reshape(4 ** k, 4 ** k))
    src = rho.buffer.compute()
    out = src.empty_like()
    nat.call("qf_apply_gate", nat.ptr(src.data), nat.ptr(out.data), src.n, gate_layout(src), 2 * k,
             nat.int_array(axes), m.view(np.float64).reshape(-1).ctypes.data_as(nat._dp),
             nat.stream_handle(src.device))
    return Density(out, rho.qubits, rho._memory)


def _evolve_by_choi(rho: Density, superop: np.ndarray, qubits: Qubits) -> Density:
    """Channels on three or more qubits (whose 2k-qubit superoperator is above
    the engine's 5-qubit dense gates): the Choi matrix's eigen-decomposition
    gives sum_i l_i K_i (.) K_i^dagger (K_i = the i-th eigenvector as a
    2^k x 2^k matrix, the reshaping of quantumflow/channels.py:181-203), and
    every term is one k-qubit gate pair on the density's ket and bra axes."""
    from .ops import Gate
    k = len(qubits)
    d = 2 ** k
    choi = np.asarray(superop).reshape([d] * 4).transpose(0, 2, 1, 3).reshape(d * d, d * d)
    if not np.allclose(choi, choi.conj().T, atol=1e-10):
        raise ValueError("channel does not preserve Hermiticity")
    evals, evecs = np.linalg.eigh(choi)
    acc = None
    for lam, vec in zip(evals, evecs.T):
        if abs(lam) < 1e-14:
            continue
        term = evolve_gates(rho, [Gate(vec.reshape(d, d), qubits=qubits)])
        t = term.buffer.complex().to(torch.complex128) * float(lam)
        acc = t if acc is None else acc + t
    if acc is None:
        acc = torch.zeros(2 ** rho.buffer.n, dtype=torch.complex128, device=rho.buffer.device)
    out = Density(acc.reshape([2] * rho.buffer.n), rho.qubits, rho._memory)
    return out if rho.dtype == "complex128" else Density(acc.to(torch.complex64).reshape([2] * rho.buffer.n),
                                                         rho.qubits, rho._memory)


# ----------------------------------------------------------- constructors --
def mixed_density(qubits: Union[int, Qubits], dtype: str = "complex128") -> Density:
    """The completely mixed state I / 2^N (quantumflow/states.py:322-326)."""
    N, qubits = qubits_count_tuple(qubits)
    m = torch.eye(2 ** N, dtype=_DTYPES[dtype], device=_device()) / 2 ** N
    return Density(m, qubits)


def random_density(qubits: Union[int, Qubits], dtype: str = "complex128") -> Density:
    """A Hilbert-Schmidt random density matrix: G G^dagger / tr, G Ginibre
    (quantumflow/states.py:329-346; numpy's global generator, as there)."""
    N, qubits = qubits_count_tuple(qubits)
    size = (2 ** N, 2 ** N)
    g = (np.random.normal(size=size) + 1j * np.random.normal(size=size)) / np.sqrt(2.0)
    m = g @ np.conj(g).T
    m /= np.trace(m)
    return Density(m.astype(np.complex64 if dtype == "complex64" else np.complex128), qubits)


def join_densities(*densities: Density) -> Density:
    """Tensor product of densities on disjoint qubits (quantumflow/states.py:349-355)."""
    vec = reduce(outer_product, [rho.vec for rho in densities])
    memory = dict(ChainMap(*[rho.memory for rho in densities]))
    return Density(vec.tensor, vec.qubits, memory)


def asdensity(state: State) -> Density:
    """|psi><psi| (quantumflow/states.py:162-165), formed on the device."""
    t = state.buffer.complex().reshape(-1)
    return Density(torch.outer(t, t.conj()).contiguous(), state.qubits, state._memory)
