"""Circuits (quantumflow/circuits.py:35-138).

``Circuit.run`` hands the whole gate list to ``qf_run_circuit`` in one call;
the native planner fuses consecutive gates into blocks and sweeps the state
once per block instead of once per gate (the reference loops
``ket = elem.run(ket)`` at quantumflow/circuits.py:97-98).
"""
from typing import Iterable, Iterator

import numpy as np

from . import _native as nat
from . import config
from .gates import identity_gate
from .ops import Gate, Operation
from .qubits import Qubits
from .states import Buffer, State, compute_layout, gate_layout, zero_state

__all__ = ["Circuit", "count_operations", "map_gate", "reversal_circuit", "qft_circuit", "control_circuit",
           "ccnot_circuit", "zyz_circuit", "phase_estimation_circuit", "addition_circuit", "ghz_circuit"]


class Circuit(Operation):
    """A sequence of operations (quantumflow/circuits.py:35-138)."""

    def __init__(self, elements: Iterable[Operation] = None) -> None:
        self.elements = list(elements) if elements is not None else []
        self._pack_key = None
        self._pack = None

    def add(self, other: "Circuit") -> "Circuit":
        return Circuit(self.elements + other.elements)

    def extend(self, other: Operation) -> None:
        if isinstance(other, Circuit):
            self.elements.extend(other.elements)
        else:
            self.elements.append(other)

    def __add__(self, other: "Circuit") -> "Circuit":
        return self.add(other)

    def __iadd__(self, other: Operation) -> "Circuit":
        self.extend(other)
        return self

    def __iter__(self) -> Iterator[Operation]:
        return self.elements.__iter__()

    def size(self) -> int:
        return len(self.elements)

    @property
    def qubits(self) -> Qubits:
        """Sorted union of element qubits (quantumflow/circuits.py:75-85)."""
        qbs = [q for elem in self.elements for q in elem.qubits]
        return tuple(sorted(set(qbs)))

    def gates(self):
        """Flattened gate list (nested circuits expanded)."""
        out = []
        for e in self.elements:
            if isinstance(e, Circuit):
                out.extend(e.gates())
            else:
                out.append(e)
        return out

    def packed(self, qubits: Qubits):
        """(op_k, op_axes, op_mats) arrays of the C ABI for a state on `qubits`."""
        flat = self.gates()
        key = (tuple(qubits), tuple(id(g) for g in flat))
        if key == self._pack_key:
            return self._pack
        index = {q: i for i, q in enumerate(qubits)}
        ks, axes, mats = [], [], []
        for g in flat:
            if not isinstance(g, Gate):
                raise TypeError(f"{type(g).__name__} cannot run inside a fused circuit")
            ks.append(g.qubit_nb)
            axes.extend(index[q] for q in g.qubits)
            mats.append(g.matrix_doubles())
        op_k = np.asarray(ks, dtype=np.int32)
        op_axes = np.asarray(axes, dtype=np.int32)
        op_mats = np.ascontiguousarray(np.concatenate(mats) if mats else np.zeros(1))
        self._pack_key, self._pack = key, (op_k, op_axes, op_mats, len(flat))
        return self._pack

    def run(self, ket: State = None, fusion_k: int = None) -> State:
        """Apply the circuit (quantumflow/circuits.py:87-99); default initial
        state |0...0> on the sorted circuit qubits."""
        fusion_k = config.FUSION_K if fusion_k is None else fusion_k
        fresh = ket is None
        if fresh:
            ket = zero_state(self.qubits)
        flat = self.gates()
        if any(not isinstance(g, Gate) or g.qubit_nb > nat.MAX_GATE_QUBITS for g in flat):
            # mixed operations: each run of consecutive gates is one fused
            # launch, other operations (and gates wider than the fused
            # engine takes) run on their own in between
            pending = []
            for elem in flat:
                if isinstance(elem, Gate) and elem.qubit_nb <= nat.MAX_GATE_QUBITS:
                    pending.append(elem)
                    continue
                if pending:
                    ket = Circuit(pending).run(ket, fusion_k)
                    pending = []
                ket = elem.run(ket)
            if pending:
                ket = Circuit(pending).run(ket, fusion_k)
            return ket
        op_k, op_axes, op_mats, nops = self.packed(ket.qubits)
        src = ket.buffer.compute()
        out = src if (fresh or src is not ket.buffer) else src.empty_like()
        passes = (nat.ctypes.c_int * 1)()
        nat.call("qf_run_circuit", nat.ptr(src.data), nat.ptr(out.data), src.n, gate_layout(src), nops,
                 op_k.ctypes.data_as(nat._ip), op_axes.ctypes.data_as(nat._ip),
                 op_mats.ctypes.data_as(nat._dp), int(fusion_k), passes, nat.stream_handle(src.device))
        self.last_passes = passes[0]
        return State(out, ket.qubits, ket._memory)

    def evolve(self, rho=None):
        """Apply the circuit to a density matrix (quantumflow/circuits.py
        Circuit.evolve); each run of consecutive gates is one fused launch on
        the density's ket and bra axes.  Default: |0...0><0...0|."""
        from .densities import evolve_gates
        if rho is None:
            rho = zero_state(self.qubits).asdensity()
        pending = []
        for elem in self.gates():
            if isinstance(elem, Gate):
                pending.append(elem)
                continue
            if pending:
                rho = evolve_gates(rho, pending)
                pending = []
            rho = elem.evolve(rho)
        return evolve_gates(rho, pending) if pending else rho

    def aschannel(self):
        """Composite superoperator of the elements, in order."""
        from .channels import gate_aschannel
        out = gate_aschannel(identity_gate(self.qubits))
        for elem in self.elements:
            out = elem.aschannel() @ out
        return out

    def asgate(self) -> Gate:
        gate = identity_gate(self.qubits)
        for elem in self.elements:
            gate = elem.asgate() @ gate
        return gate

    @property
    def H(self) -> "Circuit":
        """Reversed circuit of element inverses (quantumflow/circuits.py:128-133)."""
        return Circuit([elem.H for elem in self.elements[::-1]])

    def __str__(self) -> str:
        return "\n".join(str(elem) for elem in self.elements)


def count_operations(elements) -> dict:
    """Count operation types (quantumflow/circuits.py count_operations)."""
    out = {}
    for e in elements:
        out[type(e)] = out.get(type(e), 0) + 1
    return out


# ------------------------------------------------------- circuit library ----
# The constructions below follow the reference gate for gate
# (quantumflow/circuits.py:152-372), so that their states match it.
def map_gate(gate: Gate, args) -> Circuit:
    """The same gate on each qubit list of ``args`` (quantumflow/circuits.py:152-167)."""
    return Circuit([gate.relabel(qubits) for qubits in args])


def reversal_circuit(qubits) -> Circuit:
    """SWAPs that reverse the qubit order (quantumflow/circuits.py:187-193)."""
    from .stdgates import SWAP
    N = len(qubits)
    return Circuit([SWAP(qubits[n], qubits[N - 1 - n]) for n in range(N // 2)])


def qft_circuit(qubits) -> Circuit:
    """Quantum Fourier transform: H and CPHASE(pi / 2^d) ladders, then the
    qubit reversal (quantumflow/circuits.py:170-184)."""
    from math import pi
    from .stdgates import CPHASE, H
    qubits = list(qubits)
    N = len(qubits)
    circ = Circuit()
    for n0 in range(N):
        circ += H(qubits[n0])
        for n1 in range(n0 + 1, N):
            circ += CPHASE(pi / 2 ** (n1 - n0), qubits[n1], qubits[n0])
    circ.extend(reversal_circuit(qubits))
    return circ


def control_circuit(controls, gate: Gate) -> Circuit:
    """A gate controlled by several qubits, Barenco et al. 1995 sec. 7.2
    (quantumflow/circuits.py:196-224)."""
    from .gates import control_gate
    from .stdgates import CNOT, X
    circ = Circuit()
    if len(controls) == 1:
        q0 = controls[0]
        circ += CNOT(q0, gate.qubits[0]) if isinstance(gate, X) else control_gate(q0, gate)
    else:
        circ += control_circuit(controls[-1:], gate ** 0.5)
        circ += control_circuit(controls[0:-1], X(controls[-1]))
        circ += control_circuit(controls[-1:], gate ** -0.5)
        circ += control_circuit(controls[0:-1], X(controls[-1]))
        circ += control_circuit(controls[0:-1], gate ** 0.5)
    return circ


def ccnot_circuit(qubits) -> Circuit:
    """Toffoli as six CNOTs with H and T gates, Nielsen & Chuang
    (quantumflow/circuits.py:227-257)."""
    from .stdgates import CNOT, H, T
    if len(qubits) != 3:
        raise ValueError("Expected 3 qubits")
    q0, q1, q2 = qubits
    return Circuit([H(q2), CNOT(q1, q2), T(q2).H, CNOT(q0, q2), T(q2), CNOT(q1, q2), T(q2).H, CNOT(q0, q2),
                    T(q1), T(q2), H(q2), CNOT(q0, q1), T(q0), T(q1).H, CNOT(q0, q1)])


def zyz_circuit(t0: float, t1: float, t2: float, q0) -> Circuit:
    """TZ TY TZ (quantumflow/circuits.py:260-266)."""
    from .stdgates import TY, TZ
    return Circuit([TZ(t0, q0), TY(t1, q0), TZ(t2, q0)])


def phase_estimation_circuit(gate: Gate, outputs) -> Circuit:
    """Quantum phase estimation (quantumflow/circuits.py:269-303)."""
    from .gates import control_gate
    from .stdgates import H
    outputs = list(outputs)
    circ = Circuit()
    circ += map_gate(H(), list(zip(outputs)))
    for cq in reversed(outputs):
        circ += control_gate(cq, gate)
        gate = gate @ gate
    circ += qft_circuit(outputs).H
    return circ


def addition_circuit(addend0, addend1, carry) -> Circuit:
    """Ripple-carry adder, Cuccaro et al. 2004 (quantumflow/circuits.py:306-356);
    the sum replaces addend1."""
    from itertools import chain
    from .stdgates import CCNOT, CNOT
    if len(addend0) != len(addend1):
        raise ValueError("Number of addend qubits must be equal")
    if len(carry) != 2:
        raise ValueError("Expected 2 carry qubits")

    def maj(q0, q1, q2):
        return Circuit([CNOT(q2, q1), CNOT(q2, q0), CCNOT(q0, q1, q2)])

    def uma(q0, q1, q2):
        return Circuit([CCNOT(q0, q1, q2), CNOT(q2, q0), CNOT(q0, q1)])

    qubits = [carry[0]] + list(chain.from_iterable(zip(reversed(list(addend1)), reversed(list(addend0))))) \
        + [carry[1]]
    circ = Circuit()
    for n in range(0, len(qubits) - 3, 2):
        circ += maj(*qubits[n:n + 3])
    circ += CNOT(qubits[-2], qubits[-1])
    for n in reversed(range(0, len(qubits) - 3, 2)):
        circ += uma(*qubits[n:n + 3])
    return circ


def ghz_circuit(qubits) -> Circuit:
    """H then a CNOT chain (quantumflow/circuits.py:359-370)."""
    from .stdgates import CNOT, H
    qubits = list(qubits)
    circ = Circuit([H(qubits[0])])
    for i in range(len(qubits) - 1):
        circ += CNOT(qubits[i], qubits[i + 1])
    return circ
