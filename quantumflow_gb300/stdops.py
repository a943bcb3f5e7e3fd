"""Measurement, reset and classical operations of hybrid programs
(quantumflow/stdops.py:30-341).

The quantum parts run on the GPU: ``Measure`` reads both outcome
probabilities of its qubit with one reduction (``qf_qubit_probabilities``)
and collapses the state with one diagonal pass that also renormalises;
``Reset`` applies the (non-unitary) map |0><0| + |0><1| to each qubit in one
fused launch and renormalises.  Classical operations act on
``State.memory`` on the host, with the reference's semantics.
"""
import math
import operator
from numbers import Number
from typing import Callable, Union

import numpy as np

from .cbits import Addr
from .circuits import Circuit
from .ops import Gate, Operation
from .qubits import Qubit, Qubits
from .states import State, _reduce

__all__ = ["Measure", "Reset", "Barrier", "If",
           "Neg", "Not",
           "And", "Ior", "Or", "Xor",
           "Add", "Mul", "Sub", "Div",
           "Move", "Exchange",
           "EQ", "LT", "GT", "LE", "GE", "NE"]


class Measure(Operation):
    """Measure a qubit in the computational basis and copy the outcome to a
    classical bit (quantumflow/stdops.py:38-82)."""

    def __init__(self, qubit: Qubit, cbit: Addr = None) -> None:
        self.qubit = qubit
        self.cbit = cbit

    def quil(self) -> str:
        if self.cbit is not None:
            return f"{self.name.upper()} {self.qubit} {self.cbit}"
        return f"{self.name.upper()} {self.qubit}"

    @property
    def qubits(self) -> Qubits:
        return [self.qubit]

    def run(self, ket: State) -> State:
        axis = ket.qubits.index(self.qubit)
        buf = ket.buffer.compute()
        p0, p1 = _reduce("qf_qubit_probabilities", buf, nout=2, extra=(axis,))
        # the reference rolls np.random.random() against P(0)
        if np.random.random() < p0:
            outcome, scale = 0, 1.0 / math.sqrt(p0)
            proj = np.array([[scale, 0.0], [0.0, 0.0]], dtype=np.complex128)
        else:
            outcome, scale = 1, 1.0 / math.sqrt(p1)
            proj = np.array([[0.0, 0.0], [0.0, scale]], dtype=np.complex128)
        ket = Gate(proj, qubits=[self.qubit]).run(State(buf, ket.qubits, ket._memory))
        if self.cbit is not None:
            ket = ket.update({self.cbit: outcome})
        return ket

    def evolve(self, rho):
        """Projective measurement of a density matrix, as the reference does
        it (quantumflow/stdops.py:66-82): the outcome-0 weight it rolls
        against is the norm (sum |rho'_ij|^2) of the projected density
        rho' = P0 rho P0, and the kept branch is renormalised by its trace."""
        from .gates import P0, P1
        r0 = P0(self.qubit).evolve(rho)
        if np.random.random() < r0.norm():
            rho, outcome = r0.normalize(), 0
        else:
            rho, outcome = P1(self.qubit).evolve(rho).normalize(), 1
        if self.cbit is not None:
            rho = rho.update({self.cbit: outcome})
        return rho


class Reset(Operation):
    """Reset qubits (all of the state's qubits if none are given) to |0>,
    whatever their state (quantumflow/stdops.py:85-127)."""

    _MAP = np.array([[1.0, 1.0], [0.0, 0.0]], dtype=np.complex128)

    def __init__(self, *qubits: Qubit) -> None:
        self._qubits = tuple(qubits)

    @property
    def qubits(self) -> Qubits:
        return self._qubits

    @property
    def H(self) -> "Reset":
        return self  # Hermitian

    def run(self, ket: State) -> State:
        qubits = self.qubits if self.qubits else ket.qubits
        circ = Circuit([Gate(self._MAP, qubits=[q]) for q in qubits])
        return circ.run(ket).normalize()

    def evolve(self, rho):
        raise TypeError("Not yet implemented")  # as the reference (quantumflow/stdops.py:114-116)

    def asgate(self) -> Gate:
        raise TypeError("Reset not convertible to Gate")

    def aschannel(self):
        raise TypeError("Reset not convertible to Channel")

    def quil(self) -> str:
        if self.qubits:
            return "RESET " + " ".join(str(q) for q in self.qubits)
        return "RESET"


class Barrier(Operation):
    """Prevents reordering across it; no effect on the state
    (quantumflow/stdops.py:130-148)."""

    def __init__(self, *qubits: Qubit) -> None:
        self._qubits = tuple(qubits)

    @property
    def qubits(self) -> Qubits:
        return self._qubits

    @property
    def H(self) -> "Barrier":
        return self

    def run(self, ket: State) -> State:
        return ket

    def evolve(self, rho):
        return rho

    def quil(self) -> str:
        return self.name.upper() + " " + " ".join(str(q) for q in self.qubits)


class If(Operation):
    """Run an element when a classical bit equals ``value``
    (quantumflow/stdops.py:151-170)."""

    def __init__(self, elem: Operation, condition: Addr, value: bool = True) -> None:
        self.element = elem
        self.value = value
        self.condition = condition

    @property
    def qubits(self) -> Qubits:
        return self.element.qubits

    def run(self, ket: State) -> State:
        if ket.memory[self.condition] == self.value:
            ket = self.element.run(ket)
        return ket

    def evolve(self, rho):
        if rho.memory[self.condition] == self.value:
            rho = self.element.evolve(rho)
        return rho


# ----------------------------------------------------- classical operations --
class _Classical(Operation):
    """Classical memory operations act alike on states and densities."""

    def evolve(self, rho):
        return self.run(rho)


class Neg(_Classical):
    """Negate a value in classical memory."""

    def __init__(self, target: Addr) -> None:
        self.target = target
        self.addresses = [target]

    def run(self, ket: State) -> State:
        return ket.update({self.target: -ket.memory[self.target]})

    def quil(self) -> str:
        return f"{self.name.upper()} {self.target}"


class Not(_Classical):
    """Logical NOT of a classical bit."""

    def __init__(self, target: Addr) -> None:
        self.target = target

    def run(self, ket: State) -> State:
        return ket.update({self.target: int(not ket.memory[self.target])})

    def quil(self) -> str:
        return f"{self.name.upper()} {self.target}"


class BinaryOP(_Classical):
    """target <- op(target, source); source is an address or a number."""
    _op: Callable = None

    def __init__(self, target: Addr, source: Union[Addr, Number]) -> None:
        self.target = target
        self.source = source

    def _source(self, ket: State):
        if isinstance(self.source, Addr):
            return ket.memory[self.source]
        return self.source

    def quil(self) -> str:
        return f"{self.name.upper()} {self.target} {self.source}"

    def run(self, ket: State) -> State:
        res = type(self)._op(ket.memory[self.target], self._source(ket))
        return ket.update({self.target: res})


class And(BinaryOP):
    """Logical AND; result in target."""
    _op = operator.and_


class Ior(BinaryOP):
    """Inclusive OR; result in target."""
    _op = operator.or_


class Or(BinaryOP):
    """Inclusive OR (the deprecated Quil spelling of IOR)."""
    _op = operator.or_


class Xor(BinaryOP):
    """Exclusive OR; result in target."""
    _op = operator.xor


class Add(BinaryOP):
    _op = operator.add


class Sub(BinaryOP):
    _op = operator.sub


class Mul(BinaryOP):
    _op = operator.mul


class Div(BinaryOP):
    _op = operator.truediv


class Move(BinaryOP):
    """Copy source into target."""

    def run(self, ket: State) -> State:
        return ket.update({self.target: self._source(ket)})


class Exchange(BinaryOP):
    """Swap two classical cells."""

    def run(self, ket: State) -> State:
        if not isinstance(self.source, Addr):
            raise TypeError("Exchange needs two addresses")
        return ket.update({self.target: ket.memory[self.source], self.source: ket.memory[self.target]})


class Comparison(_Classical):
    """target <- op(memory[left], memory[right])."""
    _op: Callable = None

    def __init__(self, target: Addr, left: Addr, right: Addr) -> None:
        self.target = target
        self.left = left
        self.right = right

    def quil(self) -> str:
        return f"{self.name} {self.target} {self.left} {self.right}"

    def run(self, ket: State) -> State:
        res = type(self)._op(ket.memory[self.left], ket.memory[self.right])
        return ket.update({self.target: res})


class EQ(Comparison):
    _op = operator.eq


class GT(Comparison):
    _op = operator.gt


class GE(Comparison):
    _op = operator.ge


class LT(Comparison):
    _op = operator.lt


class LE(Comparison):
    _op = operator.le


class NE(Comparison):
    _op = operator.ne
