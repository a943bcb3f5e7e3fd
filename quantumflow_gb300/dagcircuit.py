"""Directed-acyclic-graph view of a circuit (quantumflow/dagcircuit.py:25-172).

Every qubit is a wire from an ('in', q) node through the operations on it to
an ('out', q) node.  The graph is kept as per-operation predecessor and
successor maps keyed by qubit (no graph library), in the circuit's own
order, which is a topological order.  ``layers()`` groups operations by
their depth (operations in one layer act on disjoint qubits and commute);
running a DAGCircuit runs its layers as one fused circuit launch.
"""
from typing import Dict, Iterable, Iterator, List

from .circuits import Circuit
from .ops import Gate, Operation
from .qubits import Qubit, Qubits

__all__ = ["DAGCircuit"]


class DAGCircuit(Operation):
    """quantumflow/dagcircuit.py:25-172."""

    def __init__(self, elements: Iterable[Operation]) -> None:
        self._ops: List[Operation] = []
        self._prev: Dict[int, Dict[Qubit, object]] = {}
        self._next: Dict[int, Dict[Qubit, object]] = {}
        last: Dict[Qubit, object] = {}
        for elem in elements:
            if isinstance(elem, tuple):  # in / out nodes of another DAG's graph
                continue
            self._ops.append(elem)
            key = id(elem)
            self._prev[key] = {}
            self._next[key] = {}
            for q in elem.qubits:
                prev = last.get(q, ("in", q))
                self._prev[key][q] = prev
                if not isinstance(prev, tuple):
                    self._next[id(prev)][q] = elem
                last[q] = elem
        for q, elem in last.items():
            if not isinstance(elem, tuple):
                self._next[id(elem)][q] = ("out", q)
        self._wires = sorted(last) if last else []

    # -- structure ------------------------------------------------------
    @property
    def qubits(self) -> Qubits:
        return tuple(self._wires)

    @property
    def qubit_nb(self) -> int:
        return len(self._wires)

    def __iter__(self) -> Iterator[Operation]:
        return iter(self._ops)

    def size(self) -> int:
        """Number of operations."""
        return len(self._ops)

    def _depths(self, ops) -> Dict[int, int]:
        depth: Dict[int, int] = {}
        for elem in ops:
            d = 0
            for prev in self._prev[id(elem)].values():
                if not isinstance(prev, tuple) and id(prev) in depth:
                    d = max(d, depth[id(prev)] + 1)
            depth[id(elem)] = d
        return depth

    def depth(self, local: bool = True) -> int:
        """Longest chain of operations; with local=False one-qubit operations
        are left out (quantumflow/dagcircuit.py:97-113)."""
        if local:
            ops = self._ops
            depth = self._depths(ops)
        else:
            sub = DAGCircuit(e for e in self._ops if len(e.qubits) > 1)
            return sub.depth()
        return (max(depth.values()) + 1) if depth else 0

    def component_nb(self) -> int:
        """Number of independent components (qubit groups linked by operations)."""
        return len(self._component_qubits())

    def _component_qubits(self) -> List[set]:
        parent = {q: q for q in self._wires}

        def find(q):
            while parent[q] != q:
                parent[q] = parent[parent[q]]
                q = parent[q]
            return q

        for elem in self._ops:
            qs = list(elem.qubits)
            for q in qs[1:]:
                ra, rb = find(qs[0]), find(q)
                if ra != rb:
                    parent[rb] = ra
        groups: Dict[Qubit, set] = {}
        for q in self._wires:
            groups.setdefault(find(q), set()).add(q)
        return list(groups.values())

    def components(self) -> List["DAGCircuit"]:
        """Split into independent components (quantumflow/dagcircuit.py:124-127)."""
        out = []
        for qs in self._component_qubits():
            out.append(DAGCircuit(e for e in self._ops if set(e.qubits) & qs))
        return out

    def layers(self) -> Circuit:
        """A Circuit of Circuits, one per depth; operations within a layer act
        on different qubits (quantumflow/dagcircuit.py:129-151)."""
        depth = self._depths(self._ops)
        nlayers = (max(depth.values()) + 1) if depth else 0
        groups: List[List[Operation]] = [[] for _ in range(nlayers)]
        for elem in self._ops:
            groups[depth[id(elem)]].append(elem)
        return Circuit([Circuit(g) for g in groups])

    def next_element(self, elem: Operation, qubit: Qubit = None):
        nxt = self._next[id(elem)]
        return nxt[qubit] if qubit is not None else next(iter(nxt.values()))

    def prev_element(self, elem: Operation, qubit: Qubit = None):
        prv = self._prev[id(elem)]
        return prv[qubit] if qubit is not None else next(iter(prv.values()))

    # -- action ---------------------------------------------------------
    @property
    def H(self) -> "DAGCircuit":
        return DAGCircuit(Circuit(self._ops).H)

    def run(self, ket):
        """Run layer by layer as one fused circuit."""
        return self.layers().run(ket)

    def evolve(self, rho):
        return self.layers().evolve(rho)

    def asgate(self) -> Gate:
        return Circuit(self._ops).asgate()

    def aschannel(self):
        return Circuit(self._ops).aschannel()
