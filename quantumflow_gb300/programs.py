"""Hybrid quantum-classical programs (quantumflow/programs.py:29-523).

A :class:`Program` is a list of Quil instructions run by a program-counter
loop over ``State.memory`` (labels, jumps, halts, classical memory), with
the same instruction classes and semantics as the reference.  The GB300
difference is in how the quantum instructions reach the GPU: the reference
runs every ``Call`` as its own ``Gate.run`` (one einsum per gate,
quantumflow/programs.py:429-439); here each maximal run of consecutive gate
instructions (``Call``, ``Gate``, ``Circuit``) between two classical or
control-flow instructions is executed as one fused circuit launch
(``qf_run_circuit``: gate merging, warp-tile passes).  Jumps only land on
labels, and labels end a run, so a run is always entered at its start.
"""
from abc import ABC
from typing import Dict, Generator, List, Tuple, Union

from sympy import Symbol as Parameter

from .cbits import Addr, Register
from .circuits import Circuit
from .ops import Gate, Operation
from .qubits import Qubits
from .states import State, zero_state
from .stdgates import STDGATES

__all__ = ["Instruction", "Program", "DefCircuit", "Wait", "Nop", "Halt",
           "Label", "Jump", "JumpWhen", "JumpUnless", "Pragma", "Include", "Call",
           "Declare", "Load", "Store", "Parameter"]

# Private register holding the program state (quantumflow/programs.py:45-49)
_prog_state_ = Register("_prog_state_")
PC = _prog_state_["pc"]
NAMEDGATES = _prog_state_["namedgates"]
TARGETS = _prog_state_["targets"]
WAIT = _prog_state_["wait"]

HALTED = -1  # program counter of a finished program


class Instruction(ABC):
    """An instruction of a hybrid program (quantumflow/programs.py:54-87)."""

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

    def quil(self) -> str:
        return self.name

    def __str__(self) -> str:
        return self.quil()

    def run(self, ket: State) -> State:
        raise NotImplementedError()

    def evolve(self, rho):
        """Classical and control instructions act alike on densities
        (quantumflow/programs.py:82-87)."""
        return self.run(rho)


def _is_gate_instruction(instr) -> bool:
    return isinstance(instr, (Call, Gate, Circuit))


class Program(Instruction):
    """A Quil program (quantumflow/programs.py:90-171)."""

    def __init__(self, instructions: List[Instruction] = None, name: str = None, params: dict = None) -> None:
        self.instructions = list(instructions) if instructions is not None else []

    def quil(self) -> str:
        items = [str(i) for i in self.instructions]
        items.append("")
        return "\n".join(items)

    @property
    def qubits(self) -> Qubits:
        qubits = {q for instr in self.instructions for q in instr.qubits}
        return sorted(qubits)

    def __iadd__(self, other: Instruction) -> "Program":
        self.instructions.append(other)
        return self

    def __len__(self) -> int:
        return len(self.instructions)

    def __getitem__(self, key: int) -> Instruction:
        return self.instructions[key]

    def __iter__(self) -> Generator[Instruction, None, None]:
        yield from self.instructions

    def _initilize(self, state: State) -> State:
        """Program state: PC, label targets and the named gates
        (quantumflow/programs.py:140-150)."""
        targets = {instr.target: pc for pc, instr in enumerate(self) if isinstance(instr, Label)}
        return state.update({PC: 0, TARGETS: targets, NAMEDGATES: STDGATES.copy()})

    def _gate_run_end(self, pc: int) -> int:
        """End (exclusive) of the run of gate instructions starting at pc."""
        end = pc
        while end < len(self.instructions) and _is_gate_instruction(self.instructions[end]):
            end += 1
        return end

    def run(self, ket: State = None) -> State:
        """Run the program; the default initial state is |0...0> on the
        program's qubits with empty memory (quantumflow/programs.py:152-171)."""
        if ket is None:
            ket = zero_state(self.qubits)
        ket = self._initilize(ket)
        pc = 0
        while 0 <= pc < len(self):
            instr = self.instructions[pc]
            if _is_gate_instruction(instr):
                end = self._gate_run_end(pc)
                namedgates = ket.memory[NAMEDGATES]
                gates = []
                for g in self.instructions[pc:end]:
                    gates.extend(g.gates() if isinstance(g, Circuit) else
                                 [g.asgate_from(namedgates) if isinstance(g, Call) else g])
                ket = ket.update({PC: end})
                ket = Circuit(gates).run(ket)
            else:
                ket = ket.update({PC: pc + 1})
                ket = instr.run(ket)
            pc = ket.memory[PC]
        return ket

    def evolve(self, rho=None):
        """Run the program on a density matrix (quantumflow/programs.py:175-191);
        runs of gate instructions are fused as in :meth:`run`."""
        from .densities import evolve_gates
        if rho is None:
            rho = zero_state(self.qubits).asdensity()
        rho = self._initilize(rho)
        pc = 0
        while 0 <= pc < len(self):
            instr = self.instructions[pc]
            if _is_gate_instruction(instr):
                end = self._gate_run_end(pc)
                namedgates = rho.memory[NAMEDGATES]
                gates = []
                for g in self.instructions[pc:end]:
                    gates.extend(g.gates() if isinstance(g, Circuit) else
                                 [g.asgate_from(namedgates) if isinstance(g, Call) else g])
                rho = rho.update({PC: end})
                rho = Circuit(gates).evolve(rho)
            else:
                rho = rho.update({PC: pc + 1})
                rho = instr.evolve(rho)
            pc = rho.memory[PC]
        return rho


class DefCircuit(Program):
    """A named, parameterised sub-circuit definition
    (quantumflow/programs.py:177-233; recorded, as in the reference)."""

    def __init__(self, name: str, params: Dict[str, float], qubits: Qubits = None,
                 instructions: List[Instruction] = None) -> None:
        super().__init__(instructions)
        self.progname = name
        self.params = params
        self._qubits = list(qubits) if qubits is not None else []

    @property
    def qubits(self) -> Qubits:
        return self._qubits

    def quil(self) -> str:
        fparams = "(" + ",".join(map(str, self.params)) + ")" if self.params else ""
        fqubits = " " + " ".join(map(str, self.qubits)) if self.qubits else ""
        result = f"{self.name} {self.progname}{fparams}{fqubits}:\n"
        for instr in self.instructions:
            result += "    " + str(instr) + "\n"
        return result


class Wait(Instruction):
    """Return control to the caller (a no-op here, as in the reference)."""

    def run(self, ket: State) -> State:
        return ket


class Nop(Instruction):
    """No operation."""

    def run(self, ket: State) -> State:
        return ket


class Halt(Instruction):
    """Stop the program."""

    def run(self, ket: State) -> State:
        return ket.update({PC: HALTED})


class Load(Instruction):
    """The LOAD instruction (not executable in the reference either)."""

    def __init__(self, target: Addr, left: str, right: Addr) -> None:
        self.target, self.left, self.right = target, left, right

    def quil(self) -> str:
        return f"{self.name} {self.target} {self.left} {self.right}"

    def run(self, ket: State) -> State:
        raise NotImplementedError()


class Store(Instruction):
    """The STORE instruction (not executable in the reference either)."""

    def __init__(self, target: str, left: Addr, right: Union[int, Addr]) -> None:
        self.target, self.left, self.right = target, left, right

    def quil(self) -> str:
        return f"{self.name} {self.target} {self.left} {self.right}"

    def run(self, ket: State) -> State:
        raise NotImplementedError()


class Label(Instruction):
    """A jump target."""

    def __init__(self, target: str) -> None:
        self.target = target

    def quil(self) -> str:
        return f"{self.name} @{self.target}"

    def run(self, ket: State) -> State:
        return ket


class Jump(Instruction):
    """Unconditional jump to a label."""

    def __init__(self, target: str) -> None:
        self.target = target

    def quil(self) -> str:
        return f"{self.name} @{self.target}"

    def run(self, ket: State) -> State:
        return ket.update({PC: ket.memory[TARGETS][self.target]})


class JumpWhen(Instruction):
    """Jump to a label if a classical bit is one."""

    def __init__(self, target: str, condition: Addr) -> None:
        self.target = target
        self.condition = condition

    @property
    def name(self) -> str:
        return "JUMP-WHEN"

    def quil(self) -> str:
        return f"{self.name} @{self.target} {self.condition}"

    def run(self, ket: State) -> State:
        if ket.memory[self.condition]:
            return ket.update({PC: ket.memory[TARGETS][self.target]})
        return ket


class JumpUnless(Instruction):
    """Jump to a label if a classical bit is zero."""

    def __init__(self, target: str, condition: Addr) -> None:
        self.target = target
        self.condition = condition

    @property
    def name(self) -> str:
        return "JUMP-UNLESS"

    def quil(self) -> str:
        return f"{self.name} @{self.target} {self.condition}"

    def run(self, ket: State) -> State:
        if not ket.memory[self.condition]:
            return ket.update({PC: ket.memory[TARGETS][self.target]})
        return ket


class Pragma(Instruction):
    """PRAGMA <command> <arg>* "<freeform>"? (no effect)."""

    def __init__(self, command: str, args: List[float] = None, freeform: str = None) -> None:
        self.command = command
        self.args = args
        self.freeform = freeform

    def quil(self) -> str:
        ret = [f"PRAGMA {self.command}"]
        if self.args:
            ret.extend(str(a) for a in self.args)
        if self.freeform:
            ret.append(f'"{self.freeform}"')
        return " ".join(ret)

    def run(self, ket: State) -> State:
        return ket


class Include(Instruction):
    """INCLUDE of another Quil file (recorded, not acted upon)."""

    def __init__(self, filename: str, program: Program = None) -> None:
        self.filename = filename
        self.program = program

    def quil(self) -> str:
        return f'{self.name} "{self.filename}"'

    def run(self, ket: State) -> State:
        raise NotImplementedError()


class Call(Instruction):
    """Apply a named gate (quantumflow/programs.py:417-439)."""

    def __init__(self, name: str, params: List[Parameter], qubits: Qubits) -> None:
        self.gatename = name
        self.params = list(params)
        self._qubits = list(qubits)

    def quil(self) -> str:
        fqubits = " " + " ".join(str(q) for q in self.qubits) if self.qubits else ""
        fparams = "(" + ", ".join(str(p) for p in self.params) + ")" if self.params else ""
        return f"{self.gatename}{fparams}{fqubits}"

    def asgate_from(self, namedgates: dict) -> Gate:
        if self.gatename not in namedgates:
            raise RuntimeError("Unknown named gate")
        gate = namedgates[self.gatename](*self.params)
        return gate.relabel(self.qubits)

    def run(self, ket: State) -> State:
        return self.asgate_from(ket.memory[NAMEDGATES]).run(ket)

    def evolve(self, rho):
        return self.asgate_from(rho.memory[NAMEDGATES]).evolve(rho)


class Declare(Instruction):
    """Declare classical memory, zero-initialised."""

    def __init__(self, memory_name: str, memory_type: str, memory_size: int, shared_region: str = None,
                 offsets: List[Tuple[int, str]] = None) -> None:
        self.memory_name = memory_name
        self.memory_type = memory_type
        self.memory_size = memory_size
        self.shared_region = shared_region
        self.offsets = offsets

    def quil(self) -> str:
        ql = ["DECLARE", self.memory_name, self.memory_type]
        if self.memory_size != 1:
            ql.append(f"[{self.memory_size}]")
        if self.shared_region is not None:
            ql += ["SHARING", self.shared_region]
        return " ".join(ql)

    def run(self, ket: State) -> State:
        reg = Register(self.memory_name, self.memory_type)
        return ket.update({reg[idx]: 0 for idx in range(self.memory_size)})
