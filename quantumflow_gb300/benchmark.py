"""GOPS benchmark: gate operations per second (tools/benchmark.py).

The circuit of the reference tool (tools/benchmark.py:31-45): H on every
qubit, then (gates - N) // 3 rounds of X on a random qubit, T on another
and CNOT between them.  ``benchmark`` applies it gate by gate through
``Gate.run``, as the reference does, or as one fused ``Circuit.run`` launch
sequence (``fused=True``); ``benchmark_gops`` times it.

    python -m quantumflow_gb300.benchmark 16 20 24 [--gates 100] [--reps 1] [--fused]

prints ``N<tab>GOPS`` lines like the reference tool.
"""
import argparse
import random
import timeit

import torch

from .circuits import Circuit
from .states import zero_state
from .stdgates import CNOT, H, T, X

GATES = 100
REPS = 1
QUBITS = 16


def benchmark_circuit(N: int, gates: int, seed=None) -> Circuit:
    """The benchmark's gate list (tools/benchmark.py:31-43)."""
    rng = random.Random(seed)
    qubits = list(range(N))
    elems = [H(n) for n in range(N)]
    for _ in range((gates - N) // 3):
        q0, q1 = rng.sample(qubits, 2)
        elems += [X(q0), T(q1), CNOT(q0, q1)]
    return Circuit(elems)


def benchmark(N: int, gates: int, fused: bool = False, seed=None) -> torch.Tensor:
    """Run the benchmark circuit on |0...0> and return the final amplitudes
    (a [2]*N device tensor, synchronised so the work is complete)."""
    circ = benchmark_circuit(N, gates, seed)
    if fused:
        ket = circ.run(zero_state(N))
    else:
        ket = zero_state(N)
        for gate in circ:
            ket = gate.run(ket)
    out = ket.tensor
    torch.cuda.synchronize()
    return out


def benchmark_gops(N: int, gates: int = GATES, reps: int = REPS, fused: bool = False) -> float:
    """Gate operations per second, rounded to 2 decimals as the reference
    does (tools/benchmark.py:48-53); one untimed run first, so that device
    and library start-up are not timed."""
    benchmark(N, gates, fused)
    t = timeit.timeit(lambda: benchmark(N, gates, fused), number=reps)
    gops = gates * reps / t
    return int(gops * 100 + 0.5) / 100.0


def _cli(argv=None):
    parser = argparse.ArgumentParser(description="QuantumFlow GB300 benchmark, in GOPS "
                                                 "(gate operations per second)")
    parser.add_argument("qubits", nargs="*", type=int, default=[QUBITS])
    parser.add_argument("--gates", type=int, default=GATES)
    parser.add_argument("--reps", type=int, default=REPS)
    parser.add_argument("--fused", action="store_true", help="one Circuit.run instead of gate by gate")
    opts = parser.parse_args(argv)
    print("# N\tGOPS")
    for N in opts.qubits:
        print(N, "\t", benchmark_gops(N, opts.gates, opts.reps, opts.fused))


if __name__ == "__main__":
    _cli()
