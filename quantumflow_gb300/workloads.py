"""Small reproducible QAOA workloads for timing and profiling.

    python -m quantumflow_gb300.workloads adjoint --n 24 --p 8 [--dtype complex128] [--reps 2]
        expectation + adjoint gradient of QAOA MAXCUT on a seeded random
        3-regular graph (single instance: k_qaoaw forward, k_adjw adjoint)
    python -m quantumflow_gb300.workloads batch --count 32 --n 20 --p 6 [--dtype complex64] [--reps 3]
        batched evaluation of `count` seeded random 3-regular instances
        (multi-instance wave passes above the shared-memory tile)

Each prints one line with the mean wall time per evaluation.
"""
import argparse
import time

import numpy as np
import torch

from . import qaoa
from .batched import QAOABatch


def adjoint(n: int, p: int, dtype: str = "complex128", reps: int = 2) -> float:
    g = qaoa.random_regular_graph(3, n, seed=3)
    rng = np.random.default_rng(0)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    prob = qaoa.QAOAMaxCut(g, p, dtype=dtype)
    prob.expectation_and_grad(beta, gamma)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        prob.expectation_and_grad(beta, gamma)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def batch(count: int, n: int, p: int, dtype: str = "complex64", reps: int = 3) -> float:
    rng = np.random.default_rng(20)
    graphs = [qaoa.random_regular_graph(3, n, seed=int(rng.integers(1 << 30))) for _ in range(count)]
    b, g = qaoa.linear_ramp_angles(p)
    bt = QAOABatch(graphs, p, dtype=dtype)
    bt.set_angles([b] * count, [g] * count)
    bt.launch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        bt.launch()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("kind", choices=["adjoint", "batch"])
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--count", type=int, default=32)
    ap.add_argument("--dtype", default=None, choices=["complex64", "complex128"])
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)
    if a.kind == "adjoint":
        s = adjoint(a.n, a.p, a.dtype or "complex128", a.reps)
        print(f"adjoint n={a.n} p={a.p}: {s * 1e3:.3f} ms per expectation + gradient")
    else:
        s = batch(a.count, a.n, a.p, a.dtype or "complex64", a.reps)
        print(f"batch {a.count} x n={a.n} p={a.p}: {s * 1e3:.3f} ms per evaluation")


if __name__ == "__main__":
    main()
