"""Small reproducible workloads for timing and profiling (the commands of
the summaries under profiles/ run these).

    python workloads.py adjoint --n 24 --p 8 [--dtype complex128] [--reps 2]
        expectation + adjoint gradient of QAOA MAXCUT on a seeded random
        3-regular graph (single instance: k_qaoaw forward, k_adjw adjoint)
    python workloads.py batch --count 32 --n 20 --p 6 [--dtype complex64] [--reps 3]
        batched evaluation of `count` seeded random 3-regular instances
        (multi-instance wave passes above the shared-memory tile)
    python workloads.py layers --n 24 --layers 10 [--arith fx|ff|fp64] [--reps 2]
        the benchmark's random-layer circuit (bench.py c2_circuit_ops) at a
        size small enough for a profiler capture
    python workloads.py dense --n 22 --k 6 [--reps 2] [--cuda-cores]
        a dense k-qubit unitary on an n-qubit complex64 state through
        qf_apply_dense_gate (tensor cores, or the CUDA-core kernel)

Each prints one line with the mean wall time per evaluation.
"""
import argparse
import os
import sys
import time

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from quantumflow_gb300 import qaoa  # noqa: E402
from quantumflow_gb300.batched import QAOABatch  # noqa: E402


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


def layers(n: int, nlayers: int, arith: str = None, reps: int = 2) -> float:
    import bench
    import quantumflow_gb300 as qf
    if arith:
        qf.config.C128_ARITHMETIC = arith
    circ = bench.build_circuit(bench.c2_circuit_ops(n, nlayers, 2018))
    circ.run(qf.zero_state(n))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        circ.run(qf.zero_state(n))
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def dense(n: int, k: int, reps: int = 2, cuda_cores: bool = False) -> float:
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(6)
    u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
    axes = [int(a) for a in rng.choice(n, size=k, replace=False)]
    dmat = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    psi = torch.zeros(2 ** n, dtype=torch.complex64, device="cuda")
    psi[0] = 1
    out = torch.empty_like(psi)
    nat.call("qf_set_dense_tensor_cores", 0 if cuda_cores else 1)

    def run():
        nat.call("qf_apply_dense_gate", nat.ptr(psi), nat.ptr(out), n, nat.LAYOUT_C64, k, nat.int_array(axes),
                 nat.ptr(dmat), nat.stream_handle())
    run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        run()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("kind", choices=["adjoint", "batch", "layers", "dense"])
    ap.add_argument("--k", type=int, default=6)
    ap.add_argument("--cuda-cores", action="store_true")
    ap.add_argument("--layers", type=int, default=10)
    ap.add_argument("--arith", default=None, choices=["fx", "ff", "fp64"])
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--count", type=int, default=32)
    ap.add_argument("--dtype", default=None, choices=["complex64", "complex128"])
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)
    if a.kind == "dense":
        s = dense(a.n, a.k, a.reps, a.cuda_cores)
        print(f"dense k={a.k} on n={a.n} complex64: {s * 1e3:.3f} ms per gate")
    elif a.kind == "layers":
        s = layers(a.n, a.layers, a.arith, a.reps)
        print(f"layers n={a.n} x {a.layers}: {s * 1e3:.3f} ms per circuit")
    elif a.kind == "adjoint":
        s = adjoint(a.n, a.p, a.dtype or "complex128", a.reps)
        print(f"adjoint n={a.n} p={a.p}: {s * 1e3:.3f} ms per expectation + gradient")
    else:
        s = batch(a.count, a.n, a.p, a.dtype or "complex64", a.reps)
        print(f"batch {a.count} x n={a.n} p={a.p}: {s * 1e3:.3f} ms per evaluation")


if __name__ == "__main__":
    main()
