"""Generate the golden fixtures in this directory from the reference itself.

Runs only where a read-only QuantumFlow reference checkout exists; its path
is given by the ``QF_REFERENCE`` environment variable (the script stops when
it is unset).  The GPU tests never run this script: they only read the
``.npz`` files it wrote.

What it does:

* imports the reference ``quantumflow`` package on its default numpy backend.
  ``quantumflow/__init__.py`` imports every submodule, and three of them pull
  in packages absent here (``cvxpy`` in ``measures.py``, ``PIL`` in
  ``forest/__init__.py``, ``pyquil`` in ``forest/pyquil.py`` and ``meta.py``).
  A ``sys.meta_path`` finder hands out inert stub modules for exactly those
  three top-level names, so the import succeeds and every hot-path function
  (``Gate.run``, ``tensormul``, ``Circuit.run``, ``State.expectation``,
  ``qubo_circuit``, ``graph_cuts``) runs unmodified;
* reads the literal known-answer vectors out of the reference's own test files
  with ``ast`` (as data; nothing from them is executed except the helpers
  named below);
* runs the reference on seeded inputs and stores inputs and outputs.

Usage:  QF_REFERENCE=<checkout> PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [name ...]
"""
import ast
import importlib.abc
import importlib.machinery
import os
import sys
import types

import numpy as np

REF = os.environ.get("QF_REFERENCE")
HERE = os.path.dirname(os.path.abspath(__file__))
STUBBED = ("pyquil", "cvxpy", "PIL")


# ---------------------------------------------------------------- stubs ----
class _AnyMeta(type):
    def __getattr__(cls, name):
        return _Any


class _Any(metaclass=_AnyMeta):
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Any()

    def __getattr__(self, name):
        return _Any


class _StubModule(types.ModuleType):
    __all__ = []

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Any


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in STUBBED:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        mod = _StubModule(spec.name)
        mod.__path__ = []
        return mod

    def exec_module(self, module):
        pass


def import_reference():
    """Import the reference package (numpy backend) with the stubs above."""
    if not REF or not os.path.isdir(os.path.join(REF, "quantumflow")):
        sys.exit("set QF_REFERENCE to a QuantumFlow checkout (the directory holding quantumflow/)")
    os.environ.setdefault("QUANTUMFLOW_BACKEND", "numpy")
    sys.dont_write_bytecode = True
    sys.meta_path.insert(0, _StubFinder())
    sys.path.insert(0, REF)
    import quantumflow as qf  # noqa: E402
    assert qf.backend.name == "numpy", qf.backend.name
    return qf


# ------------------------------------------------- literal KATs via ast ----
def _literal_in_function(path, func, target_kind):
    """Return the first list literal assigned/passed inside ``func``."""
    tree = ast.parse(open(path).read())
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == func:
            for sub in ast.walk(node):
                if isinstance(sub, ast.List) and len(sub.elts) >= 4:
                    if target_kind == "complex":
                        return [complex(eval(compile(ast.Expression(e), "<kat>", "eval")))
                                for e in sub.elts]
                    return [float(eval(compile(ast.Expression(e), "<kat>", "eval")))
                            for e in sub.elts]
    raise KeyError(func)


def _all_float_lists(path, func):
    tree = ast.parse(open(path).read())
    out = []
    for node in ast.walk(tree):
        if isinstance(node, ast.FunctionDef) and node.name == func:
            for sub in ast.walk(node):
                if isinstance(sub, ast.List) and len(sub.elts) == 8 and all(
                        isinstance(e, (ast.Constant, ast.UnaryOp)) for e in sub.elts):
                    out.append([float(eval(compile(ast.Expression(e), "<kat>", "eval")))
                                for e in sub.elts])
    return out


def kat_fixtures(qf):
    t = os.path.join(REF, "tests")
    out = {}
    # tests/test_circuits.py:19-24  true_ket() amplitudes (referenceQVM)
    out["true_ket"] = np.array(_literal_in_function(
        os.path.join(t, "test_circuits.py"), "true_ket", "complex"))
    # tests/test_circuits.py:190-203  3-qubit QFT amplitudes
    out["qft3"] = np.array(_literal_in_function(
        os.path.join(t, "test_circuits.py"), "test_qft", "complex"))
    # tests/test_qaoa.py:40-55  literal cut tables (unweighted, weighted)
    tables = _all_float_lists(os.path.join(t, "test_qaoa.py"), "test_graph_cuts")
    out["cuts_unweighted"] = np.array(tables[0])
    out["cuts_weighted"] = np.array(tables[1])
    # tests/test_qaoa.py:17-37 element counts; tests/test_gates.py:150-164
    # expectation literals; these are scalars in asserts.
    out["qubo_counts"] = np.array([13, 15])
    out["expectation_literals"] = np.array([42.0, 2.5])

    # Cross-check: the reference itself reproduces its literals.
    from math import pi
    circ = qf.Circuit()
    circ += qf.RY(pi / 2, 0)
    circ += qf.RX(pi, 0)
    circ += qf.RY(pi / 2, 1)
    circ += qf.RX(pi, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.RX(-pi / 2, 1)
    circ += qf.RY(4.71572463191, 1)
    circ += qf.RX(pi / 2, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.RX(-2 * 2.74973750579, 0)
    circ += qf.RX(-2 * 2.74973750579, 1)
    ket = circ.run(qf.zero_state(2))
    assert qf.states_close(ket, qf.State(out["true_ket"].reshape(2, 2)))
    out["true_ket_ref_run"] = ket.tensor.reshape(-1)
    c = qf.Circuit()
    c += qf.X(2)
    c.extend(qf.qft_circuit([0, 1, 2]))
    ket = c.run(qf.zero_state(3))
    assert qf.states_close(ket, qf.State(out["qft3"]))
    out["qft3_ref_run"] = ket.tensor.reshape(-1)
    return out


# ----------------------------------------------------------- gate tables ----
GATE_SPECS = [
    # name, params, nqubits
    ("I", (), 1), ("X", (), 1), ("Y", (), 1), ("Z", (), 1), ("H", (), 1),
    ("S", (), 1), ("T", (), 1), ("S_H", (), 1), ("T_H", (), 1),
    ("PHASE", (0.1,), 1), ("RX", (0.2,), 1), ("RY", (0.3,), 1), ("RZ", (0.4,), 1),
    ("TX", (2.7,), 1), ("TY", (1.2,), 1), ("TZ", (0.3,), 1), ("TH", (0.3,), 1),
    ("ZYZ", (3.5, 0.9, 2.1), 1), ("RN", (0.7, 0.3, 0.4, 0.5), 1),
    ("CZ", (), 2), ("CNOT", (), 2), ("SWAP", (), 2), ("ISWAP", (), 2),
    ("CPHASE00", (0.5,), 2), ("CPHASE01", (0.6,), 2), ("CPHASE10", (0.6,), 2),
    ("CPHASE", (0.7,), 2), ("PSWAP", (0.15,), 2), ("PISWAP", (0.2,), 2),
    ("XX", (1.8,), 2), ("YY", (0.9,), 2), ("ZZ", (0.45,), 2),
    ("CAN", (0.1, 0.2, 0.3), 2), ("EXCH", (0.1,), 2),
    ("CCNOT", (), 3), ("CSWAP", (), 3),
]


def gate_fixtures(qf):
    out = {}
    for name, params, k in GATE_SPECS:
        g = getattr(qf, name)(*params)
        m = np.asarray(g.asoperator(), dtype=np.complex128)
        assert m.shape == (2 ** k, 2 ** k)
        out["gate_" + name] = m
        out["gateH_" + name] = np.asarray(g.H.asoperator(), dtype=np.complex128)
    return out


# -------------------------------------------------------- tensormul ----
def tensormul_fixtures(qf, rng):
    bk = qf.backend
    out = {}
    cases = []
    for N in (1, 2, 3, 5, 8, 10):
        for K in (1, 2, 3):
            if K > N:
                continue
            for rep in range(3):
                idx = rng.choice(N, size=K, replace=False)
                cases.append((N, K, idx))
    out["tm_count"] = np.array(len(cases))
    for c, (N, K, idx) in enumerate(cases):
        state = rng.normal(size=2 ** N) + 1j * rng.normal(size=2 ** N)
        gate = rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K))
        res = bk.tensormul(bk.astensorproduct(gate.reshape([2] * (2 * K))),
                           bk.astensorproduct(state), list(int(i) for i in idx))
        out[f"tm{c}_N"] = np.array(N)
        out[f"tm{c}_idx"] = np.array(idx)
        out[f"tm{c}_gate"] = gate
        out[f"tm{c}_state"] = state
        out[f"tm{c}_out"] = np.asarray(res).reshape(-1)
    return out


# ------------------------------------------------ random layered circuit ----
def random_layer_circuit(N, layers, rng):
    """Haar U(2) on every qubit then CZ on a random perfect matching, per layer.

    Returns a list of (kind, qubits, matrix) with matrices drawn on the host so
    every implementation replays identical inputs."""
    import scipy.stats
    ops = []
    for _ in range(layers):
        for q in range(N):
            u = scipy.stats.unitary_group.rvs(2, random_state=rng)
            ops.append((1, (q,), u))
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            ops.append((2, (int(perm[a]), int(perm[a + 1])), None))
    return ops


def circuit_fixtures(qf, rng):
    out = {}
    for N, layers in ((4, 3), (6, 4), (9, 3), (12, 2)):
        ops = random_layer_circuit(N, layers, rng)
        circ = qf.Circuit()
        mats = []
        quads = []
        for kind, qs, u in ops:
            if kind == 1:
                circ += qf.Gate(u, qubits=qs)
                mats.append(u)
                quads.append([1, qs[0], -1])
            else:
                circ += qf.CZ(*qs)
                mats.append(np.zeros((2, 2), complex))
                quads.append([2, qs[0], qs[1]])
        ket = circ.run(qf.zero_state(N))
        out[f"rc{N}_ops"] = np.array(quads)
        out[f"rc{N}_u"] = np.array(mats)
        out[f"rc{N}_state"] = np.asarray(ket.tensor).reshape(-1)
        inv = circ.H.run(ket)
        out[f"rc{N}_inverse"] = np.asarray(inv.tensor).reshape(-1)
    # tools/benchmark.py-style GOPS circuit (H on all, then X, T, CNOT triples)
    N = 8
    ket = qf.zero_state(N)
    triples = []
    for n in range(N):
        ket = qf.H(n).run(ket)
    for _ in range(10):
        q0, q1 = (int(x) for x in rng.choice(N, size=2, replace=False))
        triples.append([q0, q1])
        ket = qf.X(q0).run(ket)
        ket = qf.T(q1).run(ket)
        ket = qf.CNOT(q0, q1).run(ket)
    out["gops_pairs"] = np.array(triples)
    out["gops_state"] = np.asarray(ket.tensor).reshape(-1)
    return out


# ------------------------------------------------------------- QAOA ----
def _expect(qf, graph, p, beta, gamma, cuts):
    from quantumflow.qaoa import qubo_circuit
    circ = qubo_circuit(graph, p, beta, gamma)
    return float(np.real(circ.run().expectation(cuts)))


def qaoa_fixtures(qf, rng):
    import networkx as nx
    from quantumflow.qaoa import qubo_circuit, graph_cuts
    out = {}
    cases = []
    # the MAXCUT example size: G(6, 0.5) from a seed, p=5, angles U[0, pi)
    cases.append(("er6p5", nx.gnp_random_graph(6, 0.5, seed=7), 5, True))
    # 3-regular graphs (the gradient workload's family at oracle-friendly n) and ER graphs
    cases.append(("reg8", nx.random_regular_graph(3, 8, seed=11), 3, True))
    cases.append(("reg10", nx.random_regular_graph(3, 10, seed=12), 8, True))
    cases.append(("er9", nx.gnp_random_graph(9, 0.5, seed=13), 2, True))
    cases.append(("reg12", nx.random_regular_graph(3, 12, seed=14), 2, False))
    # the n=24, p=8 gradient workload at oracle-friendly size: 3-regular n=16, p=8 (state not stored)
    cases.append(("reg16p8", nx.random_regular_graph(3, 16, seed=16), 8, True))
    # weighted edges + node weights (RZ quirk, qaoa.py:55-58)
    g = nx.gnp_random_graph(7, 0.6, seed=21)
    for (a, b) in g.edges():
        g[a][b]["weight"] = float(rng.uniform(0.1, 2.0))
    g.nodes[2]["weight"] = 0.7
    g.nodes[5]["weight"] = -1.3
    cases.append(("w7", g, 3, True))
    h = 1e-6
    names = []
    for name, graph, p, with_grad in cases:
        n = graph.number_of_nodes()
        assert list(graph.nodes()) == list(range(n))
        beta = rng.uniform(0, np.pi, size=p)
        gamma = rng.uniform(0, np.pi, size=p)
        cuts = graph_cuts(graph)
        circ = qubo_circuit(graph, p, beta, gamma)
        ket = circ.run()
        e = float(np.real(ket.expectation(cuts)))
        edges = np.array([[a, b] for a, b in graph.edges()], dtype=np.int64).reshape(-1, 2)
        w = np.array([graph[a][b].get("weight", 1.0) for a, b in graph.edges()])
        nw = np.array([graph.nodes[q].get("weight", np.nan) for q in range(n)])
        out[f"{name}_n"] = np.array(n)
        out[f"{name}_p"] = np.array(p)
        out[f"{name}_edges"] = edges
        out[f"{name}_weights"] = w
        out[f"{name}_node_weights"] = nw
        out[f"{name}_beta"] = beta
        out[f"{name}_gamma"] = gamma
        if n <= 12:
            out[f"{name}_cuts"] = np.asarray(cuts).reshape(-1)
            out[f"{name}_state"] = np.asarray(ket.tensor).reshape(-1)
        out[f"{name}_expectation"] = np.array(e)
        out[f"{name}_nelements"] = np.array(len(circ.elements))
        if with_grad:
            gg = np.zeros(p)
            gb = np.zeros(p)
            for i in range(p):
                for arr, dst in ((gamma, gg), (beta, gb)):
                    old = arr[i]
                    arr[i] = old + h
                    ep = _expect(qf, graph, p, beta, gamma, cuts)
                    arr[i] = old - h
                    em = _expect(qf, graph, p, beta, gamma, cuts)
                    arr[i] = old
                    dst[i] = (ep - em) / (2 * h)
            out[f"{name}_fd_grad_gamma"] = gg
            out[f"{name}_fd_grad_beta"] = gb
        names.append(name)
    out["qaoa_cases"] = np.array(names)

    # the example training loop (examples/qaoa_maxcut.py): 5 gradient-ascent steps on <C>, lr=0.1, FD grads
    graph = cases[0][1]
    p = 5
    beta = out["er6p5_beta"].copy()
    gamma = out["er6p5_gamma"].copy()
    cuts = graph_cuts(graph)
    traj = []
    for step in range(5):
        gg = np.zeros(p)
        gb = np.zeros(p)
        for i in range(p):
            for arr, dst in ((gamma, gg), (beta, gb)):
                old = arr[i]
                arr[i] = old + h
                ep = _expect(qf, graph, p, beta, gamma, cuts)
                arr[i] = old - h
                em = _expect(qf, graph, p, beta, gamma, cuts)
                arr[i] = old
                dst[i] = (ep - em) / (2 * h)
        gamma = gamma + 0.1 * gg
        beta = beta + 0.1 * gb
        traj.append(_expect(qf, graph, p, beta, gamma, cuts))
    out["er6p5_gd_expectations"] = np.array(traj)
    out["er6p5_gd_beta"] = beta
    out["er6p5_gd_gamma"] = gamma
    out["er6p5_maxcut"] = np.array(float(np.max(cuts)))
    return out


# --------------------------------------------------------------- programs ----
PROGRAM_GATES = [("H", 0, 1), ("X", 0, 1), ("T", 0, 1), ("S", 0, 1), ("RX", 1, 1), ("RY", 1, 1),
                 ("RZ", 1, 1), ("PHASE", 1, 1), ("CNOT", 0, 2), ("CZ", 0, 2), ("SWAP", 0, 2),
                 ("CPHASE", 1, 2), ("ZZ", 1, 2), ("ISWAP", 0, 2), ("CCNOT", 0, 3)]


def program_fixtures(qf, rng):
    """Reference Program runs: the literal amplitudes of
    tests/test_programs.py:193-217, and seeded random Call programs run by
    quantumflow/programs.py:152-171 (Call.run :429-439)."""
    t = os.path.join(REF, "tests")
    out = {"wf_true": np.array(_literal_in_function(os.path.join(t, "test_programs.py"),
                                                      "test_qaoa_circuit", "complex"))}
    for case, (nq, ncalls) in enumerate([(3, 40), (5, 120), (7, 200)]):
        names, params, qubits = [], [], []
        prog = qf.Program()
        for _ in range(ncalls):
            name, npar, k = PROGRAM_GATES[rng.integers(len(PROGRAM_GATES))]
            qs = [int(q) for q in rng.choice(nq, size=k, replace=False)]
            ps = [float(v) for v in rng.uniform(-np.pi, np.pi, size=npar)]
            prog += qf.Call(name, ps, qs)
            names.append(name)
            params.append(ps + [np.nan] * (1 - len(ps)))
            qubits.append(qs + [-1] * (3 - len(qs)))
        ket = prog.run(qf.zero_state(nq))
        out[f"p{case}_names"] = np.array(names)
        out[f"p{case}_params"] = np.array(params)
        out[f"p{case}_qubits"] = np.array(qubits, dtype=np.int64)
        out[f"p{case}_state"] = ket.tensor.reshape(-1)
        out[f"p{case}_nq"] = np.array(nq)
    return out


# --------------------------------------------------------------- channels ----
def channel_fixtures(qf, rng):
    """Density-matrix evolution by the reference (quantumflow/ops.py:166-170
    Gate.evolve via aschannel, :354-363 Channel.evolve, channels.py Kraus /
    Damping / Depolarizing / Dephasing, states.py Density)."""
    import scipy.stats
    out = {}
    N = 4
    np.random.seed(20181205)
    rho = qf.random_density(N)
    out["rho0"] = np.asarray(rho.tensor).reshape(2 ** N, 2 ** N)
    u1 = scipy.stats.unitary_group.rvs(2, random_state=rng)
    u2 = scipy.stats.unitary_group.rvs(4, random_state=rng)
    out["u1"], out["u2"] = u1, u2
    steps = [
        ("gate1", qf.Gate(u1, qubits=[2])),
        ("gate2", qf.Gate(u2, qubits=[3, 0])),
        ("damping", qf.Damping(0.3, 1)),
        ("depolarizing", qf.Depolarizing(0.2, 3)),
        ("dephasing", qf.Dephasing(0.45, 0)),
        ("kraus2", qf.Kraus([qf.Gate(u2 * np.sqrt(0.7), qubits=[1, 2]),
                             qf.Gate(np.eye(4) * np.sqrt(0.3), qubits=[1, 2])])),
        ("chan_matmul", qf.Damping(0.1, 2).aschannel() @ qf.Dephasing(0.2, 2).aschannel()),
        ("joined", qf.join_channels(qf.Damping(0.25, 0).aschannel(), qf.Depolarizing(0.15, 3).aschannel())),
    ]
    cur = rho
    for name, op in steps:
        cur = op.evolve(cur)
        out[f"after_{name}"] = np.asarray(cur.tensor).reshape(2 ** N, 2 ** N)
    out["trace_final"] = np.array(complex(qf.asarray(cur.trace())))
    out["probs_final"] = np.asarray(cur.probabilities()).reshape(-1)
    out["ptrace_13"] = np.asarray(cur.partial_trace([1, 3]).tensor).reshape(4, 4)
    ket = qf.random_state(3)
    out["ket"] = np.asarray(ket.tensor).reshape(-1)
    out["ket_density"] = np.asarray(ket.asdensity().tensor).reshape(8, 8)
    out["damping_superop"] = np.asarray(qf.Damping(0.3, 0).aschannel().tensor).reshape(4, 4)
    out["mixed3"] = np.asarray(qf.mixed_density(3).tensor).reshape(8, 8)
    return out


# ------------------------------------ random-layer family at bench sizes ----
def layer_family_fixtures(qf, rng):
    """The benchmark's circuit family (Haar U(2) on every qubit, then CZ on a
    seeded random perfect matching, per layer) run by the reference's
    Circuit.run (quantumflow/circuits.py:87-99, one numpy einsum per gate):
    N=16 and N=20 with all 100 layers, N=24 with 2 layers.  The gates are
    stored; of the output, N=16 keeps the full state and every size keeps
    4096 amplitudes at seeded indices (first and last included), the
    probabilities of the top 8 axes (marginal over the rest) and the norm."""
    out = {}
    for N, layers in ((16, 100), (20, 100), (24, 2)):
        ops = random_layer_circuit(N, layers, rng)
        circ = qf.Circuit()
        us, pairs = [], []
        for kind, qs, u in ops:
            if kind == 1:
                circ += qf.Gate(u, qubits=qs)
                us.append(u)
            else:
                circ += qf.CZ(*qs)
                pairs.append(qs)
        ket = circ.run(qf.zero_state(N))
        psi = np.asarray(ket.tensor).reshape(-1)
        idx = np.unique(np.concatenate([[0, 2 ** N - 1], rng.choice(2 ** N, size=4094, replace=False)]))
        out[f"lf{N}_layers"] = np.array(layers)
        out[f"lf{N}_u"] = np.array(us)                      # [layers * N, 2, 2], layer-major
        out[f"lf{N}_pairs"] = np.array(pairs, dtype=np.int64).reshape(layers, N // 2, 2)
        out[f"lf{N}_idx"] = idx.astype(np.int64)
        out[f"lf{N}_amps"] = psi[idx]
        out[f"lf{N}_top8"] = (np.abs(psi) ** 2).reshape(256, -1).sum(axis=1)
        out[f"lf{N}_norm"] = np.array(float(np.vdot(psi, psi).real))
        if N <= 16:
            out[f"lf{N}_state"] = psi
        print(f"  layer family N={N}: {len(ops)} gates", flush=True)
    return out


# ---------------------------------------------------- wide tensormul ----
def tensormul_wide_fixtures(qf, rng):
    """quantumflow/backend/numpybk.py:159-214 tensormul with K = 4..7 gate
    qubits (random complex gate tensors, not unitary) on states of N <= 10
    qubits, on scattered axes."""
    bk = qf.backend
    out = {}
    cases = [(6, 4), (8, 5), (9, 6), (10, 7), (7, 7)]
    for c, (N, K) in enumerate(cases):
        idx = rng.choice(N, size=K, replace=False)
        state = rng.normal(size=2 ** N) + 1j * rng.normal(size=2 ** N)
        gate = rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K))
        res = bk.tensormul(bk.astensorproduct(gate.reshape([2] * (2 * K))),
                           bk.astensorproduct(state), list(int(i) for i in idx))
        out[f"tw{c}_N"] = np.array(N)
        out[f"tw{c}_idx"] = np.array(idx)
        out[f"tw{c}_gate"] = gate
        out[f"tw{c}_state"] = state
        out[f"tw{c}_out"] = np.asarray(res).reshape(-1)
    out["tw_count"] = np.array(len(cases))
    return out


def main():
    qf = import_reference()
    rng = np.random.default_rng(20181203)
    files = {
        "kat.npz": lambda: kat_fixtures(qf),
        "gates.npz": lambda: gate_fixtures(qf),
        "tensormul.npz": lambda: tensormul_fixtures(qf, rng),
        "circuits.npz": lambda: circuit_fixtures(qf, rng),
        "qaoa.npz": lambda: qaoa_fixtures(qf, rng),
        "programs.npz": lambda: program_fixtures(qf, np.random.default_rng(20181204)),
        "channels.npz": lambda: channel_fixtures(qf, np.random.default_rng(20181205)),
        "layers.npz": lambda: layer_family_fixtures(qf, np.random.default_rng(20181206)),
        "tensormul_wide.npz": lambda: tensormul_wide_fixtures(qf, np.random.default_rng(20181207)),
    }
    only = set(sys.argv[1:])  # e.g. `programs` to rewrite programs.npz alone
    for fname, arrays in files.items():
        if only and fname[:-4] not in only:
            continue
        arrays = arrays()
        path = os.path.join(HERE, fname)
        np.savez_compressed(path, **arrays)
        print(f"wrote {fname}: {len(arrays)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
