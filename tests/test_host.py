"""Host-side logic (no GPU): gate matrices against the reference's, gate
algebra, circuit structure, QAOA circuit construction, graph generators."""
import numpy as np
import pytest

import quantumflow_gb300 as qf
from tests.conftest import load_golden

GATE_SPECS = [
    ("I", ()), ("X", ()), ("Y", ()), ("Z", ()), ("H", ()), ("S", ()), ("T", ()), ("S_H", ()),
    ("T_H", ()), ("PHASE", (0.1,)), ("RX", (0.2,)), ("RY", (0.3,)), ("RZ", (0.4,)), ("TX", (2.7,)),
    ("TY", (1.2,)), ("TZ", (0.3,)), ("TH", (0.3,)), ("ZYZ", (3.5, 0.9, 2.1)), ("RN", (0.7, 0.3, 0.4, 0.5)),
    ("CZ", ()), ("CNOT", ()), ("SWAP", ()), ("ISWAP", ()), ("CPHASE00", (0.5,)), ("CPHASE01", (0.6,)),
    ("CPHASE10", (0.6,)), ("CPHASE", (0.7,)), ("PSWAP", (0.15,)), ("PISWAP", (0.2,)), ("XX", (1.8,)),
    ("YY", (0.9,)), ("ZZ", (0.45,)), ("CAN", (0.1, 0.2, 0.3)), ("EXCH", (0.1,)), ("CCNOT", ()),
    ("CSWAP", ()),
]


@pytest.mark.parametrize("name,params", GATE_SPECS)
def test_gate_matrix_matches_reference(name, params):
    g = load_golden("gates.npz")
    gate = getattr(qf, name)(*params)
    np.testing.assert_allclose(gate.asoperator(), g["gate_" + name], atol=1e-14)
    np.testing.assert_allclose(gate.H.asoperator(), g["gateH_" + name], atol=1e-12)


def test_gate_algebra():
    for gate in (qf.RX(0.3), qf.ZZ(0.45), qf.CAN(0.1, 0.2, 0.3), qf.PHASE(0.4)):
        assert qf.gates_close(gate.H, gate ** -1)
        half = gate ** 0.5
        assert qf.gates_close(gate, half @ half)
    assert qf.almost_unitary(qf.random_gate(3))


def test_qubo_circuit_counts():
    # tests/test_qaoa.py:17-37 (13 and 15 elements)
    kat = load_golden("kat.npz")
    g = qf.Graph()
    g.add_edge(0, 1, weight=0.1)
    g.add_edge(1, 2, weight=0.4)
    assert len(qf.qubo_circuit(g, 2, [1, 1], [2, 2]).elements) == kat["qubo_counts"][0]
    g.nodes[0]["weight"] = 4
    assert len(qf.qubo_circuit(g, 2, [1, 1], [2, 2]).elements) == kat["qubo_counts"][1]


def test_circuit_structure():
    c = qf.Circuit()
    c += qf.TY(1 / 2, 0)
    c += qf.TX(1, 10)
    c += qf.CNOT(0, 4)
    assert c.qubits == (0, 4, 10)
    assert c.size() == 3
    assert [type(e).__name__ for e in c.H.elements] == ["CNOT", "TX", "TY"]
    op_k, op_axes, op_mats, nops = c.packed(c.qubits)
    assert list(op_k) == [1, 1, 2] and list(op_axes) == [0, 2, 0, 1] and nops == 3
    assert op_mats.size == 8 + 8 + 32


def test_graph_generators():
    g = qf.qaoa.random_regular_graph(3, 24, seed=5)
    assert g.number_of_nodes() == 24 and g.number_of_edges() == 36
    assert all(g.degree(q) == 3 for q in range(24))
    g2 = qf.qaoa.gnp_random_graph(20, 0.5, seed=1)
    assert 60 < g2.number_of_edges() < 130
    with pytest.raises(ValueError):
        qf.qaoa.random_regular_graph(3, 7)


def test_wave_plan_host_logic():
    """The multi-instance pass planner runs on the host only: pass counts
    1 + p (m - 1) per sweep (m register-bit groups), the output count, and
    the rejection of instances it cannot run."""
    import ctypes
    from quantumflow_gb300 import _native as nat
    from quantumflow_gb300.batched import _Instance
    inst = (_Instance * 2)(_Instance(20, 6, 30, 0, 0, 0), _Instance(16, 3, 24, 30, 12, 13))
    hb, db = ctypes.c_size_t(), ctypes.c_size_t()
    assert nat.lib.qf_wave_plan(ctypes.addressof(inst), 2, nat.LAYOUT_C64, None, 0,
                                ctypes.byref(hb), ctypes.byref(db)) == 0
    plan = np.zeros(hb.value, np.uint8)
    assert nat.lib.qf_wave_plan(ctypes.addressof(inst), 2, nat.LAYOUT_C64, plan.ctypes.data, hb.value,
                                None, None) == 0
    magic, layout, rbf, rba, ninst, nwaves, nfwd, nadj, nsegs, nout = plan[:40].view(np.int32)
    assert (layout, rbf, rba, ninst) == (nat.LAYOUT_C64, 4, 3, 2)
    # forward: n=20 -> 4 groups of <= 4 high bits: 1 + 6*3; n=16 -> 3 groups: 1 + 3*2
    # adjoint: n=20 -> 5 groups of <= 3: 1 + 6*4; n=16 -> 4 groups: 1 + 3*3
    assert nfwd == 19 + 7 and nadj == 25 + 10 and nwaves == max(19 + 25, 7 + 10)
    assert nout == (2 * 6 + 1) + (2 * 3 + 1)
    # the device workspace holds both states and the cut table of each instance
    assert db.value > (2 * 8 + 2) * (2 ** 20 + 2 ** 16)
    assert nat.lib.qf_wave_plan(ctypes.addressof(inst), 2, nat.LAYOUT_C64, plan.ctypes.data, 16,
                                None, None) == 8
    bad = (_Instance * 1)(_Instance(6, 2, 5, 0, 0, 0))  # below the warp tile
    assert nat.lib.qf_wave_plan(ctypes.addressof(bad), 1, nat.LAYOUT_C64, None, 0,
                                ctypes.byref(hb), ctypes.byref(db)) == 1
    bad = (_Instance * 1)(_Instance(12, 0, 5, 0, 0, 0))  # p = 0
    assert nat.lib.qf_wave_plan(ctypes.addressof(bad), 1, nat.LAYOUT_FF, None, 0,
                                ctypes.byref(hb), ctypes.byref(db)) == 1
    assert nat.lib.qf_wave_min_qubits(nat.LAYOUT_C64) == 9 and nat.lib.qf_wave_min_qubits(nat.LAYOUT_FF) == 8


def test_graph6_round_trip_and_networkx_agreement():
    """graph6 encoding (size prefixes up to 258047 nodes, upper-triangle bits
    column by column) round-trips, and matches networkx's encoder."""
    from quantumflow_gb300 import datasets
    graphs = [qf.qaoa.gnp_random_graph(n, 0.5, seed=n) for n in (1, 2, 6, 13, 32, 63, 70)]
    text = datasets.write_graph6(graphs)
    back = datasets.read_graph6(text)
    assert len(back) == len(graphs)
    for g, h in zip(graphs, back):
        assert len(h) == len(g)
        assert {tuple(sorted(e)) for e in g.edges()} == {tuple(sorted(e)) for e in h.edges()}
    one = datasets.read_graph6(datasets.write_graph6(graphs[2:3], header=True))
    assert len(one) == 6
    nx = pytest.importorskip("networkx")
    for g in graphs:
        G = nx.Graph()
        G.add_nodes_from(range(len(g)))
        G.add_edges_from(g.edges())
        assert nx.to_graph6_bytes(G, header=False).strip() == datasets.graph_to_graph6(g)
    assert len(datasets.load_stdgraphs(12)) == 100
    with pytest.raises(ValueError):
        datasets.load_stdgraphs(5)


def test_graph6_reads_reference_datasets():
    """The reference's own graph sets (quantumflow/datasets/data/*.g6) read
    the same as networkx reads them (runs where QF_REFERENCE names a
    reference checkout)."""
    import os
    from quantumflow_gb300 import datasets
    ref = os.environ.get("QF_REFERENCE", "")
    data = os.path.join(ref, "quantumflow", "datasets", "data")
    if not ref or not os.path.isdir(data):
        pytest.skip("reference datasets not present")
    nx = pytest.importorskip("networkx")
    for size in (6, 17, 32):
        ours = datasets.load_stdgraphs(size, path=data)
        theirs = nx.read_graph6(os.path.join(data, f"graph{size}er100.g6"))
        assert len(ours) == len(theirs) == 100
        for g, G in zip(ours, theirs):
            assert {tuple(sorted(e)) for e in g.edges()} == {tuple(sorted(e)) for e in G.edges()}


def test_plan_circuit_host_only():
    """The pass planner runs on the host: gate merging turns U.CZ.U of two
    random layers into one dense 2-qubit block per matched pair, and every
    high bit of a pass fits the warp tile."""
    import ctypes
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(1)
    N = 12
    circ = qf.Circuit()
    for layer in range(4):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))

    def plan(merge):
        nat.lib.qf_set_gate_merging(merge)
        stats = np.zeros(8 * 512, np.int32)
        nb = ctypes.c_int()
        rc = nat.lib.qf_plan_circuit(N, nat.LAYOUT_FF, nops, op_k.ctypes.data, op_axes.ctypes.data,
                                     op_mats.ctypes.data, 0, stats.ctypes.data, 512, ctypes.byref(nb))
        assert rc == 0
        return stats[:8 * nb.value].reshape(-1, 8)

    try:
        merged, plain = plan(1), plan(0)
    finally:
        nat.lib.qf_set_gate_merging(1)
    assert plain[:, 0].sum() == nops                 # every gate planned once
    assert merged[:, 0].sum() < nops                 # merging removed gates
    assert merged[:, 2].sum() >= N // 2                # dense 4x4 blocks from U.CZ.U
    assert len(merged) < len(plain)
    assert (merged[:, 6] <= 2).all() and set(merged[:, 7]) <= {0, 1, 2, 3, 4}
    # float-float fused passes of dense gates and CZ signs become shape passes
    # (kernel 4): one or two dense gates each, no other ops
    shape = merged[merged[:, 7] == 4]
    assert len(shape) > 0
    assert ((shape[:, 1] + shape[:, 2]) >= 1).all() and ((shape[:, 1] + shape[:, 2]) <= 2).all()
    assert (shape[:, 5] == 0).all()
    nat.lib.qf_set_tile_kernel(5)  # default order without group or shape passes
    try:
        assert not {3, 4} & set(plan(1)[:, 7])
    finally:
        nat.lib.qf_set_tile_kernel(0)
        nat.lib.qf_set_gate_merging(1)


def test_shape_width_splits_passes():
    """The shape-width setting (qf_set_shape_bits) decides where a fused
    float-float pass is cut: two 4x4 gates on four distinct lane bits are one
    four-bit shape pass at width 4, two single-gate passes at the default
    width 3, and one interpreted pass with shapes off (width 0)."""
    import ctypes
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    N = 12
    rng = np.random.default_rng(3)
    # axes N-1..N-4 are bits 0..3 (lane bits); CZs keep the gates unmerged
    circ = qf.Circuit([qf.random_gate([N - 1, N - 2], random_state=rng), qf.CZ(N - 1, 0),
                       qf.random_gate([N - 3, N - 4], random_state=rng)])
    op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))

    def plan():
        stats = np.zeros(8 * 64, np.int32)
        nb = ctypes.c_int()
        assert nat.lib.qf_plan_circuit(N, nat.LAYOUT_FF, nops, op_k.ctypes.data, op_axes.ctypes.data,
                                       op_mats.ctypes.data, 0, stats.ctypes.data, 64, ctypes.byref(nb)) == 0
        return stats[:8 * nb.value].reshape(-1, 8)

    try:
        assert nat.lib.qf_set_shape_bits(4) == 0
        wide = plan()
        assert len(wide) == 1 and wide[0, 7] == 4 and wide[0, 2] == 2
        assert nat.lib.qf_set_shape_bits(3) == 0
        default = plan()
        assert len(default) == 2 and set(default[:, 7]) <= {1, 4} and default[:, 2].sum() == 2
        assert nat.lib.qf_set_shape_bits(0) == 0
        off = plan()
        assert len(off) == 1 and off[0, 7] == 3  # the interpreted group kernel
        assert nat.lib.qf_set_shape_bits(5) != 0  # out of range
    finally:
        nat.lib.qf_set_shape_bits(3)


def test_gops_benchmark_circuit():
    """tools/benchmark.py's circuit: H on every qubit, then X, T, CNOT
    triples on random distinct qubit pairs (host only)."""
    from quantumflow_gb300 import benchmark as bm
    circ = list(bm.benchmark_circuit(16, 100, seed=1))
    assert len(circ) == 16 + 3 * 28
    assert [type(g).__name__ for g in circ[:16]] == ["H"] * 16
    for i in range(16, len(circ), 3):
        x, t, cnot = circ[i:i + 3]
        assert (type(x).__name__, type(t).__name__, type(cnot).__name__) == ("X", "T", "CNOT")
        assert cnot.qubits == (x.qubits[0], t.qubits[0]) and x.qubits != t.qubits


def test_shape_split_keeps_every_op():
    """Cutting fused passes into shapes only re-partitions the op list: over
    random programs, every shape width (0, 2, 3, 4) plans the same merged ops
    (same totals per op class), and no shape pass holds more than two dense
    gates."""
    import ctypes
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    N = 13
    rng = np.random.default_rng(11)
    try:
        for trial in range(12):
            circ = qf.Circuit()
            for _ in range(int(rng.integers(10, 60))):
                qs = [int(q) for q in rng.choice(N, 2, replace=False)]
                pick = rng.random()
                if pick < 0.35:
                    circ += qf.random_gate([qs[0]], random_state=rng)
                elif pick < 0.6:
                    circ += qf.random_gate(qs, random_state=rng)
                elif pick < 0.9:
                    circ += qf.CZ(*qs)
                else:
                    circ += qf.RZ(float(rng.uniform(0, 3)), qs[0])
            op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))
            totals = []
            for bits in (0, 2, 3, 4):
                assert nat.lib.qf_set_shape_bits(bits) == 0
                stats = np.zeros(8 * 512, np.int32)
                nb = ctypes.c_int()
                assert nat.lib.qf_plan_circuit(N, nat.LAYOUT_FF, nops, op_k.ctypes.data, op_axes.ctypes.data,
                                               op_mats.ctypes.data, 0, stats.ctypes.data, 512, ctypes.byref(nb)) == 0
                s = stats[:8 * nb.value].reshape(-1, 8)
                totals.append(tuple(s[:, :6].sum(0)))
                shape = s[s[:, 7] == 4]
                assert ((shape[:, 1] + shape[:, 2]) <= 2).all()
            assert len(set(totals)) == 1, totals
    finally:
        nat.lib.qf_set_shape_bits(3)


def test_backend_module_interface():
    """``qf.backend`` exposes the reference backend-module names
    (quantumflow/backend/__init__.py:25-35) as the reference package does."""
    import quantumflow_gb300 as qf
    required = ["tensormul", "inner", "outer", "astensor", "astensorproduct", "evaluate", "rank", "size",
                "reshape", "transpose", "conj", "absolute", "real", "imag", "sum", "matmul", "diag", "trace",
                "productdiag", "getitem", "ccast", "fcast", "cis", "exp", "cos", "sin", "sqrt", "arccos",
                "minimum", "einsum", "set_random_seed", "gpu_available", "TL", "CTYPE", "FTYPE", "TENSOR",
                "DEVICE", "MAX_QUBITS", "EINSUM_SUBSCRIPTS", "BKTensor", "TensorLike", "name", "version"]
    missing = [n for n in required if not hasattr(qf.backend, n)]
    assert not missing, missing
    assert qf.backend.MAX_QUBITS >= 32


def test_state_cbits_from_memory():
    """State.cbits / cbit_nb (quantumflow/states.py:88-97): the sorted BIT
    addresses of the classical memory (host only: they read the memory
    dict, not the amplitudes)."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300.states import State
    ro = qf.Register("ro")
    re = qf.Register("re", "REAL")
    st = State.__new__(State)
    st._memory = {ro[1]: 1, re[0]: 0.5, ro[0]: 0}
    assert st.cbits == (ro[0], ro[1])
    assert st.cbit_nb == 2
    st._memory = {}
    assert st.cbits == () and st.cbit_nb == 0


def test_bench_workload_definition():
    """The benchmark's random-layer circuit: per layer a unitary 2x2 on every
    qubit, then CZ on a perfect matching of all qubits; seeded and
    deterministic; N=28 x 100 layers = 4200 gates."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    N, L = 28, 3
    ops = bench.c2_circuit_ops(N, L, 2018)
    again = bench.c2_circuit_ops(N, L, 2018)
    assert len(ops) == L * (N + N // 2)
    for layer in range(L):
        chunk = ops[layer * (N + N // 2):(layer + 1) * (N + N // 2)]
        ones, czs = chunk[:N], chunk[N:]
        assert [qs for _, qs, _ in ones] == [(q,) for q in range(N)]
        for kind, qs, u in ones:
            assert kind == 1 and np.allclose(u @ u.conj().T, np.eye(2), atol=1e-12)
        assert all(kind == 2 for kind, _, _ in czs)
        assert sorted(q for _, qs, _ in czs for q in qs) == list(range(N))  # a perfect matching
    for (k1, q1, u1), (k2, q2, u2) in zip(ops, again):
        assert k1 == k2 and q1 == q2 and (u1 is None and u2 is None or np.array_equal(u1, u2))
    assert len(bench.c2_circuit_ops(N, 100, 2018)) == 4200
