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
