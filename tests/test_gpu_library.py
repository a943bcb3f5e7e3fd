"""Circuit library, DAG circuits and density measures on the GPU engine: the
checks the reference's own tests make (tests/test_dagcircuit.py,
tests/test_circuits.py, tests/test_measures.py of the reference) plus the
reference-computed QFT amplitudes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _test_circ(qf):
    circ = qf.Circuit()
    circ += qf.TY(1 / 2, 0)
    circ += qf.TX(1, 0)
    circ += qf.TY(1 / 2, 1)
    circ += qf.TX(1, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.TX(-1 / 2, 1)
    circ += qf.TY(4.71572463191 / np.pi, 1)
    circ += qf.TX(1 / 2, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.TX(-2 * 2.74973750579 / np.pi, 0)
    circ += qf.TX(-2 * 2.74973750579 / np.pi, 1)
    return circ


def test_dagcircuit(golden):
    import quantumflow_gb300 as qf
    assert qf.DAGCircuit([]).size() == 0
    dag = qf.DAGCircuit(_test_circ(qf))
    ket0 = qf.random_state(2)
    assert qf.states_close(ket0, dag.H.run(dag.run(ket0)))
    assert qf.states_close(dag.run(qf.zero_state(2)), qf.State(golden["kat"]["true_ket"].reshape(2, 2)))
    circ0 = qf.ghz_circuit(range(5))
    dag = qf.DAGCircuit(circ0)
    assert tuple(qf.Circuit(dag).qubits) == (0, 1, 2, 3, 4) and dag.qubits == circ0.qubits and dag.qubit_nb == 5
    assert dag.depth() == 5 and dag.depth(local=False) == 4 and len(dag.layers().elements) == dag.depth()
    assert qf.DAGCircuit(qf.qft_circuit([0, 1, 2, 3])).depth() == 8
    assert qf.gates_close(qf.ZYZ(0.1, 2.2, 0.5), qf.DAGCircuit(qf.zyz_circuit(0.1, 2.2, 0.5, 0)).asgate())
    rho0 = qf.random_state(3).asdensity()
    rho1 = qf.CCNOT(0, 1, 2).evolve(rho0)
    dag = qf.DAGCircuit(qf.ccnot_circuit([0, 1, 2]))
    assert qf.densities_close(rho1, dag.evolve(rho0))
    assert qf.densities_close(rho1, dag.aschannel().evolve(rho0))
    circ = qf.Circuit([qf.H(0), qf.H(1)])
    assert qf.DAGCircuit(circ).component_nb() == 2
    circ += qf.CNOT(0, 1)
    assert qf.DAGCircuit(circ).component_nb() == 1
    circ = qf.Circuit()
    circ.extend(qf.ghz_circuit([0, 2, 4, 6, 8]))
    circ.extend(qf.ghz_circuit([1, 3, 5, 7, 9]))
    assert qf.DAGCircuit(circ).component_nb() == 2
    circ.extend(qf.qft_circuit([0, 2, 4, 6]))
    circ.extend(qf.ghz_circuit([1, 3, 5, 7]))
    circ += qf.H(10)
    dag = qf.DAGCircuit(circ)
    assert dag.component_nb() == 3 and len(dag.components()) == 3
    circ = qf.ghz_circuit([0, 2, 4, 6, 8])
    elem = circ.elements[3]
    dag = qf.DAGCircuit(circ)
    assert dag.next_element(elem, elem.qubits[1]) is circ.elements[4]
    assert dag.prev_element(elem, elem.qubits[0]) is circ.elements[2]
    assert dag.next_element(elem, elem.qubits[0]) == ("out", 4)
    assert dag.prev_element(elem, elem.qubits[1]) == ("in", 6)


def test_circuit_library(golden):
    import quantumflow_gb300 as qf
    c = qf.Circuit([qf.X(2)])
    c.extend(qf.qft_circuit([0, 1, 2]))
    np.testing.assert_allclose(c.run(qf.zero_state(3)).asarray().reshape(-1), golden["kat"]["qft3"], atol=1e-8)
    assert qf.states_close(qf.ghz_circuit(range(6)).run(qf.zero_state(6)), qf.ghz_state(6))
    assert qf.gates_close(qf.ccnot_circuit([0, 1, 2]).asgate(), qf.CCNOT(0, 1, 2))
    # controlled-controlled-Z by the Barenco construction
    cz = qf.control_circuit([0, 1], qf.Z(2))
    assert qf.gates_close(cz.asgate(), qf.Gate(np.diag([1, 1, 1, 1, 1, 1, 1, -1]).astype(complex), [0, 1, 2]))
    # phase estimation of RZ(-4 pi phase): the output register reads the phase
    N, phase = 6, 1 / 4
    circ = qf.phase_estimation_circuit(qf.RZ(-4 * np.pi * phase, N), range(N))
    probs = circ.run(qf.zero_state(N + 1)).probabilities().cpu().numpy().reshape(2 ** N, 2)
    est = np.argmax(probs.sum(axis=1)) / 2 ** N
    assert est == phase
    # ripple-carry addition on basis states: addend1 <- addend0 + addend1
    a0, a1, carry = [0, 1], [2, 3], [4, 5]
    add = qf.addition_circuit(a0, a1, carry)
    for x, y in ((1, 2), (3, 3), (2, 1)):
        bits = [(x >> 1) & 1, x & 1, (y >> 1) & 1, y & 1, 0, 0]
        idx = int("".join(map(str, bits)), 2)
        out = add.run(qf.basis_state(6, idx)).probabilities().cpu().numpy().reshape(-1)
        res = int(np.argmax(out))
        rb = [int(b) for b in format(res, "06b")]
        total = (rb[2] << 1 | rb[3]) + (rb[5] << 2)
        assert total == x + y, (x, y, rb)


def test_density_measures():
    import quantumflow_gb300 as qf
    N = 3
    pure = qf.random_state(N).asdensity()
    mixed = qf.mixed_density(N)
    assert abs(qf.purity(pure) - 1) < 1e-12 and abs(qf.purity(mixed) - 1 / 2 ** N) < 1e-12
    assert abs(qf.fidelity(pure, pure) - 1) < 1e-8
    assert abs(qf.entropy(mixed) - N * np.log(2)) < 1e-10 and abs(qf.entropy(mixed, base=2) - N) < 1e-10
    assert abs(qf.entropy(pure)) < 1e-8
    bell = qf.ghz_circuit([0, 1]).run(qf.zero_state(2)).asdensity()
    assert abs(qf.mutual_info(bell, [0], [1]) - 2 * np.log(2)) < 1e-10
    assert qf.densities_close(pure, pure.permute(pure.qubits))
    assert qf.bures_angle(pure, pure) < 1e-4
    assert qf.channels_close(qf.Damping(0.2, 0).aschannel(), qf.Damping(0.2, 0).aschannel())
