"""The CPU oracle against the reference's own outputs (tests/golden, made by
running the reference) and the literal known answers of its test suite."""
import numpy as np
import pytest

from oracle import qf_oracle as orc


def test_tensormul_matches_reference(golden):
    g = golden["tensormul"]
    for c in range(int(g["tm_count"])):
        out = orc.tensormul(g[f"tm{c}_gate"], g[f"tm{c}_state"], list(g[f"tm{c}_idx"]))
        np.testing.assert_allclose(out.reshape(-1), g[f"tm{c}_out"], rtol=0, atol=1e-12)


def test_tensormul_planar_matches_reference(golden):
    """The torch backend's permute + matmul tensormul (the multi-threaded CPU
    baseline) against the same reference outputs."""
    g = golden["tensormul"]
    for c in range(int(g["tm_count"])):
        st = g[f"tm{c}_state"]
        out = orc.tensormul_planar(g[f"tm{c}_gate"], orc.planar(st), [int(i) for i in g[f"tm{c}_idx"]])
        np.testing.assert_allclose(orc.from_planar(out).reshape(-1), g[f"tm{c}_out"], rtol=0, atol=1e-12)


def test_kat_true_ket():
    # tests/test_circuits.py:43-60 circuit, KAT amplitudes from
    # tests/test_circuits.py:19-24 (referenceQVM)
    import quantumflow_gb300.stdgates as sg
    from math import pi
    ops = [(sg.RY(pi / 2).asoperator(), (0,)), (sg.RX(pi).asoperator(), (0,)),
           (sg.RY(pi / 2).asoperator(), (1,)), (sg.RX(pi).asoperator(), (1,)),
           (orc.CNOT(), (0, 1)), (sg.RX(-pi / 2).asoperator(), (1,)),
           (sg.RY(4.71572463191).asoperator(), (1,)), (sg.RX(pi / 2).asoperator(), (1,)),
           (orc.CNOT(), (0, 1)), (sg.RX(-2 * 2.74973750579).asoperator(), (0,)),
           (sg.RX(-2 * 2.74973750579).asoperator(), (1,))]
    from tests.conftest import load_golden
    kat = load_golden("kat.npz")
    st = orc.run_ops(orc.zero_state(2), ops).reshape(-1)
    np.testing.assert_allclose(st, kat["true_ket_ref_run"], atol=1e-13)
    # the literal KAT is printed to ~1e-8 precision
    assert orc.fidelity(st, kat["true_ket"] / np.linalg.norm(kat["true_ket"])) > 1 - 1e-12


def test_graph_cuts_literals(golden):
    kat = golden["kat"]
    # tests/test_qaoa.py:40-55
    np.testing.assert_allclose(orc.graph_cuts(3, [(0, 1), (1, 2)]).reshape(-1), kat["cuts_unweighted"])
    np.testing.assert_allclose(
        orc.graph_cuts(3, [(0, 1), (1, 2), (0, 2)], [0.1, 0.4, 0.35]).reshape(-1), kat["cuts_weighted"])


def test_qaoa_against_reference(golden):
    q = golden["qaoa"]
    for name in q["qaoa_cases"]:
        n, p = int(q[f"{name}_n"]), int(q[f"{name}_p"])
        edges = [tuple(e) for e in q[f"{name}_edges"]]
        w = q[f"{name}_weights"]
        nw = [None if np.isnan(v) else float(v) for v in q[f"{name}_node_weights"]]
        beta, gamma = q[f"{name}_beta"], q[f"{name}_gamma"]
        cuts = orc.graph_cuts(n, edges, w)
        st = orc.run_ops(orc.zero_state(n), orc.qubo_ops(n, edges, p, beta, gamma, w, nw))
        if f"{name}_state" in q:
            np.testing.assert_allclose(cuts.reshape(-1), q[f"{name}_cuts"], atol=1e-12)
            np.testing.assert_allclose(st.reshape(-1), q[f"{name}_state"], atol=1e-12)
        e = orc.expectation(st, cuts)
        assert abs(e - float(q[f"{name}_expectation"])) < 1e-10
        ops = orc.qubo_ops(n, edges, p, beta, gamma, w, nw)
        assert len(ops) == int(q[f"{name}_nelements"])
        if f"{name}_fd_grad_gamma" in q and n <= 8:
            gg, gb = orc.qaoa_fd_gradient(n, edges, p, beta, gamma, 1e-6, w, nw)
            np.testing.assert_allclose(gg, q[f"{name}_fd_grad_gamma"], atol=1e-6)
            np.testing.assert_allclose(gb, q[f"{name}_fd_grad_beta"], atol=1e-6)


def test_random_layer_circuits(golden):
    c = golden["circuits"]
    for N in (4, 6, 9, 12):
        ops = orc.cz_layer_ops(c[f"rc{N}_ops"], c[f"rc{N}_u"])
        st = orc.run_ops(orc.zero_state(N), ops).reshape(-1)
        np.testing.assert_allclose(st, c[f"rc{N}_state"], atol=1e-12)


def test_er6p5_gradient_ascent(golden):
    # examples/qaoa_maxcut.py:37-87 semantics with FD gradients, lr 0.1, 5 steps
    q = golden["qaoa"]
    n, p = int(q["er6p5_n"]), int(q["er6p5_p"])
    edges = [tuple(e) for e in q["er6p5_edges"]]
    beta, gamma = q["er6p5_beta"].copy(), q["er6p5_gamma"].copy()
    traj = []
    for _ in range(5):
        gg, gb = orc.qaoa_fd_gradient(n, edges, p, beta, gamma)
        gamma, beta = gamma + 0.1 * gg, beta + 0.1 * gb
        traj.append(orc.qaoa_expectation(n, edges, p, beta, gamma))
    np.testing.assert_allclose(traj, q["er6p5_gd_expectations"], atol=1e-8)


def test_oracle_matches_reference_programs(golden):
    """Seeded Call programs run by the reference's Program.run reproduce in
    the oracle; the literal amplitudes of its program test agree too."""
    g = golden["programs"]
    for case in range(3):
        nq = int(g[f"p{case}_nq"])
        ops = orc.program_ops(g[f"p{case}_names"], g[f"p{case}_params"], g[f"p{case}_qubits"])
        st = orc.run_ops(orc.zero_state(nq), ops).reshape(-1)
        assert np.max(np.abs(st - g[f"p{case}_state"])) < 1e-12
    np.testing.assert_allclose(g["wf_true"], golden["kat"]["true_ket"], atol=1e-12)


def _channel_steps(c):
    """(superop, axes) of each fixture step, built from the published channel
    definitions (quantumflow/channels.py:128-166)."""
    I2, X, Y, Z = np.eye(2), orc.X(), np.array([[0, -1j], [1j, 0]]), np.diag([1.0, -1.0])
    def damp(p):
        return orc.kraus_superop([np.array([[1, 0], [0, np.sqrt(1 - p)]]), np.array([[0, np.sqrt(p)], [0, 0]])])
    def depol(p):
        return orc.kraus_superop([I2, X, Y, Z], [1 - p, p / 3, p / 3, p / 3])
    def deph(p):
        return orc.kraus_superop([I2, Z], [1 - p / 2, p / 2])
    u1, u2 = c["u1"], c["u2"]
    # Gate(u2, qubits=[3, 0]): matrix MSB on qubit 3
    return [
        ("gate1", orc.gate_superop(u1), [2]),
        ("gate2", orc.gate_superop(u2), [3, 0]),
        ("damping", damp(0.3), [1]),
        ("depolarizing", depol(0.2), [3]),
        ("dephasing", deph(0.45), [0]),
        ("kraus2", orc.kraus_superop([u2 * np.sqrt(0.7), np.eye(4) * np.sqrt(0.3)]), [1, 2]),
        ("chan_matmul", damp(0.1) @ deph(0.2), [2]),
    ]


def test_oracle_matches_reference_channels(golden):
    """Density evolution by superoperators in the oracle reproduces the
    reference's Gate.evolve / Kraus channels / channel composition."""
    c = golden["channels"]
    rho = c["rho0"]
    for name, sop, axes in _channel_steps(c):
        rho = orc.evolve_density(rho, sop, axes)
        assert np.max(np.abs(rho - c[f"after_{name}"])) < 1e-12, name
    np.testing.assert_allclose(orc.kraus_superop([np.array([[1, 0], [0, np.sqrt(0.7)]]),
                                                  np.array([[0, np.sqrt(0.3)], [0, 0]])]),
                               c["damping_superop"], atol=1e-15)
    ket = c["ket"]
    np.testing.assert_allclose(np.outer(ket, ket.conj()), c["ket_density"], atol=1e-15)


def test_layer_family_n16_matches_reference():
    """The benchmark's circuit family at N=16, all 100 layers (2400 gates),
    against the reference's Circuit.run output."""
    from tests.conftest import load_golden
    lf = load_golden("layers.npz")
    ops = orc.layer_family_ops(lf["lf16_u"], lf["lf16_pairs"])
    assert len(ops) == 2400
    st = orc.run_ops(orc.zero_state(16), ops).reshape(-1)
    np.testing.assert_allclose(st, lf["lf16_state"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(st[lf["lf16_idx"]], lf["lf16_amps"], rtol=0, atol=1e-13)


def test_tensormul_wide_matches_reference():
    """tensormul with K = 4..7 gate qubits (numpybk.py:159-214) against the
    reference's outputs."""
    from tests.conftest import load_golden
    g = load_golden("tensormul_wide.npz")
    for c in range(int(g["tw_count"])):
        out = orc.tensormul(g[f"tw{c}_gate"], g[f"tw{c}_state"], [int(i) for i in g[f"tw{c}_idx"]])
        np.testing.assert_allclose(out.reshape(-1), g[f"tw{c}_out"], rtol=0, atol=1e-11)
