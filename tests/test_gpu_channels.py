"""Density matrices and channels on the GPU engine against the reference's
own results (tests/golden/channels.npz, computed by the reference's
Gate.evolve, Kraus channels and Density methods) and against pure-state
runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _steps(qf, c):
    return [
        ("gate1", qf.Gate(c["u1"], qubits=[2])),
        ("gate2", qf.Gate(c["u2"], qubits=[3, 0])),
        ("damping", qf.Damping(0.3, 1)),
        ("depolarizing", qf.Depolarizing(0.2, 3)),
        ("dephasing", qf.Dephasing(0.45, 0)),
        ("kraus2", qf.Kraus([qf.Gate(c["u2"] * np.sqrt(0.7), qubits=[1, 2]),
                             qf.Gate(np.eye(4) * np.sqrt(0.3), qubits=[1, 2])])),
        ("chan_matmul", qf.Damping(0.1, 2).aschannel() @ qf.Dephasing(0.2, 2).aschannel()),
        ("joined", qf.join_channels(qf.Damping(0.25, 0).aschannel(), qf.Depolarizing(0.15, 3).aschannel())),
    ]


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 2e-6)])
def test_density_evolution_vs_reference(golden, dtype, tol):
    import quantumflow_gb300 as qf
    c = golden["channels"]
    rho = qf.Density(c["rho0"].reshape([2] * 8), dtype=dtype)
    assert rho.qubits == (0, 1, 2, 3) and rho.qubit_nb == 4
    for name, op in _steps(qf, c):
        rho = op.evolve(rho)
        got = rho.asoperator().cpu().numpy()
        assert np.max(np.abs(got - c[f"after_{name}"])) < tol, name
    assert abs(rho.trace() - complex(c["trace_final"])) < tol * 10
    np.testing.assert_allclose(rho.probabilities().cpu().numpy().reshape(-1), c["probs_final"].real, atol=tol)
    pt = rho.partial_trace([1, 3])
    assert pt.qubits == (0, 2)
    np.testing.assert_allclose(pt.asoperator().cpu().numpy(), c["ptrace_13"], atol=tol * 10)


def test_density_constructors_and_channel_algebra(golden):
    import quantumflow_gb300 as qf
    c = golden["channels"]
    ket = qf.State(c["ket"].reshape(2, 2, 2))
    np.testing.assert_allclose(ket.asdensity().asoperator().cpu().numpy(), c["ket_density"], atol=1e-15)
    np.testing.assert_allclose(qf.mixed_density(3).asoperator().cpu().numpy(), c["mixed3"], atol=1e-15)
    np.testing.assert_allclose(qf.Damping(0.3, 0).aschannel().tensor.reshape(4, 4), c["damping_superop"],
                               atol=1e-15)
    assert qf.kraus_iscomplete(qf.Damping(0.2, 0)) and qf.kraus_iscomplete(qf.Depolarizing(0.3, 1))
    # Kraus -> superoperator -> Kraus -> superoperator is stable
    chan = qf.Depolarizing(0.3, 0).aschannel()
    back = qf.channel_to_kraus(chan).aschannel()
    np.testing.assert_allclose(back.tensor, chan.tensor, atol=1e-12)
    np.random.seed(1)
    r = qf.random_density(3)
    assert abs(r.trace() - 1) < 1e-12
    m = r.asoperator().cpu().numpy()
    assert np.allclose(m, m.conj().T) and np.min(np.linalg.eigvalsh(m)) > -1e-12
    j = qf.join_densities(qf.mixed_density([0]), qf.Density(c["ket_density"].reshape([2] * 6), [1, 2, 3]))
    assert j.qubits == (0, 1, 2, 3) and abs(j.trace() - 1) < 1e-12


@pytest.mark.parametrize("N", [5, 9])
def test_circuit_evolve_equals_pure_state_run(N):
    """For pure states Circuit.evolve(|psi><psi|) == |C psi><C psi|; the
    gates run as one fused launch on the ket and bra axes."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(N)
    circ = qf.Circuit()
    for _ in range(3):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        circ += qf.CNOT(0, N - 1)
        circ += qf.random_gate([1, N - 2], random_state=rng)
    ket = circ.run(qf.zero_state(N))
    rho = circ.evolve(qf.zero_state(N).asdensity())
    ref = ket.asdensity().asoperator().cpu().numpy()
    assert np.max(np.abs(rho.asoperator().cpu().numpy() - ref)) < 1e-12
    # default initial density and a channel in the middle
    circ2 = qf.Circuit([qf.H(0), qf.Damping(1.0, 0), qf.X(1)])
    out = circ2.evolve()
    probs = out.probabilities().cpu().numpy()
    assert abs(probs[0, 1] - 1) < 1e-12


def test_program_evolve_and_measure_density():
    import quantumflow_gb300 as qf
    ro = qf.Register()
    prog = qf.Program()
    prog += qf.Call("X", [], [0])
    prog += qf.Call("CNOT", [], [0, 1])
    prog += qf.Measure(1, ro[0])
    prog += qf.Not(ro[1])
    rho = prog.evolve()
    assert isinstance(rho, qf.Density)
    assert rho.memory[ro[0]] == 1 and rho.memory[ro[1]] == 1
    assert abs(rho.probabilities().cpu().numpy()[1, 1] - 1) < 1e-12
    with pytest.raises(TypeError):
        qf.Reset(0).evolve(rho)
