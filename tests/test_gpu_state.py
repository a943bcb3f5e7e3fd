"""GPU State operations: probabilities, norm, inner, expectation, sampling,
measurement, constructors (quantumflow/states.py)."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def test_expectation_literals(golden):
    # tests/test_gates.py:150-164 literals 42 and 2.5
    import quantumflow_gb300 as qf
    lit = golden["kat"]["expectation_literals"]
    M = np.zeros([2] * 4)
    M[0, 0, 0, 0] = 42
    M[1, 0, 0, 0] = 1
    M[0, 1, 0, 0] = 2
    M[0, 0, 1, 0] = 3
    M[0, 0, 0, 1] = 4
    assert qf.zero_state(4).expectation(M) == lit[0]
    assert abs(qf.w_state(4).expectation(M) - lit[1]) < 1e-14


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_reductions_against_oracle(dtype):
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(5)
    tol = 1e-12 if dtype == "complex128" else 1e-6
    for n in (1, 3, 10, 18):
        a = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        b = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
        sa, sb = qf.State(a, dtype=dtype), qf.State(b, dtype=dtype)
        a_ = a.astype(np.complex64) if dtype == "complex64" else a
        b_ = b.astype(np.complex64) if dtype == "complex64" else b
        assert abs(sa.norm() - orc.norm(a_)) < tol * orc.norm(a_)
        assert abs(qf.inner(sa, sb) - orc.inner(a_, b_)) < tol * 2 ** (n / 2) * 10
        np.testing.assert_allclose(sa.probabilities().cpu().numpy().reshape(-1),
                                   orc.probabilities(a_).reshape(-1), rtol=tol * 10, atol=0)
        d = rng.normal(size=2 ** n)
        assert abs(sa.expectation(d) - orc.expectation(a_, d)) < tol * 10 * orc.norm(a_)


def test_ff_layout_reductions():
    """Reductions read the float-float buffer directly (no conversion)."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(6)
    n = 12
    a = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    a /= np.linalg.norm(a)
    st = qf.State(qf.Buffer.from_complex(torch.from_numpy(a).cuda()).to_layout(2))
    assert abs(st.norm() - 1) < 1e-13
    d = rng.uniform(size=2 ** n)
    assert abs(st.expectation(d) - orc.expectation(a, d)) < 1e-13


def test_sample_and_measure():
    import quantumflow_gb300 as qf
    ket = qf.zero_state(2)
    ket = qf.H(0).run(ket)
    ket = qf.CNOT(0, 1).run(ket)
    counts = ket.sample(10)
    assert counts.sum() == 10  # tests/test_states.py:124-130
    assert counts[0, 1] == 0 and counts[1, 0] == 0
    for _ in range(16):  # tests/test_states.py:108-121
        res = ket.measure()
        assert res[0] == res[1]
    assert np.allclose(qf.zero_state(2).measure(), [0, 0])
    assert np.allclose(qf.X(0).run(qf.zero_state(2)).measure(), [1, 0])
    # statistics: 200k draws from a random 6-qubit state
    rng = np.random.default_rng(8)
    a = rng.normal(size=64) + 1j * rng.normal(size=64)
    st = qf.State(a / np.linalg.norm(a))
    trials = 200000
    c = st.sample(trials, seed=1234).reshape(-1)
    p = orc.probabilities(a / np.linalg.norm(a)).reshape(-1)
    chi2 = np.sum((c - trials * p) ** 2 / (trials * p))
    assert c.sum() == trials
    assert chi2 < 150  # 63 degrees of freedom; p-value ~1e-8 at 150
    ket = qf.H(0).run(qf.zero_state(1))
    assert abs(ket.expectation([0.4, 0.6]) - 0.5) < 1e-12
    assert abs(ket.expectation([0.4, 0.6], 4000) - 0.5) < 0.02


def test_constructors_and_normalize():
    import quantumflow_gb300 as qf
    ghz = qf.ghz_state(3).asarray().reshape(-1)
    assert abs(ghz[0] - 2 ** -0.5) < 1e-15 and abs(ghz[7] - 2 ** -0.5) < 1e-15
    r = qf.random_state(5)
    assert abs(r.norm() - 1) < 1e-13
    u = qf.uniform_state(4).asarray().reshape(-1)
    np.testing.assert_allclose(u, np.full(16, 0.25), atol=1e-15)
    j = qf.join_states(qf.zero_state([0]), qf.X(1).run(qf.zero_state([1])))
    assert j.qubits == (0, 1) and abs(j.asarray().reshape(-1)[1] - 1) < 1e-15
    p = qf.State(np.arange(8)).permute([2, 1, 0]).asarray()
    np.testing.assert_allclose(p, np.arange(8).reshape(2, 2, 2).transpose(2, 1, 0))


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_upload_run_download_pipelined(dtype):
    """upload_state / State.to_host on the copy streams: several steps in
    flight at once (each step's upload overlapping the previous circuit,
    each download overlapping the next) give the same amplitudes as the
    oracle, step by step, with distinct inputs per step."""
    import quantumflow_gb300 as qf
    N, steps = 12, 4
    rng = np.random.default_rng(31)
    circ = qf.Circuit()
    for layer in range(2):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(a, a + 1)
    ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
    cdt = torch.complex128 if dtype == "complex128" else torch.complex64
    ins, outs, copies = [], [], []
    for s in range(steps):
        v = rng.normal(size=2 ** N) + 1j * rng.normal(size=2 ** N)
        v /= np.linalg.norm(v)
        ins.append(torch.from_numpy(v).to(cdt).pin_memory())
        outs.append(torch.empty(2 ** N, dtype=cdt).pin_memory())
    for s in range(steps):
        ket = circ.run(qf.upload_state(ins[s], dtype=dtype))
        copies.append(ket.to_host(outs[s]))
        del ket
    tol = 1e-12 if dtype == "complex128" else 2e-5
    for s in range(steps):
        got = copies[s].result()
        assert got.shape == (2,) * N
        assert got.data_ptr() == outs[s].data_ptr()
        ref = orc.run_ops(ins[s].numpy().astype(np.complex128).reshape([2] * N), ops)
        assert np.max(np.abs(got.numpy() - ref)) < tol
    # a download into a freshly allocated pinned buffer
    ket = qf.upload_state(ins[0].numpy(), dtype=dtype)
    copy = ket.to_host()
    assert copy.tensor.is_pinned()
    np.testing.assert_array_equal(copy.result().numpy().reshape(-1), ins[0].numpy())
    with pytest.raises(ValueError):
        ket.to_host(torch.empty(2 ** N + 1, dtype=cdt))
    with pytest.raises(ValueError):
        qf.upload_state(ins[0].cuda())


def test_state_and_density_memory():
    """Classical memory through updates, gates and channels
    (tests/test_states.py:205-240 of the reference)."""
    import quantumflow_gb300 as qf
    ket0 = qf.zero_state(1)
    assert ket0.memory == {}
    ro = qf.Register("ro")
    ket1 = ket0.update({ro[1]: 1})
    assert ket0.memory == {}
    assert ket1.memory == {ro[1]: 1}
    assert ket1.cbit_nb == 1
    assert ket1.cbits == (ro[1],)
    ket2 = qf.H(0).run(ket1)
    assert ket2.memory == ket1.memory
    ket3 = ket2.update({ro[1]: 0, ro[0]: 0})
    assert ket3.memory == {ro[0]: 0, ro[1]: 0}
    assert ket3.cbits == (ro[0], ro[1])

    rho0 = qf.zero_state(1).asdensity()
    assert rho0.memory == {}
    rho1 = rho0.update({ro[1]: 1})
    assert rho0.memory == {}
    assert rho1.memory == {ro[1]: 1}
    assert rho1.cbit_nb == 1
    assert rho1.cbits == (ro[1],)
    rho2 = qf.H(0).aschannel().evolve(rho1)
    assert rho2.memory == rho1.memory
    rho3 = qf.X(0).evolve(rho1)
    assert rho3.memory == rho1.memory
