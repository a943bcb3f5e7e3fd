"""Adjoint gradient of QAOA MAXCUT against central finite differences of the
reference (tests/golden, computed by the reference's numpy backend) and of
the CPU oracle, plus torch.autograd and the gradient-ascent loop (maxcut_qaoa)."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def _graph(q, name):
    import quantumflow_gb300 as qf
    g = qf.Graph(nodes=range(int(q[f"{name}_n"])))
    for (a, b) in q[f"{name}_edges"]:
        g.add_edge(int(a), int(b))
    return g


@pytest.mark.parametrize("dtype,tol", [("complex128", 2e-7), ("complex64", 2e-3)])
def test_adjoint_vs_reference_fd(golden, dtype, tol):
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    for name in ("er6p5", "reg8", "reg10", "er9", "reg16p8"):
        g = _graph(q, name)
        p = int(q[f"{name}_p"])
        prob = qf.QAOAMaxCut(g, p, dtype=dtype)
        e, gb, gg = prob.expectation_and_grad(q[f"{name}_beta"], q[f"{name}_gamma"])
        scale = max(1.0, np.max(np.abs(q[f"{name}_fd_grad_beta"])))
        assert abs(e - float(q[f"{name}_expectation"])) < tol * 10
        np.testing.assert_allclose(gb, q[f"{name}_fd_grad_beta"], atol=tol * scale)
        np.testing.assert_allclose(gg, q[f"{name}_fd_grad_gamma"], atol=tol * scale)


def test_adjoint_node_weights_vs_oracle_fd():
    import quantumflow_gb300 as qf
    n, p = 9, 3
    g = qf.qaoa.gnp_random_graph(n, 0.5, seed=4)
    g.nodes[2]["weight"] = 0.7
    g.nodes[6]["weight"] = -1.1
    nw = [g.nodes[q].get("weight", None) for q in range(n)]
    rng = np.random.default_rng(1)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    prob = qf.QAOAMaxCut(g, p)
    e, gb, gg = prob.expectation_and_grad(beta, gamma)
    fg, fb = orc.qaoa_fd_gradient(n, g.edges(), p, beta, gamma, 1e-6, None, nw)
    assert abs(e - orc.qaoa_expectation(n, g.edges(), p, beta, gamma, None, nw)) < 1e-10
    np.testing.assert_allclose(gb, fb, atol=2e-7)
    np.testing.assert_allclose(gg, fg, atol=2e-7)


@pytest.mark.parametrize("n,p", [(14, 4), (20, 6)])
def test_adjoint_vs_gpu_fd_and_uncompute(n, p):
    """Full-size property checks: gradient equals central differences of the
    GPU expectation, and the adjoint sweep leaves psi back at |+>^n."""
    import quantumflow_gb300 as qf
    g = qf.qaoa.random_regular_graph(3, n, seed=n)
    rng = np.random.default_rng(2)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    prob = qf.QAOAMaxCut(g, p)
    e, gb, gg = prob.expectation_and_grad(beta, gamma)
    assert abs(e - prob.expectation(beta, gamma)) < 1e-9
    psi = prob._grad_bufs[1]
    plus = qf.State(psi).asarray().reshape(-1)
    assert np.max(np.abs(plus - 2 ** (-n / 2))) < 1e-12
    h = 1e-5
    for i in (0, p - 1):
        for arr, grad in ((beta, gb), (gamma, gg)):
            a0 = arr[i]
            arr[i] = a0 + h
            ep = prob.expectation(beta, gamma)
            arr[i] = a0 - h
            em = prob.expectation(beta, gamma)
            arr[i] = a0
            assert abs((ep - em) / (2 * h) - grad[i]) < 1e-6 * max(1.0, abs(grad[i]))


def test_autograd_function():
    import quantumflow_gb300 as qf
    g = qf.qaoa.random_regular_graph(3, 10, seed=1)
    prob = qf.QAOAMaxCut(g, 3)
    beta = torch.tensor([0.3, 0.5, 0.7], dtype=torch.float64, requires_grad=True)
    gamma = torch.tensor([0.4, 0.2, 0.1], dtype=torch.float64, requires_grad=True)
    e = qf.QAOAExpectation.apply(beta, gamma, prob)
    (-e).backward()
    e2, gb, gg = prob.expectation_and_grad(beta.detach().numpy(), gamma.detach().numpy())
    assert abs(float(e) - e2) < 1e-12
    np.testing.assert_allclose(-beta.grad.numpy(), gb, atol=1e-12)
    np.testing.assert_allclose(-gamma.grad.numpy(), gg, atol=1e-12)


def test_er6p5_gradient_ascent_matches_reference(golden):
    """Config 1: 5 gradient-ascent steps at lr 0.1 from the golden angles."""
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    g = _graph(q, "er6p5")
    prob = qf.QAOAMaxCut(g, int(q["er6p5_p"]))
    beta, gamma = q["er6p5_beta"].copy(), q["er6p5_gamma"].copy()
    traj = []
    for _ in range(5):
        e, gb, gg = prob.expectation_and_grad(beta, gamma)
        beta, gamma = beta + 0.1 * gb, gamma + 0.1 * gg
        traj.append(prob.expectation(beta, gamma))
    np.testing.assert_allclose(traj, q["er6p5_gd_expectations"], atol=1e-7)


def test_maxcut_qaoa_star_graph():
    """tests/test_qaoa_maxcut.py:12-21: the 4-node star reaches ratio > 0.95
    (the reference runs this only on its TensorFlow backend)."""
    import quantumflow_gb300 as qf
    g = qf.Graph([(0, 1), (1, 2), (1, 3)])
    ratio, beta, gamma, hist = qf.maxcut_qaoa(g, steps=5, learning_rate=0.01, seed=0)
    assert ratio > 0.95
    assert beta is not None and gamma is not None


def test_weighted_graph_gradient_vs_reference_fd(golden):
    """Weighted edges and node weights (w7 case): generic circuit adjoint
    against the reference's finite differences."""
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    name = "w7"
    g = qf.Graph(nodes=range(int(q[f"{name}_n"])))
    for (a, b), w in zip(q[f"{name}_edges"], q[f"{name}_weights"]):
        g.add_edge(int(a), int(b), weight=float(w))
    for i, nw in enumerate(q[f"{name}_node_weights"]):
        if not np.isnan(nw):
            g.nodes[i]["weight"] = float(nw)
    prob = qf.QAOAMaxCut(g, int(q[f"{name}_p"]))
    e, gb, gg = prob.expectation_and_grad(q[f"{name}_beta"], q[f"{name}_gamma"])
    assert abs(e - float(q[f"{name}_expectation"])) < 1e-10
    np.testing.assert_allclose(gb, q[f"{name}_fd_grad_beta"], atol=2e-7)
    np.testing.assert_allclose(gg, q[f"{name}_fd_grad_gamma"], atol=2e-7)


def _param_circuit(theta):
    import quantumflow_gb300 as qf
    t = iter(theta)
    c = qf.Circuit()
    for q in range(5):
        c += qf.H(q)
    c += qf.RX(next(t), 0)
    c += qf.RY(next(t), 1)
    c += qf.RZ(next(t), 2)
    c += qf.ZZ(next(t), 0, 3)
    c += qf.XX(next(t), 1, 4)
    c += qf.YY(next(t), 2, 0)
    c += qf.CPHASE(next(t), 3, 1)
    c += qf.PHASE(next(t), 4)
    c += qf.TX(next(t), 2)
    c += qf.CAN(next(t), next(t), next(t), 1, 3)
    c += qf.PISWAP(next(t), 0, 4)
    c += qf.CNOT(4, 2)
    c += qf.RY(next(t), 3)
    return c


def test_generic_circuit_adjoint_vs_oracle_fd():
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(3)
    theta = rng.uniform(-1.5, 1.5, 14)
    diag = rng.uniform(0, 3, 32)
    circ = _param_circuit(theta)
    e, grads = qf.adjoint.expectation_and_grad(circ, diag)
    def energy(th):
        ops = [(g.asoperator(), tuple(g.qubits)) for g in _param_circuit(th)]
        return orc.expectation(orc.run_ops(orc.zero_state(5), ops), diag)
    assert abs(e - energy(theta)) < 1e-12
    # theta index -> (gate index, parameter name)
    keys = [(5, "theta"), (6, "theta"), (7, "theta"), (8, "t"), (9, "t"), (10, "t"), (11, "theta"),
            (12, "theta"), (13, "t"), (14, "tx"), (14, "ty"), (14, "tz"), (15, "theta"), (17, "theta")]
    assert set(keys) <= set(grads)
    h = 1e-6
    for k, key in enumerate(keys):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (energy(tp) - energy(tm)) / (2 * h)
        assert abs(grads[key] - fd) < 1e-7, (key, grads[key], fd)
    assert qf.adjoint.generator(qf.RN(0.3, 0.1, 0.2, 0.9), "nx") is None
    assert qf.adjoint.generator(qf.RN(0.3, 0.6, 0.0, 0.8), "theta") is not None


def test_circuit_expectation_autograd():
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(4)
    theta = torch.tensor(rng.uniform(-1, 1, 14), dtype=torch.float64, requires_grad=True)
    diag = rng.uniform(0, 3, 32)
    keys = [(5, "theta"), (6, "theta"), (7, "theta"), (8, "t"), (9, "t"), (10, "t"), (11, "theta"),
            (12, "theta"), (13, "t"), (14, "tx"), (14, "ty"), (14, "tz"), (15, "theta"), (17, "theta")]
    e = qf.adjoint.CircuitExpectation.apply(theta, _param_circuit, lambda c: [[(k, 1.0)] for k in keys], diag)
    e.backward()
    _, grads = qf.adjoint.expectation_and_grad(_param_circuit(theta.detach().numpy()), diag)
    np.testing.assert_allclose(theta.grad.numpy(), [grads[k] for k in keys], atol=1e-12)


@pytest.mark.parametrize("arith", ["ff", "fp64", "c64"])
@pytest.mark.parametrize("n", [7, 8, 9, 12, 15])
def test_warp_adjoint_equals_shared_memory_adjoint(n, arith, monkeypatch):
    """The warp-tile adjoint (default for n >= 5 + register bits), with each
    register-bit count it offers, agrees with the shared-memory adjoint
    kernel on graphs with node weights; both leave psi at |+>^n.  Covers
    the float-float, native FP64 and complex64 layouts."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    from quantumflow_gb300 import qaoa as qaoa_mod
    dtype = "complex64" if arith == "c64" else "complex128"
    if arith == "fp64":
        monkeypatch.setattr(qaoa_mod, "compute_layout", lambda d: nat.LAYOUT_C128)
    elif arith == "ff":
        monkeypatch.setattr(qaoa_mod, "compute_layout", lambda d: nat.LAYOUT_FF)
    p = 3
    g = qf.qaoa.gnp_random_graph(n, 0.45, seed=n)
    g.nodes[1]["weight"] = 0.4
    g.nodes[n - 2]["weight"] = -0.9
    rng = np.random.default_rng(n)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    results = {}
    modes = (1, 0, 2, 3) if dtype == "complex128" else (1, 0, 3, 4)
    try:
        for mode in modes:
            nat.call("qf_set_tile_kernel", mode)
            prob = qf.QAOAMaxCut(g, p, dtype=dtype)
            e, gb, gg = prob.expectation_and_grad(beta, gamma)
            results[mode] = np.concatenate([[e], gb, gg])
            plus = qf.State(prob._grad_bufs[1]).asarray().reshape(-1)
            assert np.max(np.abs(plus - 2 ** (-n / 2))) < (1e-12 if dtype == "complex128" else 1e-5)
    finally:
        nat.call("qf_set_tile_kernel", 0)
    tol = 1e-10 if dtype == "complex128" else 2e-4
    for mode in modes[1:]:
        np.testing.assert_allclose(results[mode], results[1], atol=tol * max(1.0, np.max(np.abs(results[1]))))
    if dtype == "complex128":
        nw = [g.nodes[q].get("weight", None) for q in range(n)]
        fg, fb = orc.qaoa_fd_gradient(n, g.edges(), p, beta, gamma, 1e-6, None, nw) if n <= 9 else (None, None)
        if fg is not None:
            np.testing.assert_allclose(results[0][1:1 + p], fb, atol=2e-7)
            np.testing.assert_allclose(results[0][1 + p:], fg, atol=2e-7)
