"""Adjoint gradient of QAOA MAXCUT against central finite differences of the
reference (tests/golden, computed by the reference's numpy backend) and of
the CPU oracle, plus torch.autograd and the gradient-ascent driver."""
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
    for name in ("c1", "reg8", "reg10", "er9"):
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


def test_c1_gradient_ascent_matches_reference(golden):
    """Config 1: 5 gradient-ascent steps at lr 0.1 from the golden angles."""
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    g = _graph(q, "c1")
    prob = qf.QAOAMaxCut(g, int(q["c1_p"]))
    beta, gamma = q["c1_beta"].copy(), q["c1_gamma"].copy()
    traj = []
    for _ in range(5):
        e, gb, gg = prob.expectation_and_grad(beta, gamma)
        beta, gamma = beta + 0.1 * gb, gamma + 0.1 * gg
        traj.append(prob.expectation(beta, gamma))
    np.testing.assert_allclose(traj, q["c1_gd_expectations"], atol=1e-7)


def test_maxcut_qaoa_star_graph():
    """tests/test_qaoa_maxcut.py:12-21: the 4-node star reaches ratio > 0.95
    (the reference runs this only on its TensorFlow backend)."""
    import quantumflow_gb300 as qf
    g = qf.Graph([(0, 1), (1, 2), (1, 3)])
    ratio, beta, gamma, hist = qf.maxcut_qaoa(g, steps=5, learning_rate=0.01, seed=0)
    assert ratio > 0.95
    assert beta is not None and gamma is not None
