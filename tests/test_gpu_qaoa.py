"""GPU parity of the QAOA path (quantumflow/qaoa.py) against the reference's
own outputs: cut tables, QAOA states, expectations."""
import numpy as np
import pytest

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def _graph(q, name):
    import quantumflow_gb300 as qf
    g = qf.Graph(nodes=range(int(q[f"{name}_n"])))
    for (a, b), w in zip(q[f"{name}_edges"], q[f"{name}_weights"]):
        if w == 1.0:
            g.add_edge(int(a), int(b))
        else:
            g.add_edge(int(a), int(b), weight=float(w))
    for i, nw in enumerate(q[f"{name}_node_weights"]):
        if not np.isnan(nw):
            g.nodes[i]["weight"] = float(nw)
    return g


def test_graph_cuts_literals(golden):
    import quantumflow_gb300 as qf
    kat = golden["kat"]
    g = qf.Graph([(0, 1), (1, 2)])
    np.testing.assert_allclose(qf.graph_cuts(g).cpu().numpy().reshape(-1), kat["cuts_unweighted"])
    g = qf.Graph()
    g.add_edge(0, 1, weight=0.1)
    g.add_edge(1, 2, weight=0.4)
    g.add_edge(0, 2, weight=0.35)
    np.testing.assert_allclose(qf.graph_cuts(g).cpu().numpy().reshape(-1), kat["cuts_weighted"], atol=1e-15)


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-5)])
@pytest.mark.parametrize("path", ["fast", "circuit"])
def test_qaoa_cases(golden, dtype, tol, path):
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    for name in q["qaoa_cases"]:
        if f"{name}_state" not in q:
            continue
        g = _graph(q, name)
        p = int(q[f"{name}_p"])
        beta, gamma = q[f"{name}_beta"], q[f"{name}_gamma"]
        prob = qf.QAOAMaxCut(g, p, dtype=dtype)
        np.testing.assert_allclose(prob.cuts.cpu().numpy(), q[f"{name}_cuts"], atol=1e-12)
        if path == "fast":
            st = prob.state(beta, gamma)
            e = prob.expectation(beta, gamma)
        else:
            zero = qf.zero_state(prob.n, dtype=dtype)
            st = qf.qubo_circuit(g, p, beta, gamma).run(zero)
            e = st.expectation(qf.graph_cuts(g))
        err = np.max(np.abs(st.asarray().reshape(-1) - q[f"{name}_state"]))
        assert err < tol, (name, err)
        assert abs(e - float(q[f"{name}_expectation"])) < tol * 100, (name, e)


def test_qaoa_large_against_oracle():
    import quantumflow_gb300 as qf
    n, p = 16, 3
    g = qf.qaoa.random_regular_graph(3, n, seed=3)
    rng = np.random.default_rng(0)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    prob = qf.QAOAMaxCut(g, p)
    st = prob.state(beta, gamma).asarray().reshape(-1)
    ref = orc.run_ops(orc.zero_state(n), orc.qubo_ops(n, g.edges(), p, beta, gamma)).reshape(-1)
    assert np.max(np.abs(st - ref)) < 1e-12
    cuts = orc.graph_cuts(n, g.edges())
    assert abs(prob.expectation(beta, gamma) - orc.expectation(ref, cuts)) < 1e-10
    assert prob.maxcut == cuts.max()


@pytest.mark.parametrize("arith", ["ff", "fp64", "c64"])
@pytest.mark.parametrize("n,p", [(7, 2), (8, 3), (9, 4), (10, 1), (13, 3), (16, 2)])
def test_warp_qaoa_state_vs_engine_and_oracle(n, p, arith, monkeypatch):
    """The warp-tile QAOA forward kernel (default; merged layer boundaries,
    |+>^n generated in the first pass), at each register-bit count, equals
    the shared-memory engine path and the oracle, with node weights."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    from quantumflow_gb300 import qaoa as qaoa_mod
    dtype = "complex64" if arith == "c64" else "complex128"
    if arith != "c64":
        layout = nat.LAYOUT_C128 if arith == "fp64" else nat.LAYOUT_FF
        monkeypatch.setattr(qaoa_mod, "compute_layout", lambda d: layout)
    g = qf.qaoa.gnp_random_graph(n, 0.5, seed=n + p)
    g.nodes[0]["weight"] = 0.3
    g.nodes[n - 1]["weight"] = -1.3
    rng = np.random.default_rng(n * p)
    beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
    nw = [g.nodes[q].get("weight", None) for q in range(n)]
    ref = orc.run_ops(orc.zero_state(n), orc.qubo_ops(n, g.edges(), p, beta, gamma, None, nw)).reshape(-1)
    tol = 1e-5 if dtype == "complex64" else 1e-12
    modes = (0, 1, 2, 3) if dtype == "complex128" else (0, 1, 3, 4)
    try:
        for mode in modes:
            nat.call("qf_set_tile_kernel", mode)
            prob = qf.QAOAMaxCut(g, p, dtype=dtype)
            st = prob.state(beta, gamma).asarray().reshape(-1)
            assert np.max(np.abs(st - ref)) < tol, mode
    finally:
        nat.call("qf_set_tile_kernel", 0)
