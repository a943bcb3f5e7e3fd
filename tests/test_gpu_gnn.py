"""The angle network's CUDA forward/backward kernels against the float64
numpy checker, and its training behaviour."""
import numpy as np
import pytest
import torch

from oracle import gnn_oracle as go

pytestmark = pytest.mark.gpu


def _graphs(count, seed, nmin=4, nmax=16):
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        if i % 2 and n % 2 == 0:
            out.append(qf.qaoa.random_regular_graph(3, n, seed=int(rng.integers(1 << 30))))
        else:
            out.append(qf.qaoa.gnp_random_graph(n, 0.5, seed=int(rng.integers(1 << 30))))
    return out


def test_forward_and_gradient_match_numpy():
    import quantumflow_gb300 as qf
    p = 6
    graphs = _graphs(24, 1)
    graphs.append(qf.Graph(nodes=range(5)))  # isolated nodes
    net = qf.gnn.AngleGNN(p, seed=3)
    rng = np.random.default_rng(0)
    net.params.copy_(torch.from_numpy((net.params.cpu().numpy() + rng.normal(0, 0.05, net.nparams)).astype(np.float32)))
    batch = qf.gnn.GraphBatch(graphs)
    targets = rng.uniform(0, 1, size=(len(graphs), 2 * p)).astype(np.float32)
    loss, grad = net.gradient(batch, torch.from_numpy(targets))
    params = net.params.cpu().numpy().astype(np.float64)
    simple = [(len(list(g.nodes())), [tuple(e) for e in g.edges()]) for g in graphs]
    ref_loss, ref_grad, ref_out = go.batch_loss_grad(params, p, simple, targets.astype(np.float64))
    out = net.predict(batch)
    np.testing.assert_allclose(out, ref_out, rtol=1e-4, atol=1e-5)
    assert abs(float(loss) - ref_loss) < 1e-5 * max(1.0, ref_loss)
    g = grad.cpu().numpy()
    scale = np.max(np.abs(ref_grad))
    np.testing.assert_allclose(g, ref_grad, atol=2e-5 * scale, rtol=1e-3)


def test_training_reduces_loss_and_adam_matches_numpy():
    import quantumflow_gb300 as qf
    p = 3
    graphs = _graphs(256, 2, 6, 14)
    # a learnable target: angles that depend on the mean degree
    deg = np.array([2 * len(g.edges()) / len(list(g.nodes())) for g in graphs])
    targets = np.stack([0.3 + 0.05 * deg] * p + [0.5 - 0.03 * deg] * p, axis=1).astype(np.float32)
    net = qf.gnn.AngleGNN(p, seed=1)
    hist = net.fit(graphs, targets, epochs=40, batch_size=64, lr=3e-3)
    assert hist[-1] < 0.2 * hist[0]
    # one Adam step against a numpy restatement
    w = net.params.clone()
    g = torch.randn_like(w)
    m0, v0, step0 = net.m.clone(), net.v.clone(), net.step
    net.adam_step(g, lr=1e-3)
    t = step0 + 1
    m = 0.9 * m0 + 0.1 * g
    v = 0.999 * v0 + 0.001 * g * g
    ref = w - 1e-3 * (m / (1 - 0.9 ** t)) / (torch.sqrt(v / (1 - 0.999 ** t)) + 1e-8)
    assert torch.allclose(net.params, ref, rtol=1e-5, atol=1e-7)
