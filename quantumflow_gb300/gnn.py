"""Learned QAOA angle initialiser (graph network -> 2p angles).

The network (3 message-passing layers, hidden width 64, FP32) is described
in ``csrc/gnn.cu``; its forward, backward and Adam kernels are the
``qf_gnn_*`` / ``qf_adam_update`` entry points.  Training labels are angles
that the simulator's own batched adjoint-gradient Adam finds
(:func:`make_labels`).  The reference has no counterpart: it starts every
optimisation from N(0.5, 0.01) angles (examples/qaoa_maxcut.py:47-51).
"""
import numpy as np
import torch

from . import _native as nat
from .qaoa import _graph_arrays, linear_ramp_angles

__all__ = ["GraphBatch", "AngleGNN", "make_labels", "predict_angles"]

HIDDEN = 64
MAX_NODES = 32


class GraphBatch:
    """Graphs as device CSR arrays (node_offset, adj_offset, adj)."""

    def __init__(self, graphs, device=None):
        device = device or torch.device("cuda", torch.cuda.current_device())
        node_offset = [0]
        adj_offset = [0]
        adj = []
        self.sizes = []
        for g in graphs:
            nodes, edges, _, _ = _graph_arrays(g)
            n = len(nodes)
            if n < 1 or n > MAX_NODES:
                raise ValueError(f"graphs must have 1..{MAX_NODES} nodes")
            base = node_offset[-1]
            nbrs = [[] for _ in range(n)]
            for a, b in edges:
                if a != b:
                    nbrs[a].append(b)
                    nbrs[b].append(a)
            for v in range(n):
                adj.extend(base + u for u in sorted(nbrs[v]))
                adj_offset.append(len(adj))
            node_offset.append(base + n)
            self.sizes.append(n)
        self.count = len(self.sizes)
        self.total_nodes = node_offset[-1]
        t = lambda a: torch.tensor(a if len(a) else [0], dtype=torch.int32, device=device)
        self.node_offset = t(node_offset)
        self.adj_offset = t(adj_offset)
        self.adj = t(adj)
        self.device = device


class AngleGNN:
    """The angle network with its parameters on the GPU."""

    def __init__(self, p=6, seed=0, device=None):
        self.p = int(p)
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.nparams = int(nat.lib.qf_gnn_param_count(self.p))
        self.params = torch.from_numpy(self._init(seed)).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0

    def _init(self, seed):
        """Glorot-uniform weights, zero biases, output bias at the linear-ramp
        angles so an untrained network already predicts the plain start."""
        rng = np.random.default_rng(seed)
        H, p = HIDDEN, self.p
        parts = []

        def glorot(rows, cols):
            lim = np.sqrt(6.0 / (rows + cols))
            return rng.uniform(-lim, lim, size=(rows, cols)).reshape(-1)

        parts += [glorot(H, 3), np.zeros(H)]
        for _ in range(3):
            parts += [glorot(H, H), glorot(H, H), np.zeros(H)]
        parts += [glorot(H, H), np.zeros(H)]
        parts += [0.1 * glorot(2 * p, H)]
        b, g = linear_ramp_angles(p)
        parts += [np.concatenate([b, g])]
        flat = np.concatenate(parts).astype(np.float32)
        assert flat.size == self.nparams, (flat.size, self.nparams)
        return flat

    # ----------------------------------------------------------- kernels ---
    def forward(self, batch: GraphBatch, activations=None) -> torch.Tensor:
        out = torch.empty((batch.count, 2 * self.p), dtype=torch.float32, device=self.device)
        nat.call("qf_gnn_forward", nat.ptr(self.params), self.p, batch.count, batch.total_nodes,
                 nat.ptr(batch.node_offset), nat.ptr(batch.adj_offset), nat.ptr(batch.adj), nat.ptr(out),
                 nat.ptr(activations) if activations is not None else None, nat.stream_handle(self.device))
        return out

    def gradient(self, batch: GraphBatch, target: torch.Tensor):
        """(mean squared error, d loss / d params) on one batch."""
        nact = int(nat.lib.qf_gnn_activation_floats(batch.total_nodes, batch.count))
        acts = torch.empty(nact, dtype=torch.float32, device=self.device)
        out = self.forward(batch, acts)
        grad = torch.zeros_like(self.params)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        target = target.to(device=self.device, dtype=torch.float32).contiguous()
        nat.call("qf_gnn_backward", nat.ptr(self.params), self.p, batch.count, batch.total_nodes,
                 nat.ptr(batch.node_offset), nat.ptr(batch.adj_offset), nat.ptr(batch.adj), nat.ptr(out),
                 nat.ptr(target), nat.ptr(acts), nat.ptr(grad), nat.ptr(loss), nat.stream_handle(self.device))
        return loss / (batch.count * 2 * self.p), grad

    def adam_step(self, grad, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.step += 1
        nat.call("qf_adam_update", nat.ptr(self.params), nat.ptr(grad), nat.ptr(self.m), nat.ptr(self.v),
                 self.nparams, lr, betas[0], betas[1], eps, self.step, nat.stream_handle(self.device))

    # ------------------------------------------------------------- use ---
    def predict(self, graphs) -> np.ndarray:
        """Angles (len(graphs), 2p): beta_0..beta_{p-1}, gamma_0..gamma_{p-1}."""
        batch = graphs if isinstance(graphs, GraphBatch) else GraphBatch(graphs, self.device)
        return self.forward(batch).double().cpu().numpy()

    def fit(self, graphs, labels, epochs=60, batch_size=512, lr=2e-3, seed=0, verbose=False):
        """Mini-batch Adam on the mean squared angle error; returns the loss
        history (one mean per epoch)."""
        rng = np.random.default_rng(seed)
        labels = np.asarray(labels, dtype=np.float32)
        graphs = list(graphs)
        nb = (len(graphs) + batch_size - 1) // batch_size
        cached = []  # four shuffles are built once and cycled (CSR building is host work)
        hist = []
        for ep in range(epochs):
            if ep < 4:
                perm = rng.permutation(len(graphs))
                cached.append([(perm[s:s + batch_size],
                                GraphBatch([graphs[i] for i in perm[s:s + batch_size]], self.device))
                               for s in range(0, len(graphs), batch_size)])
            tot, cnt = 0.0, 0
            for k in range(nb):
                idx, b = cached[ep % 4][k]
                loss, grad = self.gradient(b, torch.from_numpy(labels[idx]))
                self.adam_step(grad, lr=lr)
                tot += float(loss) * len(idx)
                cnt += len(idx)
            hist.append(tot / cnt)
            if verbose:
                print(f"epoch {ep} loss {hist[-1]:.5f}")
        return hist

    def save(self, path):
        np.savez_compressed(path, params=self.params.cpu().numpy(), p=self.p)

    @classmethod
    def load(cls, path, device=None):
        d = np.load(path)
        net = cls(int(d["p"]), device=device)
        net.params.copy_(torch.from_numpy(d["params"]))
        return net


def make_labels(graphs, p=6, steps=200, lr=0.05, dtype="complex64", init=None):
    """Simulator-optimised angles: every graph starts from the linear ramp
    (or ``init`` = (betas, gammas)) and runs ``steps`` Adam steps of batched
    adjoint gradients; returns (angles (B, 2p), final <C> per graph)."""
    from .batched import QAOABatch
    batch = QAOABatch(graphs, p, dtype=dtype)
    if init is None:
        b, g = linear_ramp_angles(p)
        betas, gammas = [b] * len(graphs), [g] * len(graphs)
    else:
        betas, gammas = init
    batch.set_angles(betas, gammas)
    batch.optimize(steps, lr=lr)
    es, _, _ = batch.evaluate()
    betas, gammas = batch.get_angles()
    return np.concatenate([np.stack(betas), np.stack(gammas)], axis=1), es


def predict_angles(net, graphs):
    """Network angles split into (betas, gammas) lists."""
    a = net.predict(graphs)
    p = net.p
    return [r[:p] for r in a], [r[p:] for r in a]
