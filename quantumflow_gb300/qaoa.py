"""QAOA for QUBO / MAXCUT (quantumflow/qaoa.py:22-81) on the GPU.

* ``qubo_circuit`` builds the same gate sequence as the reference: H on every
  node; per step ZZ(-w*gamma/pi) per edge in ``graph.edges()`` order,
  RZ(node weight) where a node has one (not scaled by gamma, as in the
  reference), then RX(beta) on every node.
* ``graph_cuts`` returns the cut value of every basis state, computed by the
  ``qf_cut_values`` kernel instead of the reference's O(E 2^N) Python loop.
* ``QAOAMaxCut`` is the fast path: the cut table stays on the device and each
  cost layer is one diagonal-phase lookup exp(i gamma (W/2 - C(x))) fused with
  the RX mixer layer (``qf_qaoa_state``).

Graphs may be networkx graphs or the dependency-free :class:`Graph` below
(any object with ``nodes()``, ``edges()``, ``graph[u][v]`` and
``graph.nodes[u]`` attribute dicts).
"""
import math
from typing import Sequence

import numpy as np
import torch

from . import _native as nat
from . import config
from .circuits import Circuit
from .states import Buffer, State, _device, _reduce
from .stdgates import H, RX, RZ, ZZ

__all__ = ["qubo_circuit", "graph_cuts", "Graph", "gnp_random_graph", "random_regular_graph",
           "QAOAMaxCut", "QAOAExpectation", "maxcut_qaoa", "linear_ramp_angles"]


# ------------------------------------------------------------------ graph ---
class _NodeView:
    def __init__(self, g):
        self._g = g

    def __call__(self):
        return list(self._g._nodes)

    def __getitem__(self, q):
        return self._g._nodes[q]

    def __iter__(self):
        return iter(self._g._nodes)

    def __len__(self):
        return len(self._g._nodes)


class Graph:
    """A small undirected graph with the networkx accessors QAOA uses."""

    def __init__(self, edges=(), nodes=()):
        self._nodes = {}
        self._adj = {}
        self._edges = []
        for q in nodes:
            self.add_node(q)
        for e in edges:
            self.add_edge(*e)

    def add_node(self, q, **attr):
        if q not in self._nodes:
            self._nodes[q] = {}
            self._adj[q] = {}
        self._nodes[q].update(attr)

    def add_edge(self, u, v, **attr):
        self.add_node(u)
        self.add_node(v)
        if v in self._adj[u]:
            self._adj[u][v].update(attr)
            return
        d = dict(attr)
        self._adj[u][v] = d
        self._adj[v][u] = d
        self._edges.append((u, v))

    @property
    def nodes(self):
        return _NodeView(self)

    def edges(self):
        return list(self._edges)

    def __getitem__(self, u):
        return self._adj[u]

    def __len__(self):
        return len(self._nodes)

    def number_of_nodes(self):
        return len(self._nodes)

    def number_of_edges(self):
        return len(self._edges)

    def degree(self, q):
        return len(self._adj[q])


def gnp_random_graph(n: int, p: float, seed=None) -> Graph:
    """Erdos-Renyi G(n, p): each of the n(n-1)/2 edges present with prob. p."""
    rng = np.random.default_rng(seed)
    g = Graph(nodes=range(n))
    for i in range(n):
        for j in range(i + 1, n):
            if rng.random() < p:
                g.add_edge(i, j)
    return g


def random_regular_graph(d: int, n: int, seed=None, max_tries: int = 10000) -> Graph:
    """Uniform d-regular simple graph by the pairing (configuration) model with
    rejection of self-loops and multi-edges.  n*d must be even."""
    if (n * d) % 2 or d >= n:
        raise ValueError("no d-regular graph on n nodes")
    rng = np.random.default_rng(seed)
    for _ in range(max_tries):
        stubs = rng.permutation(np.repeat(np.arange(n), d))
        pairs = stubs.reshape(-1, 2)
        if np.any(pairs[:, 0] == pairs[:, 1]):
            continue
        key = np.sort(pairs, axis=1)
        if len(np.unique(key, axis=0)) != len(key):
            continue
        g = Graph(nodes=range(n))
        for a, b in key[np.lexsort((key[:, 1], key[:, 0]))]:
            g.add_edge(int(a), int(b))
        return g
    raise RuntimeError("random_regular_graph: too many rejections")


def compute_layout(dtype: str) -> int:
    """Element layout of the QAOA kernels' state buffers: complex64, or for
    complex128 float-float pairs, or native FP64 when that is configured
    (config.C128_ARITHMETIC == "fp64")."""
    if dtype == "complex64":
        return nat.LAYOUT_C64
    return nat.LAYOUT_C128 if config.C128_ARITHMETIC == "fp64" else nat.LAYOUT_FF


def _graph_arrays(graph):
    nodes = sorted(graph.nodes())
    axis = {q: i for i, q in enumerate(nodes)}
    edges = [(axis[a], axis[b]) for a, b in graph.edges()]
    weights = [float(graph[a][b].get("weight", 1.0)) for a, b in graph.edges()]
    node_w = [graph.nodes[q].get("weight", None) for q in nodes]
    return nodes, edges, weights, node_w


# ---------------------------------------------------------- reference API ---
def qubo_circuit(graph, steps: int, beta: Sequence, gamma: Sequence) -> Circuit:
    """QAOA circuit for QUBO / Ising problems (quantumflow/qaoa.py:22-64)."""
    qubits = list(graph.nodes())
    circ = Circuit()
    for q0 in qubits:
        circ += H(q0)
    for p in range(steps):
        for q0, q1 in graph.edges():
            weight = graph[q0][q1].get("weight", 1.0)
            circ += ZZ(-weight * gamma[p] / np.pi, q0, q1)
        for q0 in qubits:
            node_weight = graph.nodes[q0].get("weight", None)
            if node_weight is not None:
                circ += RZ(node_weight, q0)
        for q0 in qubits:
            circ += RX(beta[p], q0)
    return circ


def _cut_table(n, edges, weights, device):
    """(uint16 table or None, float64 table) of cut values on the device."""
    e = nat.int_array([a for ab in edges for a in ab])
    stream = nat.stream_handle(device)
    if all(w == 1.0 for w in weights):
        c16 = torch.empty(2 ** n, dtype=torch.int16, device=device)  # uint16 bits; cuts <= 2048
        nat.call("qf_cut_values", nat.ptr(c16), n, len(edges), e, stream)
        return c16, c16.to(torch.float64)
    c64 = torch.empty(2 ** n, dtype=torch.float64, device=device)
    nat.call("qf_cut_values_weighted", nat.ptr(c64), n, len(edges), e, nat.double_array(weights), stream)
    return None, c64


def graph_cuts(graph) -> torch.Tensor:
    """Cut value of every basis state as a [2]*N float64 CUDA tensor
    (quantumflow/qaoa.py:68-81)."""
    nodes, edges, weights, _ = _graph_arrays(graph)
    n = len(nodes)
    _, table = _cut_table(n, edges, weights, _device())
    return table.reshape([2] * n)


# ------------------------------------------------------------- fast path ---
class QAOAMaxCut:
    """QAOA MAXCUT on one graph with the cut table resident on the GPU.

    ``state(beta, gamma)`` equals ``qubo_circuit(graph, p, beta, gamma).run()``
    and ``expectation(beta, gamma)`` equals ``.expectation(graph_cuts(graph))``.
    """

    def __init__(self, graph, p: int, dtype: str = "complex128", fusion_k: int = None):
        self.graph = graph
        self.p = int(p)
        self.dtype = dtype
        self.fusion_k = config.FUSION_K if fusion_k is None else fusion_k
        self.nodes, self.edges, self.weights, node_w = _graph_arrays(graph)
        self.n = len(self.nodes)
        self.device = _device()
        self.cuts16, self.cuts = _cut_table(self.n, self.edges, self.weights, self.device)
        self.node_theta = None
        if any(w is not None for w in node_w):
            self.node_theta = np.array([np.nan if w is None else float(w) for w in node_w])
        self.total_weight = float(sum(self.weights))
        self._maxcut = None

    @property
    def unweighted(self) -> bool:
        return self.cuts16 is not None

    @property
    def maxcut(self) -> float:
        if self._maxcut is None:
            self._maxcut = float(self.cuts.max())
        return self._maxcut

    def circuit(self, beta, gamma) -> Circuit:
        return qubo_circuit(self.graph, self.p, beta, gamma)

    def state(self, beta, gamma) -> State:
        beta = np.asarray(beta, dtype=np.float64)
        gamma = np.asarray(gamma, dtype=np.float64)
        if not self.unweighted:
            return self.circuit(beta, gamma).run(fusion_k=self.fusion_k)
        buf = Buffer.empty(self.n, compute_layout(self.dtype), self.device)
        nt = nat.double_array(self.node_theta) if self.node_theta is not None else None
        nat.call("qf_qaoa_state", nat.ptr(buf.data), self.n, buf.layout, nat.ptr(self.cuts16),
                 len(self.edges), self.p, nat.double_array(beta), nat.double_array(gamma), nt,
                 int(self.fusion_k), nat.stream_handle(self.device))
        return State(buf, tuple(self.nodes))

    def expectation(self, beta, gamma) -> float:
        st = self.state(beta, gamma)
        buf = st.buffer
        if self.unweighted:
            return _reduce("qf_expectation_cuts", buf, nout=1, extra=(nat.ptr(self.cuts16),))[0]
        return _reduce("qf_expectation_diag", buf, nout=1, extra=(nat.ptr(self.cuts),))[0]

    def ratio(self, beta, gamma) -> float:
        return self.expectation(beta, gamma) / self.maxcut

    # ------------------------------------------------------------ gradient --
    def expectation_and_grad(self, beta, gamma):
        """(<C>, d<C>/d beta, d<C>/d gamma) by the adjoint method
        (qf_qaoa_expectation_grad): one forward sweep, then every layer undone
        on psi and lambda = C psi; two state vectors whatever p is."""
        p = self.p
        if not self.unweighted:
            return self._weighted_grad(beta, gamma)
        beta = np.ascontiguousarray(beta, dtype=np.float64)
        gamma = np.ascontiguousarray(gamma, dtype=np.float64)
        if beta.shape != (p,) or gamma.shape != (p,):
            raise ValueError(f"expected {p} betas and {p} gammas")
        layout = compute_layout(self.dtype)
        if getattr(self, "_grad_bufs", None) is None or self._grad_bufs[0] != layout:
            nbytes = nat.lib.qf_qaoa_grad_workspace_bytes(self.n, p, layout)
            psi = Buffer.empty(self.n, layout, self.device)
            ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            out = torch.empty(2 * p + 1, dtype=torch.float64, device=self.device)
            self._grad_bufs = (layout, psi, ws, nbytes, out)
        _, psi, ws, nbytes, out = self._grad_bufs
        nt = nat.double_array(self.node_theta) if self.node_theta is not None else None
        nat.call("qf_qaoa_expectation_grad", nat.ptr(psi.data), self.n, layout, nat.ptr(self.cuts16),
                 len(self.edges), p, beta.ctypes.data_as(nat._dp), gamma.ctypes.data_as(nat._dp), nt,
                 int(self.fusion_k), nat.ptr(out), nat.ptr(ws), nbytes, nat.stream_handle(self.device))
        o = out.cpu().numpy()
        return float(o[2 * p]), o[p:2 * p].copy(), o[:p].copy()


def _weighted_grad_impl(prob, beta, gamma):
    """Weighted edges: the generic circuit adjoint over qubo_circuit, with the
    chain rule for the shared angles (ZZ(t), t = -w gamma / pi; RX(beta))."""
    from .adjoint import expectation_and_grad
    circ = prob.circuit(beta, gamma)
    e, grads = expectation_and_grad(circ, prob.cuts, dtype=prob.dtype)
    p = prob.p
    gb, gg = np.zeros(p), np.zeros(p)
    nodes = list(prob.graph.nodes())
    weighted_nodes = sum(1 for q in nodes if prob.graph.nodes[q].get("weight", None) is not None)
    k = len(nodes)  # the H layer
    for l in range(p):
        for w in prob.weights:
            gg[l] += grads.get((k, "t"), 0.0) * (-w / np.pi)
            k += 1
        k += weighted_nodes
        for _ in nodes:
            gb[l] += grads.get((k, "theta"), 0.0)
            k += 1
    return e, gb, gg


QAOAMaxCut._weighted_grad = lambda self, beta, gamma: _weighted_grad_impl(self, beta, gamma)


class QAOAExpectation(torch.autograd.Function):
    """<C>(beta, gamma) as a differentiable torch function.

    The forward pass runs the fused forward + adjoint kernels once and keeps
    the gradient; backward scales it by the incoming gradient.  Inputs are
    1-D float64 tensors of length p (any device)."""

    @staticmethod
    def forward(ctx, beta, gamma, problem):
        e, gb, gg = problem.expectation_and_grad(beta.detach().cpu().numpy(), gamma.detach().cpu().numpy())
        ctx.save_for_backward(torch.from_numpy(gb).to(beta.device), torch.from_numpy(gg).to(gamma.device))
        return torch.tensor(e, dtype=torch.float64, device=beta.device)

    @staticmethod
    def backward(ctx, grad_out):
        gb, gg = ctx.saved_tensors
        return grad_out * gb, grad_out * gg, None


def linear_ramp_angles(p: int, dt: float = 0.75):
    """Plain initialisation: gamma ramps up and beta ramps down linearly over
    the p layers (the discretised-annealing start for QAOA)."""
    t = (np.arange(p) + 0.5) / p
    return dt * (1 - t), dt * t  # beta, gamma


def maxcut_qaoa(graph, steps: int = 5, learning_rate: float = 0.01, init=None, max_iters: int = 10000,
                block: int = 10, min_difference: float = 1e-4, target_ratio: float = None,
                dtype: str = "complex128", seed=None, verbose: bool = False):
    """QAOA MAXCUT by gradient ascent on <C> (examples/qaoa_maxcut.py:37-87).

    ``init``: None draws beta, gamma ~ N(0.5, 0.01) as the reference does;
    'ramp' uses :func:`linear_ramp_angles`; or a (beta, gamma) pair.  Every
    ``block`` steps the ratio <C>/max C is checked and the loop stops when it
    improved by less than ``min_difference`` (reference :70-82) or reached
    ``target_ratio``.  Returns (ratio, beta, gamma, history) where history
    holds (step, ratio, seconds) per check."""
    import time
    prob = graph if isinstance(graph, QAOAMaxCut) else QAOAMaxCut(graph, steps, dtype=dtype)
    p = prob.p
    if init is None:
        rng = np.random.default_rng(seed)
        beta = rng.normal(loc=0.5, scale=0.01, size=p)
        gamma = rng.normal(loc=0.5, scale=0.01, size=p)
    elif isinstance(init, str) and init == "ramp":
        beta, gamma = linear_ramp_angles(p)
    else:
        beta, gamma = (np.array(a, dtype=np.float64) for a in init)
    maxcut = prob.maxcut
    history = []
    last = -1.0
    t0 = time.perf_counter()
    ratio = prob.expectation(beta, gamma) / maxcut
    history.append((0, ratio, 0.0))
    for step in range(0, max_iters, block):
        for _ in range(block):
            e, gb, gg = prob.expectation_and_grad(beta, gamma)
            beta = beta + learning_rate * gb
            gamma = gamma + learning_rate * gg
        ratio = prob.expectation(beta, gamma) / maxcut
        history.append((step + block, ratio, time.perf_counter() - t0))
        if verbose:
            print("# step: {}  ratio: {:.4f}".format(step + block, ratio))
        if target_ratio is not None and ratio >= target_ratio:
            break
        if ratio - last < min_difference:
            break
        last = ratio
    return ratio, beta, gamma, history
