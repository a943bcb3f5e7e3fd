"""Batched QAOA MAXCUT: thousands of uneven instances per launch.

``QAOABatch`` uploads the instances once (graphs as axis pairs, depths,
angle and output offsets) and evaluates every instance's <C> and adjoint
gradient: the instances that fit one CTA's shared memory in one persistent
kernel (``qf_batch_qaoa_grad``), the larger ones as multi-instance
warp-tile passes (``qf_wave_qaoa_grad``, one launch per pass index).  The launch (a counter reset plus the kernel) and
an optional on-device Adam update are captured in a CUDA graph and replayed.

The reference evaluates one circuit at a time (quantumflow/qaoa.py:22-81,
examples/qaoa_maxcut.py:37-87); each instance here computes exactly that
circuit's expectation and its gradient.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from .qaoa import _graph_arrays

__all__ = ["QAOABatch"]


class _Instance(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("p", ctypes.c_int32), ("nedges", ctypes.c_int32),
                ("edge_offset", ctypes.c_int32), ("angle_offset", ctypes.c_int32),
                ("out_offset", ctypes.c_int32)]


_LAYOUTS = {"complex64": nat.LAYOUT_C64, "complex128": nat.LAYOUT_FF}


class QAOABatch:
    """Forward expectation + adjoint gradient of many QAOA MAXCUT instances.

    Args:
        graphs: unweighted graphs (networkx or :class:`qaoa.Graph`).
        ps: QAOA depth per graph (int or sequence).
        dtype: 'complex64' (FP32) or 'complex128' (float-float arithmetic).
        tile_bits, ctas: kernel shape; None takes the autotuned or default
            values (see :mod:`quantumflow_gb300.autotune`).
        wave_min: smallest n run as multi-instance passes (default: every
            instance above tile_bits); a larger value keeps more instances in
            the persistent kernel.
    """

    def __init__(self, graphs, ps, dtype="complex64", tile_bits=None, ctas=None, device=None, wave_min=None):
        if dtype not in _LAYOUTS:
            raise ValueError("dtype must be complex64 or complex128")
        self.dtype = dtype
        self.layout = _LAYOUTS[dtype]
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        graphs = list(graphs)
        ps = [int(ps)] * len(graphs) if np.isscalar(ps) else [int(p) for p in ps]
        if len(ps) != len(graphs):
            raise ValueError("one depth per graph")
        self.count = len(graphs)
        self.ns = np.zeros(self.count, dtype=np.int64)
        self.ps = np.asarray(ps, dtype=np.int64)
        self.nedges = np.zeros(self.count, dtype=np.int64)
        edges_all = []
        for i, g in enumerate(graphs):
            nodes, edges, weights, node_w = _graph_arrays(g)
            if any(w != 1.0 for w in weights) or any(w is not None for w in node_w):
                raise ValueError("the batched kernel handles unweighted graphs without node weights")
            self.ns[i] = len(nodes)
            self.nedges[i] = len(edges)
            edges_all.append(np.asarray(edges, dtype=np.uint8).reshape(-1, 2))
        self.max_n = int(self.ns.max()) if self.count else 1
        ts_max = 12 if self.layout == nat.LAYOUT_C64 else 11
        if self.max_n > 30:
            raise ValueError("instances above 30 qubits are not supported by the batched engine")
        # offsets in the caller's (input) order; launch order is largest first
        self.angle_offset = np.concatenate([[0], np.cumsum(2 * self.ps)[:-1]]).astype(np.int64)
        self.out_offset = np.concatenate([[0], np.cumsum(2 * self.ps + 1)[:-1]]).astype(np.int64)
        self.edge_offset = np.concatenate([[0], np.cumsum(self.nedges)[:-1]]).astype(np.int64)
        edges = np.concatenate(edges_all) if edges_all else np.zeros((0, 2), np.uint8)
        self.d_edges = torch.from_numpy(np.ascontiguousarray(edges).reshape(-1)).to(self.device)
        if self.d_edges.numel() == 0:
            self.d_edges = torch.zeros(2, dtype=torch.uint8, device=self.device)
        self.angles = torch.zeros(int(2 * self.ps.sum()), dtype=torch.float64, device=self.device)
        self.out = torch.zeros(int((2 * self.ps + 1).sum()), dtype=torch.float64, device=self.device)
        # index maps: angles (beta..., gamma...) <- out (dgamma..., dbeta..., E)
        gsrc = np.zeros(self.angles.numel(), dtype=np.int64)
        esrc = np.zeros(self.count, dtype=np.int64)
        for i in range(self.count):
            p, a, o = int(self.ps[i]), int(self.angle_offset[i]), int(self.out_offset[i])
            gsrc[a:a + p] = o + p + np.arange(p)      # beta  <- dbeta
            gsrc[a + p:a + 2 * p] = o + np.arange(p)  # gamma <- dgamma
            esrc[i] = o + 2 * p
        self._gsrc = torch.from_numpy(gsrc).to(self.device)
        self._esrc = torch.from_numpy(esrc).to(self.device)
        # instance of every angle (masked updates)
        self._ainst = torch.from_numpy(np.repeat(np.arange(self.count), 2 * self.ps)).to(self.device)
        self._skip_on = False
        from . import autotune
        cfg = autotune.batch_config(self) if (tile_bits is None or ctas is None) else {}
        self.tile_bits = int(tile_bits if tile_bits is not None else cfg.get("tile_bits", ts_max))
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.ctas = int(ctas if ctas is not None else cfg.get("ctas", 2 * sms))
        self.wave_min = int(wave_min) if wave_min is not None else 0
        self._alloc_workspace()
        self._graph = None

    def _alloc_workspace(self):
        """Split the instances for the current tile size and size both
        workspaces.  Instances with n <= tile_bits live in one CTA's shared
        memory (``qf_batch_qaoa_grad``, largest first); the larger ones run
        as multi-instance warp-tile passes (``qf_wave_qaoa_grad``), which
        keep psi, lambda and the cut table of each in device memory."""
        self.ctas = max(8, (self.ctas // 8) * 8)
        cost = lambda i: -(2 ** int(self.ns[i])) * (int(self.ps[i]) + 1)
        wmin = max(self.tile_bits + 1, self.wave_min)
        to_wave = lambda i: self.ns[i] >= wmin and self.ps[i] > 0
        waves = sorted(i for i in range(self.count) if to_wave(i))
        # persistent kernel: cluster-shared instances (n >= tile + 4) first,
        # then the rest, each group largest first
        coop_min = self.tile_bits + 4
        large = sorted((i for i in range(self.count) if not to_wave(i) and self.ns[i] >= coop_min),
                       key=lambda i: (cost(i), i))
        small = sorted((i for i in range(self.count) if not to_wave(i) and self.ns[i] < coop_min),
                       key=lambda i: (cost(i), i))
        self.nlarge = len(large)
        self.nsmall = len(large) + len(small)
        inst = (_Instance * max(1, self.nsmall))()
        for k, i in enumerate(large + small):
            inst[k] = self._inst(i)
        raw = np.frombuffer(bytes(inst), dtype=np.uint8)
        self.d_inst = torch.from_numpy(raw.copy()).to(self.device)
        small_n = int(max((self.ns[i] for i in large + small), default=1))
        self.ws_bytes = nat.lib.qf_batch_workspace_bytes(small_n, self.layout, self.ctas)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        self.small_max_n = small_n
        # multi-instance passes
        self.nwave = len(waves)
        self._wave_plan = None
        # plan order is input order: skip[k] leaves instance waves[k] out
        self._wave_idx = torch.as_tensor(waves, dtype=torch.int64).to(self.device)
        self._wave_skip = torch.zeros(max(1, self.nwave), dtype=torch.int32, device=self.device)
        if self.nwave:
            winst = (_Instance * self.nwave)(*[self._inst(i) for i in waves])
            hb, db = ctypes.c_size_t(), ctypes.c_size_t()
            nat.call("qf_wave_plan", ctypes.addressof(winst), self.nwave, self.layout, None, 0,
                     ctypes.byref(hb), ctypes.byref(db))
            plan = np.zeros(hb.value, dtype=np.uint8)
            nat.call("qf_wave_plan", ctypes.addressof(winst), self.nwave, self.layout, plan.ctypes.data,
                     hb.value, None, None)
            self._wave_plan = plan
            self.wave_ws_bytes = db.value
            self.wave_ws = torch.empty(max(db.value, 256), dtype=torch.uint8, device=self.device)
            nat.call("qf_wave_prepare", plan.ctypes.data, nat.ptr(self.d_edges), nat.ptr(self.wave_ws),
                     self.wave_ws_bytes, nat.stream_handle(self.device))
        self._graph = None

    def _inst(self, i):
        return _Instance(int(self.ns[i]), int(self.ps[i]), int(self.nedges[i]), int(self.edge_offset[i]),
                         int(self.angle_offset[i]), int(self.out_offset[i]))

    # ------------------------------------------------------------ angles ---
    def set_angles(self, betas, gammas):
        """Per-instance beta and gamma sequences (lists of length-p arrays)."""
        host = np.zeros(self.angles.numel())
        for i in range(self.count):
            p, a = int(self.ps[i]), int(self.angle_offset[i])
            host[a:a + p] = np.asarray(betas[i], dtype=np.float64).reshape(p)
            host[a + p:a + 2 * p] = np.asarray(gammas[i], dtype=np.float64).reshape(p)
        self.angles.copy_(torch.from_numpy(host))

    def get_angles(self):
        host = self.angles.cpu().numpy()
        betas, gammas = [], []
        for i in range(self.count):
            p, a = int(self.ps[i]), int(self.angle_offset[i])
            betas.append(host[a:a + p].copy())
            gammas.append(host[a + p:a + 2 * p].copy())
        return betas, gammas

    # ------------------------------------------------------------ launch ---
    def launch(self, stream=None):
        """Enqueue one evaluation (asynchronous)."""
        stream = stream or nat.stream_handle(self.device)
        if self.nsmall:
            nat.call("qf_batch_qaoa_grad", nat.ptr(self.d_inst), self.nsmall, self.nlarge, nat.ptr(self.d_edges),
                     nat.ptr(self.angles), nat.ptr(self.out), self.layout, self.small_max_n, self.tile_bits,
                     self.ctas, nat.ptr(self.ws), self.ws_bytes, stream)
        if self.nwave:
            skip = nat.ptr(self._wave_skip) if self._skip_on else None
            nat.call("qf_wave_qaoa_grad", self._wave_plan.ctypes.data, nat.ptr(self.wave_ws), self.wave_ws_bytes,
                     nat.ptr(self.angles), nat.ptr(self.out), skip, stream)

    def expectations(self) -> torch.Tensor:
        """<C> per instance (device tensor, input order) from the last launch."""
        return self.out[self._esrc]

    def angle_gradients(self) -> torch.Tensor:
        """d<C>/d angles in the layout of ``self.angles`` (device)."""
        return self.out[self._gsrc]

    def evaluate(self):
        """Run once; return (E, dbetas, dgammas) on the host (input order)."""
        self.launch()
        o = self.out.cpu().numpy()
        es, dbs, dgs = [], [], []
        for i in range(self.count):
            p, off = int(self.ps[i]), int(self.out_offset[i])
            dgs.append(o[off:off + p].copy())
            dbs.append(o[off + p:off + 2 * p].copy())
            es.append(o[off + 2 * p])
        return np.array(es), dbs, dgs

    # ------------------------------------------------------------ Adam -----
    def optimizer_reset(self, maxcut=None, target=None):
        """Fresh Adam state; optional per-instance max cut and target ratio
        for recording the first step each instance reaches the target."""
        self._opt = {
            "m": torch.zeros_like(self.angles), "v": torch.zeros_like(self.angles),
            "t": torch.zeros(1, dtype=torch.float64, device=self.device),
            "first": torch.full((self.count,), -1, dtype=torch.int64, device=self.device),
            "mc": None if maxcut is None else torch.as_tensor(np.asarray(maxcut, dtype=np.float64),
                                                              device=self.device),
            "target": None if target is None else float(target),
        }
        self._wave_skip.zero_()
        self._graph = None
        self._graph_key = None

    def _opt_step(self, lr, b1, b2, eps, stop=False):
        o = self._opt
        self.launch(nat.stream_handle(self.device))
        if o["mc"] is not None and o["target"] is not None:
            hit = (self.out[self._esrc] / o["mc"] >= o["target"]) & (o["first"] < 0)
            o["first"].copy_(torch.where(hit, o["t"].to(torch.int64).expand_as(o["first"]), o["first"]))
        g = self.out[self._gsrc]
        o["t"].add_(1.0)
        o["m"].mul_(b1).add_(g, alpha=1 - b1)
        o["v"].mul_(b2).addcmul_(g, g, value=1 - b2)
        mhat = o["m"] / (1 - b1 ** o["t"])
        vhat = o["v"] / (1 - b2 ** o["t"])
        step = lr * mhat / (vhat.sqrt() + eps)
        if stop:
            # instances at the target keep their angles and leave the passes
            live = o["first"] < 0
            step = torch.where(live[self._ainst], step, torch.zeros_like(step))
            self._wave_skip[:self.nwave].copy_((~live[self._wave_idx]).to(torch.int32))
        self.angles.add_(step)

    def optimize(self, steps, lr=0.05, betas=(0.9, 0.999), eps=1e-8, maxcut=None, target=None,
                 use_graph=True, reset=True, stop_at_target=False):
        """Gradient ascent on every instance's <C> with Adam, entirely on the
        device: each step is one batched forward + adjoint launch and the
        update, replayed from a CUDA graph.  ``reset=False`` continues the
        previous optimizer state (chunked runs).

        With ``maxcut`` (per instance, input order) and ``target`` the step at
        which each instance first has <C>/maxcut >= target is recorded (-1 if
        never; the ratio is that of the angles a step starts from).  Returns
        (ratios or <C> at the final angles, first_step).

        ``stop_at_target=True`` (needs maxcut and target) also stops each
        instance once it reaches the target: its angles stay where they
        reached it and its multi-instance passes are skipped, so a batch costs
        the steps each instance needs rather than the slowest one's."""
        if reset or getattr(self, "_opt", None) is None:
            self.optimizer_reset(maxcut, target)
        if stop_at_target and (self._opt["mc"] is None or self._opt["target"] is None):
            raise ValueError("stop_at_target needs maxcut and target")
        b1, b2 = betas
        stop = bool(stop_at_target)
        key = (float(lr), b1, b2, eps, stop)
        self._skip_on = stop
        try:
            if steps > 0:
                if not use_graph:
                    for _ in range(steps):
                        self._opt_step(lr, b1, b2, eps, stop)
                else:
                    done = 0
                    if self._graph is None or self._graph_key != key:
                        self._opt_step(lr, b1, b2, eps, stop)  # outside capture: sets attributes, caches
                        done = 1
                        torch.cuda.synchronize(self.device)
                        graph = torch.cuda.CUDAGraph()
                        s = torch.cuda.Stream(self.device)
                        s.wait_stream(torch.cuda.current_stream(self.device))
                        with torch.cuda.stream(s):
                            with torch.cuda.graph(graph, stream=s):
                                self._opt_step(lr, b1, b2, eps, stop)  # recorded, not run
                        torch.cuda.current_stream(self.device).wait_stream(s)
                        self._graph, self._graph_key = graph, key
                    for _ in range(steps - done):
                        self._graph.replay()
            o = self._opt
            self.launch()
        finally:
            self._skip_on = False
        e = self.out[self._esrc]
        first = o["first"]
        if o["mc"] is not None and o["target"] is not None:
            ratio = e / o["mc"]
            hit = (ratio >= o["target"]) & (first < 0)
            first = torch.where(hit, o["t"].to(torch.int64).expand_as(first), first)
            o["first"].copy_(first)
            return ratio.cpu().numpy(), first.cpu().numpy()
        return e.cpu().numpy(), first.cpu().numpy()

    def adam(self, steps, lr=0.05, betas=(0.9, 0.999), eps=1e-8, use_graph=True):
        """Adam ascent on every instance's <C> (see :meth:`optimize`)."""
        self.optimize(steps, lr=lr, betas=betas, eps=eps, use_graph=use_graph)
