"""float64 numpy restatement of the angle network in
quantumflow_gb300/csrc/gnn.cu -- TEST INFRASTRUCTURE ONLY.

The network has no counterpart in the reference; this is the CPU checker for
its CUDA forward and backward kernels (used only by tests/)."""
import numpy as np

H = 64


def unpack(params, p):
    o = 0
    out = {}

    def take(name, shape):
        nonlocal o
        size = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + size], dtype=np.float64).reshape(shape)
        o += size

    take("W0", (H, 3))
    take("b0", (H,))
    for l in range(3):
        take(f"Ws{l}", (H, H))
        take(f"Wn{l}", (H, H))
        take(f"b{l + 1}", (H,))
    take("Wr", (H, H))
    take("br", (H,))
    take("Wo", (2 * p, H))
    take("bo", (2 * p,))
    assert o == len(params)
    return out


def forward(params, p, n, edges):
    """Returns (out, cache) for one graph with nodes 0..n-1."""
    P = unpack(params, p)
    nbrs = [[] for _ in range(n)]
    for a, b in edges:
        if a != b:
            nbrs[a].append(b)
            nbrs[b].append(a)
    deg = np.array([len(x) for x in nbrs], dtype=np.float64)
    X = np.stack([np.ones(n), deg / 8.0, np.full(n, n / 16.0)], axis=1)
    hs = [np.maximum(X @ P["W0"].T + P["b0"], 0.0)]
    aggs = []
    for l in range(3):
        h = hs[-1]
        A = np.zeros_like(h)
        for v in range(n):
            if nbrs[v]:
                A[v] = h[nbrs[v]].mean(axis=0)
        aggs.append(A)
        hs.append(np.maximum(h @ P[f"Ws{l}"].T + A @ P[f"Wn{l}"].T + P[f"b{l + 1}"], 0.0))
    g = hs[-1].mean(axis=0)
    r = np.maximum(P["Wr"] @ g + P["br"], 0.0)
    out = P["Wo"] @ r + P["bo"]
    return out, dict(P=P, X=X, hs=hs, aggs=aggs, g=g, r=r, nbrs=nbrs, deg=deg, n=n)


def backward(cache, dout):
    """Gradient dict for the loss whose d/dout is ``dout``."""
    P, hs, aggs, nbrs, deg, n = cache["P"], cache["hs"], cache["aggs"], cache["nbrs"], cache["deg"], cache["n"]
    G = {k: np.zeros_like(v) for k, v in P.items()}
    r, g = cache["r"], cache["g"]
    G["Wo"] += np.outer(dout, r)
    G["bo"] += dout
    dr = (P["Wo"].T @ dout) * (r > 0)
    G["Wr"] += np.outer(dr, g)
    G["br"] += dr
    dg = P["Wr"].T @ dr
    dh = np.tile(dg / n, (n, 1))
    for l in (2, 1, 0):
        dz = dh * (hs[l + 1] > 0)
        G[f"Ws{l}"] += dz.T @ hs[l]
        G[f"Wn{l}"] += dz.T @ aggs[l]
        G[f"b{l + 1}"] += dz.sum(axis=0)
        da = dz @ P[f"Wn{l}"]
        dh = dz @ P[f"Ws{l}"]
        for w in range(n):
            if nbrs[w]:
                for u in nbrs[w]:
                    dh[u] += da[w] / deg[w]
    dz = dh * (hs[0] > 0)
    G["W0"] += dz.T @ cache["X"]
    G["b0"] += dz.sum(axis=0)
    return G


def flat(G, p):
    order = ["W0", "b0"] + [k for l in range(3) for k in (f"Ws{l}", f"Wn{l}", f"b{l + 1}")] + ["Wr", "br", "Wo", "bo"]
    return np.concatenate([G[k].reshape(-1) for k in order])


def batch_loss_grad(params, p, graphs, targets):
    """Mean squared error over a batch and its gradient (flat)."""
    B = len(graphs)
    grad = None
    loss = 0.0
    outs = []
    for (n, edges), t in zip(graphs, targets):
        out, cache = forward(params, p, n, edges)
        outs.append(out)
        d = out - t
        loss += float(np.sum(d * d))
        G = backward(cache, 2 * d / (B * 2 * p))
        f = flat(G, p)
        grad = f if grad is None else grad + f
    return loss / (B * 2 * p), grad, np.array(outs)
