"""CPU oracle for the quantumflow_gb300 parity tests -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this module, and only as the checker (or the timed CPU
baseline), never as a product path.  It is a numpy restatement of the
reference QuantumFlow (rigetti/quantumflow) algorithms on the state-vector
path; each function cites the reference file:line it restates.

Parity pin: ``tests/golden/*.npz`` were produced by running the reference
package itself (numpy backend) with ``tests/golden/make_golden.py``;
``tests/test_oracle.py`` checks every function here against those outputs
and against the literal known-answer vectors of the reference's own tests.
"""
import numpy as np

EINSUM_SUBSCRIPTS = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"


# ------------------------------------------------------------ core ---------
def tensormul(gate, state, indices, dtype=np.complex128):
    """Contract a K-qubit gate with an N-axis tensor on ``indices``.

    Restates quantumflow/backend/numpybk.py:159-214: the gate's bra axes are
    summed against the state axes ``indices`` and its ket axes written back
    at the same positions (out of place).  ``gate`` is (2^K, 2^K) or
    [2]*2K; ``state`` is [2]*N or flat.  ``dtype`` np.clongdouble evaluates
    the same contraction in the host's extended precision (an accuracy
    yardstick for the tests; the reference computes in complex128)."""
    gate = np.asarray(gate, dtype=dtype)
    state = np.asarray(state, dtype=dtype)
    K = len(indices)
    N = int(round(np.log2(state.size)))
    g = gate.reshape([2] * (2 * K))
    s = state.reshape([2] * N)
    out = list(EINSUM_SUBSCRIPTS[:N])
    left_in = list(EINSUM_SUBSCRIPTS[N:N + K])
    left_out = [out[i] for i in indices]
    right = list(out)
    for i, c in zip(indices, left_in):
        right[i] = c
    sub = "".join(left_out + left_in) + "," + "".join(right) + "->" + "".join(out)
    return np.einsum(sub, g, s)


# The reference's torch backend holds a complex tensor as a planar float64
# stack [real, imag] of shape [2, 2, ..., 2] (quantumflow/backend/torchbk.py);
# its tensormul is a permute -> matmul -> inverse permute on that layout,
# multi-threaded on the CPU, and limited to 24 qubits (torchbk.py:60).
def planar(state):
    """Complex array -> the torch backend's planar float64 tensor [2, 2, ..., 2]."""
    import torch
    a = np.asarray(state, dtype=np.complex128)
    n = int(round(np.log2(a.size)))
    return torch.from_numpy(np.stack([a.real, a.imag]).reshape([2] + [2] * n).copy())


def from_planar(t):
    """The planar tensor back to a complex [2]*N numpy array."""
    t = t.numpy()
    return t[0] + 1j * t[1]


def tensormul_planar(gate, tensor, indices):
    """quantumflow/backend/torchbk.py:243-261 tensormul on planar tensors: the
    state axes ``indices`` are permuted to the front (transpose, :180-186),
    the tensor is reshaped to [2^K, 2^(N-K)] and multiplied by the gate with
    four real matmuls (matmul, :198-205), then reshaped and permuted back.
    ``gate`` is a complex (2^K, 2^K) array, ``tensor`` a planar state."""
    import torch
    K = len(indices)
    N = tensor.dim() - 1
    g = np.asarray(gate, dtype=np.complex128).reshape(2 ** K, 2 ** K)
    g_re, g_im = torch.from_numpy(g.real.copy()), torch.from_numpy(g.imag.copy())
    perm = list(indices) + [n for n in range(N) if n not in indices]
    inv_perm = [int(i) for i in np.argsort(perm)]
    re = tensor[0].permute(*perm).contiguous().view(2 ** K, 2 ** (N - K))
    im = tensor[1].permute(*perm).contiguous().view(2 ** K, 2 ** (N - K))
    new_re = g_re @ re - g_im @ im
    new_im = g_re @ im + g_im @ re
    shape = [2] * N
    return torch.stack((new_re.view(shape).permute(*inv_perm).contiguous(),
                        new_im.view(shape).permute(*inv_perm).contiguous()))


def run_ops(state, ops, dtype=np.complex128):
    """Apply (matrix, axes) pairs in order (quantumflow/circuits.py:87-99)."""
    for m, axes in ops:
        state = tensormul(m, state, list(axes), dtype)
    return state


def zero_state(n):
    """|0...0> (quantumflow/states.py:186-191)."""
    s = np.zeros(2 ** n, dtype=np.complex128)
    s[0] = 1
    return s.reshape([2] * n)


def probabilities(state):
    """|psi|^2 (quantumflow/states.py:113-119)."""
    a = np.abs(state)
    return a * a


def expectation(state, diag):
    """sum Re(h) p (quantumflow/states.py:131-147)."""
    return float(np.sum(np.real(np.asarray(diag)).reshape(-1) * probabilities(state).reshape(-1)))


def norm(state):
    """|<psi|psi>| (quantumflow/qubits.py:180-182)."""
    return float(np.abs(np.vdot(state, state)))


def inner(a, b):
    """np.vdot (quantumflow/backend/numpybk.py:125-128)."""
    return complex(np.vdot(a, b))


def fidelity(a, b):
    """|<a|b>|^2 (quantumflow/measures.py:32-36)."""
    return abs(inner(a, b)) ** 2


# ------------------------------------------------------------ gates --------
def cis(x):
    return np.exp(1j * x)


def H():
    """quantumflow/stdgates.py:91-109."""
    return np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)


def X():
    return np.array([[0, 1], [1, 0]], dtype=np.complex128)


def T():
    """quantumflow/stdgates.py:133-151."""
    return np.array([[1, 0], [0, cis(np.pi / 4)]], dtype=np.complex128)


def RX(theta):
    """quantumflow/stdgates.py:179-205."""
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)


def RZ(theta):
    """quantumflow/stdgates.py:236-262."""
    return np.array([[cis(-theta / 2), 0], [0, cis(theta / 2)]], dtype=np.complex128)


def ZZ(t):
    """quantumflow/stdgates.py:944-968: diag(cis(-pi t/2), cis(pi t/2), cis(pi t/2), cis(-pi t/2))."""
    th = np.pi * t
    return np.diag([cis(-th / 2), cis(th / 2), cis(th / 2), cis(-th / 2)]).astype(np.complex128)


def CZ():
    """quantumflow/stdgates.py:267-288."""
    return np.diag([1, 1, 1, -1]).astype(np.complex128)


def CNOT():
    """quantumflow/stdgates.py:291-312."""
    return np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)


def S():
    """quantumflow/stdgates.py:112-125."""
    return np.array([[1, 0], [0, 1j]], dtype=np.complex128)


def PHASE(theta):
    """quantumflow/stdgates.py:154-166."""
    return np.array([[1, 0], [0, cis(theta)]], dtype=np.complex128)


def RY(theta):
    """quantumflow/stdgates.py:208-224."""
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return np.array([[c, -s], [s, c]], dtype=np.complex128)


def SWAP():
    """quantumflow/stdgates.py:315-338."""
    return np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def ISWAP():
    """quantumflow/stdgates.py:341-362."""
    return np.array([[1, 0, 0, 0], [0, 0, 1j, 0], [0, 1j, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def CPHASE(theta):
    """quantumflow/stdgates.py:431-446: diag(1, 1, 1, e^{i theta})."""
    return np.diag([1, 1, 1, cis(theta)]).astype(np.complex128)


def CCNOT():
    """quantumflow/stdgates.py:519-556: Toffoli, control qubits first."""
    m = np.eye(8, dtype=np.complex128)
    m[6:, 6:] = [[0, 1], [1, 0]]
    return m


NAMED = {"H": H, "X": X, "T": T, "S": S, "RX": RX, "RY": RY, "RZ": RZ, "PHASE": PHASE, "CNOT": CNOT,
         "CZ": CZ, "SWAP": SWAP, "CPHASE": CPHASE, "ZZ": ZZ, "ISWAP": ISWAP, "CCNOT": CCNOT}


def program_ops(names, params, qubits):
    """Gate list of a program of named-gate calls (quantumflow/programs.py
    Call.run :429-439: the named gate class, its parameters, its qubits)."""
    ops = []
    for name, ps, qs in zip(names, params, qubits):
        ps = [p for p in ps if not np.isnan(p)]
        qs = [int(q) for q in qs if q >= 0]
        ops.append((NAMED[str(name)](*ps), tuple(qs)))
    return ops


# ------------------------------------------------------ density matrices --
def gate_superop(u):
    """Superoperator of a k-qubit gate as a (4^k, 4^k) matrix, rows (ket-out,
    bra-out), columns (ket-in, bra-in): outer(U, U^dagger) with index groups
    (0, 3, 1, 2) (quantumflow/ops.py:244-253)."""
    u = np.asarray(u, dtype=np.complex128)
    d = u.shape[0]
    t = np.multiply.outer(u, np.conj(u).T).reshape(d, d, d, d).transpose(0, 3, 1, 2)
    return t.reshape(d * d, d * d)


def kraus_superop(ops, weights=None):
    """sum_k w_k superop(K_k) for operators on the same qubits
    (quantumflow/channels.py:58-68)."""
    weights = [1.0] * len(ops) if weights is None else weights
    return sum(w * gate_superop(k) for k, w in zip(ops, weights))


def evolve_density(rho, superop, axes):
    """rho (2^N x 2^N) after a channel on qubit axes `axes`: the superoperator
    contracted with the ket and bra axes of rho as a 2N-index tensor
    (quantumflow/ops.py:354-363, tensormul of numpybk.py:159-214)."""
    rho = np.asarray(rho, dtype=np.complex128)
    M = rho.shape[0]
    N = int(round(np.log2(M)))
    t = rho.reshape([2] * (2 * N))
    out = tensormul(np.asarray(superop).reshape([2] * (4 * len(axes))), t, list(axes) + [N + a for a in axes])
    return out.reshape(M, M)


# ------------------------------------------------------------- QAOA --------
def qubo_ops(n, edges, p, beta, gamma, weights=None, node_weights=None):
    """Gate list of quantumflow/qaoa.py:22-64 qubo_circuit for nodes 0..n-1:
    H on every node; per step ZZ(-w*gamma/pi) per edge (given order),
    RZ(node weight) where present (not gamma-scaled), RX(beta) per node."""
    ops = [(H(), (q,)) for q in range(n)]
    weights = [1.0] * len(edges) if weights is None else list(weights)
    for s in range(p):
        for (a, b), w in zip(edges, weights):
            ops.append((ZZ(-w * gamma[s] / np.pi), (a, b)))
        if node_weights is not None:
            for q in range(n):
                nw = node_weights[q]
                if nw is not None and not (isinstance(nw, float) and np.isnan(nw)):
                    ops.append((RZ(nw), (q,)))
        for q in range(n):
            ops.append((RX(beta[s]), (q,)))
    return ops


def graph_cuts(n, edges, weights=None):
    """Cut value of every basis state, [2]*n float64.

    Restates quantumflow/qaoa.py:68-81 (for each edge add its weight where the
    two node bits differ), vectorised over all 2^n states; node q is axis q,
    i.e. bit n-1-q of the flat index."""
    x = np.arange(2 ** n, dtype=np.int64)
    out = np.zeros(2 ** n, dtype=np.float64)
    weights = [1.0] * len(edges) if weights is None else list(weights)
    for (a, b), w in zip(edges, weights):
        diff = ((x >> (n - 1 - a)) ^ (x >> (n - 1 - b))) & 1
        out += w * diff
    return out.reshape([2] * n)


def qaoa_expectation(n, edges, p, beta, gamma, weights=None, node_weights=None):
    """<C> of the QAOA state (examples/qaoa_maxcut.py:56-58 objective)."""
    st = run_ops(zero_state(n), qubo_ops(n, edges, p, beta, gamma, weights, node_weights))
    return expectation(st, graph_cuts(n, edges, weights))


def qaoa_fd_gradient(n, edges, p, beta, gamma, h=1e-6, weights=None, node_weights=None):
    """Central finite differences of <C> w.r.t. (gamma, beta); the gradient
    oracle for the adjoint kernel (the reference differentiates only with its
    TensorFlow backends, quantumflow/backend/tensorflowbk.py)."""
    beta = np.array(beta, dtype=np.float64)
    gamma = np.array(gamma, dtype=np.float64)
    gg, gb = np.zeros(p), np.zeros(p)
    for i in range(p):
        for arr, dst in ((gamma, gg), (beta, gb)):
            old = arr[i]
            arr[i] = old + h
            ep = qaoa_expectation(n, edges, p, beta, gamma, weights, node_weights)
            arr[i] = old - h
            em = qaoa_expectation(n, edges, p, beta, gamma, weights, node_weights)
            arr[i] = old
            dst[i] = (ep - em) / (2 * h)
    return gg, gb


# --------------------------------------------------- random-layer circuit --
def layer_family_ops(umats, pairs):
    """The random-layer family (a U(2) on every qubit, then CZ on each pair of
    a perfect matching, per layer) from its stored gates: umats [L*N, 2, 2]
    layer-major, pairs [L, N/2, 2]."""
    L, half = pairs.shape[0], pairs.shape[1]
    N = umats.shape[0] // L
    out = []
    for layer in range(L):
        for q in range(N):
            out.append((umats[layer * N + q], (q,)))
        for a, b in pairs[layer]:
            out.append((CZ(), (int(a), int(b))))
    assert half == N // 2
    return out


def cz_layer_ops(ops_array, umats):
    """Decode the (kind, q0, q1) op table of the golden random-layer circuits
    into (matrix, axes) pairs."""
    out = []
    for (kind, a, b), u in zip(ops_array, umats):
        if kind == 1:
            out.append((u, (int(a),)))
        else:
            out.append((CZ(), (int(a), int(b))))
    return out
