"""Complex128 passes on the tensor cores (csrc/tcfx.cu, the default for
complex128 states of at least 2^11 amplitudes): bit-for-bit agreement with
the CPU model of the digit arithmetic (tests/txarith.py), parity with the
oracle (the reference's numpy backend restated) at 1e-12 on circuits with
every op class the pass takes, sign ops on both sides of the gates, in and
out of place.  The planner's routing is tested on the CPU
(tests/test_tensor_fx_plan.py)."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc
import txarith as tx

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture
def tensor_cores():
    from quantumflow_gb300 import _native as nat
    nat.call("qf_set_fx_tensor_cores", 1)
    yield nat
    nat.call("qf_set_fx_tensor_cores", 1)


def _rand_state(n, rng, spread=False):
    s = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    if spread:  # amplitudes over many binades, some exact zeros
        s *= 10.0 ** rng.uniform(-9, 0, size=2 ** n)
        s[rng.integers(0, 2 ** n, 2 ** (n - 4))] = 0
    return s / np.linalg.norm(s)


def _apply(state, mat, axes, inplace=False):
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    n = int(np.log2(state.size))
    t = torch.from_numpy(state.reshape(-1).astype(np.complex128)).to("cuda")
    src = qf.Buffer.from_complex(t).to_layout(nat.LAYOUT_FX)
    out = src if inplace else src.empty_like()
    m = np.ascontiguousarray(np.asarray(mat, dtype=np.complex128)).view(np.float64).reshape(-1)
    nat.call("qf_apply_gate", nat.ptr(src.data), nat.ptr(out.data), n, nat.LAYOUT_FX, len(axes),
             nat.int_array(axes), m.ctypes.data_as(nat._dp), nat.stream_handle())
    return out.complex().cpu().numpy().astype(np.complex128)


def _model(state, mat, axes):
    """The CPU model of one tensor-core pass of a single 4x4 gate (a lone
    2x2 gate takes the CUDA-core sweep): the window is the gate's bits
    (matrix MSB first) padded with the highest other bits."""
    n = int(np.log2(state.size))
    k = len(axes)
    gb = [n - 1 - a for a in axes]
    wb = list(gb)
    b = n - 1
    while len(wb) < 4:
        if b not in wb:
            wb.append(b)
        b -= 1
    mat = np.asarray(mat, dtype=np.complex128)

    def local(c):
        r = 0
        for j in range(k):
            r = (r << 1) | ((c >> j) & 1)
        return r
    U = np.zeros((16, 16), dtype=np.complex128)
    for r in range(16):
        for c in range(16):
            if (r >> k) == (c >> k):
                U[r, c] = mat[local(r), local(c)]
    g = tx.gate_integers(U)
    gd = tx.gate_digits(g)
    off = np.array([sum(((c >> j) & 1) << wb[j] for j in range(4)) for c in range(16)], dtype=np.int64)
    wmask = sum(1 << w for w in wb)
    psi = state.reshape(-1)
    out = np.empty_like(psi)
    for base in range(2 ** n):
        if base & wmask:
            continue
        idx = base | off
        out[idx] = tx.pass_row(g, psi[idx], gd)
    return out


@pytest.mark.parametrize("n,axes", [(11, [3, 9]), (11, [0, 7]), (12, [10, 2]), (12, [11, 0])])
def test_single_gate_bit_exact_against_model(tensor_cores, n, axes):
    rng = np.random.default_rng(7 + n + axes[0])
    st = _rand_state(n, rng, spread=True)
    k = len(axes)
    u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
    got = _apply(st, u, axes)
    want = _model(st, u, axes)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), \
        float(np.max(np.abs(got - want)))
    ref = orc.tensormul(u, st.reshape([2] * n), axes).reshape(-1)
    assert np.max(np.abs(got - ref)) < TOL


@pytest.mark.parametrize("n", [11, 13, 16])
def test_single_gates_every_kind_against_oracle(tensor_cores, n):
    rng = np.random.default_rng(n)
    st = _rand_state(n, rng)
    gates = [orc.H(), orc.RX(0.7) @ orc.RZ(1.3), np.diag([1, np.exp(0.3j)]),
             np.array([[0, 1], [1, 0]]), orc.CNOT(), np.diag([1, 1, 1, -1]),
             np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0]]
    for i, u in enumerate(gates):
        k = int(np.log2(u.shape[0]))
        axes = list(rng.choice(n, k, replace=False))
        for inplace in (False, True):
            got = _apply(st, u, axes, inplace)
            ref = orc.tensormul(np.asarray(u, dtype=np.complex128), st.reshape([2] * n), axes).reshape(-1)
            assert np.max(np.abs(got - ref)) < TOL, (i, axes, inplace)


def _layers_with_signs(N, layers, rng):
    """Random layers whose CZs straddle every fused window: signs before and
    after the dense gates of a pass, inside and outside its bits."""
    import quantumflow_gb300 as qf
    circ = qf.Circuit()
    for _ in range(layers):
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
        circ += qf.CPHASE(0.37, int(perm[0]), int(perm[1]))
        circ += qf.ZZ(0.21, int(perm[2]), int(perm[3]))
        circ += qf.T(int(perm[4]))
        circ += qf.SWAP(int(perm[0]), int(perm[5]))
        circ += qf.CNOT(int(perm[6]), int(perm[1]))
    return circ


@pytest.mark.parametrize("N", [11, 14, 18])
@pytest.mark.parametrize("fusion_k", [2, 4])
def test_fused_circuits_against_oracle(tensor_cores, N, fusion_k, monkeypatch):
    import quantumflow_gb300 as qf
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", "fx")
    rng = np.random.default_rng(300 + N)
    circ = _layers_with_signs(N, 3, rng)
    got = circ.run(qf.zero_state(N), fusion_k=fusion_k).asarray().reshape(-1)
    ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
    ref = orc.run_ops(orc.zero_state(N), ops).reshape(-1)
    err = float(np.max(np.abs(got - ref)))
    assert err < TOL, (N, fusion_k, err)
    # the same circuit with the CUDA-core fixed-point kernels
    tensor_cores.call("qf_set_fx_tensor_cores", 0)
    alt = circ.run(qf.zero_state(N), fusion_k=fusion_k).asarray().reshape(-1)
    assert float(np.max(np.abs(alt - ref))) < TOL


@pytest.mark.parametrize("n", [11, 14])
def test_three_and_four_qubit_gates_against_oracle(tensor_cores, n):
    """Unitary gates on 3 and 4 qubits (dense, and permutations with phases
    such as CCNOT) run as tensor-core windows of their own: against the
    oracle at 1e-12, in and out of place."""
    rng = np.random.default_rng(60 + n)
    st = _rand_state(n, rng)
    gates = [np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0],
             np.linalg.qr(rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16)))[0],
             orc.CCNOT(),
             np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, 8)))[[3, 1, 2, 0, 6, 7, 4, 5]]]
    for i, u in enumerate(gates):
        k = int(np.log2(u.shape[0]))
        axes = [int(a) for a in rng.choice(n, k, replace=False)]
        for inplace in (False, True):
            got = _apply(st, u, axes, inplace)
            ref = orc.tensormul(np.asarray(u, dtype=np.complex128), st.reshape([2] * n), axes).reshape(-1)
            assert np.max(np.abs(got - ref)) < TOL, (i, axes, inplace)



def test_extreme_rows_bit_exact_against_model(tensor_cores):
    """Rows over the whole exponent range: all-zero rows, rows whose largest
    part is below 2^-959 (they become 0, as in the CUDA-core fixed point),
    rows near 2^900 and rows with parts 600 binades apart -- bit for bit
    against the CPU model."""
    n = 11
    rng = np.random.default_rng(77)
    st = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    scale = np.ones(2 ** n)
    gb = [n - 1 - a for a in (4, 9)]
    wb = gb + [b for b in range(n - 1, -1, -1) if b not in gb][:2]
    wmask = sum(1 << w for w in wb)
    bases = [b for b in range(2 ** n) if not b & wmask]
    off = [sum(((c >> j) & 1) << wb[j] for j in range(4)) for c in range(16)]
    for i, base in enumerate(bases):
        kind = i % 5
        idx = [base | o for o in off]
        if kind == 0:
            scale[idx] = 0.0
        elif kind == 1:
            scale[idx] = 1e-300
        elif kind == 2:
            scale[idx] = 2.0 ** 900
        elif kind == 3:
            scale[idx] = 10.0 ** rng.uniform(-180, 0, 16)
    st = st * scale
    u = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0]
    got = _apply(st, u, [4, 9])
    want = _model(st, u, [4, 9])
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    assert np.all(np.isfinite(got))
