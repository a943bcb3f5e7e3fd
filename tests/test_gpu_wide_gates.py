"""Dense gates on more than five qubits (qf_apply_dense_gate): the
reference's tensormul takes any K up to the state's rank
(quantumflow/backend/numpybk.py:159-214); wide gates come from
Gate.__matmul__ (quantumflow/ops.py:187-198) and Circuit.asgate
(quantumflow/circuits.py:111-118).  Checked against the reference's own
tensormul outputs (K = 4..7) and the oracle (K up to 10), in every layout,
through Gate.run, Circuit.run and the reference-backend module."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu

TOL = {0: 1e-5, 1: 1e-12, 2: 1e-12, 3: 1e-12}


def _dense(state_np, mat, axes, layout):
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    n = int(np.log2(state_np.size))
    dt = torch.complex64 if layout == 0 else torch.complex128
    t = torch.from_numpy(state_np.reshape(-1).astype(np.complex128)).to("cuda").to(dt)
    src = qf.Buffer.from_complex(t).to_layout(layout)
    out = src.empty_like()
    dmat = torch.from_numpy(np.ascontiguousarray(mat, dtype=np.complex128)).cuda()
    nat.call("qf_apply_dense_gate", nat.ptr(src.data), nat.ptr(out.data), n, layout, len(axes),
             nat.int_array(axes), nat.ptr(dmat), nat.stream_handle())
    return out.complex().cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("layout", [0, 1, 2, 3])
def test_reference_wide_tensormul_fixtures(layout):
    from tests.conftest import load_golden
    g = load_golden("tensormul_wide.npz")
    for c in range(int(g["tw_count"])):
        ref = g[f"tw{c}_out"]
        out = _dense(g[f"tw{c}_state"], g[f"tw{c}_gate"], [int(i) for i in g[f"tw{c}_idx"]], layout)
        err = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
        assert err < TOL[layout] * 10, (c, err)


@pytest.mark.parametrize("layout", [0, 1, 3])
@pytest.mark.parametrize("n,k", [(10, 8), (12, 10), (9, 9), (13, 6)])
def test_wide_unitaries_against_oracle(layout, n, k):
    rng = np.random.default_rng(n * 16 + k)
    st = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    st /= np.linalg.norm(st)
    u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
    axes = [int(a) for a in rng.choice(n, size=k, replace=False)]
    ref = orc.tensormul(u, st, axes).reshape(-1)
    assert np.max(np.abs(_dense(st, u, axes, layout) - ref)) < TOL[layout]


def test_in_place_and_api_paths():
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(3)
    n, k = 11, 7
    st = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    st /= np.linalg.norm(st)
    u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
    axes = [3, 0, 9, 5, 10, 1, 7]
    ref = orc.tensormul(u, st, axes).reshape(-1)
    # in place (psi_out == psi_in)
    buf = qf.Buffer.from_complex(torch.from_numpy(st).cuda())
    dmat = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    nat.call("qf_apply_dense_gate", nat.ptr(buf.data), nat.ptr(buf.data), n, 1, k, nat.int_array(axes),
             nat.ptr(dmat), nat.stream_handle())
    assert np.max(np.abs(buf.data.cpu().numpy() - ref)) < 1e-12
    # Gate.run and Circuit.run (a wide gate between fused runs of small ones)
    ket = qf.State(st.reshape([2] * n))
    g = qf.Gate(u.reshape([2] * (2 * k)), qubits=axes)
    assert np.max(np.abs(g.run(ket).asarray().reshape(-1) - ref)) < 1e-12
    h = qf.H(2)
    circ = qf.Circuit([h, g, qf.CNOT(4, 6)])
    want = orc.tensormul(orc.CNOT(), orc.tensormul(u, orc.tensormul(h.asoperator(), st, [2]), axes), [4, 6])
    got = circ.run(ket).asarray().reshape(-1)
    assert np.max(np.abs(got - want.reshape(-1))) < 1e-12
    # Circuit.asgate on 7 qubits, applied as one wide gate
    c2 = qf.Circuit([qf.random_gate([q], random_state=rng) for q in range(7)] +
                    [qf.CZ(0, 6), qf.ISWAP(2, 5), qf.CCNOT(1, 3, 4)])
    z = qf.zero_state(7)
    a = c2.run(z).asarray().reshape(-1)
    b = c2.asgate().run(z).asarray().reshape(-1)
    assert np.max(np.abs(a - b)) < 1e-12


def test_reference_backend_wide_tensormul():
    """The reference-backend module (what unmodified reference code calls)
    contracting a 6-qubit gate tensor into a 12-axis tensor, as
    Gate.__matmul__ does for two 6-qubit gates."""
    from quantumflow_gb300 import refbackend as bk
    rng = np.random.default_rng(6)
    K, N = 6, 12
    a = rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K))
    b = rng.normal(size=2 ** N) + 1j * rng.normal(size=2 ** N)
    idx = [0, 1, 2, 3, 4, 5]
    out = bk.tensormul(bk.astensorproduct(a.reshape([2] * (2 * K))), bk.astensorproduct(b), idx)
    ref = orc.tensormul(a, b, idx).reshape(-1)
    got = bk.evaluate(out).reshape(-1)
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-13


@pytest.mark.parametrize("n,k", [(12, 5), (13, 6), (16, 6), (20, 5), (22, 6)])
def test_tensor_core_dense_gates_c64(n, k):
    """Dense complex64 gates on 5 and 6 qubits on the tensor cores (tcgen05,
    split-TF32 operands) against the oracle and against the CUDA-core kernel,
    out of place and in place, on scattered and on the lowest bits."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(n * 8 + k)
    st = (rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n))
    st /= np.linalg.norm(st)
    u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
    for axes in ([int(a) for a in rng.choice(n, size=k, replace=False)], list(range(n - k, n))):
        ref = orc.tensormul(u, st, axes).reshape(-1)
        scale = np.max(np.abs(ref))
        tc = _dense(st, u, axes, 0)
        assert np.max(np.abs(tc - ref)) / scale < 1e-5, axes
        try:
            nat.call("qf_set_dense_tensor_cores", 0)
            cc = _dense(st, u, axes, 0)
        finally:
            nat.call("qf_set_dense_tensor_cores", 1)
        assert np.max(np.abs(tc - cc)) / scale < 1e-5
        # in place
        buf = qf.Buffer.from_complex(torch.from_numpy(st.astype(np.complex64)).cuda())
        dmat = torch.from_numpy(np.ascontiguousarray(u)).cuda()
        nat.call("qf_apply_dense_gate", nat.ptr(buf.data), nat.ptr(buf.data), n, 0, k, nat.int_array(axes),
                 nat.ptr(dmat), nat.stream_handle())
        got = buf.data.cpu().numpy().astype(np.complex128)
        assert np.max(np.abs(got - ref)) / scale < 1e-5
    assert nat.device_error() == 0
