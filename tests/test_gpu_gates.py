"""GPU parity: single-gate application (the tensormul hot path) through the
C ABI against the CPU oracle and the reference's own outputs."""
import itertools

import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu

# tolerances: complex128 (FP64, float-float and fixed-point arithmetic) 1e-12
# max amplitude error, complex64 1e-5 (the parity bar of this backend)
TOL = {0: 1e-5, 1: 1e-12, 2: 1e-12, 3: 1e-12}
LAYOUTS = [0, 1, 2, 3]


def _run(state_np, mat, axes, layout):
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    n = int(np.log2(state_np.size))
    dt = torch.complex64 if layout == 0 else torch.complex128
    t = torch.from_numpy(state_np.reshape(-1).astype(np.complex128)).to("cuda").to(dt)
    src = qf.Buffer.from_complex(t).to_layout(layout)
    out = src.empty_like()
    m = np.ascontiguousarray(np.asarray(mat, dtype=np.complex128)).view(np.float64).reshape(-1)
    nat.call("qf_apply_gate", nat.ptr(src.data), nat.ptr(out.data), n, layout, len(axes),
             nat.int_array(axes), m.ctypes.data_as(nat._dp), nat.stream_handle())
    return out.complex().cpu().numpy().astype(np.complex128)


def _rand_state(n, rng):
    s = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    return s / np.linalg.norm(s)


@pytest.mark.parametrize("layout", LAYOUTS)
def test_reference_tensormul_fixtures(golden, layout):
    g = golden["tensormul"]
    for c in range(int(g["tm_count"])):
        st = g[f"tm{c}_state"]
        scale = np.max(np.abs(g[f"tm{c}_out"]))
        out = _run(st, g[f"tm{c}_gate"], list(g[f"tm{c}_idx"]), layout)
        err = np.max(np.abs(out - g[f"tm{c}_out"])) / scale
        assert err < TOL[layout] * 10, (c, err)


@pytest.mark.parametrize("layout", LAYOUTS)
def test_every_axis_1q_2q(layout):
    rng = np.random.default_rng(1)
    for n in (1, 2, 3, 5, 6, 7, 9):
        st = _rand_state(n, rng)
        for a in range(n):
            u = orc.RX(0.7) @ orc.RZ(1.3) @ orc.H()
            ref = orc.tensormul(u, st, [a]).reshape(-1)
            assert np.max(np.abs(_run(st, u, [a], layout) - ref)) < TOL[layout]
        if n >= 2:
            for a, b in itertools.permutations(range(n), 2):
                u = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0]
                ref = orc.tensormul(u, st, [a, b]).reshape(-1)
                assert np.max(np.abs(_run(st, u, [a, b], layout) - ref)) < TOL[layout]


@pytest.mark.parametrize("layout", LAYOUTS)
def test_structured_gates(layout):
    """Diagonal, sign, permutation and dense k=3..5 classes of the planner."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(2)
    n = 8
    st = _rand_state(n, rng)
    gates = [qf.CZ(1, 6), qf.CNOT(7, 0), qf.SWAP(2, 5), qf.ISWAP(3, 4), qf.ZZ(0.3, 0, 7),
             qf.CCNOT(1, 4, 6), qf.CSWAP(7, 2, 0), qf.T(3), qf.X(0), qf.Y(5), qf.PHASE(0.2, 6),
             qf.CPHASE(0.9, 2, 1), qf.PSWAP(0.4, 6, 3)]
    for g in gates:
        axes = list(g.qubits)
        ref = orc.tensormul(g.asoperator(), st, axes).reshape(-1)
        assert np.max(np.abs(_run(st, g.asoperator(), axes, layout) - ref)) < TOL[layout], g.name
    for k in (3, 4, 5):
        u = np.linalg.qr(rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k)))[0]
        axes = list(rng.choice(n, size=k, replace=False))
        ref = orc.tensormul(u, st, axes).reshape(-1)
        assert np.max(np.abs(_run(st, u, axes, layout) - ref)) < TOL[layout] * 4, k


@pytest.mark.parametrize("layout", LAYOUTS)
def test_large_state_low_and_high_bits(layout):
    """N=20: shuffle path (bits < 5) and strided path, against the oracle."""
    rng = np.random.default_rng(3)
    n = 20
    st = _rand_state(n, rng)
    u = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))[0]
    for a in (0, 7, 15, 17, 19):
        ref = orc.tensormul(u, st, [a]).reshape(-1)
        assert np.max(np.abs(_run(st, u, [a], layout) - ref)) < TOL[layout]


def test_gate_run_api_and_in_place_aliasing():
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    ket = qf.zero_state(3)
    ket = qf.H(0).run(ket)
    ket = qf.CNOT(0, 1).run(ket)
    probs = ket.probabilities().cpu().numpy().reshape(-1)
    np.testing.assert_allclose(probs, [0.5, 0, 0, 0, 0, 0, 0.5, 0], atol=1e-14)
    # in place: psi_out == psi_in
    rng = np.random.default_rng(4)
    st = _rand_state(10, rng)
    buf = qf.Buffer.from_complex(torch.from_numpy(st).cuda()).to_layout(2)
    u = orc.RX(0.4)
    m = np.ascontiguousarray(u).view(np.float64).reshape(-1)
    nat.call("qf_apply_gate", nat.ptr(buf.data), nat.ptr(buf.data), 10, 2, 1, nat.int_array([3]),
             m.ctypes.data_as(nat._dp), nat.stream_handle())
    ref = orc.tensormul(u, st, [3]).reshape(-1)
    assert np.max(np.abs(buf.complex().cpu().numpy() - ref)) < 1e-12


def test_errors_raise():
    import quantumflow_gb300 as qf
    from quantumflow_gb300._native import NativeError
    ket = qf.zero_state(3)
    with pytest.raises(ValueError):
        qf.H(7).run(ket)  # unknown qubit label (reference ops.py:164 list.index)
    from quantumflow_gb300 import _native as nat
    fake = nat._vp(0x10000)
    m = np.eye(64, dtype=np.complex128).view(np.float64).reshape(-1)
    # host-matrix entry point: k > 5 is for qf_apply_dense_gate
    assert nat.lib.qf_apply_gate(fake, fake, 8, 1, 6, nat.int_array(range(6)), m.ctypes.data_as(nat._dp),
                                 None) == 6
    # device-matrix entry point: k above QF_MAX_DENSE_QUBITS, misaligned matrix
    assert nat.lib.qf_apply_dense_gate(fake, fake, 14, 1, 13, nat.int_array(range(13)), fake, None) == 6
    assert nat.lib.qf_apply_dense_gate(fake, fake, 8, 1, 6, nat.int_array(range(6)), nat._vp(0x10008),
                                       None) == 4
    with pytest.raises(NativeError):  # unknown layout
        nat.call("qf_apply_dense_gate", fake, fake, 8, 9, 6, nat.int_array(range(6)), fake, None)
    assert nat.device_error() == 0
