"""Host-side routing of complex128 (QF_LAYOUT_FX) passes to the tensor-core
kernel, read through qf_plan_circuit on the CPU (no GPU needed): fused
passes of dense gates and CZ-like signs go to the tensor cores (plan kind
6); a lone 2x2 gate, a sign that sits between two dense gates on its
window bits with a bit outside the window, states below 2^11 amplitudes
and the switch qf_set_fx_tensor_cores(0) keep the CUDA-core kernels."""
import numpy as np
import pytest


@pytest.fixture
def nat():
    from quantumflow_gb300 import _native as nat
    nat.call("qf_set_fx_tensor_cores", 1)
    yield nat
    nat.call("qf_set_fx_tensor_cores", 1)


def _kinds(nat, circ, N, fusion_k=0):
    op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))
    stats = (nat.ctypes.c_int32 * (8 * 4096))()
    nb = nat.ctypes.c_int(0)
    nat.call("qf_plan_circuit", N, nat.LAYOUT_FX, nops, op_k.ctypes.data_as(nat._ip),
             op_axes.ctypes.data_as(nat._ip), op_mats.ctypes.data_as(nat._dp), fusion_k, stats, 4096,
             nat.ctypes.byref(nb))
    return [stats[8 * b + 7] for b in range(nb.value)]


def _random_layers(N, layers, seed):
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(seed)
    circ = qf.Circuit()
    for _ in range(layers):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    return circ


def test_random_layers_run_on_tensor_cores(nat):
    """The benchmark's circuit family at N=20: every fused pass is a
    tensor-core pass; with the switch off the same blocks are cut into
    CUDA-core fixed-point shape passes (more of them)."""
    circ = _random_layers(20, 4, 5)
    on = _kinds(nat, circ, 20)
    assert set(on) == {6}, on
    nat.call("qf_set_fx_tensor_cores", 0)
    off = _kinds(nat, circ, 20)
    assert 6 not in off and len(off) >= len(on)


def test_small_states_and_lone_2x2_gates_keep_cuda_cores(nat):
    import quantumflow_gb300 as qf
    circ = _random_layers(10, 2, 6)
    assert 6 not in _kinds(nat, circ, 10)       # 2^10 amplitudes: below the tensor-core tile
    lone = qf.Circuit([qf.RX(0.3, 7)])
    assert _kinds(nat, lone, 16) == [1]         # the streaming 2x2 sweep
    pair = qf.Circuit([qf.CNOT(3, 9)])
    assert _kinds(nat, pair, 16) == [6]


def test_sign_placement(nat):
    """Signs with a bit outside the window are moved to the inputs (before
    every dense gate on their window bits) or the outputs (after all of
    them); one that sits between two such gates keeps the block off the
    tensor cores."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(9)
    u = lambda q: qf.random_gate([q], random_state=rng)
    N = 16
    before = qf.Circuit([qf.CZ(2, 12), u(2), u(3), qf.CZ(2, 3)])
    after = qf.Circuit([u(2), u(3), qf.CZ(2, 3), qf.CZ(3, 14)])
    inside = qf.Circuit([u(2), qf.CZ(2, 3), u(3), u(2)])
    between = qf.Circuit([u(2), qf.CZ(2, 12), u(2)])
    for c in (before, after, inside):
        assert _kinds(nat, c, N, fusion_k=4) == [6], c
    k = _kinds(nat, between, N, fusion_k=4)
    assert 6 not in k and k, k


def test_three_and_four_qubit_gates_take_the_tensor_cores(nat):
    """A unitary gate on 3 or 4 qubits (a dense unitary, or a permutation
    with phases such as CCNOT) is one tensor-core window of its own; below
    2^11 amplitudes, or with the switch off, it runs in native FP64 (plan
    kind 5)."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(4)
    u3 = np.linalg.qr(rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8)))[0]
    u4 = np.linalg.qr(rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16)))[0]
    circ = qf.Circuit([qf.H(0), qf.CCNOT(1, 5, 9), qf.Gate(u3, qubits=(2, 7, 11)),
                       qf.Gate(u4, qubits=(3, 4, 12, 13)), qf.CNOT(0, 1)])
    k = _kinds(nat, circ, 16)
    assert k.count(6) >= 3 and 5 not in k, k
    small = qf.Circuit([qf.H(0), qf.CCNOT(1, 5, 9), qf.Gate(u3, qubits=(2, 7, 8)),
                        qf.Gate(u4, qubits=(3, 4, 6, 0))])
    assert _kinds(nat, small, 10).count(5) == 3
    nat.call("qf_set_fx_tensor_cores", 0)
    assert _kinds(nat, circ, 16).count(5) == 3
