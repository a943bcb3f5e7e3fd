"""The fixed-point complex128 arithmetic (QF_LAYOUT_FX, the default for
complex128 gates): parity with the oracle on every pass kind, routing of
non-unitary gates to native FP64, and accuracy against an extended-precision
evaluation of the same circuit, side by side with native FP64 arithmetic."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _run_circuit(circ, N, arith, fusion_k=None, monkeypatch=None):
    import quantumflow_gb300 as qf
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", arith)
    return circ.run(qf.zero_state(N), fusion_k=fusion_k).asarray().reshape(-1)


def _mixed_circuit(N, layers, rng):
    import quantumflow_gb300 as qf
    circ = qf.Circuit()
    for _ in range(layers):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
        circ += qf.random_gate([int(perm[0]), int(perm[3])], random_state=rng)
        circ += qf.CNOT(int(perm[1]), int(perm[2]))
        circ += qf.CPHASE(0.37, int(perm[4]), int(perm[0]))
        circ += qf.ZZ(0.21, int(perm[2]), int(perm[5]))
        circ += qf.T(int(perm[3]))
        circ += qf.PHASE(-0.8, int(perm[1]))
        circ += qf.SWAP(int(perm[0]), int(perm[5]))
        circ += qf.CCNOT(int(perm[1]), int(perm[4]), int(perm[2]))
    return circ


@pytest.mark.parametrize("N", [6, 12, 17])
@pytest.mark.parametrize("fusion_k", [1, 2, 3, 4])
def test_fx_mixed_circuits_against_oracle(N, fusion_k, monkeypatch):
    rng = np.random.default_rng(100 + N)
    circ = _mixed_circuit(N, 4, rng)
    got = _run_circuit(circ, N, "fx", fusion_k, monkeypatch)
    ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
    ref = orc.run_ops(orc.zero_state(N), ops).reshape(-1)
    err = float(np.max(np.abs(got - ref)))
    assert err < TOL, (N, fusion_k, err)


def test_fx_plan_uses_fixed_point_passes():
    """The planner's view of a merged random-layer circuit: passes of at
    most four gate bits, no native-FP64 pass for unitary gates (with the
    tensor cores off, the 3-qubit permutations run natively)."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(5)
    N = 20
    circ = _mixed_circuit(N, 3, rng)
    op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))
    stats = (nat.ctypes.c_int32 * (8 * 4096))()
    nb = nat.ctypes.c_int(0)
    nat.call("qf_plan_circuit", N, nat.LAYOUT_FX, nops, op_k.ctypes.data_as(nat._ip),
             op_axes.ctypes.data_as(nat._ip), op_mats.ctypes.data_as(nat._dp), 0, stats, 4096,
             nat.ctypes.byref(nb))
    kinds = [stats[8 * b + 7] for b in range(nb.value)]
    # CCNOT (a 3-qubit permutation) takes a tensor-core window of its own
    assert kinds.count(5) == 0
    assert set(kinds) <= {0, 1, 3, 4, 6}
    assert nb.value < nops
    # with the tensor cores off it is the one op class that runs natively
    nat.call("qf_set_fx_tensor_cores", 0)
    try:
        nat.call("qf_plan_circuit", N, nat.LAYOUT_FX, nops, op_k.ctypes.data_as(nat._ip),
                 op_axes.ctypes.data_as(nat._ip), op_mats.ctypes.data_as(nat._dp), 0, stats, 4096,
                 nat.ctypes.byref(nb))
    finally:
        nat.call("qf_set_fx_tensor_cores", 1)
    kinds = [stats[8 * b + 7] for b in range(nb.value)]
    assert kinds.count(5) == 3
    assert set(kinds) <= {0, 1, 3, 4, 5}


def test_fx_non_unitary_gates_run_natively():
    """Gates that are not unitary (here random complex matrices, as in the
    reference's tensormul tests) take the native FP64 kernels and match."""
    from quantumflow_gb300 import _native as nat
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(8)
    n = 9
    st = rng.normal(size=2 ** n) + 1j * rng.normal(size=2 ** n)
    for k in (1, 2):
        g = rng.normal(size=(2 ** k, 2 ** k)) + 1j * rng.normal(size=(2 ** k, 2 ** k))
        axes = [int(a) for a in rng.choice(n, size=k, replace=False)]
        src = qf.Buffer.from_complex(torch.from_numpy(st).cuda())
        out = src.empty_like()
        m = np.ascontiguousarray(g).view(np.float64).reshape(-1)
        nat.call("qf_apply_gate", nat.ptr(src.data), nat.ptr(out.data), n, nat.LAYOUT_FX, k,
                 nat.int_array(axes), m.ctypes.data_as(nat._dp), nat.stream_handle())
        ref = orc.tensormul(g, st, axes).reshape(-1)
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(out.data.cpu().numpy() - ref)) / scale < 1e-14


@pytest.mark.parametrize("N", [10, 14])
def test_fx_accuracy_against_extended_precision(N, monkeypatch):
    """The same random-layer circuit in fixed point and in native FP64, both
    against an extended-precision (np.clongdouble) evaluation: the fixed-point
    result is at least as close as FP64's (within a factor 1.5), and both
    are far inside the 1e-12 parity bar."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(N)
    circ = qf.Circuit()
    for _ in range(20):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
    exact = orc.run_ops(orc.zero_state(N).astype(np.clongdouble), ops, np.clongdouble).reshape(-1)
    errs = {}
    for arith in ("fx", "fp64", "ff"):
        got = _run_circuit(circ, N, arith, None, monkeypatch).astype(np.clongdouble)
        errs[arith] = float(np.max(np.abs(got - exact)))
    print(f"N={N}, {len(ops)} gates, max |amp - extended|: " +
          ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert errs["fx"] < 1e-14
    assert errs["fx"] <= 1.5 * errs["fp64"], errs
