"""GPU parity: fused circuit execution against the reference's outputs, and
size-independent properties at large N."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def _circuit_from_fixture(c, N):
    import quantumflow_gb300 as qf
    circ = qf.Circuit()
    for (kind, a, b), u in zip(c[f"rc{N}_ops"], c[f"rc{N}_u"]):
        circ += qf.Gate(u, qubits=[int(a)]) if kind == 1 else qf.CZ(int(a), int(b))
    return circ


@pytest.fixture(params=["fx", "ff", "fp64"])
def arith(request, monkeypatch):
    """complex128 arithmetic: fixed point (default), float-float, native FP64."""
    import quantumflow_gb300 as qf
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", request.param)
    return request.param


@pytest.fixture(params=[0, 1, 2, 4], ids=["default", "smem_tiles", "warp_rb2", "warp_rb4"])
def tile_kernel(request):
    from quantumflow_gb300 import _native as nat
    nat.call("qf_set_tile_kernel", request.param)
    yield request.param
    nat.call("qf_set_tile_kernel", 0)


@pytest.mark.parametrize("dtype,tol", [("complex128", 1e-12), ("complex64", 1e-5)])
@pytest.mark.parametrize("fusion_k", [1, 2, 4, 6, 8])
def test_reference_random_layer_circuits(golden, dtype, tol, fusion_k, tile_kernel, arith):
    import quantumflow_gb300 as qf
    c = golden["circuits"]
    for N in (4, 6, 9, 12):
        circ = _circuit_from_fixture(c, N)
        ket = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=fusion_k)
        got = ket.asarray().reshape(-1)
        err = np.max(np.abs(got - c[f"rc{N}_state"]))
        assert err < tol, (N, err)
        # fidelity against the reference's FP64 state
        assert 1 - orc.fidelity(got.astype(np.complex128), c[f"rc{N}_state"]) < 10 * tol, N
        back = circ.H.run(ket, fusion_k=fusion_k)
        err = np.max(np.abs(back.asarray().reshape(-1) - c[f"rc{N}_inverse"]))
        assert err < tol * 2, (N, err)


@pytest.mark.parametrize("c128", ["fx", "ff", "fp64"])
def test_kat_circuits(golden, c128, monkeypatch):
    import quantumflow_gb300 as qf
    from math import pi
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", c128)
    kat = golden["kat"]
    circ = qf.Circuit()
    circ += qf.RY(pi / 2, 0)
    circ += qf.RX(pi, 0)
    circ += qf.RY(pi / 2, 1)
    circ += qf.RX(pi, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.RX(-pi / 2, 1)
    circ += qf.RY(4.71572463191, 1)
    circ += qf.RX(pi / 2, 1)
    circ += qf.CNOT(0, 1)
    circ += qf.RX(-2 * 2.74973750579, 0)
    circ += qf.RX(-2 * 2.74973750579, 1)
    ket = circ.run(qf.zero_state(2))
    np.testing.assert_allclose(ket.asarray().reshape(-1), kat["true_ket_ref_run"], atol=1e-13)
    assert qf.states_close(ket, qf.State(kat["true_ket"].reshape(2, 2)))
    # gates one at a time give the same state (Gate.run path)
    k2 = qf.zero_state(2)
    for g in circ:
        k2 = g.run(k2)
    np.testing.assert_allclose(k2.asarray(), ket.asarray(), atol=1e-14)


def test_gops_circuit(golden):
    import quantumflow_gb300 as qf
    c = golden["circuits"]
    circ = qf.Circuit([qf.H(n) for n in range(8)])
    for q0, q1 in c["gops_pairs"]:
        circ += qf.X(int(q0))
        circ += qf.T(int(q1))
        circ += qf.CNOT(int(q0), int(q1))
    ket = circ.run(qf.zero_state(8))
    assert np.max(np.abs(ket.asarray().reshape(-1) - c["gops_state"])) < 1e-12


@pytest.mark.parametrize("N", [13, 16, 22])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_fused_equals_unfused_and_oracle(N, dtype, tile_kernel, arith):
    """Mixed gate classes through every fused-kernel instruction: 1q gates on
    lane, register and warp bits, 2q dense gates, permutations, diagonals."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(N)
    circ = qf.Circuit()
    for layer in range(3):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
        circ += qf.random_gate([N - 6, N - 8], random_state=rng)
        circ += qf.random_gate([1, N - 1], random_state=rng)
        circ += qf.random_gate([3, 2], random_state=rng)
        circ += qf.CNOT(N - 7, 2)
        circ += qf.ZZ(0.3, 0, N - 2)
        circ += qf.CCNOT(5, 0, N - 3)
        circ += qf.random_gate([6, 7, 8], random_state=rng)
    tol = 1e-12 if dtype == "complex128" else 2e-5
    fused = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=6)
    unfused = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=1)
    assert circ.last_passes == len(circ.elements)
    a, b = fused.asarray(), unfused.asarray()
    assert np.max(np.abs(a - b)) < tol
    if N <= 16:
        ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
        ref = orc.run_ops(orc.zero_state(N), ops)
        assert np.max(np.abs(a - ref)) < tol


@pytest.mark.parametrize("N", [26])
def test_large_round_trip(N):
    """Size-independent properties at large N: norm 1 after a random circuit,
    and circuit.H restores |0...0> (complex128 and complex64)."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(7)
    circ = qf.Circuit()
    for q in range(N):
        circ += qf.random_gate([q], random_state=rng)
    for a in range(0, N - 1, 2):
        circ += qf.CZ(a, a + 1)
    for q in range(N):
        circ += qf.random_gate([q], random_state=rng)
    for dtype, tol in (("complex128", 1e-12), ("complex64", 2e-5)):
        ket = circ.run(qf.zero_state(N, dtype=dtype))
        assert abs(ket.norm() - 1) < tol * 10
        back = circ.H.run(ket)
        probs = back.probabilities()
        assert abs(float(probs.reshape(-1)[0]) - 1) < tol * 10
        del ket, back, probs
        torch.cuda.empty_cache()


@pytest.mark.parametrize("N", [9, 12, 17])
@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
@pytest.mark.parametrize("fusion_k", [0, 3])
def test_gate_merging_equals_unmerged_and_oracle(N, dtype, fusion_k, tile_kernel, arith):
    """Host gate merging (blocks of <= 2 qubits) and the warp kernel's lane
    exchanges for 2-qubit gates on lane bits: the merged run equals the
    unmerged run and the oracle."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(100 + N)
    circ = qf.Circuit()
    for layer in range(4):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
        circ += qf.random_gate([0, 3], random_state=rng)          # two lane bits
        circ += qf.random_gate([N - 2, 1], random_state=rng)      # high, lane
        circ += qf.random_gate([4, N - 1], random_state=rng)      # lane, high
        circ += qf.CNOT(2, N - 3)
        circ += qf.SWAP(1, N - 4)
        circ += qf.RZ(0.4, 3)
        circ += qf.X(N - 5)
        circ += qf.ZZ(0.7, 0, 4)
        circ += qf.T(N - 1)
    tol = 1e-12 if dtype == "complex128" else 2e-5
    try:
        nat.call("qf_set_gate_merging", 1)
        merged = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=fusion_k).asarray().reshape(-1)
        nat.call("qf_set_gate_merging", 2)
        packed = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=fusion_k).asarray().reshape(-1)
        nat.call("qf_set_gate_merging", 0)
        plain = circ.run(qf.zero_state(N, dtype=dtype), fusion_k=fusion_k).asarray().reshape(-1)
    finally:
        nat.call("qf_set_gate_merging", 1)
    assert np.max(np.abs(merged - plain)) < tol
    assert np.max(np.abs(packed - plain)) < tol
    if N <= 12:
        ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
        ref = orc.run_ops(orc.zero_state(N), ops).reshape(-1)
        assert np.max(np.abs(merged - ref)) < tol


def test_gate_merging_random_layers_n20():
    """The random-layer workload (Haar U(2) on every qubit, CZ on a matching)
    merged vs unmerged at N=20, complex128 and complex64."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    N = 20
    rng = np.random.default_rng(5)
    circ = qf.Circuit()
    for layer in range(6):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    for dtype, tol in (("complex128", 1e-12), ("complex64", 2e-5)):
        try:
            nat.call("qf_set_gate_merging", 1)
            merged = circ.run(qf.zero_state(N, dtype=dtype)).asarray().reshape(-1)
            nat.call("qf_set_gate_merging", 0)
            plain = circ.run(qf.zero_state(N, dtype=dtype)).asarray().reshape(-1)
        finally:
            nat.call("qf_set_gate_merging", 1)
        assert np.max(np.abs(merged - plain)) < tol


@pytest.mark.parametrize("merge", [0, 1])
def test_shape_passes_random_programs(merge, monkeypatch):
    """Float-float fused passes split into straight-line shape kernels (one
    or two dense gates with CZ signs around them): random programs of Haar
    1- and 2-qubit gates and CZs, mostly on the low (lane) bits where the
    fused passes form, against the oracle, with shapes of up to three
    (default) and four gate bits, and against the same programs without
    group/shape passes (tile mode 5)."""
    import ctypes
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", "ff")
    N = 12
    rng = np.random.default_rng(77 + merge)
    low = list(range(N - 5, N))  # axes of bits 0..4
    nat.call("qf_set_gate_merging", merge)
    seen_shapes = 0
    try:
        for trial in range(24):
            circ = qf.Circuit()
            for _ in range(int(rng.integers(6, 30))):
                pick = rng.random()
                qs = [int(q) for q in rng.choice(low if rng.random() < 0.8 else range(N), 2, replace=False)]
                if pick < 0.35:
                    circ += qf.random_gate([qs[0]], random_state=rng)
                elif pick < 0.65:
                    circ += qf.random_gate(qs, random_state=rng)
                else:
                    circ += qf.CZ(*qs)
            op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))
            stats = np.zeros(8 * 256, np.int32)
            nb = ctypes.c_int()
            assert nat.lib.qf_plan_circuit(N, nat.LAYOUT_FF, nops, op_k.ctypes.data, op_axes.ctypes.data,
                                           op_mats.ctypes.data, 0, stats.ctypes.data, 256, ctypes.byref(nb)) == 0
            seen_shapes += int((stats[:8 * nb.value].reshape(-1, 8)[:, 7] == 4).sum())
            got = circ.run(qf.zero_state(N)).asarray().reshape(-1)
            ops = [(g.asoperator(), tuple(g.qubits)) for g in circ]
            ref = orc.run_ops(orc.zero_state(N), ops).reshape(-1)
            assert np.max(np.abs(got - ref)) < 1e-12, trial
            nat.call("qf_set_shape_bits", 4)  # the four-bit shape as well
            try:
                wide = circ.run(qf.zero_state(N)).asarray().reshape(-1)
            finally:
                nat.call("qf_set_shape_bits", 3)
            assert np.max(np.abs(wide - ref)) < 1e-12, trial
            nat.call("qf_set_tile_kernel", 5)
            try:
                old = circ.run(qf.zero_state(N)).asarray().reshape(-1)
            finally:
                nat.call("qf_set_tile_kernel", 0)
            assert np.max(np.abs(got - old)) < 1e-12, trial
    finally:
        nat.call("qf_set_gate_merging", 1)
    assert seen_shapes >= 10


@pytest.mark.parametrize("c128", ["ff", "fx", "fx_cuda_cores"])
def test_index_paths_above_2_31_amplitudes(c128, monkeypatch):
    """States of more than 2^31 amplitudes take the 64-bit-index forms of the
    4x4 sweep and the shape kernels (float-float), of the tensor-core passes
    (fixed point, the default) or of the fixed-point shape kernels (tensor
    cores off): N=32 complex128 (64 GB per state, 128 GB at the peak), two
    merged random layers and their inverse must return |0...0> -- norm and
    single-qubit marginals by device reductions, no host copy of the
    state."""
    import ctypes
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    from quantumflow_gb300.states import _reduce
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", "ff" if c128 == "ff" else "fx")
    layout = nat.LAYOUT_FF if c128 == "ff" else nat.LAYOUT_FX
    N = 32
    free, _ = torch.cuda.mem_get_info()
    if free < 150 * 2 ** 30:
        pytest.skip("needs 150 GB of free device memory")
    rng = np.random.default_rng(32)
    circ = qf.Circuit()
    for layer in range(2):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    for q in range(N):
        circ += qf.random_gate([q], random_state=rng)
    op_k, op_axes, op_mats, nops = circ.packed(tuple(range(N)))
    stats = np.zeros(8 * 512, np.int32)
    nb = ctypes.c_int()
    if c128 == "fx_cuda_cores":
        nat.call("qf_set_fx_tensor_cores", 0)
    try:
        assert nat.lib.qf_plan_circuit(N, layout, nops, op_k.ctypes.data, op_axes.ctypes.data,
                                       op_mats.ctypes.data, 0, stats.ctypes.data, 512, ctypes.byref(nb)) == 0
        kinds = set(stats[:8 * nb.value].reshape(-1, 8)[:, 7])
        # lone sweeps and shape passes (float-float) / tensor-core passes /
        # fixed-point shape passes
        assert {"ff": {1, 4}, "fx": {6}, "fx_cuda_cores": {4}}[c128] <= kinds
        ket = circ.run(qf.zero_state(N))
        assert abs(ket.norm() - 1) < 1e-11
        back = circ.H.run(ket)
        del ket
        assert abs(back.norm() - 1) < 1e-11
        for axis in (0, 7, 26, 31):
            p0, p1 = _reduce("qf_qubit_probabilities", back.buffer, nout=2, extra=(axis,))
            assert abs(p0 - 1) < 1e-11 and abs(p1) < 1e-11
        del back
    finally:
        nat.call("qf_set_fx_tensor_cores", 1)
        torch.cuda.empty_cache()


def test_gops_benchmark_tool():
    """The GOPS benchmark (tools/benchmark.py): gate by gate and fused give
    the same state; the oracle agrees at N=10; GOPS is positive."""
    from quantumflow_gb300 import benchmark as bm
    N, gates = 10, 100
    a = bm.benchmark(N, gates, fused=False, seed=5).cpu().numpy().reshape(-1)
    b = bm.benchmark(N, gates, fused=True, seed=5).cpu().numpy().reshape(-1)
    assert np.max(np.abs(a - b)) < 1e-12
    circ = bm.benchmark_circuit(N, gates, seed=5)
    assert len(list(circ)) == N + 3 * ((gates - N) // 3)
    ref = orc.run_ops(orc.zero_state(N), [(g.asoperator(), tuple(g.qubits)) for g in circ]).reshape(-1)
    assert np.max(np.abs(a - ref)) < 1e-12
    assert bm.benchmark_gops(N, gates, 1) > 0 and bm.benchmark_gops(N, gates, 1, fused=True) > 0


def test_autotune_fusion_and_shape_width(tmp_path, monkeypatch):
    """tune_fusion searches fusion width, kernel mode and (float-float)
    shape width on the caller's circuit, caches the winner, restores the
    process-wide settings, and use_fusion_config applies it; the result of
    the tuned configuration equals the default's."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import autotune
    monkeypatch.setenv("QUANTUMFLOW_GB300_AUTOTUNE_CACHE", str(tmp_path / "at.json"))
    N = 13
    rng = np.random.default_rng(4)
    circ = qf.Circuit()
    for layer in range(3):
        for q in range(N):
            circ += qf.random_gate([q], random_state=rng)
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            circ += qf.CZ(int(perm[a]), int(perm[a + 1]))
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", "ff")  # shape widths are a float-float setting
    best = autotune.tune_fusion(circ, N, candidates=(0, 2), modes=(0,), reps=1)
    assert {t["shape_bits"] for t in best["trials"]} == {2, 3, 4}
    cached = autotune.fusion_config("complex128", N)
    assert (cached["fusion_k"], cached["mode"], cached["shape_bits"]) == \
        (best["fusion_k"], best["mode"], best["shape_bits"])
    ref = circ.run(qf.zero_state(N)).asarray()
    try:
        k = autotune.use_fusion_config(best)
        got = circ.run(qf.zero_state(N), fusion_k=k).asarray()
    finally:
        autotune.use_fusion_config({})
    assert np.max(np.abs(got - ref)) < 1e-12
