"""The reference-API backend module (refbackend) on the GPU, checked against
numpy semantics the way the reference's own backend tests check theirs
(tests/test_backend.py of the reference: inner vs vdot, outer, absolute and
productdiag literals), plus tensormul against the oracle."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def test_backend_primitives():
    import quantumflow_gb300.refbackend as bk
    rng = np.random.default_rng(0)
    v0 = rng.normal(size=[2, 2, 2, 2]) + 1j * rng.normal(size=[2, 2, 2, 2])
    v1 = rng.normal(size=[2, 2, 2, 2]) + 1j * rng.normal(size=[2, 2, 2, 2])
    assert abs(np.vdot(v0, v1) - complex(bk.evaluate(bk.inner(bk.astensor(v0), bk.astensor(v1))))) < 1e-12
    s0 = rng.normal(size=[2, 2]) + 1j * rng.normal(size=[2, 2])
    s1 = rng.normal(size=[2, 2, 2]) + 1j * rng.normal(size=[2, 2, 2])
    res = bk.astensorproduct(bk.outer(bk.astensor(s0), bk.astensor(s1)))
    assert bk.rank(res) == 5
    assert np.allclose(bk.evaluate(res), np.outer(s0, s1).reshape([2] * 5))
    t = bk.absolute(bk.astensor([-2.25 + 4.75j, -3.25 + 5.75j]))
    assert np.allclose(bk.evaluate(t), [5.25594902, 6.60492229])
    t = bk.astensorproduct([[0., 0., 0., 6.], [0., 1., 0., 0.], [0., 0., 2., 1.], [4., 0., 1., 3.]])
    assert np.allclose(bk.evaluate(bk.productdiag(t)), [[0, 1], [2, 3]])
    tr = bk.evaluate(bk.trace(bk.reshape(bk.astensor(np.asarray([[1, 0, 0, 0], [0, -1, 0, 0], [0, 0, 2.7, 1],
                                                                    [0, 0, 1, 0.3j]])), (4, 4))))
    assert abs(tr - (2.7 + 0.3j)) < 1e-12
    x = bk.astensor([1.0 + 2.0j, 0.5 - 0.2j])
    assert np.allclose(bk.evaluate(bk.real(x)), [1.0, 0.5]) and np.allclose(bk.evaluate(bk.imag(x)), [2.0, -0.2])
    assert bk.size(bk.astensor(np.eye(4))) == 16
    assert bk.gpu_available()
    assert abs(bk.cis(0.3) - np.exp(0.3j)) < 1e-15


@pytest.mark.parametrize("N,K", [(3, 1), (6, 2), (9, 3), (12, 2), (8, 5)])
def test_tensormul_against_oracle(N, K):
    import quantumflow_gb300.refbackend as bk
    rng = np.random.default_rng(N * 10 + K)
    state = rng.normal(size=[2] * N) + 1j * rng.normal(size=[2] * N)
    gate = rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K))
    idx = [int(i) for i in rng.choice(N, size=K, replace=False)]
    out = bk.tensormul(bk.astensorproduct(gate.reshape([2] * (2 * K))), bk.astensorproduct(state), idx)
    ref = orc.tensormul(gate, state, idx)
    assert tuple(out.shape) == (2,) * N
    assert np.max(np.abs(bk.evaluate(out) - ref)) < 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("K", [2, 3, 4])
def test_unitary_tensormul_on_tensor_cores(K):
    """Unitary gates through the backend module on a 12-qubit state: the
    complex128 tensor-core pass (unmodified reference code reaches it
    through Gate.run -> bk.tensormul)."""
    import quantumflow_gb300.refbackend as bk
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(90 + K)
    N = 12
    state = rng.normal(size=[2] * N) + 1j * rng.normal(size=[2] * N)
    gate = np.linalg.qr(rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K)))[0]
    idx = [int(i) for i in rng.choice(N, size=K, replace=False)]
    nat.timing_collect()
    nat.timing_enable(True)
    try:
        out = bk.tensormul(bk.astensorproduct(gate.reshape([2] * (2 * K))), bk.astensorproduct(state), idx)
        res = bk.evaluate(out)
    finally:
        nat.timing_enable(False)
    assert nat.timing_collect()["fx_tensor"][1] == 1
    ref = orc.tensormul(gate, state, idx)
    assert np.max(np.abs(res - ref)) < 1e-12 * np.max(np.abs(ref))


def test_reference_fixture_tensormul(golden):
    import quantumflow_gb300.refbackend as bk
    g = golden["tensormul"]
    for c in range(int(g["tm_count"])):
        K = len(g[f"tm{c}_idx"])
        out = bk.tensormul(bk.astensorproduct(g[f"tm{c}_gate"].reshape([2] * (2 * K))),
                           bk.astensorproduct(g[f"tm{c}_state"]), list(g[f"tm{c}_idx"]))
        assert np.max(np.abs(bk.evaluate(out).reshape(-1) - g[f"tm{c}_out"])) < 1e-11
