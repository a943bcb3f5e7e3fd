"""Batched QAOA (one persistent launch for many uneven instances) against the
single-instance adjoint path, the CPU oracle, and reference fixtures."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu


def _mixed_instances(count, seed, nmin=4, nmax=13, pmax=4):
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(seed)
    graphs, ps = [], []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        if i % 2 and n % 2 == 0 and n > 3:
            g = qf.qaoa.random_regular_graph(3, n, seed=int(rng.integers(1 << 30)))
        else:
            g = qf.qaoa.gnp_random_graph(n, 0.5, seed=int(rng.integers(1 << 30)))
        graphs.append(g)
        ps.append(int(rng.integers(1, pmax + 1)))
    return graphs, ps, rng


@pytest.mark.parametrize("dtype,tol", [("complex64", 2e-4), ("complex128", 1e-9)])
def test_batch_matches_single_instance(dtype, tol):
    import quantumflow_gb300 as qf
    graphs, ps, rng = _mixed_instances(40, 5)
    betas = [rng.uniform(0, np.pi, p) for p in ps]
    gammas = [rng.uniform(0, np.pi, p) for p in ps]
    batch = qf.batched.QAOABatch(graphs, ps, dtype=dtype)
    batch.set_angles(betas, gammas)
    es, dbs, dgs = batch.evaluate()
    for i in range(len(graphs)):
        prob = qf.QAOAMaxCut(graphs[i], ps[i])
        e, gb, gg = prob.expectation_and_grad(betas[i], gammas[i])
        scale = max(1.0, abs(e))
        assert abs(es[i] - e) < tol * scale, (i, es[i], e)
        np.testing.assert_allclose(dbs[i], gb, atol=tol * scale * 4)
        np.testing.assert_allclose(dgs[i], gg, atol=tol * scale * 4)
    from quantumflow_gb300 import _native as nat
    assert nat.device_error() == 0


@pytest.mark.parametrize("tile_bits", [8, 9, 10])
def test_batch_large_instances_tiled(tile_bits):
    """With multi-instance passes held back, instances above the tile size
    run the persistent kernel's global-scratch tiled passes (clusters of 8
    CTAs from tile + 4 qubits)."""
    import quantumflow_gb300 as qf
    rng = np.random.default_rng(9)
    graphs = [qf.qaoa.random_regular_graph(3, n, seed=n) for n in (12, 14, 16, 10)]
    ps = [3, 2, 2, 4]
    betas = [rng.uniform(0, np.pi, p) for p in ps]
    gammas = [rng.uniform(0, np.pi, p) for p in ps]
    batch = qf.batched.QAOABatch(graphs, ps, dtype="complex128", tile_bits=tile_bits, ctas=16, wave_min=99)
    assert batch.nwave == 0
    assert batch.nlarge == sum(n >= tile_bits + 4 for n in (12, 14, 16, 10))
    batch.set_angles(betas, gammas)
    es, dbs, dgs = batch.evaluate()
    for i, g in enumerate(graphs):
        e, gb, gg = qf.QAOAMaxCut(g, ps[i]).expectation_and_grad(betas[i], gammas[i])
        assert abs(es[i] - e) < 1e-9
        np.testing.assert_allclose(dbs[i], gb, atol=1e-8)
        np.testing.assert_allclose(dgs[i], gg, atol=1e-8)


@pytest.mark.parametrize("dtype,tol", [("complex64", 2e-4), ("complex128", 1e-9)])
@pytest.mark.parametrize("tile_bits", [8, 10])
def test_batch_wave_passes_match_single_instance(dtype, tol, tile_bits):
    """Uneven instances above the tile size (n up to 18, p 1..5) as
    multi-instance warp-tile passes, mixed with shared-memory instances in
    one evaluation, against the single-instance adjoint path."""
    import quantumflow_gb300 as qf
    graphs, ps, rng = _mixed_instances(24, 17, nmin=6, nmax=18, pmax=5)
    betas = [rng.uniform(0, np.pi, p) for p in ps]
    gammas = [rng.uniform(0, np.pi, p) for p in ps]
    batch = qf.batched.QAOABatch(graphs, ps, dtype=dtype, tile_bits=tile_bits, ctas=152)
    assert batch.nwave == sum(g.number_of_nodes() > tile_bits for g in graphs)
    assert 0 < batch.nwave < len(graphs)
    batch.set_angles(betas, gammas)
    es, dbs, dgs = batch.evaluate()
    for i in range(len(graphs)):
        e, gb, gg = qf.QAOAMaxCut(graphs[i], ps[i]).expectation_and_grad(betas[i], gammas[i])
        scale = max(1.0, abs(e))
        assert abs(es[i] - e) < tol * scale, (i, es[i], e)
        np.testing.assert_allclose(dbs[i], gb, atol=tol * scale * 4)
        np.testing.assert_allclose(dgs[i], gg, atol=tol * scale * 4)
    # a second evaluation with other angles reuses the uploaded plan
    batch.set_angles(gammas, betas)
    es2, _, _ = batch.evaluate()
    for i in (0, len(graphs) - 1):
        e = qf.QAOAMaxCut(graphs[i], ps[i]).expectation(gammas[i], betas[i])
        assert abs(es2[i] - e) < tol * max(1.0, abs(e))


def test_batch_wave_graph_replay():
    """Adam steps replayed from a CUDA graph over multi-instance passes equal
    the eager steps (the coefficient tables follow the device angles)."""
    import quantumflow_gb300 as qf
    graphs, ps, rng = _mixed_instances(12, 23, nmin=13, nmax=17, pmax=3)
    batch = qf.batched.QAOABatch(graphs, ps, dtype="complex64", tile_bits=10)
    assert batch.nwave == len(graphs)
    betas = [np.full(p, 0.3) for p in ps]
    gammas = [np.full(p, 0.3) for p in ps]
    batch.set_angles(betas, gammas)
    e0, _, _ = batch.evaluate()
    batch.adam(12, lr=0.05, use_graph=True)
    e1, _, _ = batch.evaluate()
    assert np.mean(e1 - e0) > 0.05
    batch.set_angles(betas, gammas)
    batch.adam(12, lr=0.05, use_graph=False)
    e2, _, _ = batch.evaluate()
    np.testing.assert_allclose(e2, e1, rtol=1e-5, atol=1e-5)


def test_batch_reference_fixtures(golden):
    import quantumflow_gb300 as qf
    q = golden["qaoa"]
    names = ["er6p5", "reg8", "reg10", "er9", "reg16p8"]
    graphs = []
    for name in names:
        g = qf.Graph(nodes=range(int(q[f"{name}_n"])))
        for a, b in q[f"{name}_edges"]:
            g.add_edge(int(a), int(b))
        graphs.append(g)
    ps = [int(q[f"{name}_p"]) for name in names]
    batch = qf.batched.QAOABatch(graphs, ps, dtype="complex128")
    batch.set_angles([q[f"{n}_beta"] for n in names], [q[f"{n}_gamma"] for n in names])
    es, dbs, dgs = batch.evaluate()
    for i, name in enumerate(names):
        assert abs(es[i] - float(q[f"{name}_expectation"])) < 1e-10
        np.testing.assert_allclose(dbs[i], q[f"{name}_fd_grad_beta"], atol=2e-7)
        np.testing.assert_allclose(dgs[i], q[f"{name}_fd_grad_gamma"], atol=2e-7)


def test_batch_adam_graph_replay_improves_all():
    import quantumflow_gb300 as qf
    graphs, ps, rng = _mixed_instances(64, 3, nmin=6, nmax=12, pmax=3)
    batch = qf.batched.QAOABatch(graphs, ps, dtype="complex64")
    betas = [np.full(p, 0.3) for p in ps]
    gammas = [np.full(p, 0.3) for p in ps]
    batch.set_angles(betas, gammas)
    e0, _, _ = batch.evaluate()
    batch.adam(30, lr=0.05, use_graph=True)
    e1, _, _ = batch.evaluate()
    assert np.all(e1 >= e0 - 1e-4)
    assert np.mean(e1 - e0) > 0.05
    # the graph replays equal eager steps
    batch.set_angles(betas, gammas)
    batch.adam(30, lr=0.05, use_graph=False)
    e2, _, _ = batch.evaluate()
    np.testing.assert_allclose(e2, e1, rtol=1e-5, atol=1e-5)


def test_batch_stop_at_target_skips_finished_instances():
    """optimize(stop_at_target=True) freezes each instance at the step it
    reaches the target and leaves it out of the multi-instance passes: the
    first-hit steps equal those of the unmasked run, the instances that never
    reach the target follow bit-identical trajectories, and the stopped ones
    report a ratio at or above the target."""
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import learned_init as li
    graphs, ps, rng = _mixed_instances(12, 17, nmin=10, nmax=17, pmax=3)
    mc = li.max_cuts(graphs)
    betas = [np.full(p, 0.3) for p in ps]
    gammas = [np.full(p, 0.4) for p in ps]

    def run(target, stop, use_graph=True):
        batch = qf.batched.QAOABatch(graphs, ps, dtype="complex64")
        assert batch.nwave > 0 and batch.nsmall > 0
        batch.set_angles(betas, gammas)
        ratio, first = batch.optimize(0, maxcut=mc, target=target, reset=True, stop_at_target=stop)
        for steps in (1, 2, 4, 5):
            ratio, first = batch.optimize(steps, lr=0.05, reset=False, stop_at_target=stop, use_graph=use_graph)
        return ratio, first

    # a target that splits the batch: the median ratio the unmasked run ends at
    r_free, _ = run(2.0, False)
    target = float(np.median(r_free))
    r0, f0 = run(target, False)
    r1, f1 = run(target, True)
    r2, f2 = run(target, True, use_graph=False)
    assert np.array_equal(f0, f1) and np.array_equal(f1, f2)
    done = f1 >= 0
    assert done.any() and (~done).any()
    assert np.all(r1[done] >= target)
    assert np.array_equal(r0[~done], r1[~done])
    np.testing.assert_allclose(r2, r1, rtol=1e-6, atol=1e-6)


def test_batch_malformed_instance_is_skipped():
    import ctypes
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    g = qf.qaoa.gnp_random_graph(6, 0.5, seed=1)
    batch = qf.batched.QAOABatch([g, g], [2, 2], dtype="complex64")
    raw = batch.d_inst.cpu().numpy().view(np.int32).reshape(-1, 6).copy()
    raw[0, 0] = 40  # n above max_n
    batch.d_inst.copy_(torch.from_numpy(raw.view(np.uint8).reshape(-1)))
    batch.set_angles([np.ones(2)] * 2, [np.ones(2)] * 2)
    es, _, _ = batch.evaluate()
    assert np.isnan(es).sum() == 1
    assert nat.device_error() == 2


def test_autotune_batch(tmp_path, monkeypatch):
    import quantumflow_gb300 as qf
    monkeypatch.setenv("QUANTUMFLOW_GB300_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    graphs, ps, rng = _mixed_instances(32, 7, nmin=8, nmax=14)
    batch = qf.batched.QAOABatch(graphs, ps, dtype="complex64", tile_bits=12, ctas=152)
    best = qf.autotune.tune_batch(batch, ctas_per_sm=(1, 2), reps=1)
    assert best["tile_bits"] >= 8 and best["ctas"] > 0 and len(best["trials"]) >= 2
    again = qf.batched.QAOABatch(graphs, ps, dtype="complex64")
    assert (again.tile_bits, again.ctas) == (best["tile_bits"], best["ctas"])
