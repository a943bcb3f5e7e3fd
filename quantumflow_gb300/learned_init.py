"""Train and evaluate the learned QAOA angle initialiser.

Training set: seeded graphs with n uniform in {8..16}, half G(n, 0.5) and
half random 3-regular (odd n, which has no 3-regular graph, falls back to
G(n, 0.5)); each is labelled with the angles that ``steps`` Adam steps of
batched adjoint gradients (complex64) reach from the linear-ramp start.
Evaluation: unseen graphs with n uniform in {12..22}; every graph is
optimised from the network's angles and from the linear ramp, recording the
initial ratio <C>/max C and the steps and wall time to reach a target ratio.

Usage:  python -m quantumflow_gb300.learned_init [--count 20000] [--out PATH]
        python -m quantumflow_gb300.learned_init --evaluate [--eval-count 1000] [--report PATH]
The default weights live in ``quantumflow_gb300/data/angle_gnn_p6.npz``;
``--evaluate`` evaluates them without training, and the 1,000-graph report
of that run is ``quantumflow_gb300/data/angle_gnn_p6_eval.json``.
"""
import argparse
import json
import os
import time

import numpy as np
import torch

from .gnn import AngleGNN, make_labels, predict_angles
from .qaoa import QAOAMaxCut, gnp_random_graph, linear_ramp_angles, random_regular_graph

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "angle_gnn_p6.npz")


def seeded_graphs(count, nmin, nmax, seed):
    rng = np.random.default_rng(seed)
    graphs = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        s = int(rng.integers(1 << 31))
        if i % 2 == 1 and n % 2 == 0:
            graphs.append(random_regular_graph(3, n, seed=s))
        else:
            graphs.append(gnp_random_graph(n, 0.5, seed=s))
    return graphs


def max_cuts(graphs):
    return np.array([QAOAMaxCut(g, 1, dtype="complex64").maxcut for g in graphs])


def train(p=6, count=20000, nmin=8, nmax=16, label_steps=200, label_lr=0.05, epochs=120, batch_size=512,
          lr=2e-3, seed=2018, out=WEIGHTS, log=print):
    t0 = time.perf_counter()
    graphs = seeded_graphs(count, nmin, nmax, seed)
    labels, es = make_labels(graphs, p, steps=label_steps, lr=label_lr)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    mc = max_cuts(graphs)
    log(f"labels: {count} graphs x {label_steps} Adam steps in {t1 - t0:.1f} s; "
        f"mean labelled ratio {np.mean(es / mc):.4f}")
    net = AngleGNN(p, seed=seed)
    hist = net.fit(graphs, labels, epochs=epochs, batch_size=batch_size, lr=lr, seed=seed)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    log(f"training: {epochs} epochs in {t2 - t1:.1f} s; loss {hist[0]:.4f} -> {hist[-1]:.5f}")
    if out:
        os.makedirs(os.path.dirname(out), exist_ok=True)
        net.save(out)
    return net, {"label_seconds": t1 - t0, "train_seconds": t2 - t1, "loss_first": hist[0],
                 "loss_last": hist[-1], "labelled_ratio": float(np.mean(es / mc))}


def evaluate(net, count=1000, nmin=12, nmax=22, target=0.9, steps=300, lr=0.05, seed=777):
    """Optimise every unseen graph from learned and from plain angles (batched
    adjoint gradients, complex64); returns per-start statistics."""
    from .batched import QAOABatch
    graphs = seeded_graphs(count, nmin, nmax, seed)
    mc = max_cuts(graphs)
    p = net.p
    out = {}
    for name in ("plain", "learned"):
        batch = QAOABatch(graphs, p, dtype="complex64")
        if name == "plain":
            b, g = linear_ramp_angles(p)
            betas, gammas = [b] * count, [g] * count
        else:
            betas, gammas = predict_angles(net, graphs)
        batch.set_angles(betas, gammas)
        e0, _, _ = batch.evaluate()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ratio, first = batch.optimize(steps, lr=lr, maxcut=mc, target=target)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        reached = first >= 0
        out[name] = {"initial_ratio": float(np.mean(e0 / mc)), "final_ratio": float(np.mean(ratio)),
                     "reached_fraction": float(np.mean(reached)),
                     "mean_steps_to_target": float(np.mean(first[reached])) if reached.any() else None,
                     "steps_all_reached": int(first.max()) if reached.all() else None,
                     "seconds": dt, "seconds_per_step": dt / steps}
    return out


def adam_single(prob, beta, gamma, maxcut, target, max_steps, lr=0.05, betas=(0.9, 0.999), eps=1e-8):
    """Plain per-graph optimisation: Adam on the single-instance adjoint
    gradient (one forward + adjoint launch per step); returns the steps to
    reach ``target`` (or None) and the final ratio."""
    m = np.zeros(2 * prob.p)
    v = np.zeros(2 * prob.p)
    x = np.concatenate([beta, gamma]).astype(np.float64)
    b1, b2 = betas
    for t in range(max_steps):
        e, gb, gg = prob.expectation_and_grad(x[:prob.p], x[prob.p:])
        if e / maxcut >= target:
            return t, e / maxcut
        g = np.concatenate([gb, gg])
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        x = x + lr * (m / (1 - b1 ** (t + 1))) / (np.sqrt(v / (1 - b2 ** (t + 1))) + eps)
    e = prob.expectation(x[:prob.p], x[prob.p:])
    return (max_steps if e / maxcut >= target else None), e / maxcut


def time_to_ratio(net, graphs, p=6, target=0.9, max_steps=400, lr=0.05, chunk=10, dtype="complex64"):
    """Wall time for every graph to reach <C>/max C >= target:
    (a) plain linear-ramp start, one graph at a time with the single-instance
        adjoint gradient;
    (b) plain start, all graphs at once with the batched adjoint gradient;
    (c) learned start (network inference included), batched adjoint gradient.
    Max-cut values (the yardstick, not part of any method) are computed
    first."""
    from .batched import QAOABatch
    mc = max_cuts(graphs)
    res = {}
    # (a)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps_a, reached_a = [], 0
    b, g = linear_ramp_angles(p)
    for gr, m in zip(graphs, mc):
        prob = QAOAMaxCut(gr, p, dtype=dtype)
        k, _ = adam_single(prob, b, g, m, target, max_steps, lr)
        if k is not None:
            reached_a += 1
            steps_a.append(k)
    torch.cuda.synchronize()
    res["plain_single"] = {"seconds": time.perf_counter() - t0, "reached": reached_a,
                           "mean_steps": float(np.mean(steps_a)) if steps_a else None}

    def batched(start):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if start == "learned":
            betas, gammas = predict_angles(net, graphs)
        else:
            betas, gammas = [b] * len(graphs), [g] * len(graphs)
        batch = QAOABatch(graphs, p, dtype=dtype)
        batch.set_angles(betas, gammas)
        batch.optimizer_reset(mc, target)
        done = 0
        ratio, first = batch.optimize(0, lr=lr, reset=False, stop_at_target=True)
        step = 1  # chunks of 1, 2, 4, ... up to `chunk` steps: few wasted steps past the target
        while (first < 0).any() and done < max_steps:
            # each instance stops at the target, as the one-at-a-time loop does
            ratio, first = batch.optimize(step, lr=lr, reset=False, stop_at_target=True)
            done += step
            step = min(2 * step, chunk)
        dt = time.perf_counter() - t0
        reached = first >= 0
        return {"seconds": dt, "reached": int(reached.sum()),
                "mean_steps": float(np.mean(first[reached])) if reached.any() else None,
                "launched_steps": done}

    res["plain_batched"] = batched("plain")
    res["learned_batched"] = batched("learned")
    res["graphs"] = len(graphs)
    res["target"] = target
    return res


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--count", type=int, default=20000)
    ap.add_argument("--label-steps", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=120)
    ap.add_argument("--eval-count", type=int, default=1000)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--report", default=None)
    ap.add_argument("--evaluate", action="store_true", help="evaluate the stored weights, no training")
    args = ap.parse_args()
    if args.evaluate:
        net = AngleGNN.load(args.out)
        stats = {"weights": os.path.basename(args.out), "eval_count": args.eval_count, "eval_n": [12, 22],
                 "eval_seed": 777, "target": 0.9, "steps": 300, "lr": 0.05, "dtype": "complex64"}
    else:
        net, stats = train(count=args.count, label_steps=args.label_steps, epochs=args.epochs, out=args.out)
    ev = evaluate(net, count=args.eval_count)
    stats["evaluation"] = ev
    print(json.dumps(stats, indent=1))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(stats, f, indent=1)


if __name__ == "__main__":
    main()
