"""Benchmark: random-layer state-vector sweep at N=28 (complex128) on GB300.

Workload (one step): a seeded random circuit on N qubits, L layers, each
layer = a Haar-random U(2) on every qubit then CZ on a random perfect
matching (N=28, L=100: 4200 gates), run by ``Circuit.run`` from |0...0>.
The state (16 * 2^28 B = 4 GiB) is far larger than L2, so every pass streams
from HBM; no flush is needed between steps.  complex128 gates compute in
the library's default arithmetic: FP64 storage with 64-bit integer
fixed-point products (at least as accurate as FP64 arithmetic per pass);
``--arith ff`` / ``fp64`` select float-float or native FP64.

Reported (one JSON line on rank 0):
  value      effective gate GB/s = gates x (2 * 16 * 2^N bytes) / step time,
             i.e. the HBM bandwidth an unfused simulator would need to match
             this speed (fusion can lift it above the HBM peak);
  roofline   the kernel class with the most time (on this workload the
             merged dense 4x4 sweep): bytes moved per launch (2 * 16 * 2^N)
             / its mean CUDA-event duration, against the measured HBM copy
             bandwidth;
  e2e        the same metric through the public API with the initial state
             uploaded from pinned host memory and the final state read back
             every step, on the library's copy streams;
  qaoa       QAOA MAXCUT time to ratio 0.90 (learned start + batched adjoint
             against plain start + per-graph adjoint), the batched evaluation
             times and the single-instance adjoint gradient rate;
  cpu_baseline  the faster of two CPU oracle ports on a bounded sample of the
             same circuit at N=28 (a walk over its first layer, one gate per
             step, the reference arm's rule): the reference numpy backend's
             einsum (one thread) and its torch backend's permute + matmul
             (all threads); the other is reported under "other".

``--impl reference`` times the CPU oracle port alone on this workload.
With ``torchrun --nproc-per-node N`` each rank runs an independent replica.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "gate GB/s vs HBM peak at N=28; QAOA time-to-0.9-ratio, learned vs plain init"


def c2_circuit_ops(N, layers, seed):
    """(kind, qubits, matrix) list: Haar U(2) on every qubit then CZ on a
    seeded random perfect matching, per layer."""
    import scipy.stats
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(layers):
        for q in range(N):
            ops.append((1, (q,), scipy.stats.unitary_group.rvs(2, random_state=rng)))
        perm = rng.permutation(N)
        for a in range(0, N - 1, 2):
            ops.append((2, (int(perm[a]), int(perm[a + 1])), None))
    return ops


def build_circuit(ops):
    import quantumflow_gb300 as qf
    circ = qf.Circuit()
    for kind, qs, u in ops:
        circ += qf.Gate(u, qubits=qs) if kind == 1 else qf.CZ(*qs)
    return circ


# DRAM bytes (read, write) per launch measured by ncu on the random-layer
# workload at N=24 complex128 (profiles/); the write shortfall is dirty L2
# lines still resident when the kernel ends.  Scaled by the state size.
KERNEL_TRAFFIC_N24 = {
    "dense2": (268.485120e6, 206.819072e6),
    "warp_tile": (268.507904e6, 207.091712e6),
    "shape": (268.482560e6, 206.890240e6),
    # fixed-point straight-line pass k_fxshape<4, 132, 110> (mean of 3 launches)
    "fx_shape": (268.601941e6, 208.636416e6),
    # tensor-core complex128 pass k_txpipe (one launch, --set full)
    "fx_tensor": (268.577024e6, 212.714240e6),
    "fx_group": (268.538240e6, 209.662080e6),
}


def kernel_traffic(kind, N, S):
    """ncu-measured DRAM bytes per launch of `kind`, scaled to N qubits."""
    if S != 16 or kind not in KERNEL_TRAFFIC_N24:
        return None
    rd, wr = KERNEL_TRAFFIC_N24[kind]
    return (rd + wr) * 2 ** (N - 24)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"qf_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def walk_sample(layer, step, per_step):
    """Gates [per_step*step, per_step*(step+1)) of one layer of the circuit,
    modulo its length: successive steps walk every qubit's U(2) and every CZ
    of the layer, so a timed sample covers all axes (cheap low axes and
    costly high ones alike) in the proportions of the workload."""
    return [layer[(per_step * step + i) % len(layer)] for i in range(per_step)]


def cpu_sample_rates(N, seed, first_step, steps, per_step):
    """The reference's two CPU paths as oracle ports on the same bounded
    sample of the random-layer circuit at N qubits: its numpy backend's
    tensormul (np.einsum, one thread; numpybk.py:159-214) and its torch
    backend's permute + four-matmul tensormul (torch's intra-op threads, all
    host cores; torchbk.py:243-261).  Step s applies walk_sample(layer 0, s,
    per_step); steps first_step .. first_step+steps-1 are timed.  Returns one
    record per port, the faster first."""
    import torch
    from oracle import qf_oracle as orc
    layer = c2_circuit_ops(N, 1, seed)
    cz = orc.CZ()
    gate_bytes = 2 * 16 * 2 ** N
    recs = []
    for name, mul, st, cores in (
            ("numpy-backend einsum port", orc.tensormul, orc.zero_state(N), 1),
            ("torch-backend permute+matmul port (planar float64)", orc.tensormul_planar,
             orc.planar(orc.zero_state(N)), torch.get_num_threads())):
        t = 0.0
        for s in range(first_step, first_step + steps):
            sample = walk_sample(layer, s, per_step)
            t0 = time.perf_counter()
            for kind, qs, u in sample:
                st = mul(u if kind == 1 else cz, st, list(qs))
            t += time.perf_counter() - t0
        del st
        recs.append({"value": steps * per_step * gate_bytes / t / 1e9, "unit": "GB/s", "cores": cores,
                     "kind": "port", "ms_per_step": t / steps * 1e3,
                     "sample": f"{name}, N={N} complex128, steps {first_step}..{first_step + steps - 1} of a "
                               f"walk over layer 0 of the random-layer circuit ({per_step} gates per step: "
                               f"gates [{per_step}s, {per_step}s+{per_step}) mod {len(layer)}), "
                               f"{t:.1f} s, {cores} thread(s)"})
    recs.sort(key=lambda r: -r["value"])
    return recs


def qaoa_time_to_ratio(args):
    """Second half of the metric: QAOA MAXCUT, n=20, p=6, on seeded random
    3-regular graphs, wall time until every graph has <C>/max C >= 0.90:
    plain linear-ramp start with per-graph adjoint gradients, against the
    learned start (network inference included) with batched adjoint
    gradients.  Adam, lr 0.05, complex64."""
    import torch
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import learned_init as li
    if not os.path.exists(li.WEIGHTS):
        return {"unavailable": "angle network weights missing"}
    net = qf.gnn.AngleGNN.load(li.WEIGHTS)
    rng = np.random.default_rng(20)
    graphs = [qf.qaoa.random_regular_graph(3, 20, seed=int(rng.integers(1 << 30))) for _ in range(args.qaoa_graphs)]
    li.time_to_ratio(net, graphs[:2], p=6, target=0.9, max_steps=20)  # warm-up (kernel attributes, caches)
    torch.cuda.synchronize()
    res = li.time_to_ratio(net, graphs, p=6, target=0.9, max_steps=400)
    mc = li.max_cuts(graphs)
    b, g = qf.qaoa.linear_ramp_angles(6)
    betas, gammas = qf.gnn.predict_angles(net, graphs)
    init_plain = float(np.mean([qf.QAOAMaxCut(gr, 6, dtype="complex64").expectation(b, g) / m
                                for gr, m in zip(graphs, mc)]))
    init_learned = float(np.mean([qf.QAOAMaxCut(gr, 6, dtype="complex64").expectation(bb, gg) / m
                                  for gr, m, bb, gg in zip(graphs, mc, betas, gammas)]))
    plain_s = res["plain_single"]["seconds"]
    learned_s = res["learned_batched"]["seconds"]
    # adjoint gradient throughput, random 3-regular n=24, p=8, complex128
    g24 = qf.qaoa.random_regular_graph(3, 24, seed=24)
    prob24 = qf.QAOAMaxCut(g24, 8)
    b24, g24a = rng.uniform(0, np.pi, 8), rng.uniform(0, np.pi, 8)
    prob24.expectation_and_grad(b24, g24a)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        prob24.expectation_and_grad(b24, g24a)
    grad_rate = reps / (time.perf_counter() - t0)
    # the same gradient in native FP64 arithmetic (the QAOA kernels compute
    # complex128 in float-float unless native FP64 is configured)
    old_arith = qf.config.C128_ARITHMETIC
    qf.config.C128_ARITHMETIC = "fp64"
    try:
        prob64 = qf.QAOAMaxCut(g24, 8)
        prob64.expectation_and_grad(b24, g24a)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            prob64.expectation_and_grad(b24, g24a)
        grad_rate_fp64 = reps / (time.perf_counter() - t0)
        del prob64
    finally:
        qf.config.C128_ARITHMETIC = old_arith
    # batched evaluation of 4096 uneven instances (n 10..20, p 1..6; half
    # G(n, 0.5), half random 3-regular where n is even): <C> and adjoint
    # gradient of every instance per evaluation
    c4 = {}
    rng4 = np.random.default_rng(4096)
    g4, p4 = [], []
    for i in range(4096):
        n = int(rng4.integers(10, 21))
        if i % 2 and n % 2 == 0:
            g4.append(qf.qaoa.random_regular_graph(3, n, seed=int(rng4.integers(1 << 30))))
        else:
            g4.append(qf.qaoa.gnp_random_graph(n, 0.5, seed=int(rng4.integers(1 << 30))))
        p4.append(int(rng4.integers(1, 7)))
    b4 = [rng4.uniform(0, np.pi, p) for p in p4]
    gm4 = [rng4.uniform(0, np.pi, p) for p in p4]
    for dt in ("complex64", "complex128"):
        batch = qf.batched.QAOABatch(g4, p4, dtype=dt)
        batch.set_angles(b4, gm4)
        batch.launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            batch.launch()
        e1.record()
        torch.cuda.synchronize()
        c4[dt] = e0.elapsed_time(e1) / 3
        del batch
        torch.cuda.empty_cache()
    return {"workload": f"{len(graphs)} random 3-regular graphs, n=20, p=6, target ratio 0.90, complex64",
            "batched_4096_uneven_eval_ms": c4,
            "plain_init_single_s": plain_s, "plain_init_batched_s": res["plain_batched"]["seconds"],
            "learned_init_batched_s": learned_s, "speedup_learned_batched_vs_plain_single": plain_s / learned_s,
            "initial_ratio_plain": init_plain, "initial_ratio_learned": init_learned,
            "mean_steps_plain": res["plain_single"]["mean_steps"],
            "mean_steps_learned": res["learned_batched"]["mean_steps"],
            "reached": {k: res[k]["reached"] for k in ("plain_single", "plain_batched", "learned_batched")},
            "adjoint_grad_evals_per_s_n24_p8_c128": grad_rate,
            "adjoint_grad_arith": "float-float (48-bit)",
            "adjoint_grad_evals_per_s_n24_p8_c128_fp64": grad_rate_fp64}


def dense_gate_c64(N=26, K=6, reps=5, seed=6):
    """A dense K-qubit gate (random unitary, scattered axes) on an N-qubit
    complex64 state through qf_apply_dense_gate: the tcgen05 tensor-core
    kernel against the CUDA-core kernel, CUDA-event timed on the launch
    stream (state 8 * 2^N bytes > L2)."""
    import torch
    from quantumflow_gb300 import _native as nat
    rng = np.random.default_rng(seed)
    u = np.linalg.qr(rng.normal(size=(2 ** K, 2 ** K)) + 1j * rng.normal(size=(2 ** K, 2 ** K)))[0]
    axes = [int(a) for a in rng.choice(N, size=K, replace=False)]
    dmat = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    psi = torch.zeros(2 ** N, dtype=torch.complex64, device="cuda")
    psi[0] = 1
    out = torch.empty_like(psi)
    stream = torch.cuda.current_stream()
    res = {}
    for name, tc in (("tensor_cores", 1), ("cuda_cores", 0)):
        nat.call("qf_set_dense_tensor_cores", tc)
        try:
            def run():
                nat.call("qf_apply_dense_gate", nat.ptr(psi), nat.ptr(out), N, nat.LAYOUT_C64, K,
                         nat.int_array(axes), nat.ptr(dmat), nat.stream_handle())
            run()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                run()
            e1.record(stream)
            torch.cuda.synchronize()
        finally:
            nat.call("qf_set_dense_tensor_cores", 1)
        ms = e0.elapsed_time(e1) / reps
        res[name] = {"ms": ms, "gbs": 2 * 8 * 2 ** N / (ms * 1e-3) / 1e9,
                     "useful_tflops": 8 * 2 ** K * 2 ** N / (ms * 1e-3) / 1e12}
    res["tensor_flops_per_useful"] = 3  # hi.hi + hi.lo + lo.hi
    res["workload"] = f"dense {K}-qubit unitary on a {N}-qubit complex64 state, axes {axes}"
    return res


def max_over_ranks(ms, dist, device):
    """The slowest rank's step time, on every rank (replicas: the whole job
    is done when the last replica is)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    """Reference arm: the reference's two CPU paths as oracle ports (the
    reference is pure Python): its numpy backend's tensormul (np.einsum, one
    thread) and its torch backend's permute + matmul tensormul (torch's
    intra-op threads), each on the same bounded sample (cpu_sample_rates:
    W untimed steps of the walk over the first layer, then K timed ones);
    the faster is reported, the other under "other"."""
    if rank != 0:
        return
    N = args.ref_n
    per_step = args.ref_gates
    from oracle import qf_oracle as orc  # noqa: F401  (the ports live there)
    # warm-up: the first W steps of the walk, untimed; then K timed steps
    cpu_sample_rates(N, args.seed, 0, args.warmup, per_step)
    best, other = cpu_sample_rates(N, args.seed, args.warmup, args.steps, per_step)
    value, dt, sample = best["value"], best["ms_per_step"] * 1e-3, best["sample"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64)", "data": "synthetic",
        "config": {"workload": f"random-layer circuit N={N} (Haar U(2) per qubit + CZ matching), "
                               f"bounded sample of {per_step} gates per step walking layer 0"},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": best["cores"], "kind": "port", "sample": sample,
                         "other": other},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=28)
    ap.add_argument("--layers", type=int, default=100)
    ap.add_argument("--dtype", default="complex128", choices=["complex128", "complex64"])
    ap.add_argument("--arith", default=None, choices=["fx", "ff", "fp64"],
                    help="complex128 arithmetic (default: the library's, fixed point)")
    ap.add_argument("--fusion", type=int, default=0, help="0 = library default per element type")
    ap.add_argument("--seed", type=int, default=2018)
    ap.add_argument("--tile-mode", type=int, default=0, help="qf_set_tile_kernel mode (0 = default)")
    ap.add_argument("--shape-bits", type=int, default=None, help="qf_set_shape_bits (default: library)")
    ap.add_argument("--fx-occupancy", type=int, default=None, help="qf_set_fx_occupancy (default: library)")
    ap.add_argument("--merge", type=int, default=1, choices=[0, 1, 2],
                    help="qf_set_gate_merging: 1 merge (default), 2 merge + pass packing, 0 off")
    ap.add_argument("--no-qaoa", action="store_true", help="skip the QAOA time-to-ratio measurement")
    ap.add_argument("--qaoa-graphs", type=int, default=32)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-dense", action="store_true", help="skip the wide dense-gate comparison")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ref-n", type=int, default=28)
    ap.add_argument("--ref-gates", type=int, default=1, help="gates per reference-arm step (CPU sample)")
    ap.add_argument("--cpu-steps", type=int, default=2, help="timed steps of the cpu_baseline sample")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    if args.arith:
        os.environ["QUANTUMFLOW_GB300_C128"] = args.arith
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    if args.arith:
        qf.config.C128_ARITHMETIC = args.arith
    nat.call("qf_set_tile_kernel", args.tile_mode)
    if args.shape_bits is not None:
        nat.call("qf_set_shape_bits", args.shape_bits)
    nat.call("qf_set_gate_merging", args.merge)
    if args.fx_occupancy is not None:
        nat.call("qf_set_fx_occupancy", args.fx_occupancy)

    N, S = args.n, (16 if args.dtype == "complex128" else 8)
    sweep_bytes = 2 * S * 2 ** N
    ops = c2_circuit_ops(N, args.layers, args.seed)
    circ = build_circuit(ops)
    ngates = len(ops)

    def step():
        return circ.run(qf.zero_state(N, dtype=args.dtype), fusion_k=args.fusion)

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        ket = step()
        del ket
    torch.cuda.synchronize()
    passes = circ.last_passes

    # ---- timed region (device events on the launch stream) ------------
    clocks = ClockSampler(local)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nat.timing_collect()
    nat.timing_enable(True)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        ket = step()
        del ket
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clock_info = clocks.stop()
    nat.timing_enable(False)
    kt = nat.timing_collect()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, dist, "cuda")
    value = world * ngates * sweep_bytes / (ms * 1e-3) / 1e9
    launches = sum(c for _, c in kt.values()) + args.steps  # + one |0> fill per step

    # unfused 2x2 sweeps on every qubit (the plain gate-sweep kernel) under
    # the same per-launch CUDA-event timing
    sweep = None
    if rank == 0:
        sweep_circ = build_circuit([op for op in ops[:N] if op[0] == 1])
        ket = sweep_circ.run(qf.zero_state(N, dtype=args.dtype), fusion_k=1)
        del ket
        torch.cuda.synchronize()
        nat.timing_collect()
        nat.timing_enable(True)
        for _ in range(2):
            ket = sweep_circ.run(qf.zero_state(N, dtype=args.dtype), fusion_k=1)
            del ket
        torch.cuda.synchronize()
        nat.timing_enable(False)
        sk = nat.timing_collect()
        kind = next((k for k in ("fx_dense1", "fx_tensor", "dense1") if sk[k][1]), "dense1")
        sms, scount = sk[kind]
        if scount:
            sweep_ach = sweep_bytes / (sms / scount * 1e-3) / 1e9
            kname = {"fx_dense1": "k_fxdense1", "fx_tensor": "k_txpipe", "dense1": "k_dense1"}[kind]
            sweep = {"kernel": f"{kname} (one 2x2 gate per pass, all {N} qubits)", "achieved": sweep_ach,
                     "peak": None, "unit": "GB/s", "frac": None, "launches_timed": scount}

    peak, peak_kind = measured_peaks()
    if sweep is not None:
        sweep["peak"], sweep["frac"] = peak, sweep["achieved"] / peak
    dom = max(kt, key=lambda k: kt[k][0])
    dom_ms, dom_n = kt[dom]
    achieved = sweep_bytes / (dom_ms / dom_n * 1e-3) / 1e9 if dom_n else None
    total_kernel_ms = sum(m for m, _ in kt.values())
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
        "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
        "traffic": kernel_traffic(dom, N, S), "launches_timed": dom_n,
        "share_of_kernel_time": dom_ms / total_kernel_ms if total_kernel_ms else None,
        "bytes_per_launch": sweep_bytes,
    }

    # ---- end to end: host state in, host state out ----------------------
    e2e = None
    if not args.no_e2e and rank == 0:
        cdt = torch.complex128 if args.dtype == "complex128" else torch.complex64
        host_in = torch.zeros(2 ** N, dtype=cdt).pin_memory()
        host_in[0] = 1
        host_out = torch.empty(2 ** N, dtype=cdt).pin_memory()

        def e2e_step():
            # upload and download run on the library's copy streams, so one
            # step's copies overlap the neighbouring steps' circuits
            ket = qf.upload_state(host_in, dtype=args.dtype)
            ket = circ.run(ket, fusion_k=args.fusion)
            return ket.to_host(host_out)

        e2e_step().result()
        torch.cuda.synchronize()
        # at least 6 steps: only the first upload and the last download are
        # exposed, and they are spread over the steps timed
        e2e_steps = max(6, args.steps)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(e2e_steps):
            copy = e2e_step()
        copy.wait(stream)
        f1.record(stream)
        torch.cuda.synchronize()
        ems = f0.elapsed_time(f1) / e2e_steps
        nbytes = host_in.numel() * host_in.element_size()
        e2e = {"value": ngates * sweep_bytes / (ems * 1e-3) / 1e9, "unit": "GB/s",
               "ms_per_step": ems, "steps": e2e_steps, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}
        del host_in, host_out

    qaoa = None
    if not args.no_qaoa and rank == 0:
        qaoa = qaoa_time_to_ratio(args)
    dense = dense_gate_c64() if rank == 0 and not args.no_dense else None

    cpu = None
    if not args.no_cpu and rank == 0:
        # both of the reference's CPU paths, as oracle ports, on the sample
        # rule of the reference arm (a walk over the first layer at the
        # workload's N); the faster is the baseline
        best, other = cpu_sample_rates(N, args.seed, 0, args.cpu_steps, args.ref_gates)
        cpu = dict(best, other=other)

    if rank == 0:
        arith = qf.config.C128_ARITHMETIC if args.dtype == "complex128" else "fp32"
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fx": "c128 (FP64 storage; fused passes as 61-bit fixed-point integer digits on fp16 "
                            "tensor-core MMAs with exact FP32 accumulation, one FP64 rounding per pass)",
                      "ff": "c128 (float-float arithmetic)", "fp64": "c128 (FP64)",
                      "fp32": "c64 (FP32)"}[arith],
            "data": "synthetic",
            "config": {"workload": f"random-layer circuit N={N}, {args.layers} layers x (Haar U(2) on "
                                   f"every qubit + CZ on a seeded perfect matching), {ngates} gates, "
                                   f"fusion k={args.fusion}, gate merging {['off', 'on', 'on, passes packed'][args.merge]}",
                       "state_bytes": S * 2 ** N, "l2": "state larger than L2 (no flush needed)",
                       "parallelism": f"replicas x{world}"},
            "gate_apps_per_s": world * ngates / (ms * 1e-3),
            "passes_per_step": passes,
            "pass_gbs": world * passes * sweep_bytes / (ms * 1e-3) / 1e9,
            "roofline": roofline,
            "sweep_roofline": sweep,
            "kernel_ms_per_step": {k: m / args.steps for k, (m, c) in kt.items() if c},
            "qaoa": qaoa,
            "dense_gate_c64": dense,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clock_info,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
