"""Parity at the benchmark's configuration: the random-layer circuit family
(a Haar U(2) on every qubit, then CZ on a seeded random perfect matching,
per layer) against the reference's own Circuit.run outputs at N=16 and N=20
(all 100 layers) and N=24 (2 layers), in every complex128 arithmetic and in
complex64; and the benchmarked N=28 x 100-layer circuit itself in the
default (fixed-point) and float-float arithmetic against native FP64.

Tolerances: complex128 1e-12 max amplitude error, complex64 1e-5 (absolute),
as in every parity test of this backend.  The observed errors are printed
(run with -s to see them)."""
import numpy as np
import pytest
import torch

from oracle import qf_oracle as orc

pytestmark = pytest.mark.gpu

ARITH = ["fx", "ff", "fp64"]


def _family_circuit(lf, N):
    import quantumflow_gb300 as qf
    circ = qf.Circuit()
    for m, axes in orc.layer_family_ops(lf[f"lf{N}_u"], lf[f"lf{N}_pairs"]):
        circ += qf.Gate(m, qubits=axes) if len(axes) == 1 else qf.CZ(*axes)
    return circ


@pytest.fixture(scope="module")
def layers():
    from tests.conftest import load_golden
    return load_golden("layers.npz")


@pytest.mark.parametrize("N", [16, 20, 24])
@pytest.mark.parametrize("arith", ARITH + ["c64"])
def test_layer_family_against_reference(layers, N, arith, monkeypatch):
    import quantumflow_gb300 as qf
    dtype = "complex64" if arith == "c64" else "complex128"
    if arith != "c64":
        monkeypatch.setattr(qf.config, "C128_ARITHMETIC", arith)
    tol = 1e-5 if arith == "c64" else 1e-12
    circ = _family_circuit(layers, N)
    ket = circ.run(qf.zero_state(N, dtype=dtype))
    flat = ket.tensor.reshape(-1)
    idx = torch.from_numpy(layers[f"lf{N}_idx"]).to(flat.device)
    got = flat[idx].cpu().numpy().astype(np.complex128)
    err = float(np.max(np.abs(got - layers[f"lf{N}_amps"])))
    probs = (flat.abs() ** 2).to(torch.float64).reshape(256, -1).sum(dim=1).cpu().numpy()
    err_top8 = float(np.max(np.abs(probs - layers[f"lf{N}_top8"])))
    norm = float((flat.abs() ** 2).to(torch.float64).sum().item())
    line = f"N={N} {arith}: max amp err {err:.2e} (4096 sampled), top-8 marginal err {err_top8:.2e}"
    if f"lf{N}_state" in layers:
        full = flat.cpu().numpy().astype(np.complex128)
        ref = layers[f"lf{N}_state"]
        err = max(err, float(np.max(np.abs(full - ref))))
        line += f", full-state max err {float(np.max(np.abs(full - ref))):.2e}, " \
                f"1 - fidelity {1 - orc.fidelity(full, ref):.2e}"
    print(line)
    assert err < tol, line
    assert err_top8 < 10 * tol, line
    assert abs(norm - float(layers[f"lf{N}_norm"])) < 10 * tol


def test_bench_circuit_n28_against_fp64(monkeypatch):
    """The benchmarked circuit (N=28, 100 layers, 4200 gates; bench.py
    c2_circuit_ops seed 2018) in the default fixed-point arithmetic and in
    float-float, against the same circuit in native FP64 (whose kernels the
    reference fixtures pin at smaller N)."""
    import bench
    import quantumflow_gb300 as qf
    ops = bench.c2_circuit_ops(28, 100, 2018)
    circ = bench.build_circuit(ops)
    monkeypatch.setattr(qf.config, "C128_ARITHMETIC", "fp64")
    ref = circ.run(qf.zero_state(28)).tensor.reshape(-1)
    report = []
    for arith in ("fx", "ff"):
        monkeypatch.setattr(qf.config, "C128_ARITHMETIC", arith)
        got = circ.run(qf.zero_state(28)).tensor.reshape(-1)
        err = float((got - ref).abs().max().item())
        ov = torch.vdot(ref, got)
        fid = float((ov.abs() ** 2).item())
        report.append(f"{arith}: max |amp - fp64| {err:.2e}, 1 - fidelity {1 - fid:.2e}")
        assert err < 1e-12, report[-1]
        assert 1 - fid < 1e-11, report[-1]
        del got
        torch.cuda.empty_cache()
    print("N=28, 100 layers: " + "; ".join(report))
