"""qf_expectation_cuts_noalloc: the expectation entry point that allocates
nothing, for callers that cannot obtain device workspace (a host whose pool
owns all GPU memory, code that must not call cudaMalloc).  Its partial sums
live in a fixed array inside the library; this checks that it returns what
the workspace-taking qf_expectation_cuts returns, on consecutive calls, for
each element layout.  This file sorts last so a run that stops at the first
failure has already run every other test."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _workspace_result(nat, buf, cuts):
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    nbytes = nat.lib.qf_reduce_workspace_bytes(buf.n)
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    nat.call("qf_expectation_cuts", nat.ptr(buf.data), buf.n, buf.layout, nat.ptr(cuts), nat.ptr(out),
             nat.ptr(ws), nbytes, nat.stream_handle())
    return float(out.item())


def _noalloc_result(nat, buf, cuts):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    nat.call("qf_expectation_cuts_noalloc", nat.ptr(buf.data), buf.n, buf.layout, nat.ptr(cuts),
             nat.ptr(out), nat.stream_handle())
    return float(out.item())


@pytest.mark.parametrize("layout", [0, 1, 2, 3])
def test_noalloc_matches_workspace_entry_point(layout):
    import quantumflow_gb300 as qf
    from quantumflow_gb300 import _native as nat
    tol = 1e-5 if layout == 0 else 1e-12  # relative, as in the other parity tests
    rng = np.random.default_rng(11)
    # calls in a row with different sizes: n=24 fills the array up to the
    # block cap of the reduction (8 blocks per SM), the later ones use fewer
    # blocks, so stale partial sums from the earlier calls sit in the
    # shared array
    for n, p in ((24, 1), (18, 2), (12, 3), (12, 3)):
        g = qf.qaoa.random_regular_graph(3, n, seed=n)
        prob = qf.QAOAMaxCut(g, p, dtype="complex64" if layout == 0 else "complex128")
        beta, gamma = rng.uniform(0, np.pi, p), rng.uniform(0, np.pi, p)
        buf = prob.state(beta, gamma).buffer.to_layout(layout)
        want = _workspace_result(nat, buf, prob.cuts16)
        got1 = _noalloc_result(nat, buf, prob.cuts16)
        got2 = _noalloc_result(nat, buf, prob.cuts16)
        assert abs(got1 - want) <= tol * abs(want), (n, got1, want)
        assert got1 == got2
    assert nat.device_error() == 0


def test_noalloc_rejects_bad_arguments():
    from quantumflow_gb300 import _native as nat
    fake = nat._vp(0x10000)
    assert nat.lib.qf_expectation_cuts_noalloc(fake, 40, 1, fake, fake, None) == 5  # too large
    assert nat.lib.qf_expectation_cuts_noalloc(fake, 10, 9, fake, fake, None) == 2  # layout
    assert nat.lib.qf_expectation_cuts_noalloc(None, 10, 1, fake, fake, None) == 1  # null
