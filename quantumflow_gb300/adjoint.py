"""Adjoint gradients of <H> for general circuits of one-parameter gates.

For a diagonal observable H (a real array over basis states, as the
reference's ``State.expectation`` takes, quantumflow/states.py:131-147) and a
circuit whose gates are ``U_k(theta)``, the state psi = U_m ... U_1 |ket>
is computed once; then with lambda = H psi each gate is undone in reverse on
both vectors, and for a gate with U(theta) = exp(i theta K) U(0)

    d<H>/d theta = 2 Re <lambda| i K U |phi> = -2 Im <lambda| K |psi_after>

is read off before the gate is undone.  Two state vectors (plus one scratch)
are held whatever the circuit depth.  The generator K of every parameter is
found on the host from the gate's own matrices, ``K = -i logm(U(theta+d)
U(theta)^dagger) / d``, and the one-parameter-group property is verified
(U(theta+2d) = exp(2 i d K) U(theta)); parameters without it (e.g. the axis
of RN) are reported as not trainable.

Every amplitude operation runs on the GPU through the C ABI
(``qf_apply_gate``, ``qf_inner``, ``qf_expectation_diag``); the reference
differentiates only through TensorFlow (quantumflow/backend/tensorflowbk.py).
"""
import numpy as np
import scipy.linalg
import torch

from . import _native as nat
from .circuits import Circuit
from .ops import Gate
from .states import Buffer, State, _reduce, zero_state

__all__ = ["generator", "trainable_parameters", "expectation_and_grad", "CircuitExpectation"]

_DELTA = 0.125


def generator(gate: Gate, name: str):
    """Hermitian K with dU/dtheta = i K U for parameter ``name`` of ``gate``,
    or None if the parameter does not generate a one-parameter group."""
    params = dict(gate.params)
    if name not in params:
        raise KeyError(name)
    keys = list(params)

    def rebuild(value):
        p = dict(params)
        p[name] = value
        return type(gate)(*[p[k] for k in keys], *gate.qubits).asoperator()

    try:
        u0 = rebuild(params[name])
        u1 = rebuild(params[name] + _DELTA)
        u2 = rebuild(params[name] + 2 * _DELTA)
    except TypeError:
        return None
    step = u1 @ u0.conj().T
    K = -1j * scipy.linalg.logm(step) / _DELTA
    K = 0.5 * (K + K.conj().T)
    if np.max(np.abs(scipy.linalg.expm(2j * _DELTA * K) @ u0 - u2)) > 1e-9:
        return None
    if np.max(np.abs(step @ u0 - u1)) > 1e-12:
        return None
    return K


def trainable_parameters(circuit: Circuit):
    """[(gate index, parameter name)] of every parameter with a generator."""
    out = []
    for i, g in enumerate(circuit.gates()):
        for name in getattr(g, "params", {}):
            if generator(g, name) is not None:
                out.append((i, name))
    return out


def _apply(buf: Buffer, mat: np.ndarray, axes, out: Buffer = None):
    out = buf if out is None else out
    m = np.ascontiguousarray(np.asarray(mat, dtype=np.complex128)).view(np.float64).reshape(-1)
    nat.call("qf_apply_gate", nat.ptr(buf.data), nat.ptr(out.data), buf.n, buf.layout, len(axes),
             nat.int_array(axes), m.ctypes.data_as(nat._dp), nat.stream_handle(buf.device))
    return out


def expectation_and_grad(circuit: Circuit, diag, ket: State = None, dtype: str = "complex128"):
    """(<H>, {(gate index, parameter name): d<H>/d parameter}).

    ``diag``: real diagonal of H over the circuit's qubits (any array-like of
    2^n values, e.g. ``graph_cuts``).  ``ket``: initial state (default
    |0...0> on the sorted circuit qubits).  complex128 runs in FP64
    arithmetic (layout C128), complex64 in FP32."""
    gates = circuit.gates()
    if ket is None:
        ket = zero_state(circuit.qubits, dtype=dtype)
    qubits = ket.qubits
    layout = nat.LAYOUT_C64 if ket.dtype == "complex64" else nat.LAYOUT_C128
    psi = ket.buffer.to_layout(layout)
    psi = Buffer(psi.data.clone(), psi.n, psi.layout) if psi is ket.buffer else psi
    for g in gates:
        _apply(psi, g.asoperator(), [qubits.index(q) for q in g.qubits])
    h = torch.as_tensor(np.real(np.asarray(diag.cpu() if hasattr(diag, "cpu") else diag)),
                        dtype=torch.float64).reshape(-1).to(psi.device)
    if h.numel() != 2 ** psi.n:
        raise ValueError("Incompatibility between tensor and qubits")
    energy = _reduce("qf_expectation_diag", psi, nout=1, extra=(nat.ptr(h),))[0]
    lam = Buffer(psi.data * h.to(psi.data.dtype), psi.n, psi.layout)
    tmp = psi.empty_like()
    grads = {}
    for i in range(len(gates) - 1, -1, -1):
        g = gates[i]
        axes = [qubits.index(q) for q in g.qubits]
        for name in getattr(g, "params", {}):
            K = generator(g, name)
            if K is None:
                continue
            _apply(psi, K, axes, out=tmp)
            re, im = _reduce("qf_inner", lam, nout=2, other=tmp)
            grads[(i, name)] = -2.0 * im
        ginv = g.asoperator().conj().T
        _apply(psi, ginv, axes)
        _apply(lam, ginv, axes)
    return energy, grads


class CircuitExpectation(torch.autograd.Function):
    """<H>(theta) for a circuit built by ``build(theta)`` from a 1-D float64
    tensor; backward uses :func:`expectation_and_grad`.  ``param_map(circuit)``
    returns, for each entry of theta, a list of ((gate index, parameter
    name), d parameter / d theta) pairs (the chain rule for shared angles)."""

    @staticmethod
    def forward(ctx, theta, build, param_map, diag):
        circ = build(theta.detach().cpu().numpy())
        e, grads = expectation_and_grad(circ, diag)
        g = np.zeros(theta.numel())
        for t, uses in enumerate(param_map(circ)):
            g[t] = sum(grads.get(key, 0.0) * scale for key, scale in uses)
        ctx.save_for_backward(torch.from_numpy(g).to(theta.device))
        return torch.tensor(e, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None, None, None
