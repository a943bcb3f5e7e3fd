"""A QuantumFlow tensor-library backend that runs on the GB300 kernels.

The reference selects one backend module at import time
(quantumflow/backend/__init__.py:14-23) and reaches it through the names in
its ``__all__`` (:25-35) with numpy semantics.  This module provides those
names over torch CUDA tensors (complex128, like the reference's numpy
backend, quantumflow/backend/numpybk.py:40); ``tensormul`` -- the
"critical computational core" (numpybk.py:186) -- and ``inner`` on state
vectors run the C-ABI kernels (``qf_apply_gate``, ``qf_inner``).  Everything
else is element-wise plumbing on the device.  Plain Python numbers and numpy
arrays (gate parameters) stay on the host, as with the numpy backend.

Install it into an unmodified reference with :func:`quantumflow_gb300.shim.install`.
"""
import math
import string
import typing

import numpy as np
import torch

from . import _native as nat
from . import config as _config
from .config import version as _version

BACKEND = "gb300"
TL = torch
name = "quantumflow_gb300"
version = _version
DEVICE = "gpu"
CTYPE = torch.complex128
FTYPE = torch.float64
TENSOR = torch.Tensor
BKTensor = typing.Any
TensorLike = typing.Any
MAX_QUBITS = 34
EINSUM_SUBSCRIPTS = string.ascii_lowercase + string.ascii_uppercase

__all__ = ["BKTensor", "CTYPE", "DEVICE", "FTYPE", "MAX_QUBITS", "TENSOR", "TL", "TensorLike", "absolute",
           "arccos", "astensor", "ccast", "cis", "conj", "cos", "diag", "evaluate", "exp", "fcast",
           "gpu_available", "imag", "inner", "minimum", "outer", "matmul", "rank", "real", "reshape",
           "set_random_seed", "sin", "sqrt", "sum", "tensormul", "trace", "transpose", "getitem",
           "astensorproduct", "productdiag", "EINSUM_SUBSCRIPTS", "einsum", "BACKEND", "name", "version"]


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("the gb300 QuantumFlow backend needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def _is_t(x):
    return isinstance(x, torch.Tensor)


def gpu_available() -> bool:
    return torch.cuda.is_available()


def ccast(value):
    return value


def fcast(value):
    return value


def astensor(array):
    """Complex128 CUDA tensor (numpybk.py:98-102 semantics)."""
    if _is_t(array):
        return array.to(device=_device(), dtype=CTYPE)
    arr = np.asarray(array, dtype=np.complex128)
    return torch.from_numpy(np.ascontiguousarray(arr)).to(_device())


def astensorproduct(array):
    """astensor reshaped to [2]*N (numpybk.py:105-112)."""
    t = astensor(array)
    N = int(math.log2(t.numel()))
    return t.reshape([2] * N)


def evaluate(tensor):
    """Host value of a tensor (numpybk.py:115-117 returns the array itself)."""
    if _is_t(tensor):
        return tensor.detach().cpu().numpy()
    return tensor


def rank(tensor) -> int:
    return len(tensor.shape)


def size(tensor) -> int:
    return int(tensor.numel()) if _is_t(tensor) else int(np.size(tensor))


def _u(tfn, nfn):
    def f(x, *a, **k):
        return tfn(x, *a, **k) if _is_t(x) else nfn(x, *a, **k)
    return f


conj = _u(torch.conj_physical, np.conj)
absolute = _u(torch.abs, np.absolute)
real = _u(torch.real, np.real)
imag = _u(torch.imag, np.imag)
exp = _u(torch.exp, np.exp)
cos = _u(torch.cos, np.cos)
sin = _u(torch.sin, np.sin)
sqrt = _u(torch.sqrt, np.sqrt)
arccos = _u(torch.arccos, np.arccos)


def minimum(a, b):
    if _is_t(a) or _is_t(b):
        a = a if _is_t(a) else torch.as_tensor(a, device=_device())
        b = b if _is_t(b) else torch.as_tensor(b, device=_device())
        return torch.minimum(a, b)
    return np.minimum(a, b)


def sum(tensor, *args, **kwargs):  # noqa: A001  (numpy name)
    return torch.sum(tensor, *args, **kwargs) if _is_t(tensor) else np.sum(tensor, *args, **kwargs)


def cis(theta):
    """exp(i theta) (numpybk.py:131-138)."""
    return torch.exp(1j * theta) if _is_t(theta) else np.exp(theta * 1.0j)


def set_random_seed(seed: int) -> None:
    np.random.seed(seed)
    torch.manual_seed(seed)


def getitem(tensor, key):
    return tensor.__getitem__(key)


def reshape(tensor, shape):
    return tensor.reshape(tuple(shape)) if _is_t(tensor) else np.reshape(tensor, shape)


def transpose(tensor, perm=None):
    if not _is_t(tensor):
        return np.transpose(tensor, perm)
    if perm is None:
        return tensor.permute(*reversed(range(tensor.dim())))
    return tensor.permute(*perm)


def matmul(a, b):
    return torch.matmul(astensor(a), astensor(b))


def diag(tensor):
    return torch.diag(tensor) if _is_t(tensor) else np.diag(tensor)


def trace(tensor):
    return torch.trace(tensor) if _is_t(tensor) else np.trace(tensor)


def outer(a, b):
    """np.outer semantics: flattened inputs, 2-D result."""
    return torch.outer(astensor(a).reshape(-1), astensor(b).reshape(-1))


def einsum(subscripts, *operands):
    return torch.einsum(subscripts, *[astensor(o) for o in operands])


def productdiag(tensor):
    """Diagonal of a product-form operator (numpybk.py:147-154)."""
    N = rank(tensor)
    t = reshape(tensor, [2 ** (N // 2), 2 ** (N // 2)])
    t = diag(t)
    return reshape(t, [2] * (N // 2))


def inner(tensor0, tensor1):
    """Flattened <a|b> (numpybk.py:125-128), reduced on the GPU."""
    a = astensor(tensor0).reshape(-1).contiguous()
    b = astensor(tensor1).reshape(-1).contiguous()
    n = int(math.log2(a.numel())) if a.numel() > 0 else 0
    if a.numel() != b.numel():
        raise ValueError("inner: size mismatch")
    if n < 1 or 2 ** n != a.numel():
        return torch.vdot(a, b)
    out = torch.empty(2, dtype=torch.float64, device=a.device)
    nbytes = nat.lib.qf_reduce_workspace_bytes(n)
    ws = nat.workspace(nbytes, a.device)
    nat.call("qf_inner", nat.ptr(a), nat.ptr(b), n, nat.LAYOUT_C128, nat.ptr(out), nat.ptr(ws), nbytes,
             nat.stream_handle(a.device))
    return torch.complex(out[0], out[1])


def tensormul(tensor0, tensor1, indices):
    """Apply a K-axis-pair gate tensor to the given axes of tensor1
    (numpybk.py:159-214), out of place, with ``qf_apply_gate``."""
    K = rank(tensor0) // 2
    assert K == len(indices)
    state = astensor(tensor1)
    shape = tuple(state.shape)
    N = len(shape)
    state = state.reshape(-1).contiguous()
    out = torch.empty_like(state)
    layout = nat.LAYOUT_FX if _config.C128_ARITHMETIC == "fx" else nat.LAYOUT_C128
    if K > nat.MAX_GATE_QUBITS:
        # wide gates: the matrix stays on (or goes to) the device
        dmat = astensor(tensor0).reshape(-1).contiguous()
        nat.call("qf_apply_dense_gate", nat.ptr(state), nat.ptr(out), N, layout, K, nat.int_array(list(indices)),
                 nat.ptr(dmat), nat.stream_handle(state.device))
        return out.reshape(shape)
    gate = tensor0.detach().to("cpu", torch.complex128) if _is_t(tensor0) else \
        torch.from_numpy(np.asarray(tensor0, dtype=np.complex128))
    mat = np.ascontiguousarray(gate.reshape(2 ** K, 2 ** K).numpy()).view(np.float64).reshape(-1)
    nat.call("qf_apply_gate", nat.ptr(state), nat.ptr(out), N, layout, K,
             nat.int_array(list(indices)), mat.ctypes.data_as(nat._dp), nat.stream_handle(state.device))
    return out.reshape(shape)
