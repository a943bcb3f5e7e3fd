"""ctypes binding of ``libqfgb300.so`` (the C ABI declared in include/qf_gb300.h).

The library is the only compute path: importing this module raises if the
library is missing or was built for a different ABI, and every wrapper raises
if a call returns a non-zero status.  Device memory and streams come from
PyTorch (``tensor.data_ptr()``, ``torch.cuda.current_stream().cuda_stream``);
nothing here computes on the host.
"""
import ctypes
import os

import torch

LIBPATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libqfgb300.so")

LAYOUT_C64 = 0
LAYOUT_C128 = 1
LAYOUT_FF = 2
LAYOUT_FX = 3  # complex128 bytes (as LAYOUT_C128); gates in 64-bit fixed point
MAX_GATE_QUBITS = 5    # qf_apply_gate / qf_run_circuit (host matrices)
MAX_DENSE_QUBITS = 12  # qf_apply_dense_gate (device matrix)

STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "unknown element layout",
    3: "CUDA runtime error",
    4: "device pointer not 16-byte aligned",
    5: "size above the supported maximum",
    6: "operation not supported",
    7: "a bounded device-side wait gave up",
    8: "workspace missing or too small",
}

ABI_VERSION = 1


class NativeError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, fn, status, cuda_error=0):
        self.fn = fn
        self.status = status
        self.cuda_error = cuda_error
        msg = f"{fn}: {STATUS.get(status, 'unknown status')} (status {status}"
        if status == 3:
            msg += f", cudaError {cuda_error}"
        super().__init__(msg + ")")


_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_u64 = ctypes.c_uint64
_c_dbl = ctypes.c_double
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_sz = ctypes.c_size_t

# name -> (restype, argtypes); mirrors include/qf_gb300.h
SIGNATURES = {
    "qf_abi_version": (_c_int, []),
    "qf_status_string": (ctypes.c_char_p, [_c_int]),
    "qf_last_cuda_error": (_c_int, []),
    "qf_get_device_error": (_c_int, [_ip, _vp]),
    "qf_reduce_workspace_bytes": (_sz, [_c_int]),
    "qf_timing_enable": (_c_int, [_c_int]),
    "qf_set_tile_kernel": (_c_int, [_c_int]),
    "qf_set_shape_bits": (_c_int, [_c_int]),
    "qf_set_gate_merging": (_c_int, [_c_int]),
    "qf_set_dense_tensor_cores": (_c_int, [_c_int]),
    "qf_set_fx_occupancy": (_c_int, [_c_int]),
    "qf_set_fx_tensor_cores": (_c_int, [_c_int]),
    "qf_plan_circuit": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _c_int, _vp, _c_int, _vp]),
    "qf_timing_collect": (_c_int, [_dp, ctypes.POINTER(ctypes.c_int64), _c_int]),
    "qf_sample_workspace_bytes": (_sz, [_c_int]),
    "qf_fill_basis": (_c_int, [_vp, _c_int, _c_int, _c_i64, _vp]),
    "qf_fill_uniform": (_c_int, [_vp, _c_int, _c_int, _vp]),
    "qf_convert": (_c_int, [_vp, _c_int, _vp, _c_int, _c_int, _vp]),
    "qf_scale": (_c_int, [_vp, _c_int, _c_int, _c_dbl, _vp]),
    "qf_apply_gate": (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _ip, _dp, _vp]),
    "qf_apply_dense_gate": (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _ip, _vp, _vp]),
    "qf_run_circuit": (_c_int, [_vp, _vp, _c_int, _c_int, _c_int, _ip, _ip, _dp, _c_int, _ip, _vp]),
    "qf_cut_values": (_c_int, [_vp, _c_int, _c_int, _ip, _vp]),
    "qf_cut_values_weighted": (_c_int, [_vp, _c_int, _c_int, _ip, _dp, _vp]),
    "qf_qaoa_state": (_c_int, [_vp, _c_int, _c_int, _vp, _c_int, _c_int, _dp, _dp, _dp, _c_int, _vp]),
    "qf_expectation_cuts": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp, _sz, _vp]),
    "qf_qaoa_grad_workspace_bytes": (_sz, [_c_int, _c_int, _c_int]),
    "qf_batch_workspace_bytes": (_sz, [_c_int, _c_int, _c_int]),
    "qf_gnn_param_count": (_sz, [_c_int]),
    "qf_gnn_activation_floats": (_sz, [_c_int, _c_int]),
    "qf_gnn_forward": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qf_gnn_backward": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qf_adam_update": (_c_int, [_vp, _vp, _vp, _vp, _c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, _c_int, _vp]),
    "qf_batch_qaoa_grad": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp, _c_int, _c_int, _c_int, _c_int, _vp, _sz,
                                    _vp]),
    "qf_wave_min_qubits": (_c_int, [_c_int]),
    "qf_wave_plan": (_c_int, [_vp, _c_int, _c_int, _vp, _sz, _vp, _vp]),
    "qf_wave_prepare": (_c_int, [_vp, _vp, _vp, _sz, _vp]),
    "qf_wave_qaoa_grad": (_c_int, [_vp, _vp, _sz, _vp, _vp, _vp, _vp]),
    "qf_qaoa_expectation_grad": (_c_int, [_vp, _c_int, _c_int, _vp, _c_int, _c_int, _dp, _dp, _dp, _c_int,
                                          _vp, _vp, _sz, _vp]),
    "qf_expectation_diag": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp, _sz, _vp]),
    "qf_expectation_cuts_noalloc": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _vp]),
    "qf_norm2": (_c_int, [_vp, _c_int, _c_int, _vp, _vp, _sz, _vp]),
    "qf_qubit_probabilities": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _sz, _vp]),
    "qf_inner": (_c_int, [_vp, _vp, _c_int, _c_int, _vp, _vp, _sz, _vp]),
    "qf_probabilities": (_c_int, [_vp, _c_int, _c_int, _vp, _vp]),
    "qf_sample": (_c_int, [_vp, _c_int, _c_int, _c_i64, _c_u64, _vp, _vp, _sz, _vp]),
}


def _load():
    if not os.path.exists(LIBPATH):
        raise ImportError(
            f"{LIBPATH} is missing: build it with `python quantumflow_gb300/build.py` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIBPATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.qf_abi_version() != ABI_VERSION:
        raise ImportError(f"{LIBPATH}: ABI {lib.qf_abi_version()} != {ABI_VERSION}")
    return lib


lib = _load()


def call(name, *args):
    """Call a status-returning entry point; raise NativeError on failure."""
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise NativeError(name, rc, lib.qf_last_cuda_error())
    return rc


def stream_handle(device=None):
    """cudaStream_t of torch's current stream as a ctypes void pointer."""
    return _vp(torch.cuda.current_stream(device).cuda_stream)


def ptr(t):
    return _vp(t.data_ptr())


def int_array(values):
    arr = (ctypes.c_int * max(1, len(values)))(*[int(v) for v in values])
    return arr


def double_array(values):
    arr = (ctypes.c_double * max(1, len(values)))(*[float(v) for v in values])
    return arr


def device_error(stream=None):
    """Read and clear the device error word (raises if it was set)."""
    flags = ctypes.c_int(0)
    call("qf_get_device_error", ctypes.byref(flags), stream or stream_handle())
    return flags.value


KERNEL_CLASSES = ("fused_tile", "dense1", "dense2", "permutation", "elementwise", "warp_tile", "group", "shape",
                  "fx_dense1", "fx_dense2", "fx_group", "fx_elementwise", "fx_shape", "fx_tensor")


def timing_enable(on=True):
    call("qf_timing_enable", 1 if on else 0)


def timing_collect():
    """{kernel class: (milliseconds, launches)} since the previous collect."""
    n = len(KERNEL_CLASSES)
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_int64 * n)()
    call("qf_timing_collect", ms, cnt, n)
    return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}


# ------------------------------------------------------------ workspaces ----
_workspaces = {}


def workspace(nbytes, device):
    """A cached device workspace of at least ``nbytes`` (uint8 tensor)."""
    key = (device.index if device.index is not None else torch.cuda.current_device())
    buf = _workspaces.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _workspaces[key] = buf
    return buf
