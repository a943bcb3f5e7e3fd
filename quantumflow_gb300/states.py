"""Quantum states on the GPU.

Mirrors quantumflow/states.py:29-219 (State, zero_state, w_state, ghz_state,
random_state, join_states, print_state, print_probabilities).  A State owns a
device buffer of 2^N amplitudes; amplitudes are never copied to the host
unless the caller asks for them (``asarray``, ``print_state``).

Element layouts (include/qf_gb300.h): complex64 states use QF_LAYOUT_C64.
complex128 states are held as complex128 (QF_LAYOUT_C128) and their gates
run in 64-bit integer fixed point (the engine's QF_LAYOUT_FX argument, the
default) or native FP64, or they are held as float-float pairs
(QF_LAYOUT_FF), see config.C128_ARITHMETIC.  An FF buffer is converted back
to complex128 only when ``State.tensor`` is read.
"""
import math
from collections import defaultdict
from functools import reduce
from typing import Any, Dict, TextIO, Union

import numpy as np
import torch

from . import _native as nat
from . import config
from .qubits import Qubits, qubits_count_tuple

__all__ = ["State", "zero_state", "w_state", "ghz_state", "random_state", "join_states",
           "print_state", "print_probabilities", "basis_state", "uniform_state",
           "upload_state", "HostCopy"]

_DTYPES = {"complex128": torch.complex128, "complex64": torch.complex64}


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("quantumflow_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def compute_layout(dtype: str) -> int:
    """Element layout of the buffers gates are applied to."""
    if dtype == "complex64":
        return nat.LAYOUT_C64
    return nat.LAYOUT_FF if config.C128_ARITHMETIC == "ff" else nat.LAYOUT_C128


def gate_layout(buf: "Buffer") -> int:
    """The layout argument of the gate-engine calls (qf_apply_gate,
    qf_run_circuit) for ``buf``: complex128 buffers run the fixed-point
    arithmetic (QF_LAYOUT_FX, same bytes) unless native FP64 is configured."""
    if buf.layout == nat.LAYOUT_C128 and config.C128_ARITHMETIC == "fx":
        return nat.LAYOUT_FX
    return buf.layout


class Buffer:
    """2^n amplitudes in one element layout on one device."""

    __slots__ = ("data", "n", "layout", "_complex")

    def __init__(self, data: torch.Tensor, n: int, layout: int):
        self.data = data
        self.n = n
        self.layout = layout
        self._complex = None

    # -- construction ----------------------------------------------------
    @staticmethod
    def empty(n: int, layout: int, device=None) -> "Buffer":
        device = device or _device()
        if layout == nat.LAYOUT_C64:
            data = torch.empty(2 ** n, dtype=torch.complex64, device=device)
        elif layout in (nat.LAYOUT_C128, nat.LAYOUT_FX):
            data = torch.empty(2 ** n, dtype=torch.complex128, device=device)
        elif layout == nat.LAYOUT_FF:
            data = torch.empty((2 ** n, 4), dtype=torch.float32, device=device)
        else:
            raise ValueError(f"unknown layout {layout}")
        return Buffer(data, n, layout)

    @staticmethod
    def from_complex(t: torch.Tensor) -> "Buffer":
        t = t.reshape(-1).contiguous()
        n = int(round(math.log2(t.numel()))) if t.numel() > 0 else 0
        if 2 ** n != t.numel():
            raise ValueError("Incompatibility between tensor and qubits")
        layout = nat.LAYOUT_C64 if t.dtype == torch.complex64 else nat.LAYOUT_C128
        return Buffer(t, n, layout)

    # -- properties ------------------------------------------------------
    @property
    def dtype(self) -> str:
        return "complex64" if self.layout == nat.LAYOUT_C64 else "complex128"

    @property
    def device(self):
        return self.data.device

    def empty_like(self) -> "Buffer":
        return Buffer.empty(self.n, self.layout, self.data.device)

    # -- layout conversion ---------------------------------------------
    def to_layout(self, layout: int) -> "Buffer":
        if layout == self.layout:
            return self
        out = Buffer.empty(self.n, layout, self.data.device)
        nat.call("qf_convert", nat.ptr(self.data), self.layout, nat.ptr(out.data), layout, self.n,
                 nat.stream_handle(self.data.device))
        return out

    def compute(self) -> "Buffer":
        """This buffer in the layout gates are applied in."""
        return self.to_layout(compute_layout(self.dtype))

    def complex(self) -> torch.Tensor:
        """Flat complex tensor (complex128 for FF buffers, converted once)."""
        if self.layout != nat.LAYOUT_FF:
            return self.data
        if self._complex is None:
            self._complex = self.to_layout(nat.LAYOUT_C128).data
        return self._complex


_IO_STREAMS = {}


def _io_streams(device):
    """(upload, download) copy streams of one device, made on first use."""
    index = torch.device(device).index
    if index is None:
        index = torch.cuda.current_device()
    if index not in _IO_STREAMS:
        with torch.cuda.device(index):
            _IO_STREAMS[index] = (torch.cuda.Stream(), torch.cuda.Stream())
    return _IO_STREAMS[index]


class HostCopy:
    """A device-to-host copy in flight (from :meth:`State.to_host`)."""

    __slots__ = ("tensor", "event", "shape")

    def __init__(self, tensor: torch.Tensor, event, shape):
        self.tensor = tensor
        self.event = event
        self.shape = shape

    def done(self) -> bool:
        return self.event.query()

    def wait(self, stream=None) -> None:
        """Order ``stream`` (default: the current stream) after the copy."""
        (stream or torch.cuda.current_stream()).wait_event(self.event)

    def result(self) -> torch.Tensor:
        """Block until the copy has landed; the host amplitudes as [2]*N."""
        self.event.synchronize()
        return self.tensor.reshape(self.shape)


def _as_complex_tensor(tensor, dtype=None) -> torch.Tensor:
    device = _device()
    if isinstance(tensor, torch.Tensor):
        t = tensor
        if dtype is None:
            dtype = "complex64" if t.dtype in (torch.complex64, torch.float32) else "complex128"
        return t.to(device=device, dtype=_DTYPES[dtype])
    arr = np.asarray(tensor)
    if dtype is None:
        dtype = "complex64" if arr.dtype in (np.complex64, np.float32) else "complex128"
    arr = np.ascontiguousarray(arr, dtype=np.complex64 if dtype == "complex64" else np.complex128)
    return torch.from_numpy(arr).to(device)


class State:
    """The quantum state of a collection of qubits (quantumflow/states.py:29-183).

    ``tensor`` may be a torch tensor, numpy array, nested list, or a
    :class:`Buffer`.  ``dtype`` ('complex128' or 'complex64') overrides the
    element type inferred from ``tensor``.
    """

    def __init__(self, tensor: Any, qubits: Qubits = None, memory: Dict = None, *, dtype=None) -> None:
        if isinstance(tensor, Buffer):
            buf = tensor
        else:
            buf = Buffer.from_complex(_as_complex_tensor(tensor, dtype))
        if qubits is None:
            qubits = range(buf.n)
        qubits = tuple(qubits)
        if len(qubits) != buf.n:
            raise ValueError("Incompatibility between tensor and qubits")
        self._buf = buf
        self._qubits = qubits
        self._memory = memory if memory is not None else {}

    # -- reference API ---------------------------------------------------
    @property
    def tensor(self) -> torch.Tensor:
        """Amplitudes as a [2]*N complex CUDA tensor."""
        return self._buf.complex().reshape([2] * self._buf.n)

    @property
    def qubits(self) -> Qubits:
        return self._qubits

    @property
    def qubit_nb(self) -> int:
        return len(self._qubits)

    @property
    def dtype(self) -> str:
        return self._buf.dtype

    @property
    def buffer(self) -> Buffer:
        return self._buf

    @property
    def memory(self) -> dict:
        return defaultdict(int, self._memory)

    @property
    def cbits(self) -> tuple:
        """The classical bit addresses in memory, sorted (quantumflow/states.py:88-92)."""
        return tuple(sorted(addr for addr in self._memory if getattr(addr, "dtype", None) == "BIT"))

    @property
    def cbit_nb(self) -> int:
        """Number of classical bits in memory (quantumflow/states.py:95-97)."""
        return len(self.cbits)

    def update(self, memory: Dict) -> "State":
        mem = self.memory
        mem.update(memory)
        return State(self._buf, self.qubits, mem)

    def asarray(self) -> np.ndarray:
        return self.tensor.detach().cpu().numpy()

    def to_host(self, out: torch.Tensor = None) -> "HostCopy":
        """Copy the amplitudes into host memory on the device's download
        stream, after the work queued so far on the current stream, and
        return at once: the copy overlaps whatever is launched next.  ``out``
        (pinned, same element count and complex dtype as ``tensor``)
        receives them; a pinned buffer is allocated when it is None.  Read
        the result through :meth:`HostCopy.result`."""
        t = self._buf.complex().reshape(-1)
        if out is None:
            out = torch.empty(t.numel(), dtype=t.dtype, pin_memory=True)
        if (out.device.type != "cpu" or out.numel() != t.numel() or out.dtype != t.dtype
                or not out.is_contiguous()):
            raise ValueError("to_host wants a contiguous host tensor with the state's element count and dtype")
        cur = torch.cuda.current_stream(t.device)
        _, down = _io_streams(t.device)
        down.wait_stream(cur)
        with torch.cuda.stream(down):
            out.reshape(-1).copy_(t, non_blocking=True)
            event = torch.cuda.Event()
            event.record(down)
        t.record_stream(down)
        return HostCopy(out, event, [2] * self._buf.n)

    def asdensity(self):
        """|psi><psi| as a Density (quantumflow/states.py:162-165)."""
        from .densities import asdensity
        return asdensity(self)

    def norm(self) -> float:
        """|<psi|psi>| (quantumflow/qubits.py:180-182)."""
        return abs(_reduce("qf_norm2", self._buf, nout=1)[0])

    def relabel(self, qubits: Qubits) -> "State":
        return State(self._buf, qubits, self._memory)

    def permute(self, qubits: Qubits) -> "State":
        """Reorder qubits (quantumflow/states.py:103-106)."""
        qubits = tuple(qubits)
        if qubits == self.qubits:
            return self
        perm = [self.qubits.index(q) for q in qubits]
        t = self.tensor.permute(perm).contiguous()
        return State(Buffer.from_complex(t), qubits, self._memory)

    def normalize(self) -> "State":
        """quantumflow/states.py:108-111."""
        src = self._buf.compute()
        out = src.empty_like()
        out.data.copy_(src.data)
        nat.call("qf_scale", nat.ptr(out.data), out.n, out.layout, 1.0 / math.sqrt(self.norm()),
                 nat.stream_handle(out.device))
        return State(out, self.qubits, self._memory)

    def probabilities(self) -> torch.Tensor:
        """|psi_x|^2 as a [2]*N float64 CUDA tensor (quantumflow/states.py:113-119)."""
        buf = self._buf
        if buf.layout == nat.LAYOUT_C128 and config.C128_ARITHMETIC == "ff":
            buf = buf  # plain complex128 input: read directly
        probs = torch.empty(2 ** buf.n, dtype=torch.float64, device=buf.device)
        nat.call("qf_probabilities", nat.ptr(buf.data), buf.n, buf.layout, nat.ptr(probs),
                 nat.stream_handle(buf.device))
        return probs.reshape([2] * buf.n)

    def sample(self, trials: int, seed: int = None) -> np.ndarray:
        """Multinomial counts over basis states (quantumflow/states.py:121-129)."""
        buf = self._buf
        counts = torch.empty(2 ** buf.n, dtype=torch.int64, device=buf.device)
        nbytes = nat.lib.qf_sample_workspace_bytes(buf.n)
        ws = torch.empty(nbytes, dtype=torch.uint8, device=buf.device)
        nat.call("qf_sample", nat.ptr(buf.data), buf.n, buf.layout, int(trials),
                 _next_seed(seed), nat.ptr(counts), nat.ptr(ws), nbytes,
                 nat.stream_handle(buf.device))
        return counts.cpu().numpy().reshape([2] * buf.n)

    def expectation(self, diag_hermitian: Any, trials: int = None) -> float:
        """sum_x Re(h_x) p_x (quantumflow/states.py:131-147); with ``trials``
        the probabilities are replaced by sampled frequencies."""
        buf = self._buf
        if isinstance(diag_hermitian, torch.Tensor):
            h = diag_hermitian.to(device=buf.device)
            h = h.real if h.is_complex() else h
            h = h.to(torch.float64).reshape(-1).contiguous()
        else:
            h = torch.from_numpy(np.ascontiguousarray(np.real(np.asarray(diag_hermitian)),
                                                      dtype=np.float64).reshape(-1)).to(buf.device)
        if h.numel() != 2 ** buf.n:
            raise ValueError("Incompatibility between tensor and qubits")
        if trials is not None:
            counts = self.sample(trials)
            return float(np.sum(h.cpu().numpy() * counts.reshape(-1)) / trials)
        return _reduce("qf_expectation_diag", buf, nout=1, extra=(nat.ptr(h),))[0]

    def measure(self, seed: int = None) -> np.ndarray:
        """One computational-basis measurement as a bit array
        (quantumflow/states.py:149-160)."""
        counts = self.sample(1, seed).reshape(-1)
        idx = int(np.nonzero(counts)[0][0])
        n = self.qubit_nb
        return np.array([(idx >> (n - 1 - i)) & 1 for i in range(n)])

    def __str__(self) -> str:
        state = self.asarray()
        s = []
        count = 0
        for index, amplitude in np.ndenumerate(state):
            if not np.isclose(amplitude, 0.0):
                ket = "|" + "".join(str(n) for n in index) + ">"
                s.append("({c.real:0.04g}{c.imag:+0.04g}i) {k}".format(c=amplitude, k=ket))
                count += 1
                if count > 64:
                    s.append("...")
                    break
        return " + ".join(s)


_seed_counter = [0]


def _next_seed(seed):
    if seed is not None:
        return int(seed) & 0xFFFFFFFFFFFFFFFF
    base = config.SEED if config.SEED is not None else int(np.random.randint(0, 2 ** 62))
    _seed_counter[0] += 1
    return (base * 1000003 + _seed_counter[0]) & 0xFFFFFFFFFFFFFFFF


def _reduce(fn, buf, nout, extra=(), other=None):
    """Run a workspace reduction and return its result(s) as Python floats."""
    out = torch.empty(2, dtype=torch.float64, device=buf.device)
    nbytes = nat.lib.qf_reduce_workspace_bytes(buf.n)
    ws = nat.workspace(nbytes, buf.device)
    args = [nat.ptr(buf.data)]
    if other is not None:
        args.append(nat.ptr(other.data))
    args += [buf.n, buf.layout, *extra, nat.ptr(out), nat.ptr(ws), nbytes, nat.stream_handle(buf.device)]
    nat.call(fn, *args)
    return out[:nout].tolist()


def inner(a: State, b: State) -> complex:
    """<a|b> for states on the same qubits in the same order."""
    ba, bb = a.buffer, b.buffer
    if ba.n != bb.n:
        raise ValueError("Incompatibly vectors. Qubits and rank must match")
    if ba.layout != bb.layout:
        lay = nat.LAYOUT_C128 if nat.LAYOUT_C64 not in (ba.layout, bb.layout) else nat.LAYOUT_C64
        if lay == nat.LAYOUT_C64 and ba.layout != bb.layout:
            lay = nat.LAYOUT_C128
        ba, bb = ba.to_layout(lay), bb.to_layout(lay)
    re, im = _reduce("qf_inner", ba, nout=2, other=bb)
    return complex(re, im)


# ----------------------------------------------------------- constructors --
def upload_state(host: torch.Tensor, qubits: Qubits = None, memory: Dict = None, *,
                 dtype: str = None) -> State:
    """A State from host amplitudes, copied on the device's upload stream.

    The copy does not wait for work already queued on the current stream,
    so with a pinned ``host`` it overlaps a circuit still running on the
    device; the current stream waits for it before the returned state's
    first use.  ``host`` must stay unchanged until that copy has run."""
    if not isinstance(host, torch.Tensor):
        host = torch.from_numpy(np.ascontiguousarray(np.asarray(host)))
    if host.device.type != "cpu":
        raise ValueError("upload_state takes host amplitudes")
    device = _device()
    up, _ = _io_streams(device)
    cur = torch.cuda.current_stream(device)
    with torch.cuda.stream(up):
        dev = host.reshape(-1).to(device, non_blocking=True)
    cur.wait_stream(up)
    dev.record_stream(cur)
    return State(dev, qubits, memory, dtype=dtype)


def basis_state(qubits: Union[int, Qubits], index: int = 0, dtype: str = "complex128") -> State:
    N, qubits = qubits_count_tuple(qubits)
    if N == 0:  # the empty register: one amplitude, 1 (kept on the host side of the ABI)
        return State(torch.ones(1, dtype=_DTYPES[dtype], device=_device()), qubits)
    buf = Buffer.empty(N, compute_layout(dtype))
    nat.call("qf_fill_basis", nat.ptr(buf.data), N, buf.layout, int(index), nat.stream_handle(buf.device))
    return State(buf, qubits)


def zero_state(qubits: Union[int, Qubits], dtype: str = "complex128") -> State:
    """|0...0> (quantumflow/states.py:186-191)."""
    return basis_state(qubits, 0, dtype)


def uniform_state(qubits: Union[int, Qubits], dtype: str = "complex128") -> State:
    """|+>^N, the output of H on every qubit of |0...0>."""
    N, qubits = qubits_count_tuple(qubits)
    buf = Buffer.empty(N, compute_layout(dtype))
    nat.call("qf_fill_uniform", nat.ptr(buf.data), N, buf.layout, nat.stream_handle(buf.device))
    return State(buf, qubits)


def w_state(qubits: Union[int, Qubits], dtype: str = "complex128") -> State:
    """quantumflow/states.py:194-202."""
    N, qubits = qubits_count_tuple(qubits)
    t = torch.zeros(2 ** N, dtype=_DTYPES[dtype], device=_device())
    for n in range(N):
        t[1 << (N - 1 - n)] = 1 / math.sqrt(N)
    return State(t, qubits)


def ghz_state(qubits: Union[int, Qubits], dtype: str = "complex128") -> State:
    """quantumflow/states.py:205-211."""
    N, qubits = qubits_count_tuple(qubits)
    t = torch.zeros(2 ** N, dtype=_DTYPES[dtype], device=_device())
    t[0] = 1 / math.sqrt(2)
    t[-1] = 1 / math.sqrt(2)
    return State(t, qubits)


def random_state(qubits: Union[int, Qubits], dtype: str = "complex128") -> State:
    """Normalised complex Gaussian state (quantumflow/states.py:214-219)."""
    N, qubits = qubits_count_tuple(qubits)
    ket = np.random.normal(size=([2] * N)) + 1j * np.random.normal(size=([2] * N))
    return State(ket, qubits, dtype=dtype).normalize()


def join_states(*states: State) -> State:
    """Tensor product of states on disjoint qubits (quantumflow/states.py:225-229)."""
    def _join(a, b):
        if not set(a.qubits).isdisjoint(b.qubits):
            raise ValueError("Overlapping qubits")
        t = torch.outer(a.tensor.reshape(-1), b.tensor.reshape(-1)).reshape(-1)
        return State(t, tuple(a.qubits) + tuple(b.qubits))
    return reduce(_join, states)


def print_state(state: State, file: TextIO = None) -> None:
    """quantumflow/states.py:234-239."""
    for index, amplitude in np.ndenumerate(state.asarray()):
        print("".join(str(n) for n in index), ":", amplitude, file=file)


def print_probabilities(state: State, ndigits: int = 4, file: TextIO = None) -> None:
    """quantumflow/states.py:243-261."""
    prob = state.probabilities().cpu().numpy()
    for index, p in np.ndenumerate(prob):
        p = round(float(p), ndigits)
        if p == 0.0:
            continue
        print("".join(str(n) for n in index), ":", p, file=file)
