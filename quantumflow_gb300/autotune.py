"""Autotuner for kernel shapes, with a JSON cache.

Candidates are timed on the caller's actual workload with CUDA events and
the fastest is stored under a key of (GPU name, workload signature) in
``~/.cache/quantumflow_gb300/autotune.json`` (override the path with
``QUANTUMFLOW_GB300_AUTOTUNE_CACHE``).  Lookups never tune implicitly:
``batch_config`` / ``fusion_config`` return cached values or ``{}`` (library
defaults); ``tune_batch`` / ``tune_fusion`` measure and store;
``use_fusion_config`` applies a fusion result.
"""
import hashlib
import json
import os
import threading

import numpy as np
import torch

_LOCK = threading.Lock()


def cache_path():
    return os.environ.get("QUANTUMFLOW_GB300_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "quantumflow_gb300", "autotune.json"))


def _load():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, value):
    with _LOCK:
        data = _load()
        data[key] = value
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _gpu():
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _batch_key(batch):
    sig = hashlib.sha1(np.stack([batch.ns, batch.ps, batch.nedges]).tobytes()).hexdigest()[:12]
    return f"{_gpu()}|batch|{batch.dtype}|{batch.count}|{batch.max_n}|{sig}"


def batch_config(batch):
    return _load().get(_batch_key(batch), {})


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def tune_batch(batch, tile_bits=None, ctas_per_sm=(1, 2, 3), reps=3):
    """Time (tile_bits, CTAs per SM) candidates for ``batch`` and keep the
    fastest; returns {"tile_bits", "ctas", "ms", "trials"}."""
    ts_max = 12 if batch.dtype == "complex64" else 11
    lo = max(8, (batch.max_n + 1) // 2)
    tile_bits = tile_bits or [t for t in range(lo, ts_max + 1)]
    sms = torch.cuda.get_device_properties(batch.device).multi_processor_count
    trials = []
    best = None
    for tb in tile_bits:
        for k in ctas_per_sm:
            batch.tile_bits, batch.ctas = tb, k * sms
            batch._alloc_workspace()
            try:
                ms = _time(batch.launch, reps)
            except RuntimeError:
                continue
            trials.append({"tile_bits": tb, "ctas": k * sms, "ms": ms})
            if best is None or ms < best["ms"]:
                best = dict(trials[-1])
    if best is None:
        raise RuntimeError("no batch configuration could run")
    batch.tile_bits, batch.ctas = best["tile_bits"], best["ctas"]
    batch._alloc_workspace()
    best["trials"] = trials
    _store(_batch_key(batch), best)
    return best


def _fusion_key(dtype, n):
    from . import config
    return f"{_gpu()}|fusion|{dtype}|{config.C128_ARITHMETIC}|{n}"


def fusion_config(dtype, n):
    return _load().get(_fusion_key(dtype, n), {})


DEFAULT_SHAPE_BITS = 3  # the library's qf_set_shape_bits default


def tune_fusion(circuit, n, dtype="complex128", candidates=(1, 2, 3, 4, 5, 6), modes=(0, 1), reps=2,
                shape_bits=None):
    """Time Circuit.run over fusion widths, fused-kernel modes
    (qf_set_tile_kernel) and, for float-float complex128 states, shape
    widths (qf_set_shape_bits; default candidates 2, 3, 4) on ``circuit``;
    stores and returns the fastest {"fusion_k", "mode", "shape_bits", "ms",
    "trials"}.  The process-wide settings are restored afterwards; apply a
    result with ``use_fusion_config``."""
    from . import _native as nat
    from . import config
    from .states import zero_state
    ff = dtype == "complex128" and config.C128_ARITHMETIC == "ff"
    if shape_bits is None:
        shape_bits = (2, 3, 4) if ff else (DEFAULT_SHAPE_BITS,)
    trials = []
    best = None
    try:
        for mode in modes:
            nat.call("qf_set_tile_kernel", mode)
            for bits in shape_bits:
                nat.call("qf_set_shape_bits", bits)
                for k in candidates:
                    ms = _time(lambda: circuit.run(zero_state(n, dtype=dtype), fusion_k=k), reps)
                    trials.append({"fusion_k": k, "mode": mode, "shape_bits": bits, "ms": ms})
                    if best is None or ms < best["ms"]:
                        best = dict(trials[-1])
    finally:
        nat.call("qf_set_tile_kernel", 0)
        nat.call("qf_set_shape_bits", DEFAULT_SHAPE_BITS)
    best["trials"] = trials
    _store(_fusion_key(dtype, n), best)
    return best


def use_fusion_config(cfg):
    """Apply a ``tune_fusion`` / ``fusion_config`` result process-wide (tile
    mode and shape width) and return its fusion width for Circuit.run
    (None, the library default, for an empty config)."""
    from . import _native as nat
    nat.call("qf_set_tile_kernel", int(cfg.get("mode", 0)))
    nat.call("qf_set_shape_bits", int(cfg.get("shape_bits", DEFAULT_SHAPE_BITS)))
    return cfg.get("fusion_k")
