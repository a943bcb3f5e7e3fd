"""Configuration, mirroring quantumflow/config.py:19-62 of the reference.

Environment variables (prefix ``QUANTUMFLOW_GB300_``):

``C128``    arithmetic for complex128 states: ``fx`` (default) keeps the
            amplitudes in FP64 and applies unitary gates in 64-bit integer
            fixed point on the integer multiply pipe (each thread's
            amplitude group shares one exponent; >= 55 significant bits
            relative to the group's largest part, one FP64 rounding per
            pass; other gates run in native FP64); ``ff`` holds each
            amplitude as float-float pairs and computes on the FP32 pipes
            (48-bit significand); ``fp64`` computes in native FP64
            (bit-for-bit IEEE double arithmetic, several times slower on
            GB300, whose FP64 FMA rate is about 1/64 of its FP32 rate).
            The QAOA fast path (qf_qaoa_state, the adjoint and batched
            kernels) computes complex128 in float-float under ``fx`` and
            ``ff``, and in native FP64 under ``fp64``.
``FUSION``  maximum number of high qubits (bit >= 5) per fused pass;
            0 (default) lets the library pick per element type, 1 disables
            fusion (one pass per gate).
``SEED``    seed for sampling (reference QUANTUMFLOW_SEED, config.py:59-62).
"""
import os

_PREFIX = "QUANTUMFLOW_GB300_"

TOLERANCE = 1e-6
"""Tolerance used in floating point comparisons (reference config.py:54)."""

C128_ARITHMETIC = os.getenv(_PREFIX + "C128", "fx")
if C128_ARITHMETIC not in ("fx", "ff", "fp64"):
    raise ValueError(f"Unknown {_PREFIX}C128={C128_ARITHMETIC} (expected fx, ff or fp64)")

FUSION_K = int(os.getenv(_PREFIX + "FUSION", "0"))

_ENVSEED = os.getenv(_PREFIX + "SEED", os.getenv("QUANTUMFLOW_SEED", None))
SEED = int(_ENVSEED) if _ENVSEED is not None else None

version = "0.1.0"
