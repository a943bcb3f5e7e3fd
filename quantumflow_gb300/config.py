"""Configuration, mirroring quantumflow/config.py:19-62 of the reference.

Environment variables (prefix ``QUANTUMFLOW_GB300_``):

``C128``    arithmetic for complex128 states: ``ff`` (default) holds each
            amplitude as float-float pairs and computes on the FP32 pipes
            (48-bit significand, results within 1e-12 of FP64); ``fp64``
            computes in native FP64 (bit-for-bit IEEE double arithmetic,
            ~3x slower on GB300 whose FP64 rate is 1/64 of FP32).
``FUSION``  maximum number of high qubits (bit >= 5) per fused pass;
            0 (default) lets the library pick per element type, 1 disables
            fusion (one pass per gate).
``SEED``    seed for sampling (reference QUANTUMFLOW_SEED, config.py:59-62).
"""
import os

_PREFIX = "QUANTUMFLOW_GB300_"

TOLERANCE = 1e-6
"""Tolerance used in floating point comparisons (reference config.py:54)."""

C128_ARITHMETIC = os.getenv(_PREFIX + "C128", "ff")
if C128_ARITHMETIC not in ("ff", "fp64"):
    raise ValueError(f"Unknown {_PREFIX}C128={C128_ARITHMETIC} (expected ff or fp64)")

FUSION_K = int(os.getenv(_PREFIX + "FUSION", "0"))

_ENVSEED = os.getenv(_PREFIX + "SEED", os.getenv("QUANTUMFLOW_SEED", None))
SEED = int(_ENVSEED) if _ENVSEED is not None else None

version = "0.1.0"
