"""The C-ABI library loads and exports every entry point include/qf_gb300.h
declares; argument validation returns status codes without touching a GPU."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qf_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qf_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_functions():
    names = declared_functions()
    assert "qf_apply_gate" in names and "qf_run_circuit" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    from quantumflow_gb300 import _native as nat
    lib = ctypes.CDLL(nat.LIBPATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from quantumflow_gb300 import _native as nat
    assert set(declared_functions()) <= set(nat.SIGNATURES), set(declared_functions()) - set(nat.SIGNATURES)


def test_status_strings_and_version():
    from quantumflow_gb300 import _native as nat
    assert nat.lib.qf_abi_version() == nat.ABI_VERSION
    for code, text in nat.STATUS.items():
        assert nat.lib.qf_status_string(code).decode() == text


def test_validation_without_gpu():
    """Every check below fails before any CUDA call is made."""
    from quantumflow_gb300 import _native as nat
    lib = nat.lib
    fake = ctypes.c_void_p(0x10000)  # aligned, never dereferenced
    mis = ctypes.c_void_p(0x10008)
    m = nat.double_array([1, 0, 0, 0, 0, 0, 1, 0])
    ax = nat.int_array([0])
    s = ctypes.c_void_p(0)
    assert lib.qf_apply_gate(fake, fake, 40, 1, 1, ax, m, s) == 5          # too large
    assert lib.qf_apply_gate(fake, fake, 4, 7, 1, ax, m, s) == 2           # layout
    assert lib.qf_apply_gate(None, fake, 4, 1, 1, ax, m, s) == 1           # null
    assert lib.qf_apply_gate(mis, mis, 4, 1, 1, ax, m, s) == 4             # alignment
    assert lib.qf_apply_gate(fake, fake, 4, 1, 1, nat.int_array([4]), m, s) == 1  # axis range
    assert lib.qf_apply_gate(fake, fake, 4, 1, 2, nat.int_array([1, 1]), m, s) == 1  # repeated
    assert lib.qf_apply_gate(fake, fake, 8, 1, 6, nat.int_array(range(6)), m, s) == 6  # k > 5
    assert lib.qf_apply_gate(fake, fake, 2, 1, 3, nat.int_array(range(3)), m, s) == 1  # k > n
    assert lib.qf_fill_basis(fake, 3, 0, 8, s) == 1                        # index range
    assert lib.qf_cut_values(fake, 4, 1, nat.int_array([0, 9]), s) == 1
    assert lib.qf_cut_values(fake, 4, 5000, nat.int_array([0, 1]), s) == 5
    assert lib.qf_norm2(fake, 4, 1, fake, None, 0, s) == 8                 # workspace
    assert lib.qf_convert(fake, 1, fake, 2, 4, s) == 1                     # aliasing
    assert lib.qf_sample_workspace_bytes(0) == 0
    assert lib.qf_reduce_workspace_bytes(10) >= 2048 * 16
