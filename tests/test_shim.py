"""The reference QuantumFlow binds the GB300 backend through the shim.

Runs where a reference checkout is named by the QF_REFERENCE environment
variable (skipped otherwise); needs no GPU because it only checks what
``import quantumflow`` binds."""
import os
import subprocess
import sys

import pytest

from tests.conftest import ROOT

REF = os.environ.get("QF_REFERENCE", "")

CHECK = r"""
import sys
sys.path.insert(0, {root!r})
sys.path.insert(0, {golden!r})
import make_golden          # stub finder for the reference's absent optional imports
import importlib.abc
sys.meta_path.insert(0, make_golden._StubFinder())
sys.path.insert(0, {ref!r})
sys.dont_write_bytecode = True
import quantumflow_gb300.shim as shim
shim.install()
import quantumflow as qf
import quantumflow_gb300.refbackend as rb
assert qf.backend is rb, qf.backend
assert qf.backend.BACKEND == "gb300"
import quantumflow.ops, quantumflow.states, quantumflow.qubits
assert quantumflow.ops.bk is rb and quantumflow.states.bk is rb and quantumflow.qubits.bk is rb
from quantumflow.backend.numpybk import EINSUM_SUBSCRIPTS
assert EINSUM_SUBSCRIPTS.startswith("abc")
print("bound")
"""


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "quantumflow")),
                    reason="QF_REFERENCE does not name a reference checkout")
def test_reference_binds_gb300_backend():
    code = CHECK.format(root=ROOT, golden=os.path.join(ROOT, "tests", "golden"), ref=REF)
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "bound" in r.stdout


def test_install_refuses_after_import(monkeypatch):
    import types
    import quantumflow_gb300.shim as shim
    monkeypatch.setitem(sys.modules, "qf_fake_pkg", types.ModuleType("qf_fake_pkg"))
    with pytest.raises(RuntimeError):
        shim.install("qf_fake_pkg")
