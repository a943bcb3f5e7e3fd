"""Drop the GB300 backend into an unmodified QuantumFlow (the reference).

QuantumFlow binds its tensor-library backend once, when ``quantumflow`` is
imported (quantumflow/backend/__init__.py:14-23, chosen by
QUANTUMFLOW_BACKEND from a fixed tuple, quantumflow/config.py:43-50).
:func:`install` pre-registers :mod:`quantumflow_gb300.refbackend` as the
module ``quantumflow.backend`` before that import, so ``Gate.run``,
``Circuit.run``, ``qubo_circuit`` and ``State.expectation`` of the reference
run on the GPU kernels without any change to its source.

Usage::

    import quantumflow_gb300.shim as shim
    shim.install()          # before the first `import quantumflow`
    import quantumflow as qf
"""
import importlib.util
import os
import sys

from . import refbackend


def install(package: str = "quantumflow") -> None:
    """Make ``<package>.backend`` resolve to the GB300 backend module.

    Must run before ``<package>`` is first imported; raises if it already
    was (its modules would hold references to the old backend)."""
    if package in sys.modules:
        if getattr(sys.modules.get(package + ".backend"), "BACKEND", None) == refbackend.BACKEND:
            return
        raise RuntimeError(f"{package} is already imported; install the GB300 backend first")
    spec = importlib.util.find_spec(package)
    if spec is None or not spec.submodule_search_locations:
        raise ImportError(f"cannot locate the {package} package")
    pkg_dir = list(spec.submodule_search_locations)[0]
    # submodules of the original backend package (e.g. numpybk, whose
    # EINSUM_SUBSCRIPTS quantumflow/qubits.py imports) stay importable
    refbackend.__path__ = [os.path.join(pkg_dir, "backend")]
    refbackend.__package__ = package + ".backend"
    sys.modules[package + ".backend"] = refbackend


def installed(package: str = "quantumflow") -> bool:
    return getattr(sys.modules.get(package + ".backend"), "BACKEND", None) == refbackend.BACKEND
