"""quantumflow_gb300: a GB300-native state-vector backend for QuantumFlow.

The public namespace mirrors the reference package ``quantumflow``
(quantumflow/__init__.py:8-22) for the state-vector path: states, gates,
standard gates, circuits, QAOA helpers and state measures.  All amplitude
arithmetic runs in the CUDA library ``_lib/libqfgb300.so`` (C ABI in
include/qf_gb300.h); importing the package fails if that library is missing.
"""
from .config import version as __version__  # noqa: F401
from . import config  # noqa: F401
from .qubits import *  # noqa: F401,F403
from .states import *  # noqa: F401,F403
from .states import inner, Buffer  # noqa: F401
from .ops import *  # noqa: F401,F403
from .gates import *  # noqa: F401,F403
from .stdgates import *  # noqa: F401,F403
from .circuits import *  # noqa: F401,F403
from .measures import *  # noqa: F401,F403
from .densities import *  # noqa: F401,F403
from .channels import *  # noqa: F401,F403
from .dagcircuit import *  # noqa: F401,F403
from .cbits import *  # noqa: F401,F403
from .stdops import *  # noqa: F401,F403
from .programs import *  # noqa: F401,F403
from .qaoa import qubo_circuit, graph_cuts, QAOAMaxCut, QAOAExpectation, Graph, maxcut_qaoa  # noqa: F401
from . import qaoa  # noqa: F401
from . import batched, autotune, gnn, adjoint, datasets  # noqa: F401
# ``qf.backend`` is the reference's backend-module interface
# (quantumflow/backend/__init__.py:25-35: tensormul, inner, astensor, ...),
# here over the kernels
from . import refbackend as backend  # noqa: F401
