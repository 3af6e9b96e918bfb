"""torchquantum_gb300: GB300-native statevector engine behind the TorchQuantum API.

Drop-in for the gate-application path of upstream torchquantum:
``import torchquantum_gb300 as tq`` / ``import torchquantum_gb300.functional as tqf``
gives ``tq.QuantumDevice``, the ``tqf`` gate functions, the ``tq.Operator`` classes,
``tq.QuantumModule`` and ``expval_joint_analytical``, executed by hand-written
sm_103a CUDA kernels (``libtqk.so``, C ABI in ``include/tqk.h``).  CUDA only: the
engine raises if its library is missing or the device is not a GPU.
"""
from .macro import *  # noqa: F401,F403
from . import gates  # noqa: F401
from . import functional  # noqa: F401
from .device import QuantumDevice, set_engine_defaults, _bind_gate_methods
from .module import QuantumModule, QuantumModuleList, QuantumModuleDict, static_support
from .operators import *  # noqa: F401,F403
from .operators import op_name_dict, fixed_ops, parameterized_ops, Operator, Operation, Observable, \
    DiagonalOperation  # noqa: F401
from . import layers as layer  # noqa: F401
from .layers import *  # noqa: F401,F403
from .encoding import GeneralEncoder, StateEncoder, Encoder, PhaseEncoder, MultiPhaseEncoder, AmplitudeEncoder, \
    MagnitudeEncoder  # noqa: F401
from .measurement import expval_joint_analytical, expval_joint_analytical_batch, expval, MeasureAll, probs  # noqa
from .measurement import measure, gen_bitstrings, MeasureMultipleTimes, MeasureMultiPauliSum, \
    MeasureMultiQubitPauliSum, find_observable_groups, expval_joint_sampling, \
    expval_joint_sampling_grouping  # noqa: F401
from . import measurement  # noqa: F401
from .density import NoiseDevice  # noqa: F401

_bind_gate_methods()


def _export_functional():
    """Upstream star-imports its functional package at the top level (``tq.rx``,
    ``tq.cnot``, ``tq.gate_wrapper``, ``tq.func_name_dict``, ...): the same names here,
    without shadowing the operator classes and modules already exported."""
    g = globals()
    names = list(functional.func_name_dict) + list(functional.__all__) + \
        [n for n in dir(functional) if n.endswith("_matrix")]
    for name in names:
        if name not in g:
            g[name] = getattr(functional, name)


_export_functional()

__version__ = "0.1.0"
