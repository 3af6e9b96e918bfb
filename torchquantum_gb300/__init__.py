"""torchquantum_gb300: GB300-native statevector engine behind the TorchQuantum API.

Drop-in for the gate-application path of upstream torchquantum:
``import torchquantum_gb300 as tq`` / ``import torchquantum_gb300.functional as tqf``
gives ``tq.QuantumDevice``, the ``tqf`` gate functions, the ``tq.Operator`` classes,
``tq.QuantumModule`` and ``expval_joint_analytical``, executed by hand-written
sm_103a CUDA kernels (``libtqk.so``, C ABI in ``include/tqk.h``).  CUDA only: the
engine raises if its library is missing or the device is not a GPU.
"""
from . import gates  # noqa: F401
from . import functional  # noqa: F401
from .device import QuantumDevice, _bind_gate_methods
from .module import QuantumModule, QuantumModuleList, QuantumModuleDict, static_support
from .operators import *  # noqa: F401,F403
from .operators import op_name_dict, fixed_ops, parameterized_ops, Operator, Operation, Observable, \
    DiagonalOperation  # noqa: F401
from . import layers as layer  # noqa: F401
from .layers import *  # noqa: F401,F403
from .encoding import GeneralEncoder, StateEncoder, Encoder  # noqa: F401
from .measurement import expval_joint_analytical, expval_joint_analytical_batch, expval, MeasureAll, probs  # noqa
from .measurement import measure, gen_bitstrings, MeasureMultipleTimes, MeasureMultiPauliSum, \
    MeasureMultiQubitPauliSum, find_observable_groups, expval_joint_sampling, \
    expval_joint_sampling_grouping  # noqa: F401
from . import measurement  # noqa: F401
from .density import NoiseDevice  # noqa: F401

_bind_gate_methods()

__version__ = "0.1.0"
