"""Operator classes (upstream ``torchquantum/operator/op_types.py:53-443`` and
``operator/standard_gates/*.py``).

Same class names, ``num_params`` / ``num_wires`` / ``op_name`` / ``func`` attributes,
parameter handling (``[1, num_params]`` ``nn.Parameter``, uniform in [-pi, pi) by
default, ``build_params``/``reset_params`` at op_types.py:377-405) and ``forward``
(op_types.py:182-264), so a trainable gate's gradient sums over the batch exactly as
upstream's broadcast matrix does.  The registry ``op_name_dict`` carries the same
names and aliases (``standard_gates/__init__.py:139-162``).
"""
from __future__ import annotations

from collections.abc import Iterable

import numpy as np
import torch
import torch.nn as nn

from . import functional as tqf
from . import gates as G
from .module import QuantumModule

__all__ = ["Operator", "Observable", "Operation", "DiagonalOperation", "op_name_dict", "fixed_ops",
           "parameterized_ops", "AnyNParams", "AnyWires", "AllWires"]

AnyNParams = -1
AnyWires = -1
AllWires = 0


class Operator(QuantumModule):
    num_params = 0
    num_wires = 1
    op_name = None
    func = None

    def __init__(self, has_params=False, trainable=False, init_params=None, n_wires=None, wires=None, inverse=False):
        super().__init__()
        self.params = None
        self.n_wires = n_wires
        self.wires = wires
        self._name = self.__class__.__name__
        self.static_matrix = None
        self.inverse = inverse
        self.clifford_quantization = False
        if trainable and not has_params:
            has_params = True
        self.has_params = has_params
        self.trainable = trainable
        if self.has_params:
            self.params = self.build_params(trainable=self.trainable)
            self.reset_params(init_params)

    @property
    def name(self):
        return self._name

    @name.setter
    def name(self, value):
        self._name = value

    @classmethod
    def _matrix(cls, params):
        return tqf.mat_dict[cls.op_name](params) if cls.op_name in tqf.mat_dict else None

    @property
    def matrix(self):
        return self._matrix(self.params)

    @classmethod
    def _eigvals(cls, params):
        return None

    @property
    def eigvals(self):
        return self._eigvals(self.params)

    def _get_unitary_matrix(self):
        return self.matrix

    def set_wires(self, wires):
        self.wires = [wires] if isinstance(wires, int) else wires

    def build_params(self, trainable):
        nparams = self.num_params if self.num_params >= 0 else 1
        p = nn.Parameter(torch.empty([1, nparams], dtype=torch.float32))
        p.requires_grad = bool(trainable)
        return p

    def reset_params(self, init_params=None):
        if init_params is not None:
            if isinstance(init_params, Iterable):
                for k, v in enumerate(init_params):
                    torch.nn.init.constant_(self.params[:, k], v)
            else:
                torch.nn.init.constant_(self.params, init_params)
        else:
            torch.nn.init.uniform_(self.params, -np.pi, np.pi)

    def forward(self, q_device, wires=None, params=None, inverse=None):
        # plain attributes are written straight into __dict__: nn.Module.__setattr__ costs
        # more than the gate itself on small circuits
        d = self.__dict__
        if inverse is not None:
            d["inverse"] = inverse
        if params is not None:
            self.params = params
        if self.params is not None and self.params.dim() == 1:
            self.params = self.params.unsqueeze(-1)
        if wires is not None:
            d["wires"] = [wires] if isinstance(wires, int) else wires
        if self.params is None:
            if self.n_wires is None:
                self.func(q_device, self.wires, inverse=self.inverse)
            else:
                self.func(q_device, self.wires, n_wires=self.n_wires, inverse=self.inverse)
        else:
            if self.n_wires is None:
                self.func(q_device, self.wires, params=self.params, inverse=self.inverse)
            else:
                self.func(q_device, self.wires, params=self.params, n_wires=self.n_wires, inverse=self.inverse)

    def __repr__(self):
        return f" class: {self.name} \n parameters: {self.params} \n wires: {self.wires} \n inverse: {self.inverse}"


class Observable(Operator):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.return_type = None

    def diagonalizing_gates(self):
        raise NotImplementedError


class Operation(Operator):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        if self.num_wires > 0:  # op_types.py:363-364
            self.n_wires = self.num_wires


class DiagonalOperation(Operation):
    @classmethod
    def _matrix(cls, params):
        return torch.diag(cls._eigvals(params))


# name of the class -> (functional gate, base class); parameters/wires from gates.GATES
_CLASSES = {
    "Hadamard": ("hadamard", "obs"), "SHadamard": ("shadamard", "op"), "CHadamard": ("chadamard", "op"),
    "PauliX": ("paulix", "obs"), "PauliY": ("pauliy", "obs"), "PauliZ": ("pauliz", "obs"), "I": ("i", "obs"),
    "S": ("s", "diag"), "SDG": ("sdg", "diag"), "T": ("t", "diag"), "TDG": ("tdg", "diag"), "SX": ("sx", "op"),
    "SXDG": ("sxdg", "op"), "CNOT": ("cnot", "op"), "CZ": ("cz", "diag"), "CY": ("cy", "op"),
    "RX": ("rx", "op"), "RY": ("ry", "op"), "RZ": ("rz", "diag"), "RXX": ("rxx", "op"), "RYY": ("ryy", "op"),
    "RZZ": ("rzz", "diag"), "RZX": ("rzx", "op"), "SWAP": ("swap", "op"), "SSWAP": ("sswap", "op"),
    "CSWAP": ("cswap", "op"), "Toffoli": ("toffoli", "op"), "PhaseShift": ("phaseshift", "diag"),
    "Rot": ("rot", "op"), "MultiRZ": ("multirz", "diag"), "CRX": ("crx", "op"), "CRY": ("cry", "op"),
    "CRZ": ("crz", "op"), "CRot": ("crot", "op"), "U1": ("u1", "diag"), "U2": ("u2", "op"), "U3": ("u3", "op"),
    "CU1": ("cu1", "diag"), "CU2": ("cu2", "op"), "CU3": ("cu3", "op"), "CU": ("cu", "op"),
    "MultiCNOT": ("multicnot", "op"), "MultiXCNOT": ("multixcnot", "op"), "Reset": ("reset", "op"),
    "SingleExcitation": ("singleexcitation", "op"), "ECR": ("ecr", "op"), "QFT": ("qft", "op"),
    "ISWAP": ("iswap", "op"), "CS": ("cs", "op"), "CSDG": ("csdg", "op"), "CSX": ("csx", "op"),
    "CCZ": ("ccz", "op"), "DCX": ("dcx", "op"), "XXMINYY": ("xxminyy", "op"), "XXPLUSYY": ("xxplusyy", "op"),
    "C3X": ("c3x", "op"), "C4X": ("c4x", "op"), "R": ("r", "op"), "GlobalPhase": ("globalphase", "op"),
    "C3SX": ("c3sx", "op"), "RCCX": ("rccx", "op"), "RC3X": ("rc3x", "op"),
}
_OP_NAMES = {"TrainableUnitary": "trainableunitary", "TrainableUnitaryStrict": "trainableunitarystrict"}
_EIGVALS = {"PauliX": [1, -1], "PauliY": [1, -1], "PauliZ": [1, -1], "Hadamard": [1, -1], "I": [1, 1]}


def _diag_gates(cls_name):
    ns = globals()
    table = {
        "PauliX": lambda: [ns["Hadamard"]()],
        "PauliY": lambda: [ns["PauliZ"](), ns["S"](), ns["Hadamard"]()],
        "PauliZ": lambda: [],
        "I": lambda: [],
        "Hadamard": lambda: [ns["RY"](has_params=True, trainable=False, init_params=-np.pi / 4)],
    }
    return table[cls_name]


def _make_class(cls_name, fname, base_kind):
    if fname == "reset":
        npar, nw = 0, -1
    else:
        gd = G.GATES[fname]
        npar, nw = gd.num_params, gd.num_wires
    base = {"obs": Observable, "op": Operation, "diag": DiagonalOperation}[base_kind]
    attrs = {
        "num_params": npar,
        "num_wires": nw,
        "op_name": _OP_NAMES.get(cls_name, fname),
        "func": staticmethod(tqf.func_name_dict[fname]),
        "__doc__": f"{cls_name} gate (upstream torchquantum.{cls_name}).",
    }
    if base_kind == "diag":
        attrs["_matrix"] = classmethod(lambda cls, params, _f=fname: tqf.mat_dict[_f](params))
    if cls_name in _EIGVALS:
        ev = torch.tensor(_EIGVALS[cls_name], dtype=torch.complex64)
        attrs["eigvals"] = ev
        attrs["_eigvals"] = classmethod(lambda cls, params, _e=ev: _e)
        attrs["diagonalizing_gates"] = lambda self, _c=cls_name: _diag_gates(_c)()
    return type(cls_name, (base,), attrs)


for _cn, (_fn, _bk) in _CLASSES.items():
    globals()[_cn] = _make_class(_cn, _fn, _bk)
    __all__.append(_cn)

# aliases (standard_gates/__init__.py and the module-level aliases upstream exports)
H, SH, CH, U, CCX = Hadamard, SHadamard, CHadamard, U3, Toffoli  # noqa: F821
EchoedCrossResonance = ECR  # noqa: F821
__all__ += ["H", "SH", "CH", "U", "CCX", "EchoedCrossResonance"]

op_name_dict = {globals()[c].op_name: globals()[c] for c in _CLASSES}
op_name_dict.update({
    "h": H, "sh": SH, "u": U3,  # noqa: F821
    "x": PauliX, "y": PauliY, "z": PauliZ, "cx": CNOT, "xx": RXX, "yy": RYY, "zz": RZZ, "zx": RZX,  # noqa: F821
    "ccx": Toffoli, "p": U1, "cp": CU1, "cr": CU1, "ch": CHadamard, "echoedcrossresonance": ECR,  # noqa: F821
})
fixed_ops = [c for c in _CLASSES if globals()[c].num_params == 0]
parameterized_ops = [c for c in _CLASSES if globals()[c].num_params > 0]


# ---------------------------------------------------------------- unitary-matrix gates
class QubitUnitary(Operation):
    """Fixed unitary matrix gate (upstream standard_gates/qubit_unitary.py)."""

    num_params = AnyNParams
    num_wires = AnyWires
    op_name = "qubitunitary"
    func = staticmethod(tqf.func_name_dict["qubitunitary"])

    @classmethod
    def _matrix(cls, params):
        return params.squeeze(0)

    def build_params(self, trainable):
        return None

    def reset_params(self, init_params=None):
        self.params = torch.as_tensor(np.asarray(init_params) if not isinstance(init_params, torch.Tensor)
                                      else init_params).to(torch.complex64)
        self.register_buffer(f"{self.name}_unitary", self.params)


class QubitUnitaryFast(QubitUnitary):
    op_name = "qubitunitaryfast"
    func = staticmethod(tqf.func_name_dict["qubitunitaryfast"])

    def __init__(self, has_params=False, trainable=False, init_params=None, n_wires=None, wires=None):
        super().__init__(has_params=True, trainable=trainable, init_params=init_params, n_wires=n_wires,
                         wires=wires)

    @classmethod
    def from_controlled_operation(cls, op, c_wires, t_wires, trainable):
        """Controlled version of ``op`` (upstream qubit_unitary.py from_controlled_operation)."""
        c = np.array(c_wires)
        t = np.array(t_wires)
        u = op.matrix
        u_wires = op.n_wires if op.n_wires is not None else int(np.log2(u.shape[-1]))
        wires = [int(c.item())] if c.ndim == 0 else [int(w) for w in c]
        twires = [int(t.item())] if t.ndim == 0 else [int(w) for w in t.flatten()]
        n_sets = 1 if t.ndim == 0 else len(twires) // u_wires
        cu = u
        for _ in range(n_sets - 1):
            cu = torch.kron(cu, u)
        n_wires = len(wires) + len(twires)
        full = torch.eye(1 << n_wires, dtype=torch.complex64)
        d = cu.shape[-1]
        full[-d:, -d:] = cu.to(torch.complex64)
        return cls(has_params=True, trainable=trainable, init_params=full, n_wires=n_wires, wires=wires + twires)


class TrainableUnitary(Operation):
    """Trainable dense unitary (upstream standard_gates/trainable_unitary.py)."""

    num_params = AnyNParams
    num_wires = AnyWires
    op_name = "trainableunitary"
    func = staticmethod(tqf.func_name_dict["qubitunitaryfast"])

    def build_params(self, trainable):
        p = nn.Parameter(torch.empty(1, 2 ** self.n_wires, 2 ** self.n_wires, dtype=torch.complex64))
        p.requires_grad = bool(trainable)
        return p

    def reset_params(self, init_params=None):
        mat = torch.randn((1, 2 ** self.n_wires, 2 ** self.n_wires), dtype=torch.complex64)
        u, _, v = torch.svd(mat)
        self.params.data.copy_(u.matmul(v.permute(0, 2, 1)))


class TrainableUnitaryStrict(TrainableUnitary):
    op_name = "trainableunitarystrict"
    func = staticmethod(tqf.func_name_dict["qubitunitarystrict"])


for _c in (QubitUnitary, QubitUnitaryFast, TrainableUnitary, TrainableUnitaryStrict):
    op_name_dict[_c.op_name] = _c
    __all__.append(_c.__name__)
