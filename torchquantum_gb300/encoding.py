"""Encoders (upstream ``torchquantum/encoding/encodings.py``).

``GeneralEncoder`` (``encodings.py:50-102``) applies ``func_name_dict[f](qdev, wires,
params=x[:, input_idx])`` per entry of its ``func_list``; the per-sample parameters
make every batch row's matrix different, which the engine handles with per-row
operands (``mat_batch == bsz``).
"""
from __future__ import annotations

from .functional import func_name_dict
from .module import QuantumModule, static_support
from .operators import op_name_dict

__all__ = ["Encoder", "GeneralEncoder", "PhaseEncoder", "MultiPhaseEncoder", "StateEncoder", "AmplitudeEncoder",
           "MagnitudeEncoder"]


class Encoder(QuantumModule):
    def __init__(self):
        super().__init__()
        self.q_device = None

    def forward(self, qdev, x):
        raise NotImplementedError


class GeneralEncoder(Encoder):
    def __init__(self, func_list):
        super().__init__()
        self.func_list = func_list

    @static_support
    def forward(self, qdev, x):
        for info in self.func_list:
            params = None
            if op_name_dict[info["func"]].num_params > 0:
                idx = info["input_idx"]
                if _consecutive(idx):  # a view: the engine reads the angles in place
                    params = x[:, idx[0]:idx[-1] + 1]
                else:
                    params = x[:, idx]
            func_name_dict[info["func"]](qdev, wires=info["wires"], params=params)


def _consecutive(idx) -> bool:
    return isinstance(idx, (list, tuple)) and len(idx) > 0 and all(isinstance(i, int) for i in idx) and \
        list(idx) == list(range(idx[0], idx[0] + len(idx)))


class PhaseEncoder(Encoder):
    """``func`` on every wire k with angle ``x[:, k]`` (upstream encodings.py:133-160)."""

    def __init__(self, func):
        super().__init__()
        self.func = func

    @static_support
    def forward(self, qdev, x):
        for k in range(qdev.n_wires):
            self.func(qdev, wires=k, params=x[:, k:k + 1])


class MultiPhaseEncoder(Encoder):
    """``funcs[k]`` on ``wires[k]`` with the next 1 / 2 / 3 columns of ``x`` for
    rx, ry, rz, u1, phaseshift / u2 / u3 (upstream encodings.py:163-205)."""

    _STRIDE = {"rx": 1, "ry": 1, "rz": 1, "u1": 1, "phaseshift": 1, "u2": 2, "u3": 3}

    def __init__(self, funcs, wires=None):
        super().__init__()
        self.funcs = list(funcs) if isinstance(funcs, (list, tuple)) else [funcs]
        self.wires = wires

    @static_support
    def forward(self, qdev, x):
        if self.wires is None:
            self.wires = list(range(qdev.n_wires)) * (len(self.funcs) // qdev.n_wires)
        col = 0
        for k, func in enumerate(self.funcs):
            if func not in self._STRIDE:
                raise ValueError(func)
            step = self._STRIDE[func]
            func_name_dict[func](qdev, wires=self.wires[k], params=x[:, col:col + step])
            col += step


class MagnitudeEncoder(Encoder):
    """Placeholder class with upstream's name (encodings.py:243-249 defines no forward)."""


class StateEncoder(Encoder):
    """Load a (zero-padded, normalised) state from ``x`` (upstream encodings.py StateEncoder)."""

    def forward(self, qdev, x):
        import torch

        pad = (1 << qdev.n_wires) - x.shape[1]
        state = torch.cat([x, torch.zeros(x.shape[0], pad, device=x.device, dtype=x.dtype)], dim=-1)
        state = state / state.abs().pow(2).sum(-1, keepdim=True).sqrt()
        qdev.set_states(state.to(torch.complex64))


AmplitudeEncoder = StateEncoder
