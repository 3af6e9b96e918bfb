"""QuantumModule and containers (upstream ``torchquantum/module/modules.py:38-368``).

Static mode keeps the upstream switch (``static_on(wires_per_block=k)`` /
``static_off``) but routes it to the engine's fused method: while a graph-top module
in static mode runs, its QuantumDevice records gates without applying them, and the
fusion planner applies them as 2^k x 2^k blocks when the state is next read.
"""
from __future__ import annotations

import functools
from typing import Iterable

import torch
import torch.nn as nn

__all__ = ["QuantumModule", "QuantumModuleList", "QuantumModuleDict", "static_support"]


def static_support(f):
    """Decorator for ``forward``: a graph-top module in static mode runs ``f`` with the
    device switched to the fused method (upstream ``graph/graphs.py:60-81``)."""

    @functools.wraps(f)
    def forward_register_graph(*args, **kwargs):
        self = args[0]
        qdev = args[1] if len(args) > 1 else kwargs.get("q_device", kwargs.get("qdev"))
        if getattr(self, "static_mode", False) and getattr(self, "is_graph_top", False) and qdev is not None \
                and hasattr(qdev, "method"):
            prev = (qdev.method, qdev.fuse_wires)
            qdev.method = "fused"
            qdev.fuse_wires = self.wires_per_block or qdev.fuse_wires
            try:
                return f(*args, **kwargs)
            finally:
                qdev._flush()
                qdev.method, qdev.fuse_wires = prev
        return f(*args, **kwargs)

    return forward_register_graph


class QuantumModule(nn.Module):
    def __init__(self) -> None:
        super().__init__()
        self.static_mode = False
        self.graph = None
        self.parent_graph = None
        self.is_graph_top = False
        self.unitary = None
        self.wires = None
        self.n_wires = None
        self.q_device = None
        self.device = None
        self.wires_per_block = None
        self.qiskit_processor = None
        self.noise_model_tq = None
        self.Operator_list = None

    def load_op_history(self, op_history):
        """Build operators from upstream op-history dicts (modules.py:92-133)."""
        from .operators import op_name_dict

        ops = []
        for op in op_history:
            cls = op_name_dict[op["name"]]
            trainable = op.get("trainable", False)
            has_params = (op.get("params", None) is not None) or trainable
            wires = op["wires"]
            n_wires = len(wires) if isinstance(wires, Iterable) else 1
            ops.append(cls(has_params=has_params, trainable=trainable, init_params=op.get("params", None),
                           n_wires=n_wires, wires=wires, inverse=op.get("inverse", False)))
        self.Operator_list = QuantumModuleList(ops)

    @classmethod
    def from_op_history(cls, op_history):
        qmodule = cls()
        qmodule.load_op_history(op_history)
        qmodule.forward = qmodule.forward_Operators_list
        return qmodule

    def forward_Operators_list(self, qdev):
        assert self.Operator_list is not None, "Operator_list should not contain nothing"
        for op in self.Operator_list:
            op(qdev)

    def set_noise_model_tq(self, noise_model_tq):
        for module in self.modules():
            module.noise_model_tq = noise_model_tq

    def set_qiskit_processor(self, processor):
        for module in self.modules():
            module.qiskit_processor = processor

    def set_wires_per_block(self, wires_per_block):
        self.wires_per_block = wires_per_block

    def static_on(self, is_graph_top=True, wires_per_block=3):
        self.wires_per_block = wires_per_block
        self.static_mode = True
        self.is_graph_top = is_graph_top
        for module in self.children():
            if isinstance(module, QuantumModule):
                module.static_on(is_graph_top=False, wires_per_block=wires_per_block)

    def static_off(self):
        self.static_mode = False
        self.is_graph_top = False
        for module in self.children():
            if isinstance(module, QuantumModule):
                module.static_off()

    def get_unitary(self, x=None):
        """Unitary of the module on ``self.n_wires`` wires (modules.py:326-354)."""
        from .device import QuantumDevice

        assert self.n_wires is not None, "n_wires should not be None"
        qdev = QuantumDevice(n_wires=self.n_wires)
        qdev.reset_identity_states()
        if x is None:
            self.forward(qdev)
        else:
            self.forward(qdev, x)
        return qdev.get_states_1d().T


class QuantumModuleList(nn.ModuleList, QuantumModule):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)


class QuantumModuleDict(nn.ModuleDict, QuantumModule):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
