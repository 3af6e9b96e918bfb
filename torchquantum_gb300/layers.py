"""Circuit templates on the hot path (upstream ``torchquantum/layer``).

``Op1QAllLayer`` (``layer/layers/layers.py:71-96``), ``Op2QAllLayer``
(``layer/entanglement/op2_layer.py:43-110``), ``Op2QDenseLayer``, ``LayerTemplate0``
(``layers.py:99-138``), ``NLocal`` / ``TwoLocal`` (``layer/nlocal/nlocal.py:37-134``,
``two_local.py:42-111``) and the TwoLocal presets ``EfficientSU2``, ``RealAmplitudes``,
``ExcitationPreserving``, and ``RandomLayer`` / ``RandomLayerAllTypes``
(``layer/layers/random_layers.py:80-298``): the same constructors and wire patterns,
built from this package's operators.
"""
from __future__ import annotations

from collections.abc import Iterable

import numpy as np

from .module import QuantumModule, QuantumModuleList, static_support
from . import operators as ops

__all__ = ["Op1QAllLayer", "Op2QAllLayer", "Op2QDenseLayer", "LayerTemplate0", "NLocal", "TwoLocal", "EfficientSU2",
           "RealAmplitudes", "ExcitationPreserving", "RandomLayer", "RandomLayerAllTypes"]


class Op1QAllLayer(QuantumModule):
    def __init__(self, op, n_wires: int, has_params=False, trainable=False):
        super().__init__()
        self.n_wires = n_wires
        self.op = op
        self.ops_all = QuantumModuleList()
        for _ in range(n_wires):
            self.ops_all.append(op(has_params=has_params, trainable=trainable))

    @static_support
    def forward(self, q_device):
        for k in range(self.n_wires):
            self.ops_all[k](q_device, wires=k)


class Op2QAllLayer(QuantumModule):
    """Pairs [k, (k+jump) % n]; n pairs if circular else n - jump."""

    def __init__(self, op, n_wires: int, has_params=False, trainable=False, wire_reverse=False, jump=1,
                 circular=False):
        super().__init__()
        self.n_wires = n_wires
        self.jump = jump
        self.circular = circular
        self.op = op
        self.wire_reverse = wire_reverse
        self.ops_all = QuantumModuleList()
        n_ops = n_wires if circular else n_wires - jump
        for _ in range(n_ops):
            self.ops_all.append(op(has_params=has_params, trainable=trainable))

    @static_support
    def forward(self, q_device):
        for k in range(len(self.ops_all)):
            wires = [k, (k + self.jump) % self.n_wires]
            if self.wire_reverse:
                wires.reverse()
            self.ops_all[k](q_device, wires=wires)


class Op2QDenseLayer(QuantumModule):
    """Every pair (i, j), i < j."""

    def __init__(self, op, n_wires: int, has_params=False, trainable=False, wire_reverse=False):
        super().__init__()
        self.n_wires = n_wires
        self.op = op
        self.wire_reverse = wire_reverse
        self.ops_all = QuantumModuleList()
        for _ in range(n_wires * (n_wires - 1) // 2):
            self.ops_all.append(op(has_params=has_params, trainable=trainable))

    @static_support
    def forward(self, q_device):
        k = 0
        for i in range(self.n_wires):
            for j in range(i + 1, self.n_wires):
                wires = [i, j]
                if self.wire_reverse:
                    wires.reverse()
                self.ops_all[k](q_device, wires=wires)
                k += 1


class LayerTemplate0(QuantumModule):
    name = None

    def __init__(self, arch: dict = None):
        super().__init__()
        self.n_wires = arch["n_wires"]
        self.arch = arch
        self.n_blocks = arch.get("n_blocks", None)
        self.n_layers_per_block = arch.get("n_layers_per_block", None)
        self.layers_all = self.build_layers()

    def build_layers(self):
        raise NotImplementedError

    @static_support
    def forward(self, q_device):
        self.q_device = q_device
        for k in range(len(self.layers_all)):
            self.layers_all[k](q_device)


class NLocal(LayerTemplate0):
    def __init__(self, rotation_ops=None, entanglement_ops=None, arch=None, rotation_layer=Op1QAllLayer,
                 entanglement_layer=Op2QAllLayer, reps=1, rotation_layer_params=None, entanglement_layer_params=None,
                 initial_circuit=None, skip_final_rotation_layer=False):
        self.rotation_ops = rotation_ops
        self.rotation_layer = rotation_layer
        self.rotation_layer_params = rotation_layer_params or {}
        self.entanglement_ops = entanglement_ops
        self.entanglement_layer = entanglement_layer
        self.entanglement_layer_params = entanglement_layer_params or {}
        self.initial_circuit = initial_circuit
        self.skip_final_rotation_layer = skip_final_rotation_layer
        self.reps = reps
        super().__init__(arch)

    def build_rotation_block(self):
        return [self.rotation_layer(op=r, n_wires=self.n_wires, **self.rotation_layer_params) for r in self.rotation_ops]

    def build_entanglement_block(self):
        return [self.entanglement_layer(op=e, n_wires=self.n_wires, **self.entanglement_layer_params)
                for e in self.entanglement_ops]

    def build_layers(self):
        layers_all = QuantumModuleList()
        if self.initial_circuit is not None:
            layers_all.append(self.initial_circuit)
        for _ in range(self.reps):
            layers_all.extend(self.build_rotation_block())
            layers_all.extend(self.build_entanglement_block())
        if not self.skip_final_rotation_layer:
            layers_all.extend(self.build_rotation_block())
        return layers_all


def _as_ops(x):
    if isinstance(x, str):
        return [ops.op_name_dict[x]]
    if isinstance(x, Iterable):
        return [ops.op_name_dict[o] if isinstance(o, str) else o for o in x]
    return [x]


class TwoLocal(NLocal):
    def __init__(self, n_wires=1, rotation_ops=None, entanglement_ops=None, rotation_layer=Op1QAllLayer,
                 entanglement_layer="linear", reps=1, entanglement_layer_params=None, initial_circuit=None,
                 skip_final_rotation_layer=False):
        params = dict(entanglement_layer_params or {})
        if entanglement_layer == "linear":
            entanglement_layer = Op2QAllLayer
        elif entanglement_layer == "reverse_linear":
            entanglement_layer, params = Op2QAllLayer, {"wire_reverse": True}
        elif entanglement_layer == "circular":
            entanglement_layer, params = Op2QAllLayer, {"circular": True}
        elif entanglement_layer == "full":
            entanglement_layer = Op2QDenseLayer
        super().__init__(arch={"n_wires": n_wires}, rotation_ops=_as_ops(rotation_ops),
                         rotation_layer=rotation_layer, rotation_layer_params={"has_params": True, "trainable": True},
                         entanglement_ops=_as_ops(entanglement_ops), entanglement_layer=entanglement_layer,
                         entanglement_layer_params=params, initial_circuit=initial_circuit, reps=reps,
                         skip_final_rotation_layer=skip_final_rotation_layer)


class EfficientSU2(TwoLocal):
    def __init__(self, n_wires=1, entanglement_layer="reverse_linear", reps=3, skip_final_rotation_layer=False):
        super().__init__(n_wires=n_wires, rotation_ops=[ops.RY, ops.RZ], entanglement_ops=[ops.CNOT],
                         entanglement_layer=entanglement_layer, reps=reps,
                         skip_final_rotation_layer=skip_final_rotation_layer)


class RealAmplitudes(TwoLocal):
    def __init__(self, n_wires=1, entanglement_layer="reverse_linear", reps=3, skip_final_rotation_layer=False):
        super().__init__(n_wires=n_wires, rotation_ops=[ops.RY], entanglement_ops=[ops.CNOT],
                         entanglement_layer=entanglement_layer, reps=reps,
                         skip_final_rotation_layer=skip_final_rotation_layer)


class ExcitationPreserving(TwoLocal):
    def __init__(self, n_wires=1, entanglement_layer="full", reps=3, skip_final_rotation_layer=False):
        super().__init__(n_wires=n_wires, rotation_ops=[ops.RZ], entanglement_ops=[ops.RXX, ops.RYY],
                         entanglement_layer=entanglement_layer, reps=reps,
                         skip_final_rotation_layer=skip_final_rotation_layer)


class RandomLayer(QuantumModule):
    """``n_ops`` (or ``n_params`` worth of) operations drawn from ``op_types`` with
    ``op_ratios`` on random wires (upstream ``random_layers.py:80-231``).  The draws use
    numpy's global generator in upstream's order (op type, then its wires without
    replacement; ``np.random.seed(seed)`` first when a seed is given) and the operators
    initialise their parameters as upstream's do, so a seeded layer rebuilds upstream's
    circuit."""

    def __init__(self, wires, n_ops=None, n_params=None, op_ratios=None,
                 op_types=(ops.RX, ops.RY, ops.RZ, ops.CNOT), seed=None, qiskit_compatible=False):
        super().__init__()
        assert n_params is not None or n_ops is not None
        self.n_ops = n_ops
        self.n_params = n_params
        self.wires = list(wires) if isinstance(wires, Iterable) else [wires]
        self.n_wires = len(self.wires)
        op_types = list(op_types) if isinstance(op_types, Iterable) else [op_types]
        if op_ratios is None:
            op_ratios = [1] * len(op_types)
        elif not isinstance(op_ratios, Iterable):
            op_ratios = [op_ratios]
        # qiskit_compatible only filters qiskit-incompatible gates upstream; every gate here
        # runs on the engine, so the list is kept as given
        self.op_types = op_types
        self.op_ratios = np.array(op_ratios) / sum(op_ratios)
        self.seed = seed
        self.op_list = QuantumModuleList()
        if seed is not None:
            np.random.seed(seed)
        self.build_random_layer()

    def rebuild_random_layer_from_op_list(self, n_ops_in, wires_in, op_list_in):
        """Rebuild from a saved op list (upstream ``random_layers.py:153-175``)."""
        self.n_ops = n_ops_in
        self.wires = wires_in
        self.op_list = QuantumModuleList()
        for op_in in op_list_in:
            self.op_list.append(ops.op_name_dict[op_in.name.lower()](
                has_params=op_in.has_params, trainable=op_in.trainable, wires=op_in.wires, n_wires=op_in.n_wires))

    def build_random_layer(self):
        op_cnt = param_cnt = 0
        while True:
            op = np.random.choice(self.op_types, p=self.op_ratios)
            k = op.num_wires
            if k > self.n_wires:
                continue
            any_wire = k == -1
            if any_wire:
                k = self.n_wires
            op_wires = list(np.random.choice(self.wires, size=k, replace=False))
            if any_wire:
                if op().name in ["MultiRZ"]:
                    operation = op(has_params=True, trainable=True, n_wires=k, wires=op_wires)
                else:
                    operation = op(n_wires=k, wires=op_wires)
            elif op().name in ops.parameterized_ops:
                operation = op(has_params=True, trainable=True, wires=op_wires)
            else:
                operation = op(wires=op_wires)
            self.op_list.append(operation)
            op_cnt += 1
            param_cnt += op.num_params
            if self.n_ops is not None and op_cnt == self.n_ops:
                break
            if self.n_ops is None and self.n_params is not None:
                if param_cnt == self.n_params:
                    break
                if param_cnt > self.n_params:  # the last op overshoots: draw another
                    op_cnt -= 1
                    param_cnt -= op.num_params
                    del self.op_list[-1]

    @static_support
    def forward(self, q_device):
        for op in self.op_list:
            op(q_device)


class RandomLayerAllTypes(RandomLayer):
    """``RandomLayer`` over upstream's full default gate list (``random_layers.py:234-298``)."""

    def __init__(self, wires, n_ops=None, n_params=None, op_ratios=None,
                 op_types=(ops.Hadamard, ops.SHadamard, ops.PauliX, ops.PauliY, ops.PauliZ, ops.S, ops.T, ops.SX,
                           ops.CNOT, ops.CZ, ops.CY, ops.RX, ops.RY, ops.RZ, ops.RZZ, ops.SWAP, ops.CSWAP,
                           ops.Toffoli, ops.PhaseShift, ops.Rot, ops.MultiRZ, ops.CRX, ops.CRY, ops.CRZ, ops.CRot,
                           ops.U1, ops.U2, ops.U3, ops.MultiCNOT, ops.MultiXCNOT),
                 seed=None, qiskit_compatible=False):
        super().__init__(wires=wires, n_ops=n_ops, n_params=n_params, op_ratios=op_ratios, op_types=op_types,
                         seed=seed, qiskit_compatible=qiskit_compatible)
