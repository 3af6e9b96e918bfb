"""Functional gates (``tqf``): the drop-in for ``torchquantum.functional``.

``gate_wrapper`` keeps the upstream signature and behaviour
(``torchquantum/functional/gate_wrapper.py:324-446``): parameter normalisation
(:361-378), op-history recording (:380-391), static-mode deferral (:393-403),
matrix construction (:406-425), inverse as conjugate transpose (:427-432) and the
wire-count assertion (:433).  Where upstream then calls ``apply_unitary_bmm``
(:441-446), this version hands a structured ``TapeOp`` to the CUDA engine: dense
1/2-wire matrices, controlled blocks, multi-controlled X, phases, diagonals and swaps
each have their own kernel.  ``comp_method`` ("bmm" / "einsum") is accepted and
ignored: both upstream methods compute the same product.

Every gate of upstream ``func_name_dict`` (``functional/__init__.py:125-218``) is
provided under the same name, plus ``func_name_dict_collect`` (``matrix_exp``,
``controlled_unitary``).
"""
from __future__ import annotations

import math
from typing import Callable, Optional

import numpy as np
import torch

from . import engine
from . import gates as G
from . import program

__all__ = ["gate_wrapper", "func_name_dict", "func_name_dict_collect", "mat_dict", "apply_unitary_bmm",
           "apply_unitary_einsum"]

_QU = ("qubitunitary", "qubitunitaryfast", "qubitunitarystrict")
# operands that are not unitary by construction: upstream's cu2 block has no 1/sqrt(2)
# (functional/u2.py), and qubitunitaryfast does not check its matrix
_MAYBE_NON_UNITARY = ("cu2", "qubitunitaryfast")
_VAR_WIRES_NOPARAM = ("multicnot", "multixcnot", "qft")


def _normalize_params(name: str, params):
    """gate_wrapper.py:361-378."""
    if params is None:
        return None
    if not isinstance(params, torch.Tensor):
        if name in _QU:
            params = torch.tensor(np.asarray(params), dtype=torch.complex64)
        else:
            params = torch.tensor(params, dtype=torch.float32)
    if name in _QU:
        params = params.unsqueeze(0) if params.dim() == 2 else params
    else:
        if params.dim() == 1:
            params = params.unsqueeze(-1)
        elif params.dim() == 0:
            params = params.unsqueeze(-1).unsqueeze(-1)
    return params


def _record(q_device, name, wires, params, inverse):
    q_device.op_history.append({
        "name": name,
        "wires": np.array(wires).squeeze().tolist(),
        "params": params.squeeze().detach().cpu().numpy().tolist() if params is not None else None,
        "inverse": inverse,
        "trainable": params.requires_grad if params is not None else False,
    })


def _op_from_matrix(name: str, matrix: torch.Tensor, wires, device) -> engine.TapeOp:
    """Turn the (batched) gate matrix into the engine op for the gate's structure.

    ``source`` keeps the operand at the matrix's own precision (complex128 when built
    for the fused method) and autograd-tracked; ``operand`` is the complex64 copy the
    plain kernels read."""
    if matrix.dim() == 2:
        matrix = matrix.unsqueeze(0)
    if matrix.device != device:
        matrix = matrix.to(device)
    if not matrix.is_complex():
        matrix = matrix.to(torch.complex64)
    gd = G.GATES.get(name)
    struct = gd.struct if gd is not None else ("dense",)
    kind = struct[0]
    k = len(wires)

    def mk(op_kind, src, **kw):
        kop = engine.kernel_operand(src.to(torch.complex64))
        if name in _MAYBE_NON_UNITARY and op_kind in (engine.KIND_DENSE, engine.KIND_CTRL):
            kw["uncompute"] = engine.kernel_operand(torch.linalg.inv(kop))
        return engine.TapeOp(op_kind, wires, operand=kop, source=src, **kw)

    if kind == "x":
        nc = struct[1] if struct[1] >= 0 else k - 1
        return engine.TapeOp(engine.KIND_X, wires, controls=wires[:nc], targets=wires[nc:], ctrl_val=struct[2])
    if kind == "swap":
        nc = struct[1]
        return engine.TapeOp(engine.KIND_SWAP, wires, controls=wires[:nc], targets=wires[nc:])
    if kind == "phase":
        return mk(engine.KIND_PHASE, matrix[:, -1, -1])
    if kind == "diag" and k <= 4:
        return mk(engine.KIND_DIAG, torch.diagonal(matrix, dim1=-2, dim2=-1))
    if kind == "ctrl":
        nc = struct[1]
        return mk(engine.KIND_CTRL, matrix[:, -2:, -2:], controls=wires[:nc], targets=wires[nc:])
    return mk(engine.KIND_DENSE, matrix)


_STRUCT_NCTRL = {"dense": 0, "diag": 0, "phase": 0}


def _native_record(cname, wires, params, inverse, q_device):
    """A NativeGate for a supported parameterised gate (operand built on the GPU)."""
    gd = G.GATES[cname]
    ntype, npar = program.NATIVE[cname]
    if params.dim() != 2 or params.shape[1] != npar or len(wires) != gd.num_wires:
        return None
    if params.device != q_device.device:
        params = params.to(q_device.device)
    if params.dtype not in (torch.float32, torch.float64):
        params = params.to(torch.float32)
    kind_name = gd.struct[0]
    kind = {"dense": engine.KIND_DENSE, "ctrl": engine.KIND_CTRL, "diag": engine.KIND_DIAG,
            "phase": engine.KIND_PHASE}[kind_name]
    nctrl = gd.struct[1] if kind_name == "ctrl" else 0
    return program.NativeGate(cname, wires, params, inverse, kind, nctrl)


# parameter-free gates: the engine op is built once per (gate, width, inverse, method,
# device) and reused with the call's wires (no per-call matrix work or copies)
_CONST_NAMES = frozenset(n for n, g in G.GATES.items()
                         if g.num_params == 0 and g.builder is None and n not in _QU and n != "globalphase")
_CONST_OPS: dict = {}


def _const_op(cname, k, wires, inverse, fused, device) -> engine.TapeOp:
    key = (cname, k, bool(inverse), bool(fused), str(device))
    tpl = _CONST_OPS.get(key)
    if tpl is None:
        matrix = G.gate_matrix(cname, None, k, dtype=torch.complex128 if fused else torch.complex64, device=device)
        if inverse:
            matrix = matrix.conj().permute(0, 2, 1)
        assert int(round(math.log2(matrix.shape[-1]))) == len(wires), f"{cname}: matrix on wires {wires}"
        tpl = _op_from_matrix(cname, matrix, list(range(len(wires))), device)
        _CONST_OPS[key] = tpl
    op = engine.TapeOp(tpl.kind, wires, controls=[wires[i] for i in tpl.controls],
                       targets=[wires[i] for i in tpl.targets], ctrl_val=tpl.ctrl_val, operand=tpl.operand,
                       source=tpl.source, uncompute=tpl.uncompute)
    return op


def gate_wrapper(name, mat, method, q_device, wires, params=None, n_wires=None, static=False, parent_graph=None,
                 inverse=False):
    """Apply gate ``name`` to ``q_device`` (upstream gate_wrapper.py:324-446)."""
    params = _normalize_params(name, params)
    wires = [wires] if isinstance(wires, int) else [int(w) for w in wires]
    fused = getattr(q_device, "method", "plain") == "fused"
    if q_device.record_op:
        _record(q_device, name, wires, params, inverse)
    if static and parent_graph is not None and hasattr(parent_graph, "add_func"):
        # a caller-provided graph object collects the op (gate_wrapper.py:393-403); without
        # one, static mode is the device's fused method (module.static_support)
        parent_graph.add_func(name=name, wires=wires, parent_graph=parent_graph, params=params, n_wires=n_wires,
                              inverse=inverse)
        return
    cname = G.canonical_name(name)
    density = getattr(q_device, "is_density", False)
    if mat is None and params is None and not density and cname in _CONST_NAMES:
        q_device._apply(_const_op(cname, n_wires if n_wires is not None else len(wires), wires, inverse, fused,
                                  q_device.device))
        return
    if mat is None and cname in program.NATIVE and isinstance(params, torch.Tensor) and not params.is_complex() \
            and not density:
        nat = _native_record(cname, wires, params, inverse, q_device)
        if nat is not None:
            q_device._apply(nat)
            return
    if isinstance(mat, Callable):
        # upstream calling convention of the builder (gate_wrapper.py:406-423)
        if n_wires is None or name in _QU:
            matrix = mat(params)
        elif name in _VAR_WIRES_NOPARAM:
            matrix = mat(n_wires)
        elif name == "multirz":
            matrix = mat(params, n_wires)
        else:
            matrix = mat(params)
    elif mat is None:
        if fused and params is not None and params.is_floating_point() and not params.is_complex():
            params = params.to(torch.float64)  # fused blocks are built in complex128
        matrix = G.gate_matrix(cname, params, n_wires if n_wires is not None else len(wires),
                               dtype=torch.complex128 if fused else torch.complex64, device=q_device.device)
    else:
        matrix = mat
    if inverse:
        matrix = matrix.conj()
        matrix = matrix.permute(0, 2, 1) if matrix.dim() == 3 else matrix.permute(1, 0)
    dim = matrix.shape[-1]
    assert int(round(math.log2(dim))) == len(wires), f"{name}: matrix of dim {dim} on wires {wires}"
    if density:  # rho -> U rho U^H (density.NoiseDevice; a global phase cancels)
        if len(wires):
            q_device._apply_matrix(matrix, wires)
        return
    if len(wires) == 0:  # globalphase: a phase on every amplitude
        ph = matrix.reshape(-1).to(q_device.device)
        q_device._apply(engine.TapeOp(engine.KIND_PHASE, [], operand=engine.kernel_operand(ph.to(torch.complex64)),
                                      source=ph))
        return
    q_device._apply(_op_from_matrix(cname if mat is None or isinstance(mat, Callable) else "qubitunitaryfast",
                                    matrix, wires, q_device.device))


class _Builder:
    """Upstream-style matrix builder callable for ``mat_dict`` (params -> matrix)."""

    def __init__(self, name):
        self.name = name

    def __call__(self, params=None, n_wires=None):
        g = G.GATES[self.name]
        if g.num_params == 0 and self.name in _VAR_WIRES_NOPARAM:
            return G.gate_matrix(self.name, None, params if n_wires is None else n_wires)
        if g.num_params == 0:
            return G.gate_matrix(self.name, None, g.num_wires).squeeze(0)
        p = _normalize_params(self.name, params)
        if self.name == "multirz":
            return G.gate_matrix(self.name, p, n_wires).squeeze(0)
        return G.gate_matrix(self.name, p, g.num_wires).squeeze(0)


mat_dict = {name: _Builder(name) for name in G.GATES}
for _a, _t in G.ALIASES.items():
    mat_dict.setdefault(_a, mat_dict[_t])
# upstream's per-gate builder names (functional/rx.py rx_matrix, u3.py u3_matrix, ...)
for _n, _b in list(mat_dict.items()):
    globals().setdefault(f"{_n}_matrix", _b)


def _make_gate(name: str):
    cname = G.canonical_name(name)

    def gate(q_device, wires, params=None, n_wires=None, static=False, parent_graph=None, inverse=False,
             comp_method="bmm"):
        gate_wrapper(name=cname, mat=None, method=comp_method, q_device=q_device, wires=wires, params=params,
                     n_wires=n_wires, static=static, parent_graph=parent_graph, inverse=inverse)

    gate.__name__ = name
    gate.__qualname__ = name
    gate.__doc__ = f"Apply the ``{cname}`` gate (upstream torchquantum.functional.{name})."
    return gate


def reset(q_device, wires, inverse=False):
    """Project ``wires`` onto |0> and renormalise each row (upstream functional/reset.py)."""
    wires = [wires] if isinstance(wires, int) else list(wires)
    q_device.reset_wires(wires)


_NAMES = list(G.GATES.keys()) + list(G.ALIASES.keys())
func_name_dict = {n: _make_gate(n) for n in _NAMES}
func_name_dict["reset"] = reset
globals().update(func_name_dict)


def matrix_exp(qdev, wires, params, n_wires=None, inverse=False, comp_method="bmm"):
    """Apply exp(params) as a dense gate (upstream functional/func_mat_exp.py:34-72)."""
    if isinstance(params, np.ndarray):
        params = torch.from_numpy(params)
    gate_wrapper(name="qubitunitaryfast", mat=None, method=comp_method, q_device=qdev, wires=wires,
                 params=torch.matrix_exp(params), inverse=inverse)


def controlled_unitary(qdev, c_wires, t_wires, params):
    """Controlled version of ``params`` (upstream functional/func_controlled_unitary.py:31-133):
    identity unless every control wire is 1; several target sets get the Kronecker
    power of the unitary."""
    if isinstance(params, np.ndarray):
        params = torch.from_numpy(params)
    c = np.array(c_wires)
    t = np.array(t_wires)
    u = params
    u_wires = int(np.log2(u.shape[-1]))
    wires = [int(c.item())] if c.ndim == 0 else [int(w) for w in c]
    if t.ndim == 0:
        twires = [int(t.item())]
    else:
        twires = [int(w) for w in t.flatten()]
    n_sets = max(1, len(twires) // u_wires)
    cu = u
    for _ in range(n_sets - 1):
        cu = torch.kron(cu, u)
    all_wires = wires + twires
    dim = 1 << len(all_wires)
    full = torch.eye(dim, dtype=torch.complex64)
    d = cu.shape[-1]
    full[-d:, -d:] = cu.to(torch.complex64)
    gate_wrapper(name="qubitunitaryfast", mat=full.to(qdev.device), method="bmm", q_device=qdev, wires=all_wires,
                 n_wires=len(all_wires))


func_name_dict_collect = {"matrix_exp": matrix_exp, "controlled_unitary": controlled_unitary}


def apply_unitary_bmm(state, mat, wires):
    """Out-of-place ``U psi`` on a ``[bsz, 2, ..., 2]`` state (upstream gate_wrapper.py:96-140),
    computed by the engine's dense kernel on a copy.  Differentiable w.r.t. ``state``
    and ``mat`` through the adjoint Function."""
    from .device import QuantumDevice

    wires = [wires] if isinstance(wires, int) else list(wires)
    n = state.dim() - 1
    q = QuantumDevice(n_wires=n, bsz=state.shape[0], device=state.device)
    q.set_states(state)
    q._apply(_op_from_matrix("qubitunitaryfast", mat, wires, q.device))
    return q.states


apply_unitary_einsum = apply_unitary_bmm
