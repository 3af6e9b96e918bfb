"""Measurement (upstream ``torchquantum/measurement/measurements.py``).

``expval_joint_analytical`` (measurements.py:232-279) builds a dense 2^n x 2^n kron
Hamiltonian upstream; here a Pauli string becomes two bit masks and one CUDA pass
over the state evaluates it (``tqk_pauli_expval``), so n = 24..28 work.  Reductions
are float64 with a fixed order.  The backward of an expval is ``2 g P psi``
(``tqk_pauli_apply_sum``), which feeds the circuit's adjoint sweep.

``expval`` / ``MeasureAll`` (measurements.py:282-343) keep upstream semantics: the
observables' diagonalizing gates are applied to the device in place, then each wire's
eigenvalue-weighted marginal is read -- here as a Z-string expectation value,
``e0 P(0) + e1 P(1) = (e0+e1)/2 + (e0-e1)/2 <Z>``.
"""
from __future__ import annotations

from typing import List, Sequence, Union

import torch

from . import _lib
from .engine import kernel_operand
from .module import QuantumModule

__all__ = ["expval_joint_analytical", "expval_joint_analytical_batch", "expval", "MeasureAll", "probs",
           "pauli_masks"]


def pauli_masks(observable: str, n: int):
    """(xmask, zmask) over the in-row index for a Pauli string; P[0] acts on wire 0 (bit n-1)."""
    x = z = 0
    for w, ch in enumerate(observable.upper()):
        bit = 1 << (n - 1 - w)
        if ch == "X":
            x |= bit
        elif ch == "Y":
            x |= bit
            z |= bit
        elif ch == "Z":
            z |= bit
        elif ch != "I":
            raise ValueError(f"invalid Pauli character {ch!r} in {observable!r}")
    return x, z


class PauliExpvalFunction(torch.autograd.Function):
    """[bsz, m] = Re <psi|P_j|psi> for a [bsz, 2^n] complex64 state."""

    @staticmethod
    def forward(ctx, state, n, xmasks, zmasks):
        ctx.n, ctx.x, ctx.z = n, xmasks, zmasks
        ctx.save_for_backward(state)
        return _lib.pauli_expval(kernel_operand(state), n, xmasks, zmasks).to(torch.float32)

    @staticmethod
    def backward(ctx, grad):
        (state,) = ctx.saved_tensors
        coef = (2.0 * grad).to(torch.float32).contiguous()
        g = _lib.pauli_apply_sum(kernel_operand(state), ctx.n, ctx.x, ctx.z, coef)
        return g, None, None, None


def _state_2d(qdev) -> torch.Tensor:
    return qdev.get_states_1d()


def expval_joint_analytical_batch(qdev, observables: Sequence[str]) -> torch.Tensor:
    """Expectation values of several Pauli strings in one pass: [bsz, m] float32."""
    n = qdev.n_wires
    masks = []
    for o in observables:
        assert len(o) == n, f"observable {o!r} must have length n_wires={n}"
        masks.append(pauli_masks(o, n))
    xs = [m[0] for m in masks]
    zs = [m[1] for m in masks]
    return PauliExpvalFunction.apply(_state_2d(qdev), n, xs, zs)


def expval_joint_analytical(qdev, observable: str) -> torch.Tensor:
    """Re <psi| P |psi> per batch row, [bsz] float32 (measurements.py:232-279)."""
    return expval_joint_analytical_batch(qdev, [observable.upper()])[:, 0]


def expval(qdev, wires: Union[int, List[int]], observables) -> torch.Tensor:
    """Per-wire expectation values after in-place basis rotation (measurements.py:282-312)."""
    if isinstance(wires, int):
        wires = [wires]
        observables = [observables]
    for wire, obs in zip(wires, observables):
        for rotation in obs.diagonalizing_gates():
            rotation(qdev, wires=wire)
    n = qdev.n_wires
    strings = ["".join("Z" if w == wire else "I" for w in range(n)) for wire in wires]
    z = expval_joint_analytical_batch(qdev, strings)  # [bsz, len(wires)]
    cols = []
    for j, obs in enumerate(observables):
        ev = obs.eigvals.real.to(z.device, torch.float32)
        cols.append((ev[0] + ev[1]) / 2 + (ev[0] - ev[1]) / 2 * z[:, j])
    return torch.stack(cols, dim=-1)


class MeasureAll(QuantumModule):
    """Expectation value of ``obs`` on every wire (measurements.py:315-343)."""

    def __init__(self, obs, v_c_reg_mapping=None):
        super().__init__()
        self.obs = obs
        self.v_c_reg_mapping = v_c_reg_mapping

    def forward(self, qdev):
        x = expval(qdev, list(range(qdev.n_wires)), [self.obs()] * qdev.n_wires)
        if self.v_c_reg_mapping is not None:
            c2v = self.v_c_reg_mapping["c2v"]
            perm = [c2v[k] for k in range(x.shape[-1]) if k in c2v.keys()]
            x = x[:, perm]
        return x

    def set_v_c_reg_mapping(self, mapping):
        self.v_c_reg_mapping = mapping


def probs(qdev) -> torch.Tensor:
    """|psi|^2 as [bsz, 2^n] float32 (no autograd; use ``get_states_1d().abs()**2`` for gradients)."""
    st = kernel_operand(_state_2d(qdev))
    return _lib.probs(st, qdev.n_wires)
