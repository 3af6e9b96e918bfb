"""Density-matrix device (upstream ``torchquantum/device/noisedevices.py:36-105`` and the
``noisedevice`` branch of ``functional/gate_wrapper.py:434-440``).

A density matrix rho on n wires is held as the 2n-wire vector vec(rho): row (ket)
wire w is vector wire w, column (bra) wire w is vector wire n + w, so the flat index is
row * 2^n + column -- upstream's ``[bsz] + [2] * 2n`` layout.  A gate U on wires W maps
rho -> U rho U^H, i.e. U on wires W and conj(U) on wires W + n of vec(rho): two dense
applications on the plain engine's kernels (``tqk_apply_matrix``), with the engine's
adjoint backward for gradients.

Upstream's bmm branch (``apply_unitary_density_bmm``, gate_wrapper.py:265-321)
multiplies the columns by conj(U) without the transpose, i.e. computes rho conj(U);
that equals rho U^H only for symmetric U (RX, RZ, H, CNOT, CZ, CRX, ...).  This device
computes U rho U^H for every gate.
"""
from __future__ import annotations

from typing import Union

import torch
from torch import nn

from . import functional as tqf
from .device import QuantumDevice

__all__ = ["NoiseDevice"]


class NoiseDevice(nn.Module):
    """``NoiseDevice(n_wires, device_name="noisedevice", bsz=1, device="cuda", record_op=False)``;
    every ``tqf`` gate is bound as a method, as on upstream's NoiseDevice."""

    is_density = True

    def __init__(self, n_wires: int, device_name: str = "noisedevice", bsz: int = 1,
                 device: Union[torch.device, str] = "cuda", record_op: bool = False):
        super().__init__()
        self.n_wires = n_wires
        self.device_name = device_name
        self.bsz = bsz
        self.record_op = record_op
        self.op_history = []
        self._vec = QuantumDevice(2 * n_wires, bsz=bsz, device=device)  # vec(|0><0|) = e_0
        self.device = self._vec.device

    # ------------------------------------------------------------------ gates
    def _apply_matrix(self, matrix: torch.Tensor, wires) -> None:
        """rho -> U rho U^H for U = ``matrix`` ([2^k, 2^k] or [B, 2^k, 2^k]) on ``wires``."""
        m = matrix if matrix.dim() == 3 else matrix.unsqueeze(0)
        m = m.to(self.device)
        if not m.is_complex():
            m = m.to(torch.complex64)
        n = self.n_wires
        self._vec._apply(tqf._op_from_matrix("qubitunitaryfast", m, list(wires), self.device))
        self._vec._apply(tqf._op_from_matrix("qubitunitaryfast", m.conj(), [w + n for w in wires], self.device))

    # ------------------------------------------------------------------ state access
    @property
    def densities(self) -> torch.Tensor:
        """[bsz] + [2] * 2n complex64 (autograd-connected to the gate parameters)."""
        return self._vec.get_states_1d().reshape([self._vec.bsz] + [2] * (2 * self.n_wires))

    @densities.setter
    def densities(self, value: torch.Tensor) -> None:
        self.set_densities(value)

    @property
    def density(self) -> torch.Tensor:
        """|0..0><0..0| as [2] * 2n (upstream's registered buffer)."""
        d = torch.zeros(1 << (2 * self.n_wires), dtype=torch.complex64, device=self.device)
        d[0] = 1
        return d.reshape([2] * (2 * self.n_wires))

    def set_densities(self, rho: torch.Tensor) -> None:
        """Start from ``rho`` ([bsz, 2^n, 2^n] or [bsz] + [2] * 2n)."""
        self._vec.set_states(rho.reshape(rho.shape[0], -1))
        self.bsz = self._vec.bsz

    def reset_states(self, bsz: int) -> None:
        self._vec.reset_states(bsz)
        self.bsz = bsz

    def get_densities_2d(self) -> torch.Tensor:
        d = 1 << self.n_wires
        return self._vec.get_states_1d().reshape(-1, d, d)

    def get_probs_1d(self) -> torch.Tensor:
        """Diagonal of every rho, [bsz, 2^n] (upstream returns it complex; so does this)."""
        return torch.diagonal(self.get_densities_2d(), offset=0, dim1=1, dim2=2)

    def get_prob_1d(self) -> torch.Tensor:
        return self.get_probs_1d()[0]

    @property
    def name(self):
        return self.__class__.__name__

    def __repr__(self):
        return (f" class: {self.name} \n device name: {self.device_name} \n number of qubits: {self.n_wires} \n"
                f" batch size: {self.bsz} \n current computing device: {self.device} \n"
                f" recording op history: {self.record_op}")


def _bind():
    for name, fn in tqf.func_name_dict.items():
        setattr(NoiseDevice, name, fn)


_bind()
