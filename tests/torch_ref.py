"""complex128 statevector reference on the GPU with plain torch ops (test infrastructure).

Used where the CPU oracle is too slow (n = 26..28): the same algorithm as the oracle's
``apply`` (gate_wrapper.py:96-140 upstream: move the gate's wire axes to the front,
multiply, move them back), in float64 complex arithmetic with torch's own CUDA kernels,
independent of the engine's kernels.  Gate matrices come from the oracle."""
from __future__ import annotations

from typing import Dict, List

import numpy as np
import torch

from oracle import statevec as O


def apply(state: torch.Tensor, mat: torch.Tensor, wires: List[int], n: int) -> torch.Tensor:
    """state [bsz, 2^n] complex128; mat [B, 2^k, 2^k] with B in {1, bsz}."""
    bsz = state.shape[0]
    k = len(wires)
    s = state.view([bsz] + [2] * n)
    perm = [0] + [1 + w for w in wires] + [1 + w for w in range(n) if w not in wires]
    s = s.permute(perm).reshape(bsz, 1 << k, -1)
    m = mat if mat.shape[0] == bsz else mat.expand(bsz, -1, -1)
    s = torch.bmm(m, s)
    inv = [0] * (n + 1)
    for i, p in enumerate(perm):
        inv[p] = i
    return s.view([bsz] + [2] * n).permute(inv).reshape(bsz, 1 << n).contiguous()


def run(n: int, bsz: int, gates: List[Dict], device) -> torch.Tensor:
    """|0..0> through oracle-format gate dicts ({name, wires, params [B, P] or None})."""
    st = torch.zeros(bsz, 1 << n, dtype=torch.complex128, device=device)
    st[:, 0] = 1
    for g in gates:
        m = O.gate_matrix(g["name"], g["params"])
        st = apply(st, torch.as_tensor(np.asarray(m), dtype=torch.complex128, device=device), g["wires"], n)
    return st


def expval_pauli(state: torch.Tensor, pauli: str, n: int) -> torch.Tensor:
    """<psi|P|psi> per row (float64) via masks: (P psi)_i = i^nY (-1)^popcount((i^x)&z) psi_{i^x}."""
    x, z, ny = O.pauli_masks(pauli, n)
    idx = torch.arange(1 << n, device=state.device, dtype=torch.int64)
    src = idx ^ x
    v = src & z
    par = torch.zeros_like(v)
    while True:  # parity by folding
        nz = v != 0
        if not bool(nz.any()):
            break
        par ^= v & 1
        v = v >> 1
    ph = (1j ** ny) * (1 - 2 * par.to(torch.float64))
    p_psi = ph.to(torch.complex128) * state[:, src]
    return (state.conj() * p_psi).sum(dim=1).real
