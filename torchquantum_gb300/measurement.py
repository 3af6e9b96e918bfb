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

``MeasureMultipleTimes`` / ``MeasureMultiPauliSum`` / ``MeasureMultiQubitPauliSum``
(measurements.py:346-456) measure a copy of the state per layer of per-wire
observables; Pauli layers become single-site strings evaluated in one fused pass.

``measure`` (measurements.py:37-74) samples bitstrings on the GPU (``tqk_sample``:
inverse-CDF draws against device-side prefix sums) instead of copying |psi|^2 to the
host for ``random.choices``.
"""
from __future__ import annotations

from collections import OrderedDict
from typing import Dict, List, Optional, Sequence, Union

import numpy as np
import torch

from . import _lib
from .engine import kernel_operand
from .module import QuantumModule

__all__ = ["expval_joint_analytical", "expval_joint_analytical_batch", "expval", "MeasureAll", "probs",
           "pauli_masks", "measure", "gen_bitstrings", "MeasureMultipleTimes", "MeasureMultiPauliSum",
           "MeasureMultiQubitPauliSum", "find_observable_groups", "expval_joint_sampling",
           "expval_joint_sampling_grouping"]


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
    evs = tuple(tuple(complex(v).real for v in obs.eigvals.reshape(-1).tolist()) for obs in observables)
    if all(e == (1.0, -1.0) for e in evs):  # Pauli eigenvalues: the Z-string values themselves
        return z
    key = (evs, str(z.device))
    ab = _EIG_CACHE.get(key)
    if ab is None:
        ab = torch.tensor([[(e0 + e1) / 2 for e0, e1 in evs], [(e0 - e1) / 2 for e0, e1 in evs]],
                          dtype=torch.float32, device=z.device)
        _EIG_CACHE[key] = ab
    return ab[0] + ab[1] * z


_EIG_CACHE: dict = {}


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


# ------------------------------------------------------------------ sampling
def gen_bitstrings(n_wires: int) -> List[str]:
    """All n-bit strings, qubit 0 first (measurements.py:33-34)."""
    return ["{:0{}b}".format(k, n_wires) for k in range(2 ** n_wires)]


FULL_DICT_MAX_WIRES = 20


def measure(qdev, n_shots: int = 1024, draw_id: Optional[int] = None, generator: Optional[torch.Generator] = None):
    """Sample ``n_shots`` bitstrings per batch row (measurements.py:37-74): a list of
    OrderedDicts bitstring -> count, sorted by bitstring, qubit 0 first.  Up to
    ``FULL_DICT_MAX_WIRES`` wires every bitstring is a key (zero counts included, as
    upstream); above that only observed bitstrings are (upstream would build 2^n keys).
    ``generator``: a CUDA torch.Generator for reproducible draws.  ``draw_id`` plots
    that row's histogram when matplotlib is installed."""
    n = qdev.n_wires
    if getattr(qdev, "is_density", False):  # sample the diagonal of rho (measurements.py:51-55)
        p = qdev.get_probs_1d().detach().real.clamp_min(0)
        st = torch.sqrt(p).to(torch.complex64).contiguous()
    else:
        st = kernel_operand(_state_2d(qdev))
    bsz = st.shape[0]
    u = torch.rand(bsz, int(n_shots), dtype=torch.float64, device=st.device, generator=generator)
    idx = _lib.sample(st, n, u)
    out = []
    if n <= FULL_DICT_MAX_WIRES:
        flat = idx + (torch.arange(bsz, device=idx.device, dtype=torch.int64) << n)[:, None]
        counts = torch.bincount(flat.reshape(-1), minlength=bsz << n).view(bsz, 1 << n).cpu().numpy()
        keys = gen_bitstrings(n)
        for b in range(bsz):
            out.append(OrderedDict(zip(keys, counts[b].tolist())))
    else:
        for b in range(bsz):
            vals, cnt = torch.unique(idx[b], return_counts=True)
            out.append(OrderedDict(("{:0{}b}".format(int(v), n), int(c)) for v, c in
                                   zip(vals.cpu().tolist(), cnt.cpu().tolist())))
    if draw_id is not None:
        try:
            import matplotlib.pyplot as plt
        except ImportError:
            plt = None
        if plt is not None:
            plt.bar(out[draw_id].keys(), out[draw_id].values())
            plt.xticks(rotation="vertical")
            plt.xlabel("bitstring [qubit0, qubit1, ..., qubitN]")
            plt.title("distribution of measured bitstrings")
            plt.show()
    return out


# ------------------------------------------------------------------ sampled expectation values
def find_observable_groups(observables: Sequence[str]) -> Dict[str, List[str]]:
    """Group Pauli strings that one measurement basis serves (measurements.py:77-111):
    each string joins the first group, in insertion order, whose basis agrees with it on
    every non-identity site (the group's identity sites take the string's Pauli); the
    grown group moves to the end of the dict.  Otherwise it starts a new group."""
    groups: Dict[str, List[str]] = {}
    for ob in observables:
        hit = None
        for g in groups:
            grown = list(g)
            ok = True
            for k, ch in enumerate(ob):
                if ch == "I" or ch == g[k]:
                    continue
                if g[k] == "I":
                    grown[k] = ch
                    continue
                ok = False
                break
            if ok:
                hit = (g, "".join(grown))
                break
        if hit is None:
            groups[ob] = [ob]
        else:
            members = groups.pop(hit[0])
            members.append(ob)
            groups[hit[1]] = members
    return groups


def _parity64(v: torch.Tensor) -> torch.Tensor:
    for sh in (32, 16, 8, 4, 2, 1):
        v = v ^ (v >> sh)
    return v & 1


def _rotated_samples(qdev, basis: str, n_shots: int, generator=None) -> torch.Tensor:
    """Outcome indices [bsz, n_shots] after rotating a copy of the state into ``basis``."""
    from .device import QuantumDevice
    from .operators import op_name_dict

    n = qdev.n_wires
    qc = QuantumDevice(n_wires=n, bsz=qdev.bsz, device=qdev.device)
    qc.set_states(qdev.get_states_1d().detach())
    names = {"X": "paulix", "Y": "pauliy", "Z": "pauliz", "I": "i"}
    for w, ch in enumerate(basis):
        for rot in op_name_dict[names[ch]]().diagonalizing_gates():
            rot(qc, wires=w)
    st = kernel_operand(_state_2d(qc))
    u = torch.rand(st.shape[0], int(n_shots), dtype=torch.float64, device=st.device, generator=generator)
    return _lib.sample(st, n, u)


def _sampled_expval(idx: torch.Tensor, observable: str, n: int) -> torch.Tensor:
    mask = 0
    for w, ch in enumerate(observable):
        if ch != "I":
            mask |= 1 << (n - 1 - w)
    par = _parity64(idx & mask)
    return (1.0 - 2.0 * par.to(torch.float64)).mean(dim=1).to(torch.float32)


def expval_joint_sampling(qdev, observable: str, n_shots: int = 1024, generator=None) -> torch.Tensor:
    """<P> estimated from ``n_shots`` basis-rotated samples per row (measurements.py:169-229),
    [bsz] float32: the share of shots with even parity on the non-identity sites minus the
    share with odd parity, counted on the GPU."""
    observable = observable.upper()
    idx = _rotated_samples(qdev, observable, n_shots, generator)
    return _sampled_expval(idx, observable, qdev.n_wires)


def expval_joint_sampling_grouping(qdev, observables: Sequence[str], n_shots_per_group: int = 1024,
                                   generator=None) -> Dict[str, torch.Tensor]:
    """Sampled <P> for several strings, one set of shots per group of
    ``find_observable_groups`` (measurements.py:114-166): {string: [bsz] float32}."""
    assert len(observables) == len(set(observables)), "each observable should be unique"
    obs = [o.upper() for o in observables]
    out = {}
    for basis, members in find_observable_groups(obs).items():
        idx = _rotated_samples(qdev, basis, n_shots_per_group, generator)
        for ob in members:
            out[ob] = _sampled_expval(idx, ob, qdev.n_wires)
    return out


# ------------------------------------------------------------------ multi-observable layers
_PAULI_CHAR = {"x": "X", "paulix": "X", "y": "Y", "pauliy": "Y", "z": "Z", "pauliz": "Z", "i": "I"}


class MeasureMultipleTimes(QuantumModule):
    """Per layer ``{'wires': [...], 'observables': [...]}``: each wire's expectation value
    of its observable (identity on unlisted wires) on a copy of the state; layers
    concatenated along the batch dimension, [layers * bsz, n_wires]
    (measurements.py:346-400)."""

    def __init__(self, obs_list, v_c_reg_mapping=None):
        super().__init__()
        self.obs_list = obs_list
        self.v_c_reg_mapping = v_c_reg_mapping

    def forward(self, qdev):
        from .device import QuantumDevice
        from .operators import op_name_dict

        n = qdev.n_wires
        res_all = []
        for layer in self.obs_list:
            names = ["i"] * n
            for wire, ob in zip(layer["wires"], layer["observables"]):
                names[wire] = ob.lower()
            if all(nm in _PAULI_CHAR for nm in names):
                # single-site Pauli strings, one fused pass per distinct X pattern
                strings = ["".join(_PAULI_CHAR[nm] if w == j else "I" for j in range(n)) for w, nm in enumerate(names)]
                res = expval_joint_analytical_batch(qdev, strings)
            else:
                qnew = QuantumDevice(n_wires=n, bsz=qdev.bsz, device=qdev.device)
                qnew.set_states(qdev.get_states_1d())
                res = expval(qnew, list(range(n)), [op_name_dict[nm]() for nm in names])
            if self.v_c_reg_mapping is not None:
                c2v = self.v_c_reg_mapping["c2v"]
                perm = [c2v[k] for k in range(res.shape[-1]) if k in c2v.keys()]
                res = res[:, perm]
            res_all.append(res)
        return torch.cat(res_all)

    def set_v_c_reg_mapping(self, mapping):
        self.v_c_reg_mapping = mapping


class MeasureMultiPauliSum(QuantumModule):
    """Sum over wires of ``MeasureMultipleTimes`` (measurements.py:403-432; upstream does
    not apply the coefficients here, and neither does this)."""

    def __init__(self, obs_list, v_c_reg_mapping=None):
        super().__init__()
        self.obs_list = obs_list
        self.v_c_reg_mapping = v_c_reg_mapping
        self.measure_multiple_times = MeasureMultipleTimes(obs_list=obs_list, v_c_reg_mapping=v_c_reg_mapping)

    def forward(self, qdev):
        return self.measure_multiple_times(qdev).sum(-1)


class MeasureMultiQubitPauliSum(QuantumModule):
    """``obs_list[0]['coefficient']`` times ``MeasureMultipleTimes(obs_list[1:])``, summed
    over the last dimension (measurements.py:435-456)."""

    def __init__(self, obs_list, v_c_reg_mapping=None):
        super().__init__()
        self.obs_list = obs_list
        self.v_c_reg_mapping = v_c_reg_mapping
        self.measure_multiple_times = MeasureMultipleTimes(obs_list=obs_list[1:], v_c_reg_mapping=v_c_reg_mapping)

    def forward(self, qdev):
        res_all = self.measure_multiple_times(qdev)
        coef = torch.as_tensor(self.obs_list[0]["coefficient"], dtype=res_all.dtype, device=res_all.device)
        return (res_all * coef).sum(-1)
