"""QuantumDevice: the statevector container, backed by one engine-owned device buffer.

Mirrors upstream ``torchquantum/device/devices.py:37-136``: same constructor, same
``states`` shape ``[bsz, 2, ..., 2]`` (complex64, |0...0> initially, wire 0 the most
significant bit), ``get_states_1d``, ``set_states``, ``clone_states``,
``reset_states``, ``reset_identity_states``, ``reset_all_eq_states``, op history and
every functional gate bound as a method.  Differences by design:

* the state lives in one contiguous ``[bsz, 2^n]`` buffer updated in place by the
  CUDA kernels (upstream rebuilds a permuted view per gate); with ``checkpoint``
  (``"auto"``: when a backward can follow and memory allows) fused tensor-core blocks
  write to new buffers and keep their inputs for the backward;
* reading ``states`` returns a tensor connected to autograd through
  ``engine.CircuitFunction`` (adjoint-method backward) instead of a per-gate graph;
* CUDA devices only: there is no CPU path.
"""
from __future__ import annotations

from typing import List, Optional, Union

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from . import engine

__all__ = ["QuantumDevice"]


# Engine settings every new QuantumDevice starts with (``set_engine_defaults``).
ENGINE_DEFAULTS = {"method": "plain", "fuse_wires": "auto", "fused_backend": "auto", "stage_low": True,
                   "checkpoint": "auto"}

# "auto" keeps the inputs of a segment's tensor-core blocks when they fit in this share of
# the device memory still available (free plus cached by torch)
CHECKPOINT_MEMORY_SHARE = 0.5


def set_engine_defaults(method: Optional[str] = None, fuse_wires=None, fused_backend: Optional[str] = None,
                        stage_low: Optional[bool] = None, checkpoint=None) -> dict:
    """Set the engine settings of QuantumDevices created from now on -- e.g. the fused
    method for models that build their devices inside ``forward`` -- and return the
    previous defaults (pass them back as keyword arguments to restore them)."""
    prev = dict(ENGINE_DEFAULTS)
    if method is not None:
        if method not in ("plain", "fused"):
            raise ValueError(f"method must be 'plain' or 'fused' (got {method!r})")
        ENGINE_DEFAULTS["method"] = method
    if fuse_wires is not None:
        if fuse_wires != "auto" and not (isinstance(fuse_wires, int) and 1 <= fuse_wires <= 6):
            raise ValueError(f"fuse_wires must be 1..6 or 'auto' (got {fuse_wires!r})")
        ENGINE_DEFAULTS["fuse_wires"] = fuse_wires
    if fused_backend is not None:
        if fused_backend not in ("auto", "tc", "cuda"):
            raise ValueError(f"fused_backend must be 'auto', 'tc' or 'cuda' (got {fused_backend!r})")
        ENGINE_DEFAULTS["fused_backend"] = fused_backend
    if stage_low is not None:
        ENGINE_DEFAULTS["stage_low"] = bool(stage_low)
    if checkpoint is not None:
        if checkpoint not in ("auto", True, False):
            raise ValueError(f"checkpoint must be 'auto', True or False (got {checkpoint!r})")
        ENGINE_DEFAULTS["checkpoint"] = checkpoint
    return prev


# Plain (non-module, non-parameter) attributes of QuantumDevice, written straight into
# the instance dict: nn.Module.__setattr__ costs more than recording a gate on small
# circuits, and `_out` is reset on every gate.
_PLAIN_ATTRS = frozenset({"n_wires", "device_name", "bsz", "device", "record_op", "op_history", "method",
                          "fuse_wires", "fused_backend", "stage_low", "checkpoint", "_tape", "_pending", "_init",
                          "_exported", "_out", "_buf", "_zero_start"})


class QuantumDevice(nn.Module):
    def __setattr__(self, name, value):
        if name in _PLAIN_ATTRS:
            self.__dict__[name] = value
        else:
            super().__setattr__(name, value)

    def __init__(self, n_wires: int, device_name: str = "default", bsz: int = 1,
                 device: Union[torch.device, str] = "cuda", record_op: bool = False):
        super().__init__()
        dev = torch.device(device)
        if dev.type != "cuda":
            raise RuntimeError(
                f"torchquantum_gb300.QuantumDevice runs on CUDA devices only (got device={device!r})")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.n_wires = int(n_wires)
        self.device_name = device_name
        self.bsz = int(bsz)
        self.device = dev
        self.record_op = record_op
        self.op_history: List[dict] = []
        d = ENGINE_DEFAULTS
        self.method = d["method"]                # "plain" | "fused" (see fusion.py)
        self.fuse_wires = d["fuse_wires"]        # fused block width 1..6, or "auto" (autotune.choose_fusion)
        self.fused_backend = d["fused_backend"]  # "auto" | "tc" (tensor cores) | "cuda" (CUDA cores)
        self.stage_low = d["stage_low"]          # plain method: runs of low-qubit gates share one pass
        # fused method: keep each tensor-core block's input state for the backward
        # ("auto": when a backward may follow and the states fit in memory)
        self.checkpoint = d["checkpoint"]
        self._tape: List[engine.TapeOp] = []
        self._pending: List[engine.TapeOp] = []   # fused method: recorded, not yet applied
        self._init: Optional[torch.Tensor] = None
        self._exported = False
        self._out: Optional[torch.Tensor] = None
        self._buf = self._zero_state(self.bsz)
        self._zero_start = True  # the tape starts from |0...0> (no initial state given)

    # ------------------------------------------------------------------ buffers
    def _zero_state(self, bsz: int) -> torch.Tensor:
        s = torch.zeros(bsz, 1 << self.n_wires, dtype=torch.complex64, device=self.device)
        s[:, 0] = 1
        return s

    def _anchor(self, states: Optional[torch.Tensor], bsz: Optional[int] = None):
        """Start a new tape from ``states`` ([bsz, 2^n]) or from |0..0>."""
        self._tape = []
        self._pending = []
        self._out = None
        self._exported = False
        self._zero_start = states is None
        if states is None:
            self._init = None
            self._buf = self._zero_state(bsz if bsz is not None else self.bsz)
        else:
            st = states.reshape(states.shape[0], 1 << self.n_wires)
            if st.device != self.device:
                st = st.to(self.device)
            st = st.to(torch.complex64)
            self._init = st if st.requires_grad else None
            self._buf = st.detach().resolve_conj().resolve_neg().clone().contiguous()
        self.bsz = int(self._buf.shape[0])

    @property
    def state(self) -> torch.Tensor:
        """The |0...0> single state [2]*n (upstream registers it as a buffer)."""
        s = torch.zeros(1 << self.n_wires, dtype=torch.complex64, device=self.device)
        s[0] = 1
        return s.reshape([2] * self.n_wires)

    # ------------------------------------------------------------------ gate path
    def _apply(self, op) -> None:
        """Record a gate (``engine.TapeOp`` or ``program.NativeGate``); it runs at the next read."""
        b = op.batch
        if b and b not in (1, self.bsz):
            raise ValueError(f"gate operand batch {b} does not match QuantumDevice bsz {self.bsz}")
        n = self.n_wires
        seen = set()
        for w in op.wires:  # same checks (and messages) as the kernels' host validation
            if w < 0 or w >= n:
                raise _lib.TQKError(1, f"wire {w} out of range for n_wires={n}")
            if w in seen:
                raise _lib.TQKError(1, f"wire {w} used twice")
            seen.add(w)
        self._pending.append(op)
        self._out = None

    def _flush(self) -> None:
        """Compile the recorded gates into a segment and apply it to the state buffer."""
        if self._pending:
            from . import program

            ops, self._pending = self._pending, []
            if self._exported:  # the buffer is referenced by an exported tensor: copy on write
                self._buf = self._buf.clone()
                self._exported = False
            seg = program.Segment(self, ops, self.method)
            self._buf = seg.apply(self._buf, self._store_block_inputs(seg),
                                  zero_input=self._zero_start and not self._tape)
            self._tape.append(seg)
            self._out = None

    def _store_block_inputs(self, seg) -> bool:
        """Whether ``seg``'s tensor-core blocks keep their input states for the backward."""
        mode = self.checkpoint
        if mode is False or not seg.blocks or not torch.is_grad_enabled():
            return False
        if not any(b.tc for b in seg.blocks):
            return False
        if not (seg.diff_inputs or self._init is not None or any(sg.diff_inputs for sg in self._tape)):
            return False  # no backward will reach this segment
        if mode is True:
            return True
        free, _ = torch.cuda.mem_get_info(self.device)
        cached = torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        return seg.stored_bytes(self._buf) <= CHECKPOINT_MEMORY_SHARE * (free + cached)

    def _output(self) -> torch.Tensor:
        """[bsz, 2^n] state as an autograd-connected tensor (cached until the next gate)."""
        self._flush()
        if self._out is not None:
            return self._out
        sources = [t for sg in self._tape for t in sg.diff_inputs]
        needs = bool(sources) or (self._init is not None and self._init.requires_grad)
        if needs and torch.is_grad_enabled():
            out = engine.CircuitFunction.apply(self._buf, self.n_wires, list(self._tape), self._init, *sources)
        else:
            out = self._buf
        self._exported = True
        self._out = out
        return out

    def reset_wires(self, wires: List[int]) -> None:
        """Project ``wires`` onto |0> and renormalise (functional/reset.py); anchors the tape."""
        from . import _lib

        self._flush()
        cur = self._output().detach().clone()
        _lib.reset(cur, self.n_wires, wires)
        self._anchor(cur)

    # ------------------------------------------------------------------ upstream API
    @property
    def states(self) -> torch.Tensor:
        return self._output().view([self.bsz] + [2] * self.n_wires)

    @states.setter
    def states(self, value: torch.Tensor) -> None:
        self._anchor(value)

    def reset_op_history(self):
        self.op_history = []

    def clone_states(self, existing_states: torch.Tensor):
        self._anchor(existing_states.clone())

    def set_states(self, states: torch.Tensor):
        self._anchor(states)

    def reset_states(self, bsz: int):
        self._anchor(None, bsz)

    def reset_identity_states(self):
        """Batch of 2^n basis states (one per row); useful for unitary extraction."""
        dim = 1 << self.n_wires
        self._anchor(torch.eye(dim, dtype=torch.complex64, device=self.device))

    def reset_all_eq_states(self, bsz: int):
        energy = np.sqrt(1 / (2 ** self.n_wires) / 2)
        s = torch.full((bsz, 1 << self.n_wires), complex(energy, energy), dtype=torch.complex64, device=self.device)
        self._anchor(s)

    def get_states_1d(self) -> torch.Tensor:
        return self._output()

    def get_state_1d(self) -> torch.Tensor:
        return self.state.reshape(1 << self.n_wires)

    @property
    def name(self):
        return self.__class__.__name__

    def __repr__(self):
        return (f" class: {self.name} \n device name: {self.device_name} \n number of qubits: {self.n_wires} \n"
                f" batch size: {self.bsz} \n current computing device: {self.device} \n"
                f" recording op history: {self.record_op} \n method: {self.method}")


def _bind_gate_methods():
    from .functional import func_name_dict, func_name_dict_collect

    for fname, fn in func_name_dict.items():
        setattr(QuantumDevice, fname, fn)
    for fname, fn in func_name_dict_collect.items():
        setattr(QuantumDevice, fname, fn)
