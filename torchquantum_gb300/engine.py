"""Gate tape and the adjoint-method autograd Function.

A ``QuantumDevice`` owns one contiguous ``[bsz, 2^n]`` complex64 device buffer and a
tape of ``TapeOp`` records.  Gates are applied to the buffer in place by the CUDA
kernels of ``libtqk.so`` as they are called (the plain method).  Nothing per gate is
kept for autograd except the small gate operand (a 2x2 / 4x4 matrix, a phase or a
diagonal); when the state is read by a measurement, ``CircuitFunction`` exposes it
to torch autograd as a function of every operand that requires grad.  Its backward
is the adjoint method: starting from the final state psi and the incoming cotangent
lam it walks the tape in reverse, uncomputing psi <- U^H psi and lam <- U^H lam and
accumulating each operand's cotangent ``sum lam_after conj(psi_before)^T`` in float64
-- two state buffers instead of one saved state per gate.  Fused tensor-core blocks
may instead keep their input states (the forward writes each block's output to a new
buffer, when memory allows): their reverse steps then read the stored input and only
update lam.  Torch autograd then
carries the operand cotangents through the differentiable matrix builders
(``gates.py``) to the gate parameters.

Replaces the per-gate ``torch.bmm``/``permute`` graph that upstream
``apply_unitary_bmm`` records (``torchquantum/functional/gate_wrapper.py:96-140``).
"""
from __future__ import annotations

from typing import List, Optional

import torch

from . import _lib

KIND_DENSE, KIND_CTRL, KIND_X, KIND_PHASE, KIND_DIAG, KIND_SWAP = "dense", "ctrl", "x", "phase", "diag", "swap"


class TapeOp:
    """One applied gate.

    ``operand`` is the detached complex64 tensor the kernel reads (``[B, D, D]``
    matrix, ``[B]`` phase or ``[B, 2^k]`` diagonal, ``B`` in {1, bsz});
    ``source`` is the autograd-tracked tensor it was taken from (or None).
    """

    def __init__(self, kind, wires, controls=(), targets=(), ctrl_val=1, operand=None, source=None, uncompute=None):
        self.kind = kind
        self.wires = list(wires)
        self.controls = list(controls)
        self.targets = list(targets)
        self.ctrl_val = int(ctrl_val)
        self.operand = operand
        self.source = source
        self.batch = 0 if operand is None else int(operand.shape[0])
        # exact inverse of a dense/controlled operand that is not unitary (psi is uncomputed
        # with it; the cotangent still propagates with U^H)
        self.uncompute = uncompute
        # tensor-core operand image of a fused 6-wire block (forward uses the tcgen05 kernel)
        self.image = None

    @property
    def needs_grad(self) -> bool:
        return self.source is not None and self.source.requires_grad

    def grad_numel(self) -> int:
        """float64 values of this op's operand cotangent (complex128 interleaved)."""
        if self.operand is None:
            return 0
        return 2 * self.operand.numel()

    def __repr__(self):
        return f"TapeOp({self.kind}, wires={self.wires}, batch={self.batch})"


def kernel_operand(t: torch.Tensor) -> torch.Tensor:
    """Detached, materialised (no lazy conj/neg bit), contiguous copy-or-view for a kernel.

    ``Tensor.conj()`` only sets a conjugation bit; ``contiguous()`` keeps that bit on an
    already-contiguous view, so the raw pointer would still address unconjugated data.
    """
    return t.detach().resolve_conj().resolve_neg().contiguous()


class StateCursor:
    """The state a reverse sweep has reached, carried from segment to segment.  It starts
    as the saved final state and, after a block whose input the forward kept, is that
    stored input: both are only read.  The sweep uncomputes in place only on its work
    buffer (one state, allocated the first time a segment needs it): the segment runner
    (``tqk_segment_backward``) copies the state there before the first such step."""

    def __init__(self, state: torch.Tensor):
        self.state = state
        self.owned = False  # state is the work buffer
        self.work = None

    def work_buffer(self) -> torch.Tensor:
        if self.work is None:
            self.work = torch.empty_like(self.state)
        return self.work


class CircuitFunction(torch.autograd.Function):
    """final_state = circuit(init_state, differentiable inputs...) with an adjoint backward.

    ``segments`` are the compiled gate runs (``program.Segment``) applied since the
    state was anchored; forward receives the already-computed final state (the device
    buffer) and returns it.  Inputs after ``init`` are every segment's
    ``diff_inputs`` in order (parameter base tensors, generic operand sources).
    backward walks the segments in reverse, each returning its inputs' gradients.
    """

    @staticmethod
    def forward(ctx, final: torch.Tensor, n: int, segments: list, init: Optional[torch.Tensor], *inputs):
        ctx.n = n
        ctx.segments = segments
        ctx.counts = [len(sg.diff_inputs) for sg in segments]
        ctx.has_init = init is not None
        # the blocks' stored input states become saved tensors of this node (the segments
        # keep weak references), so torch releases them when a backward that does not
        # retain the graph has run, as it does for its own saved tensors
        stored = [pair for sg in segments for pair in sg.take_stored_inputs()]
        ctx.stored_ops = [op for op, _ in stored]
        ctx.save_for_backward(final, *[t for _, t in stored])
        return final

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        final, *stored = ctx.saved_tensors
        inputs = {id(op): t for op, t in zip(ctx.stored_ops, stored)}
        psi = StateCursor(final.detach())
        lam = kernel_operand(grad_out.to(torch.complex64)).clone()
        per_seg = []
        for sg, cnt in zip(reversed(ctx.segments), reversed(ctx.counts)):
            per_seg.append(sg.backward(psi, lam, cnt > 0, inputs))
        grads = [g for gl in reversed(per_seg) for g in gl]
        g_init = lam if ctx.has_init else None
        return (None, None, None, g_init, *grads)
