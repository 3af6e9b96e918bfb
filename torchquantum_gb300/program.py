"""Gate programs: how a recorded sequence of gates becomes GPU work.

Gates are recorded cheaply by ``gate_wrapper`` and compiled into a ``Segment`` when
the state is read:

* every parameterised gate of a supported type (``NATIVE``) gets its operand built
  on the GPU by one ``tqk_gate_operands`` launch for the whole segment, reading its
  parameters in place through their strides (no per-gate torch ops);
* the plain method then applies each op with its kernel; the fused method plans
  blocks of up to 6 wires (``fusion.plan_blocks``; width, planner variant and kernel
  per block chosen by ``autotune.choose_fusion`` from measured pass costs when
  ``fuse_wires == "auto"``), builds every block unitary in float64 with one
  ``tqk_block_build`` launch, and applies each block with the tensor-core kernel or
  the CUDA-core dense kernel -- out of place, keeping the block's input state, when a
  backward can follow and memory allows (``QuantumDevice.checkpoint``);
* the backward walks the segment in reverse with the adjoint kernels (a tensor-core
  block with a stored input reads it instead of uncomputing the state; the images and
  cotangents of all tensor-core blocks take one launch each), turns block cotangents
  into gate-operand cotangents with ``tqk_block_unbuild``, and gate-operand cotangents
  into parameter gradients with ``tqk_param_grads`` (analytic derivatives), accumulated
  in float64 into one buffer per parameter base tensor.

Gates with no native type (qubitunitary, multirz, qft, user matrices, ...) keep the
torch-built operand and its autograd graph (``generic`` ops).
"""
from __future__ import annotations

import ctypes
import weakref
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _lib
from . import engine

# canonical gate name -> (TQK_G_* type id, number of parameters)
NATIVE = {
    "u3": (0, 3), "rx": (1, 1), "ry": (2, 1), "rz": (3, 1), "phaseshift": (4, 1), "u1": (4, 1), "rot": (5, 3),
    "u2": (6, 2), "r": (7, 2), "crx": (8, 1), "cry": (9, 1), "crz": (10, 1), "cu3": (11, 3), "cu1": (12, 1),
    "crot": (13, 3), "cu": (14, 4), "rzz": (15, 1), "rxx": (16, 1), "ryy": (17, 1), "rzx": (18, 1),
    "singleexcitation": (19, 1),
}
_DIAG_TYPES = {3: 2, 4: 1, 12: 1, 10: 4, 15: 4}  # type -> operand size for diagonal / phase operands
_WIDE_TYPES = {16, 17, 18, 19}                    # 4x4 dense operands

KIND_ID = {engine.KIND_DENSE: 0, engine.KIND_CTRL: 1, engine.KIND_X: 2, engine.KIND_PHASE: 3,
           engine.KIND_DIAG: 4, engine.KIND_SWAP: 5}


def operand_size(type_id: int) -> int:
    if type_id in _DIAG_TYPES:
        return _DIAG_TYPES[type_id]
    return 16 if type_id in _WIDE_TYPES else 4


# ---------------------------------------------------------------- ctypes descriptor layouts
class GateDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("inverse", ctypes.c_int32), ("batch", ctypes.c_int32),
                ("nparam", ctypes.c_int32), ("p", ctypes.c_void_p), ("p_row_stride", ctypes.c_int64),
                ("p_col_stride", ctypes.c_int64), ("p_is_double", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("op128", ctypes.c_void_p), ("op64", ctypes.c_void_p), ("op_grad", ctypes.c_void_p),
                ("grad", ctypes.c_void_p)]


class BlockOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nw", ctypes.c_int32), ("pos", ctypes.c_int32 * 6),
                ("nctrl", ctypes.c_int32), ("ctrl_val", ctypes.c_int32), ("batch", ctypes.c_int32),
                ("op_size", ctypes.c_int32), ("operand", ctypes.c_void_p), ("grad", ctypes.c_void_p)]


class BlockDesc(ctypes.Structure):
    _fields_ = [("first_op", ctypes.c_int32), ("num_ops", ctypes.c_int32), ("k", ctypes.c_int32),
                ("batch", ctypes.c_int32), ("u", ctypes.c_void_p), ("gu", ctypes.c_void_p)]


assert ctypes.sizeof(GateDesc) == 80 and ctypes.sizeof(BlockOp) == 64 and ctypes.sizeof(BlockDesc) == 32


def _to_device_table(structs, device) -> torch.Tensor:
    """Array of ctypes structures -> device uint8 tensor (via a pinned staging copy)."""
    n = len(structs)
    size = ctypes.sizeof(structs[0]) * n if n else 0
    host = torch.empty(max(size, 1), dtype=torch.uint8, pin_memory=True)
    arr = (type(structs[0]) * n)(*structs)
    ctypes.memmove(host.data_ptr(), ctypes.addressof(arr), size)
    dev = host.to(device, non_blocking=True)
    return dev, host  # keep the staging buffer alive until the copy has run


# ---------------------------------------------------------------- recorded native gate
class NativeGate:
    """A parameterised gate whose operand the GPU builds from ``params`` in place."""

    __slots__ = ("name", "type_id", "nparam", "wires", "params", "inverse", "kind", "nctrl", "batch")

    def __init__(self, name, wires, params, inverse, kind, nctrl):
        self.name = name
        self.type_id, self.nparam = NATIVE[name]
        self.wires = list(wires)
        self.params = params          # [B, P] float32/float64 on the device (may require grad)
        self.inverse = bool(inverse)
        self.kind = kind              # engine.KIND_*
        self.nctrl = nctrl
        self.batch = int(params.shape[0])


def _param_base(p: torch.Tensor):
    """(base tensor to differentiate, element offset of p[0, 0] inside base's storage)."""
    base = p._base if p._base is not None else p
    if base.dtype not in (torch.float32, torch.float64) or not _dense(base):
        return p, 0
    return base, p.storage_offset() - base.storage_offset()


def _dense(t: torch.Tensor) -> bool:
    try:
        return t.is_contiguous() or t.is_non_overlapping_and_dense()
    except AttributeError:
        return t.is_contiguous()


# ---------------------------------------------------------------- segment
class Segment:
    """A compiled run of gates: forward applied at construction, ``backward`` on demand."""

    def __init__(self, qdev, records: List, method: str):
        from . import fusion

        self.n = qdev.n_wires
        self.bsz = qdev.bsz
        self.device = qdev.device
        dev = self.device
        n = self.n
        # ---- native gate operands (one launch)
        natives = [r for r in records if isinstance(r, NativeGate)]
        self.natives = natives
        # operands laid out by shape: the natives of one operand shape are consecutive, so
        # their views come from one view + unbind per shape instead of per-gate slicing
        shapes = [_operand_shape(g, operand_size(g.type_id)) for g in natives]
        by_shape: Dict[tuple, List[int]] = {}
        for i, shp in enumerate(shapes):
            by_shape.setdefault(shp, []).append(i)
        offsets = [0] * len(natives)
        total = 0
        for shp, idx in by_shape.items():
            numel = int(np.prod(shp))
            for i in idx:
                offsets[i] = total
                total += numel
        self.op128 = torch.empty(max(total, 1), dtype=torch.complex128, device=dev)
        self.op64 = torch.empty(max(total, 1), dtype=torch.complex64, device=dev)
        views64, views128 = [None] * len(natives), [None] * len(natives)
        for shp, idx in by_shape.items():
            a, cnt = offsets[idx[0]], len(idx)
            size = cnt * int(np.prod(shp))
            for i, v64, v128 in zip(idx, self.op64[a:a + size].view(cnt, *shp).unbind(0),
                                    self.op128[a:a + size].view(cnt, *shp).unbind(0)):
                views64[i], views128[i] = v64, v128
        self.gate_offsets = offsets
        descs = []
        self._keep = []
        p64, p128 = self.op64.data_ptr(), self.op128.data_ptr()
        for g, off in zip(natives, offsets):
            p = g.params
            d = GateDesc()
            d.type, d.inverse, d.batch, d.nparam = g.type_id, int(g.inverse), g.batch, g.nparam
            d.p = p.data_ptr()
            d.p_row_stride = p.stride(0) if g.batch > 1 else 0
            d.p_col_stride = p.stride(1)
            d.p_is_double = int(p.dtype == torch.float64)
            d.op128 = p128 + 16 * off
            d.op64 = p64 + 8 * off
            descs.append(d)
        self.gate_descs = descs
        if descs:
            table, host = _to_device_table(descs, dev)
            self._keep += [table, host]
            _lib.gate_operands(table, len(descs), dev)
        # ---- exec ops: one TapeOp per record (operands point into op64 / op128)
        ops = []
        gi = 0
        for r in records:
            if isinstance(r, NativeGate):
                op = engine.TapeOp(r.kind, r.wires, controls=r.wires[:r.nctrl], targets=r.wires[r.nctrl:],
                                   operand=views64[gi])
                op.native = r
                op.op128 = views128[gi]
                gi += 1
            else:
                op = r
            ops.append(op)
        self.records = ops
        # ---- plan
        self.blocks = []
        if method == "fused":
            wl = planner_wires(ops, n)
            fw = qdev.fuse_wires
            backend = getattr(qdev, "fused_backend", "auto")
            tc_ok = backend != "cuda" and n >= fusion.TC_MIN_WIRES
            if fw == "auto" and self.device.type == "cuda":
                from . import autotune

                with_adj = any(isinstance(r, NativeGate) and r.params.requires_grad for r in records) or \
                    any(not isinstance(r, NativeGate) and r.needs_grad for r in records)
                stored = with_adj and getattr(qdev, "checkpoint", "auto") is not False
                # how a gate left alone by a plan runs: a dense or controlled gate may still
                # run as a tensor-core block (its own kernel is a dense pass with a
                # cotangent, and on large states a 6-wire block's forward + reverse step
                # costs less); structured gates keep their light kernels
                lone_kind = [autotune.LONE_OTHER if not fusable(op) else
                             autotune.LONE_DENSE if op.kind in (engine.KIND_DENSE, engine.KIND_CTRL) else
                             autotune.LONE_LIGHT for op in ops]
                plan, tc_flags, k, _ = autotune.choose_fusion(wl, n, self.bsz, dev, tc_ok, with_adj, stored=stored,
                                                              lone_kind=lone_kind)
                lone_tc = [len(idxs) == 1 and tc for (_, idxs), tc in zip(plan, tc_flags)]
                if backend == "tc":
                    tc_flags = [tc_ok for _ in plan]
            else:
                k = max(1, min(6 if fw == "auto" else int(fw), n, 6))
                plan = fusion.plan_cached(wl, k, 8, 4)
                tc_flags = [fusion.use_tensor_cores(qdev, len(bw)) for bw, _ in plan]
                lone_tc = [False] * len(plan)
            self.fuse_width = k
            exec_ops = []
            for (bwires, idxs), tc, lone in zip(plan, tc_flags, lone_tc):
                members = [ops[i] for i in idxs]
                if len(members) == 1 and not (lone and fusable(members[0])):  # a lone gate on its own kernel
                    exec_ops.append(members[0])
                    continue
                exec_ops.append(self._make_block(qdev, members, bwires, tc))
            self.exec_ops = exec_ops
            self._build_blocks()
        else:
            self.exec_ops = stage_runs(ops, n) if getattr(qdev, "stage_low", True) else ops
        # ---- differentiable inputs
        self.bases: Dict[int, tuple] = {}
        for g in natives:
            if g.params.requires_grad:
                base, _ = _param_base(g.params)
                self.bases.setdefault(id(base), (base, None))
        self.generic_sources = [op for op in ops if not hasattr(op, "native") and op.needs_grad]
        self.diff_inputs = [b for b, _ in self.bases.values()] + [op.source for op in self.generic_sources]

    # -------------------------------------------------------------- blocks
    def _make_block(self, qdev, members, bwires, tc):
        from . import fusion

        if len(bwires) > 6 or not all(fusable(m) for m in members):
            raise _lib.TQKError(1, f"a fused block holds at most 6 wires of fusable ops (got {len(bwires)} wires)")
        if tc:
            bwires = fusion._pad_wires(bwires, self.n)
        k = len(bwires)
        batch = max(m.batch if m.batch else 1 for m in members)
        blk = engine.TapeOp(engine.KIND_DENSE, bwires)
        blk.members = members
        blk.block_batch = batch
        blk.tc = tc
        blk.batch = batch
        blk.k = k
        self.blocks.append(blk)
        return blk

    def _build_blocks(self):
        if not self.blocks:
            return
        dev = self.device
        sizes = [b.block_batch * (1 << (2 * b.k)) for b in self.blocks]
        self.u128 = torch.empty(max(sum(sizes), 1), dtype=torch.complex128, device=dev)
        off = 0
        bdescs, bops = [], []
        for blk, sz in zip(self.blocks, sizes):
            d = 1 << blk.k
            blk.u128 = self.u128[off:off + sz].view(blk.block_batch, d, d)
            off += sz
            where = {w: blk.k - 1 - i for i, w in enumerate(blk.wires)}
            bd = BlockDesc()
            bd.first_op, bd.num_ops, bd.k, bd.batch = len(bops), len(blk.members), blk.k, blk.block_batch
            bd.u = blk.u128.data_ptr()
            bd.gu = None
            bdescs.append(bd)
            for m in blk.members:
                bops.append(self._block_op(m, where))
        self.block_descs, self.block_ops = bdescs, bops
        bt, bh = _to_device_table(bdescs, dev)
        ot, oh = _to_device_table(bops, dev)
        self._keep += [bt, bh, ot, oh]
        maxb = max(b.block_batch for b in self.blocks)
        _lib.block_build(bt, len(bdescs), maxb, ot, dev)
        for blk in self.blocks:
            if not blk.tc:
                blk.operand = blk.u128.to(torch.complex64)
        self._prepare_images(adjoint=False)
        # keep operands of non-native members alive in complex128
        self._member128 = [getattr(m, "_op128_keep", None) for b in self.blocks for m in b.members]

    def _prepare_images(self, adjoint: bool) -> None:
        """Tensor-core operand images of every block of the segment (of U, or of U^H for
        the reverse sweep) in one buffer and one launch: ``blk.image`` / ``blk.image_h``."""
        tcb = [b for b in self.blocks if b.tc]
        if not tcb:
            return
        lib = _lib.load()
        sizes = [lib.tqk_fused_image_bytes(b.block_batch) for b in tcb]
        buf = torch.empty(sum(sizes), dtype=torch.uint8, device=self.device)
        jobs, off = [], 0
        for b, sz in zip(tcb, sizes):
            img = buf[off:off + sz]  # every image is a multiple of 64 KB: offsets stay aligned
            off += sz
            setattr(b, "image_h" if adjoint else "image", img)
            j = _lib.ImageJob()
            j.u, j.image, j.u_batch, j.adjoint = b.u128.data_ptr(), img.data_ptr(), b.block_batch, int(adjoint)
            for i, w in enumerate(b.wires):
                j.wires[i] = w
            jobs.append(j)
        table, host = _to_device_table(jobs, self.device)
        # the pinned staging copy must outlive its asynchronous upload (one slot per
        # direction, so repeated reverse sweeps do not accumulate them)
        setattr(self, "_keep_images_h" if adjoint else "_keep_images", (table, host))
        _lib.fused_prepare_many(table, len(jobs), max(b.block_batch for b in tcb))

    def _block_op(self, m, where):
        bo = BlockOp()
        bo.kind = KIND_ID[m.kind]
        wires = m.wires
        bo.nw = len(wires)
        for j, w in enumerate(wires):
            bo.pos[j] = where[w]
        bo.nctrl = len(m.controls) if m.kind in (engine.KIND_CTRL, engine.KIND_X, engine.KIND_SWAP) else 0
        bo.ctrl_val = m.ctrl_val
        if m.kind in (engine.KIND_X, engine.KIND_SWAP):
            bo.batch, bo.op_size, bo.operand = 1, 1, self._dummy_ptr()
            return bo
        o128 = m.op128 if hasattr(m, "op128") else _generic128(m)
        bo.batch = int(o128.shape[0])
        bo.op_size = int(o128[0].numel())
        bo.operand = o128.data_ptr()
        bo.grad = None
        return bo

    def _dummy_ptr(self):
        if not hasattr(self, "_dummy"):
            self._dummy = torch.zeros(1, dtype=torch.complex128, device=self.device)
        return self._dummy.data_ptr()

    # -------------------------------------------------------------- forward
    def apply(self, buf: torch.Tensor, store_inputs: bool = False, zero_input: bool = False) -> torch.Tensor:
        """Run the segment on ``buf``; returns the buffer holding the result.  With
        ``store_inputs`` every tensor-core block writes its output to a new buffer and
        keeps its input for the backward (``buf`` itself may become one of those stored
        inputs, so the result is then a different tensor).  ``zero_input``: ``buf`` is
        |0...0> in every row and no initial state or earlier segment precedes it (the
        device's first segment from its default state)."""
        _lib.nvtx_push(f"tqk.segment.forward[{len(self.exec_ops)} passes]")
        try:
            return self._apply(buf, store_inputs, zero_input)
        finally:
            _lib.nvtx_pop()

    def _apply(self, buf: torch.Tensor, store_inputs: bool, zero_input: bool) -> torch.Tensor:
        recs, keep = [], []
        cur = buf
        for i, op in enumerate(self.exec_ops):
            if isinstance(op, StagedRun):
                recs.append(_staged_record(op, op.descs(), keep))
            elif getattr(op, "members", None) is not None:
                if not op.tc:
                    recs.append(_exec(_lib.X_BLOCK_DENSE, op.wires, batch=op.block_batch, operand=op.operand))
                    continue
                if zero_input and i == 0:
                    # a first block on |0...0>: its output is column 0 of U at the block's 64
                    # patterns (every other amplitude stays 0), written directly instead of a
                    # pass over the state; its reverse step needs neither its input nor the
                    # cotangent before it (nothing precedes it), so nothing is kept
                    op.zero_input = True
                    recs.append(_exec(_lib.X_BLOCK_ZERO, op.wires, batch=op.block_batch, u=op.u128))
                    continue
                r = _exec(_lib.X_BLOCK_TC, op.wires, batch=op.block_batch, image=op.image)
                out = None
                if store_inputs:
                    out = _new_state(cur)
                    if out is None:  # out of memory: the remaining blocks run in place
                        store_inputs = False
                if out is not None:
                    r.out = out.data_ptr()
                    op.stored_input = cur
                    op.kept_input = True
                    cur = out
                recs.append(r)
            else:
                recs.append(_plain_record(op))
        if recs:
            table = (_lib.ExecOp * len(recs))(*recs)
            final = _lib.segment_forward(buf, self.n, table, len(recs))
            assert final == cur.data_ptr(), "segment runner ended on an unexpected buffer"
        return cur

    def take_stored_inputs(self) -> list:
        """(block, stored input) pairs for an autograd node to save; the segment keeps weak
        references, so later nodes over the same segment still find the inputs while one
        node holds them, and the memory goes when the last node releases them."""
        out = []
        for op in self.blocks:
            t = getattr(op, "stored_input", None)
            if t is None and getattr(op, "stored_ref", None) is not None:
                t = op.stored_ref()
            if t is None:
                continue
            op.stored_ref = weakref.ref(t)
            op.stored_input = None
            out.append((op, t))
        return out

    def stored_bytes(self, state: torch.Tensor) -> int:
        """Device memory ``apply(..., store_inputs=True)`` keeps for the backward."""
        return sum(1 for b in self.blocks if b.tc) * state.numel() * state.element_size()

    # -------------------------------------------------------------- backward
    def backward(self, psi: "engine.StateCursor", lam: torch.Tensor, need_grads: bool,
                 inputs: Optional[dict] = None) -> List[Optional[torch.Tensor]]:
        """Reverse sweep over this segment (``psi`` at its end on entry, at its start on
        return; ``lam`` updated in place); ``inputs`` maps id(block) to the block's stored
        input state, where the forward kept one and it is still held.  Returns grads for
        ``self.diff_inputs``."""
        _lib.nvtx_push(f"tqk.segment.backward[{len(self.exec_ops)} passes]")
        try:
            return self._backward(psi, lam, need_grads, inputs or {})
        finally:
            _lib.nvtx_pop()

    def _backward(self, psi: "engine.StateCursor", lam: torch.Tensor, need_grads: bool,
                  inputs: dict) -> List[Optional[torch.Tensor]]:
        dev = self.device
        n = self.n
        opg = torch.zeros_like(self.op128) if (need_grads and self.natives) else None
        gslots = {}
        for op in self.generic_sources:
            gslots[id(op)] = torch.zeros(op.operand.shape, dtype=torch.complex128, device=dev)
        gu = torch.zeros_like(self.u128) if (need_grads and self.blocks) else None
        # tensor-core blocks: U^H images in one launch, one zeroed buffer for the cross
        # terms of the blocks that need a cotangent, stored-input cotangents added in one
        # launch after the sweep
        self._prepare_images(adjoint=True)
        mr_of = {}
        tc_grad = [b for b in self.blocks if b.tc and gu is not None and _block_needs_grad(b)]
        if tc_grad:
            mr_all = torch.zeros(sum(b.block_batch for b in tc_grad), 128, 128, dtype=torch.float64, device=dev)
            row = 0
            for b in tc_grad:
                mr_of[id(b)] = mr_all[row:row + b.block_batch]
                row += b.block_batch
        cross_jobs, recs, keep, stored_at = [], [], [], {}
        zero_block = None
        # a native gate's cotangent slot: the place of its operand in op128, inside opg
        dopg = opg.data_ptr() - self.op128.data_ptr() if opg is not None else 0
        for op in self.exec_ops:  # forward order; the runner walks it backwards
            if isinstance(op, StagedRun):
                slots = []
                for m in op.ops:
                    slot = None
                    if need_grads:
                        if hasattr(m, "native") and m.native.params.requires_grad:
                            slot = m.op128.data_ptr() + dopg
                        elif id(m) in gslots:
                            slot = torch.view_as_real(gslots[id(m)]).view(-1)
                    slots.append(slot)
                recs.append(_staged_record(op, op.descs(slots), keep))
                continue
            if getattr(op, "members", None) is not None:
                slot = None
                if gu is not None and _block_needs_grad(op):
                    slot = _as_real(gu, op.u128, self.u128)
                if not op.tc:
                    recs.append(_exec(_lib.X_BLOCK_DENSE, op.wires, batch=op.block_batch, operand=op.operand,
                                      grad=slot))
                    continue
                stored = inputs.get(id(op))
                mr = mr_of.get(id(op)) if slot is not None else None
                r = _exec(_lib.X_BLOCK_TC, op.wires, batch=op.block_batch, image_h=op.image_h, u=op.u128, grad=slot,
                          mr=mr)
                if getattr(op, "zero_input", False):
                    # the last reverse step of the circuit, from |0...0>: the runner stops
                    # before it; the cotangent of U is lam conj(e_0)^T (taken below)
                    r.skip_reverse = 1
                    zero_block = (op, slot)
                elif stored is not None:
                    r.stored = stored.data_ptr()
                    stored_at[stored.data_ptr()] = stored
                    if mr is not None:  # the cross term against the stored input is the cotangent
                        j = _lib.CrossJob()
                        j.mr, j.gu, j.batch = mr.data_ptr(), slot.data_ptr(), op.block_batch
                        cross_jobs.append(j)
                recs.append(r)
                continue
            slot = None
            if need_grads:
                if hasattr(op, "native") and op.native.params.requires_grad:
                    slot = op.op128.data_ptr() + dopg
                elif id(op) in gslots:
                    slot = torch.view_as_real(gslots[id(op)]).view(-1)
            recs.append(_plain_record(op, slot))
        if recs:
            # the sweep writes its state only on a work buffer: the cursor's own when it
            # already owns one, else one state more, when any reverse step uncomputes
            uncomputes = any(not (r.kind == _lib.X_BLOCK_TC and (r.stored or r.skip_reverse)) for r in recs)
            work = psi.state if psi.owned else (psi.work_buffer() if uncomputes else None)
            table = (_lib.ExecOp * len(recs))(*recs)
            start = _lib.segment_backward(psi.state, lam, work, n, table, len(recs))
            if work is not None and start == work.data_ptr():
                psi.state, psi.owned = work, True
            elif start in stored_at:
                psi.state, psi.owned = stored_at[start], False
        if zero_block is not None and zero_block[1] is not None:
            _add_zero_input_cotangent(lam, zero_block[0], zero_block[1], n)
        if cross_jobs:
            table, host = _to_device_table(cross_jobs, dev)
            self._keep_cross = (table, host)  # the cross terms themselves are stream-ordered
            _lib.fused_cross_add_many(table, len(cross_jobs), max(j.batch for j in cross_jobs))
        if not need_grads:
            return [None] * len(self.diff_inputs)
        # block cotangents -> member operand cotangents
        if self.blocks and gu is not None:
            bops = []
            bdescs = []
            for bi, blk in enumerate(self.blocks):
                bd = BlockDesc()
                src = self.block_descs[bi]
                bd.first_op, bd.num_ops, bd.k, bd.batch = src.first_op, src.num_ops, src.k, src.batch
                bd.u = blk.u128.data_ptr()
                bd.gu = gu.data_ptr() + (blk.u128.data_ptr() - self.u128.data_ptr()) \
                    if _block_needs_grad(blk) else None
                bdescs.append(bd)
                for m, src_op in zip(blk.members, self.block_ops[src.first_op:src.first_op + src.num_ops]):
                    bo = BlockOp.from_buffer_copy(src_op)
                    bo.grad = None
                    if hasattr(m, "native") and m.native.params.requires_grad:
                        bo.grad = opg.data_ptr() + (m.op128.data_ptr() - self.op128.data_ptr())
                    elif id(m) in gslots:
                        bo.grad = gslots[id(m)].data_ptr()
                    bops.append(bo)
            bt, bh = _to_device_table(bdescs, dev)
            ot, oh = _to_device_table(bops, dev)
            maxb = max(b.block_batch for b in self.blocks)
            _lib.block_unbuild(bt, len(bdescs), maxb, ot, dev)
            self._keep_bw = [bt, bh, ot, oh]
        # operand cotangents -> parameter gradients
        grads = []
        if self.natives and self.bases:
            # one float64 buffer for every base tensor's gradient (each base's part laid out
            # like the base's own storage), one conversion back to the bases' dtype
            bases = [b for b, _ in self.bases.values()]
            spans = [max(0, sum((sz - 1) * st for sz, st in zip(b.shape, b.stride()))) + 1 for b in bases]
            starts = np.cumsum([0] + spans[:-1]).tolist()
            flat = torch.zeros(max(sum(spans), 1), dtype=torch.float64, device=dev)
            start_of = {k: st for k, st in zip(self.bases.keys(), starts)}
            descs = []
            fp = flat.data_ptr()
            for g, d, off in zip(self.natives, self.gate_descs, self.gate_offsets):
                if not g.params.requires_grad:
                    continue
                base, eoff = _param_base(g.params)
                nd = GateDesc.from_buffer_copy(d)
                nd.op128 = None
                nd.op64 = None
                nd.op_grad = opg.data_ptr() + 16 * off
                nd.grad = fp + 8 * (start_of[id(base)] + eoff)
                descs.append(nd)
            if descs:
                table, host = _to_device_table(descs, dev)
                _lib.param_grads(table, len(descs), dev)
                self._keep_pg = [table, host]
            dtypes = {b.dtype for b in bases}
            conv = flat.to(bases[0].dtype) if len(dtypes) == 1 else None
            for b, st in zip(bases, starts):
                src = conv if conv is not None else flat
                gb = src.as_strided(b.shape, b.stride(), st)
                grads.append(gb if conv is not None else gb.to(b.dtype))
        else:
            grads += [None] * len(self.bases)
        for op in self.generic_sources:
            grads.append(gslots[id(op)].to(op.source.dtype).view(op.source.shape))
        return grads


_PLAIN_KIND = {engine.KIND_DENSE: _lib.X_DENSE, engine.KIND_CTRL: _lib.X_CTRL, engine.KIND_X: _lib.X_MCX,
               engine.KIND_PHASE: _lib.X_PHASE, engine.KIND_DIAG: _lib.X_DIAG, engine.KIND_SWAP: _lib.X_SWAP}


def _exec(kind: int, wires, nctrl: int = 0, ctrl_val: int = 1, batch: int = 1, operand=None, uncompute=None,
          image=None, image_h=None, u=None, grad=None, mr=None) -> "_lib.ExecOp":
    """One ``tqk_exec_op`` record (tensors, or device addresses as ints)."""
    r = _lib.ExecOp()
    r.kind, r.nw, r.nctrl, r.ctrl_val, r.batch = kind, len(wires), nctrl, ctrl_val, batch
    if len(wires) > len(r.wires):
        raise _lib.TQKError(1, f"an op on {len(wires)} wires exceeds the {len(r.wires)} one op may touch")
    for j, w in enumerate(wires):
        r.wires[j] = w
    for name, t in (("operand", operand), ("uncompute", uncompute), ("image", image), ("image_h", image_h),
                    ("u", u), ("grad", grad), ("mr", mr)):
        if t is not None:
            setattr(r, name, t if isinstance(t, int) else t.data_ptr())
    return r


def _plain_record(op, grad=None) -> "_lib.ExecOp":
    """A plain tape op (engine.TapeOp) as a ``tqk_exec_op``: wires are controls first,
    then targets, for the controlled kinds."""
    k = op.kind
    if k in (engine.KIND_CTRL, engine.KIND_X, engine.KIND_SWAP):
        wires, nctrl = op.controls + op.targets, len(op.controls)
    else:
        wires, nctrl = op.wires, 0
    return _exec(_PLAIN_KIND[k], wires, nctrl=nctrl, ctrl_val=op.ctrl_val, batch=op.batch, operand=op.operand,
                 uncompute=op.uncompute, grad=grad)


def _staged_record(run, descs, keep: list) -> "_lib.ExecOp":
    arr = (_lib.StagedOp * len(descs))(*descs)
    keep.append(arr)  # alive until the runner returns (it reads the table on the host)
    r = _lib.ExecOp()
    r.kind, r.staged, r.nstaged, r.tile_bits = _lib.X_STAGED, ctypes.addressof(arr), len(descs), run.tile_bits
    return r


def _zero_input_index(blk, n: int, device) -> torch.Tensor:
    """Amplitude offsets of a 6-wire block's 64 patterns with every other bit clear
    (wires[0] is the pattern's most significant bit), on the device; built once per block."""
    idx = getattr(blk, "_zero_idx", None)
    if idx is None:
        offs = [sum(1 << (n - 1 - w) for i, w in enumerate(blk.wires) if (j >> (5 - i)) & 1) for j in range(64)]
        # a pinned staging copy: a copy from pageable memory would block the stream (and
        # with it the host's run-ahead into the next step)
        host = torch.tensor(offs, dtype=torch.long).pin_memory()
        idx = host.to(device, non_blocking=True)
        blk._zero_idx_host = host  # alive until the copy has run
        blk._zero_idx = idx
    return idx


def _add_zero_input_cotangent(lam: torch.Tensor, blk, slot: torch.Tensor, n: int) -> None:
    """gu[b][j][0] += lam[b, offset of pattern j] for a block applied to |0...0> (wires[0] is
    the pattern's most significant bit; the sum over rows when one U serves every row)."""
    vals = lam.index_select(1, _zero_input_index(blk, n, lam.device)).to(torch.complex128)  # [bsz, 64]
    g = torch.view_as_complex(slot.view(-1, 2)).view(blk.block_batch, 64, 64)
    if blk.block_batch == 1:
        g[0, :, 0] += vals.sum(0)
    else:
        g[:, :, 0] += vals


def _new_state(like: torch.Tensor) -> Optional[torch.Tensor]:
    """A buffer for a block's output when its input is kept, or None when the device is out
    of memory (the caller then continues in place; the reverse sweep uncomputes through
    the blocks without a stored input)."""
    try:
        return torch.empty_like(like)
    except torch.cuda.OutOfMemoryError:
        return None


# ---------------------------------------------------------------- staged low-qubit runs
class StagedRun:
    """Consecutive ops whose targets lie in the lowest ``tile_bits`` index bits, applied
    in one shared-memory pass (``tqk_staged_apply``) and reversed in one adjoint pass."""

    def __init__(self, ops, tile_bits):
        self.ops = ops
        self.tile_bits = tile_bits
        self.wires = sorted({w for o in ops for w in o.wires})

    def descs(self, grads=None):
        """The run's ``tqk_staged_op`` records; ``grads``: per-op cotangent slots (tensor,
        device address or None) for the reverse pass.  The records without slots are built
        once per run (operands do not move) and copied when slots are set."""
        base = getattr(self, "_descs", None)
        if base is None:
            base = self._build_descs()
            self._descs = base
        if grads is None:
            return base
        out = []
        for d, g in zip(base, grads):
            if g is None:
                out.append(d)
                continue
            e = _lib.StagedOp.from_buffer_copy(d)
            e.grad = g if isinstance(g, int) else g.data_ptr()
            out.append(e)
        return out

    def _build_descs(self):
        out = []
        for o in self.ops:
            d = _lib.StagedOp()
            if o.kind == engine.KIND_X:
                ws, d.kind, d.ctrl_val = o.controls + o.targets, _lib.S_X, o.ctrl_val
            elif o.kind in (engine.KIND_DENSE, engine.KIND_CTRL):
                ws, d.kind = (o.controls + o.targets) if o.kind == engine.KIND_CTRL else o.wires, _lib.S_DENSE1
            elif o.kind == engine.KIND_PHASE:
                ws, d.kind = o.wires, _lib.S_PHASE
            else:
                ws, d.kind = o.wires, _lib.S_DIAG
            d.nwires = len(ws)
            for j, w in enumerate(ws):
                d.wires[j] = w
            if o.kind != engine.KIND_X:
                d.operand = o.operand.data_ptr()
                d.batch = int(o.operand.shape[0])
            else:
                d.batch = 1
            d.grad = None
            out.append(d)
        return out


def stageable(op, n: int, tile_bits: int) -> bool:
    """Ops ``tqk_staged_apply`` can run: one target inside the low tile (dense, controlled,
    controlled-X), or diagonal ops anywhere (phase on any wires, diagonal on <= 2)."""
    if getattr(op, "uncompute", None) is not None or getattr(op, "image", None) is not None:
        return False
    if not op.wires or len(op.wires) > _lib.STAGED_MAX_WIRES:
        return False
    low = n - tile_bits  # wires >= low have their bit inside the tile
    k = op.kind
    if k == engine.KIND_DENSE:
        return len(op.wires) == 1 and op.wires[0] >= low and _mat2(op)
    if k == engine.KIND_CTRL:
        return len(op.targets) == 1 and op.targets[0] >= low and _mat2(op)
    if k == engine.KIND_X:
        return len(op.targets) == 1 and op.targets[0] >= low
    if k == engine.KIND_PHASE:
        return op.operand is not None and op.operand.numel() == int(op.operand.shape[0])
    if k == engine.KIND_DIAG:
        return len(op.wires) <= 2 and op.operand is not None and op.operand.shape[-1] == (1 << len(op.wires))
    return False


def _mat2(op) -> bool:
    t = op.operand
    return t is not None and t.dtype == torch.complex64 and tuple(t.shape[1:]) == (2, 2) and t.is_contiguous()


def stage_runs(ops, n: int, min_run: int = 2):
    """Group maximal runs of consecutive stageable ops into ``StagedRun`` passes (tile of
    2^min(n, 12) amplitudes; at most ``STAGED_MAX_OPS`` ops per pass)."""
    tb = min(n, _lib.STAGED_MAX_TILE_BITS)
    out, run = [], []

    def close():
        if len(run) >= min_run:
            out.append(StagedRun(list(run), tb))
        else:
            out.extend(run)
        run.clear()

    for op in ops:
        if stageable(op, n, tb):
            run.append(op)
            if len(run) == _lib.STAGED_MAX_OPS:
                close()
        else:
            close()
            out.append(op)
    close()
    return out


def _operand_shape(r: NativeGate, sz: int):
    if r.type_id in _DIAG_TYPES:
        return (r.batch,) if sz == 1 else (r.batch, sz)
    d = 4 if r.type_id in _WIDE_TYPES else 2
    return (r.batch, d, d)


def _as_real(buf: torch.Tensor, view: torch.Tensor, base: torch.Tensor) -> torch.Tensor:
    """float64 interleaved view of ``buf`` at the position ``view`` occupies inside ``base``."""
    off = (view.data_ptr() - base.data_ptr()) // 16
    return torch.view_as_real(buf[off:off + view.numel()]).view(-1)


def _block_needs_grad(blk) -> bool:
    return any((hasattr(m, "native") and m.native.params.requires_grad) or m.needs_grad for m in blk.members)


def _generic128(m) -> torch.Tensor:
    t = m.source if m.source is not None else m.operand
    t = engine.kernel_operand(t.to(torch.complex128))
    m._op128_keep = t
    return t


def planner_wires(ops, n: int) -> List[List[int]]:
    """Wire lists the fusion planners see: an op's wires, or for an op the block kernels
    cannot hold (``fusable`` false) a barrier -- every wire (nothing moves across it) plus
    7 placeholder wires, wider than any block, so every planner leaves it alone (also when
    n <= 6, where all n wires would fit in one block)."""
    barrier = list(range(n)) + [-1 - i for i in range(7)]
    return [list(op.wires) if fusable(op) else barrier for op in ops]


def fusable(op) -> bool:
    """Ops the block kernels can fold into a fused block."""
    if not op.wires or getattr(op, "uncompute", None) is not None:
        return False
    nw = len(op.wires)
    if op.kind in (engine.KIND_X, engine.KIND_SWAP, engine.KIND_PHASE):
        return nw <= 6
    if op.kind == engine.KIND_DIAG:
        return nw <= 4
    if op.kind == engine.KIND_CTRL:
        return len(op.targets) <= 2 and nw <= 6
    return nw <= 2
