"""Fused method: group gates into k-wire blocks, build each block's unitary in
complex128, apply it with one pass over the state.

Planner: greedy and linear in the number of gates per block.  A block starts from a
seed (the first pending gate's wires, or, with lookahead, the best of a few front
gates and pairs of them); walking the pending list in order, a gate joins the block if
none of its wires is blocked by an earlier gate left out and the union of wires stays
within ``k``; otherwise its wires become blocked (gates on disjoint wires commute, so
later gates may still join).  ``plan_beam`` keeps the few best partial plans per block
instead of one.  The fusion width and planner variant are picked per segment by
``autotune.choose_fusion`` from measured per-pass costs.  Upstream's static mode instead scores every
``C(n, k)`` wire combination per block (``torchquantum/graph/graphs.py:384-532``),
which is impractical at n = 24..28.

Build: ``program.Segment`` builds every block unitary on the GPU in float64
(``tqk_block_build``); ``build_block_unitary`` here is the same product written with
torch ops, used to check it.

Apply: wide blocks on states of >= 13 wires run on the tensor-core kernel, padded to
6 wires with identity wires; otherwise the dense k-wire kernel (CUDA cores).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import torch

from . import _lib
from . import engine

__all__ = ["plan_blocks", "op_full_matrix", "build_block_unitary", "use_tensor_cores"]


def _grow(wire_lists, pending, seed, k):
    """One block from ``seed`` wires: walk ``pending`` in order, take every gate whose
    wires are unblocked and keep the union within ``k``; a gate left out blocks its
    wires for the gates after it.  Returns (block wires, taken, rest)."""
    q = set(seed)
    blocked = set()
    take, rest = [], []
    for gi in pending:
        w = set(wire_lists[gi])
        if w & blocked:
            blocked |= w
            rest.append(gi)
            continue
        if len(q | w) <= k:
            q |= w
            take.append(gi)
        else:
            blocked |= w
            rest.append(gi)
    return q, take, rest


def plan_blocks(wire_lists: Sequence[Sequence[int]], k: int, lookahead: int = 0) -> List[Tuple[List[int], List[int]]]:
    """Greedy fusion plan: list of (sorted block wires, gate indices in order).

    ``lookahead = 0``: each block is seeded with the first pending gate's wires.
    ``lookahead = m``: the first m gates of the front (pending gates no earlier pending
    gate shares a wire with) are tried as seeds, alone and in pairs that fit, and the
    seed whose block takes the most gates wins.  Cost: O(m^2 x pending) per block."""
    pending = list(range(len(wire_lists)))
    blocks = []
    while pending:
        first = set(wire_lists[pending[0]])
        if len(first) > k:  # a gate wider than the block size stays on its own
            blocks.append((sorted(first), [pending[0]]))
            pending = pending[1:]
            continue
        if lookahead <= 0:
            q, take, rest = _grow(wire_lists, pending, first, k)
        else:
            front, seen = [], set()
            for gi in pending:
                w = set(wire_lists[gi])
                if not (w & seen) and len(w) <= k:
                    front.append(w)
                seen |= w
                if len(front) >= lookahead or len(seen) >= 64:
                    break
            seeds = list(front) + [a | b for i, a in enumerate(front) for b in front[i + 1:] if len(a | b) <= k]
            best = None
            for sd in seeds:
                cand = _grow(wire_lists, pending, sd, k)
                if best is None or len(cand[1]) > len(best[1]):
                    best = cand
            q, take, rest = best
        blocks.append((sorted(q), take))
        pending = rest
    return blocks


def _front_seeds(wire_lists, pending, k, m):
    front, seen = [], set()
    for gi in pending:
        w = set(wire_lists[gi])
        if not (w & seen) and len(w) <= k:
            front.append(w)
        seen |= w
        if len(front) >= m or len(seen) >= 64:
            break
    return front + [a | b for i, a in enumerate(front) for b in front[i + 1:] if len(a | b) <= k]


def plan_beam(wire_lists: Sequence[Sequence[int]], k: int, width: int = 4, lookahead: int = 8):
    """Beam search over block sequences: each step extends every kept partial plan by one
    block per seed (front gates and pairs, as in ``plan_blocks``) and keeps the ``width``
    partial plans with the fewest gates left.  Same legality rules as ``plan_blocks``."""
    states = [([], tuple(range(len(wire_lists))))]
    while True:
        done = [st for st in states if not st[1]]
        if done:
            return min(done, key=lambda st: len(st[0]))[0]
        cand = []
        for blocks, pend in states:
            pl = list(pend)
            first = set(wire_lists[pl[0]])
            if len(first) > k:  # a gate wider than the block size stays on its own
                cand.append((blocks + [(sorted(first), [pl[0]])], tuple(pl[1:])))
                continue
            seen = set()
            for sd in _front_seeds(wire_lists, pl, k, lookahead):
                q, take, rest = _grow(wire_lists, pl, sd, k)
                key = tuple(rest)
                if key in seen:
                    continue
                seen.add(key)
                cand.append((blocks + [(sorted(q), take)], key))
        cand.sort(key=lambda st: (len(st[1]), len(st[0])))
        states, keys = [], set()
        for st in cand:
            if st[1] in keys:
                continue
            keys.add(st[1])
            states.append(st)
            if len(states) >= width:
                break


BEAM_MAX_GATES = 2000  # longer segments plan with the single-pass lookahead only
_PLAN_CACHE: dict = {}


def plan_cached(wire_lists: Sequence[Sequence[int]], k: int, lookahead: int = 0, beam: int = 0):
    """Fusion plan memoised on the wire lists (a circuit re-recorded every step plans
    once): ``beam > 1`` runs ``plan_beam`` (segments up to ``BEAM_MAX_GATES`` gates),
    otherwise ``plan_blocks``."""
    key = (tuple(tuple(w) for w in wire_lists), k, lookahead, beam)
    hit = _PLAN_CACHE.get(key)
    if hit is None:
        if len(_PLAN_CACHE) > 256:
            _PLAN_CACHE.clear()
        if beam > 1 and len(wire_lists) <= BEAM_MAX_GATES:
            hit = plan_beam(wire_lists, k, beam, max(lookahead, 1))
        else:
            hit = plan_blocks(wire_lists, k, lookahead)
        _PLAN_CACHE[key] = hit
    return hit


def op_full_matrix(op: engine.TapeOp, dtype=torch.complex128, device=None) -> torch.Tensor:
    """Full [B, 2^m, 2^m] matrix of a tape op on its own wires (differentiable in op.source)."""
    src = op.source if op.source is not None else op.operand
    k = op.kind
    m = len(op.wires)
    if k == engine.KIND_DENSE:
        return src.to(dtype)
    if k == engine.KIND_CTRL:
        blk = src.to(dtype)
        b, d = blk.shape[0], blk.shape[-1]
        full = torch.eye(1 << m, dtype=dtype, device=blk.device).repeat(b, 1, 1)
        full[:, -d:, -d:] = blk
        return full
    if k == engine.KIND_PHASE:
        ph = src.to(dtype)
        ones = torch.ones(ph.shape[0], (1 << m) - 1, dtype=dtype, device=ph.device)
        return torch.diag_embed(torch.cat([ones, ph.reshape(-1, 1)], dim=1))
    if k == engine.KIND_DIAG:
        return torch.diag_embed(src.to(dtype))
    if k in (engine.KIND_X, engine.KIND_SWAP):
        return _perm_matrix(op.kind, len(op.wires), len(op.controls), op.ctrl_val, dtype, device)
    raise ValueError(f"cannot fuse op kind {k}")


_PERM_CACHE = {}


def _perm_matrix(kind, m, nc, ctrl_val, dtype, device):
    key = (kind, m, nc, ctrl_val, dtype, str(device))
    if key in _PERM_CACHE:
        return _PERM_CACHE[key]
    mat = _perm_matrix_cpu(kind, m, nc, ctrl_val, dtype)
    if device is not None:
        mat = mat.to(device)
    _PERM_CACHE[key] = mat
    return mat


def _perm_matrix_cpu(kind, m, nc, ctrl_val, dtype):
    dim = 1 << m
    idx = torch.arange(dim)
    if kind == engine.KIND_X:
        cmask = ((1 << nc) - 1) << 1  # controls are the top nc bits of the (nc+1)-bit index
        want = cmask if ctrl_val else 0
        src = torch.where((idx & cmask) == want, idx ^ 1, idx)
    else:  # controlled swap of the last two bits
        cmask = ((1 << nc) - 1) << 2
        b1, b0 = (idx >> 1) & 1, idx & 1
        swapped = (idx & ~3) | (b0 << 1) | b1
        src = torch.where((idx & cmask) == cmask, swapped, idx)
    mat = torch.zeros(dim, dim, dtype=dtype)
    mat[idx, src] = 1
    return mat[None]


def _apply_rows(u: torch.Tensor, g: torch.Tensor, pos: List[int], k: int) -> torch.Tensor:
    """g (on row bits ``pos``, pos[0] most significant) times u, for u [B, 2^k, 2^k]."""
    b = max(u.shape[0], g.shape[0])
    d = 1 << k
    ut = u.expand(b, d, d).reshape([b] + [2] * k + [d])
    axes = [1 + p for p in pos]
    rest = [a for a in range(1, k + 1) if a not in axes]
    perm = [0] + axes + rest + [k + 1]
    up = ut.permute(perm).reshape(b, 1 << len(pos), -1)
    up = torch.matmul(g.expand(b, -1, -1), up)
    up = up.reshape([b] + [2] * k + [d])
    inv = [0] * len(perm)
    for i, p in enumerate(perm):
        inv[p] = i
    return up.permute(inv).reshape(b, d, d)


def build_block_unitary(ops: Sequence[engine.TapeOp], block_wires: List[int], device) -> torch.Tensor:
    """Product of the block's gates, [B, 2^k, 2^k] complex128 (B = 1 or bsz)."""
    k = len(block_wires)
    u = torch.eye(1 << k, dtype=torch.complex128, device=device)[None]
    where = {w: i for i, w in enumerate(block_wires)}
    for op in ops:
        g = op_full_matrix(op, device=device)
        if g.device != device:
            g = g.to(device)
        u = _apply_rows(u, g, [where[w] for w in op.wires], k)
    return u


TC_MIN_WIRES = 13     # the tensor-core kernel tiles 128 columns of 2^(n-6)
TC_MIN_BLOCK = 4      # narrower blocks are cheaper on the CUDA-core kernels


def use_tensor_cores(qdev, width: int) -> bool:
    backend = getattr(qdev, "fused_backend", "auto")
    if backend == "cuda" or qdev.n_wires < TC_MIN_WIRES:
        return False
    return width >= (1 if backend == "tc" else TC_MIN_BLOCK)


def _pad_wires(bwires: List[int], n: int) -> List[int]:
    """Extend a block to 6 wires with identity wires (lowest-numbered free wires)."""
    extra = [w for w in range(n) if w not in bwires][:6 - len(bwires)]
    return sorted(bwires + extra)
