"""Autotuner: launch shapes and fusion plans chosen from measurements on the device.

Two decisions are tuned, each measured once per GPU and workload shape and cached in a
JSON file (``$TQ_GB300_TUNE_CACHE``, default ``~/.cache/torchquantum_gb300/tune.json``;
set ``TQ_GB300_TUNE_CACHE=off`` to keep the cache in memory only):

* Circuit batches (``tune_batch``): the shared-memory tile size (2^10..2^14 amplitudes,
  which also decides how many passes a wide circuit needs), threads per CTA and
  persistent CTAs per SM.  Every candidate runs the actual batch (a warm launch, then the
  best of three CUDA-event-timed launches); the fastest wins.  Key: GPU and the batch's
  coarse signature (circuit count and per-width-band count and work, log2 buckets).
* Fused segments (``choose_fusion``): the fusion width k (4, 5 or 6 wires), the planner
  variant (first-gate seed, lookahead seeds, or a width-4 beam search) and, per block, the tensor-core kernel or
  the CUDA-core dense kernel.  Per-pass costs of every kernel the plan can use (forward
  and adjoint step of a tensor-core block, dense k-wire kernels for k = 1..6) are timed
  on a scratch state of the segment's width (``pass_costs``); each candidate plan is
  scored by the sum of its passes' costs (adjoint steps included when the segment has
  trainable inputs) and the cheapest is used.  Key: GPU, n_wires, batch size.

Qubit order: every kernel here takes its target bits where they are (the tensor-core
kernel maps any six wires onto its tiles), so no qubit-reordering pass is scheduled.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib

_LOCK = threading.Lock()
_MEM: Dict[str, dict] = {}
_LOADED = False


def _cache_path() -> Optional[str]:
    p = os.environ.get("TQ_GB300_TUNE_CACHE")
    if p == "off":
        return None
    return p or os.path.join(os.path.expanduser("~"), ".cache", "torchquantum_gb300", "tune.json")


def _load() -> None:
    global _LOADED
    if _LOADED:
        return
    _LOADED = True
    path = _cache_path()
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                _MEM.update(json.load(f))
        except (OSError, ValueError):
            pass


def _store(key: str, value: dict) -> None:
    with _LOCK:
        _MEM[key] = value
        path = _cache_path()
        if not path:
            return
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + f".{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(_MEM, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass


def lookup(key: str) -> Optional[dict]:
    with _LOCK:
        _load()
        return _MEM.get(key)


def clear(memory_only: bool = True) -> None:
    """Forget tuned results (in memory; also the cache file when ``memory_only`` is False)."""
    global _LOADED
    with _LOCK:
        _MEM.clear()
        _LOADED = memory_only
        path = _cache_path()
        if not memory_only and path and os.path.exists(path):
            os.remove(path)


def gpu_key(dev: torch.device) -> str:
    p = torch.cuda.get_device_properties(dev)
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"


def _time_ms(fn, dev, reps: int = 3) -> float:
    """Best of ``reps`` CUDA-event timings of ``fn`` on the current stream (after one warm call)."""
    stream = torch.cuda.current_stream(dev)
    fn()
    best = float("inf")
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return best


# ------------------------------------------------------------------ circuit batches
def batch_candidates(max_n: int):
    from .batch import BatchConfig

    cands = [BatchConfig(14, 512, 1), BatchConfig(13, 512, 1), BatchConfig(13, 256, 3), BatchConfig(12, 256, 4),
             BatchConfig(12, 128, 6), BatchConfig(11, 128, 8)]
    # a tile wider than every circuit only wastes shared memory
    narrow = [c for c in cands if c.tile_bits <= max(max_n, 11)]
    return narrow or cands[-1:]


def tune_batch(cb, dev: torch.device, return_states: bool = False):
    """Best ``BatchConfig`` for ``cb`` on ``dev`` (measured, cached)."""
    from .batch import BatchConfig

    key = f"batch|{gpu_key(dev)}|{','.join(map(str, cb.signature()))}|{int(return_states)}"
    hit = lookup(key)
    if hit is not None:
        return BatchConfig(**hit["config"])
    timings = []
    for cfg in batch_candidates(max(cb._n)):
        pb = cb.prepare(dev, return_states, cfg)

        def go(pb=pb):
            pb.launch()

        ms = _time_ms(go, dev)
        pb.result()  # surfaces any device-side error of this candidate
        timings.append((ms, cfg))
        del pb
    ms, best = min(timings, key=lambda t: t[0])
    _store(key, {"config": {"tile_bits": best.tile_bits, "threads": best.threads, "ctas_per_sm": best.ctas_per_sm},
                 "ms": ms, "tried": [[t[1].tile_bits, t[1].threads, t[1].ctas_per_sm, t[0]] for t in timings]})
    return best


# ------------------------------------------------------------------ fused segments
SCRATCH_AMPS = 1 << 27   # cost probes run on at most 2^27 amplitudes (1 GiB) per state buffer


def pass_costs(n: int, bsz: int, dev: torch.device, tc_ok: bool) -> dict:
    """Measured milliseconds per pass over a [bsz, 2^n] state: ``dense[k] = (fwd, adj)``
    for the CUDA-core dense k-wire kernels (k = 1..min(6, n)), ``light = (fwd, adj)`` for a
    structured two-wire gate without a cotangent (CNOT; its reverse step moves psi and
    lam) and ``tc = (fwd, adj, adj_stored)`` for the tensor-core 6-wire block kernel (if
    ``tc_ok``; adj_stored: the reverse step that reads the block's stored input).  Probes
    use min(bsz, rows that fit 2^27 amplitudes) rows and are scaled to bsz (the kernels
    stream rows independently)."""
    key = f"fusion3|{gpu_key(dev)}|n{n}|b{bsz}|tc{int(tc_ok)}"
    hit = lookup(key)
    if hit is not None:
        return hit
    _lib.nvtx_push(f"tqk.autotune.pass_costs[n={n},bsz={bsz}]")
    try:
        return _pass_costs(n, bsz, dev, tc_ok, key)
    finally:
        _lib.nvtx_pop()


def _pass_costs(n: int, bsz: int, dev: torch.device, tc_ok: bool, key: str) -> dict:
    rows = max(1, min(bsz, SCRATCH_AMPS >> n))
    scale = bsz / rows
    psi = torch.zeros(rows, 1 << n, dtype=torch.complex64, device=dev)
    psi[:, 0] = 1
    lam = psi.clone()
    rng = np.random.default_rng(0)
    out = {"dense": {}, "tc": None, "rows": rows}
    layouts = lambda k: [list(range(k)), list(range(n - k, n))]  # high bits, low bits
    for k in range(1, min(6, n) + 1):
        d = 1 << k
        z = rng.normal(size=(rows, d, d)) + 1j * rng.normal(size=(rows, d, d))
        u = torch.tensor(np.linalg.qr(z)[0], dtype=torch.complex64, device=dev)
        grad = torch.zeros(rows * d * d * 2, dtype=torch.float64, device=dev)
        f = a = 0.0
        for wires in layouts(k):
            f += _time_ms(lambda: _lib.apply_matrix(psi, n, wires, u, rows), dev)
            a += _time_ms(lambda: _lib.adjoint_matrix(psi, lam, n, wires, u, rows, grad), dev)
        out["dense"][str(k)] = (f / 2 * scale, a / 2 * scale)
    if n >= 2:
        f = 0.0
        for c, t in ((0, 1), (n - 2, n - 1)):
            f += _time_ms(lambda: _lib.apply_mcx(psi, n, [c], 1, t), dev)
        out["light"] = (f / 2 * scale, f * scale)
    if tc_ok and n >= 6:
        z = rng.normal(size=(rows, 64, 64)) + 1j * rng.normal(size=(rows, 64, 64))
        u = torch.tensor(np.linalg.qr(z)[0], dtype=torch.complex128, device=dev)
        uh = u.conj().transpose(-1, -2).contiguous()
        mr = torch.zeros(rows, 128, 128, dtype=torch.float64, device=dev)
        f = a = s = 0.0
        for wires in layouts(6):
            img, imgh = _lib.fused_prepare(u, wires), _lib.fused_prepare(uh, wires)
            f += _time_ms(lambda: _lib.fused_apply(psi, n, wires, img, rows), dev)
            a += _time_ms(lambda: _lib.fused_adjoint(psi, lam, n, wires, imgh, rows, mr), dev)
            s += _time_ms(lambda: _lib.fused_adjoint_stored(psi, lam, n, wires, imgh, rows, mr), dev)
        out["tc"] = (f / 2 * scale, a / 2 * scale, s / 2 * scale)
    _lib.check_status(dev)
    del psi, lam
    _store(key, out)
    return out


LONE_OTHER, LONE_DENSE, LONE_LIGHT = 0, 1, 2


def plan_cost(plan, costs: dict, tc_ok: bool, with_adjoint: bool, stored: bool = False,
              lone_kind: Optional[Sequence[int]] = None) -> Tuple[float, List[bool]]:
    """(cost in ms, per-block use of the tensor-core kernel) of a fusion plan; ``stored``:
    tensor-core blocks keep their inputs, so their reverse step is the stored-input one.
    A gate alone in its block runs on its own kernel, costed as a dense pass of its width,
    unless ``lone_kind[i]`` says otherwise: LONE_DENSE (a dense or controlled gate, whose
    own kernel is a dense pass with a cotangent) may run as a tensor-core block when that
    costs less; LONE_LIGHT (controlled-X, swap, phase, diagonal: structured kernels without
    a cotangent) is costed as the measured ``light`` pass."""
    total = 0.0
    tc_flags = []
    tcc = costs.get("tc") if tc_ok else None
    ct = float("inf")
    if tcc:
        adj = tcc[2] if stored and len(tcc) > 2 else tcc[1]
        ct = tcc[0] + (adj if with_adjoint else 0.0)
    for bwires, idxs in plan:
        k = len(bwires)
        dense = costs["dense"].get(str(min(k, 6)))
        cd = (dense[0] + (dense[1] if with_adjoint else 0.0)) if dense else float("inf")
        if len(idxs) == 1:  # a lone gate: its own kernel (about a dense pass of its width)
            kind = lone_kind[idxs[0]] if lone_kind is not None else LONE_OTHER
            light = costs.get("light")
            if kind == LONE_DENSE and k <= 6 and ct < cd:
                total += ct
                tc_flags.append(True)
                continue
            if kind == LONE_LIGHT and light:
                cd = light[0] + (light[1] if with_adjoint else 0.0)
            total += cd if dense else 0.0
            tc_flags.append(False)
            continue
        if k > 6:
            cd = float("inf")
        use_tc = ct < cd
        total += min(ct, cd)
        tc_flags.append(use_tc)
    return total, tc_flags


# (lookahead, beam width) of the wide beams tried for 6-wire blocks on large states
WIDE_BEAMS = ((8, 32), (16, 128))
WIDE_BEAM_MIN_AMPS = 1 << 27


def choose_fusion(wire_lists: Sequence[Sequence[int]], n: int, bsz: int, dev: torch.device, tc_ok: bool,
                  with_adjoint: bool, widths: Sequence[int] = (4, 5, 6), stored: bool = False,
                  lone_kind: Optional[Sequence[int]] = None):
    """(plan, per-block tensor-core flags, chosen width, cost table) for a segment: the
    cheapest of the candidate plans under the measured per-pass costs (``stored``: the
    tensor-core blocks are expected to keep their inputs for the backward; ``lone_kind``:
    see ``plan_cost``)."""
    from . import fusion

    try:
        costs = pass_costs(n, bsz, dev, tc_ok)
    except torch.cuda.OutOfMemoryError:
        # no room for the probe states: rank plans by pass count with the static kernel
        # rule (tensor cores for multi-gate blocks when allowed) instead of measured costs
        torch.cuda.empty_cache()
        costs = {"dense": {str(k): (1.0 + 0.25 * k, 2.0 + 0.5 * k) for k in range(1, 7)},
                 "tc": (1.0, 2.0, 1.5) if tc_ok else None, "rows": 0}
    best = None
    # on large states (a pass of >= 1 GiB) wide beams are tried too for 6-wire blocks
    # (width 32, and width 128 with a 16-gate front): they plan once per circuit structure
    # (about 1 s and 4-6 s for 400 gates, memoised) and find one to three blocks fewer per
    # 400 gates, each worth a full forward and reverse pass
    wide = (bsz << n) >= WIDE_BEAM_MIN_AMPS and len(wire_lists) <= fusion.BEAM_MAX_GATES
    for k in widths:
        k = max(1, min(k, n, 6))
        variants = ((0, 0), (8, 0), (8, 4)) + (WIDE_BEAMS if wide and k == 6 else ())
        for look, beam in variants:
            plan = fusion.plan_cached(wire_lists, k, look, beam)
            cost, flags = plan_cost(plan, costs, tc_ok, with_adjoint, stored, lone_kind)
            if best is None or cost < best[0]:
                best = (cost, plan, flags, k)
    return best[1], best[2], best[3], costs
