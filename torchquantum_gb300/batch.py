"""Persistent batches of many independent circuits of different sizes on one GPU.

Upstream runs such a batch as a Python loop over circuits, each gate a torch bmm
(functional/gate_wrapper.py:96-140).  Here a batch is compiled to a compact op list
(C ABI ``tqk_batch_op``: dense 1-qubit, controlled 1-qubit, CZ, CZ ladder), planned on
the host into shared-memory tile passes (``tqk_batch_plan``, tiles of 2^tile_bits
amplitudes), listed as (circuit, pass, tile) work items (``tqk_batch_items``) and
executed by one persistent kernel (``tqk_batch_run``): circuits with n <= tile_bits are
one item and live entirely in shared memory; the tiles of a larger circuit's pass run on
many SMs at once and its state is streamed once per pass.  The launch shape (tile size,
threads, CTAs per SM) is a ``BatchConfig``, picked by ``autotune.tune_batch`` when
``config="auto"``; ``PreparedBatch`` keeps a compiled batch on the device and replays it
from a CUDA graph.  Outputs: <Z> on one wire per circuit, each circuit's completion time
(for latency percentiles) and, on request, the final states.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from . import gates as G

OP_T = np.dtype([("kind", "<i4"), ("w0", "<i4"), ("w1", "<i4"), ("mat", "<i4")])
CIRC_T = np.dtype([("n", "<i4"), ("z_wire", "<i4"), ("first_op", "<i4"), ("num_ops", "<i4"), ("state_off", "<i8"),
                   ("first_pass", "<i4"), ("num_passes", "<i4")])
PASS_T = np.dtype([("first_op", "<i4"), ("num_ops", "<i4"), ("tile_mask", "<u4"), ("flags", "<i4")])
ITEM_T = np.dtype([("circuit", "<i4"), ("pass", "<i4"), ("tile", "<i4"), ("pad", "<i4")])
CONFIG_T = np.dtype([("tile_bits", "<i4"), ("threads", "<i4"), ("ctas_per_sm", "<i4"), ("pad", "<i4")])
DENSE1, CTRL1, CZ, CZ_LADDER = 0, 1, 2, 3
TILE_BITS = 14            # default (and largest) tile: 2^14 amplitudes = 128 KB of shared memory
MIN_TILE_BITS = 10
MAX_QUBITS = 24
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)


@dataclass(frozen=True)
class BatchConfig:
    """Launch shape of a circuit batch: shared-memory tile of 2^tile_bits amplitudes
    (circuits with n <= tile_bits run in one tile), threads per CTA and persistent CTAs
    per SM.  Chosen by ``autotune.tune_batch`` or given explicitly."""
    tile_bits: int = TILE_BITS
    threads: int = 512
    ctas_per_sm: int = 1

    def as_struct(self) -> np.ndarray:
        return np.array([(self.tile_bits, self.threads, self.ctas_per_sm, 0)], dtype=CONFIG_T)


DEFAULT_CONFIG = BatchConfig()


@dataclass
class BatchResult:
    z: np.ndarray                        # <Z_{z_wire}> per circuit (float64), in the order added
    latency_ms: np.ndarray               # completion time of each circuit after the launch started
    kernel_ms: float                     # device time of the launch (CUDA events)
    states: Optional[List[torch.Tensor]]  # final states (complex64 [2^n]) if requested


def layered_matrices(n: int, ry: np.ndarray, rz: np.ndarray) -> np.ndarray:
    """The [L * n, 2, 2] matrices RZ(rz[l, w]) RY(ry[l, w]) of ``add_layered`` (row-major
    over (layer, wire)); also what ``PreparedBatch.set_matrices`` takes for new angles."""
    ry = np.asarray(ry, np.float64).reshape(-1, n)
    rz = np.asarray(rz, np.float64).reshape(-1, n)
    c, s = np.cos(ry / 2), np.sin(ry / 2)
    em, ep = np.exp(-0.5j * rz), np.exp(0.5j * rz)
    m = np.empty(ry.shape + (2, 2), dtype=np.complex128)
    m[..., 0, 0], m[..., 0, 1] = em * c, -em * s
    m[..., 1, 0], m[..., 1, 1] = ep * s, ep * c
    return m.reshape(-1, 2, 2)


class CircuitBatch:
    """Collects circuits (``add_gates`` / ``add_layered``), then ``run`` executes them all
    with one persistent kernel launch."""

    def __init__(self):
        self._n: List[int] = []
        self._z: List[int] = []
        self._ops: List[np.ndarray] = []
        self._mats: List[np.ndarray] = []

    def __len__(self):
        return len(self._n)

    # ------------------------------------------------------------------ building
    def add_ops(self, n: int, ops: np.ndarray, mats: np.ndarray, z_wire: int = 0) -> int:
        """A circuit in the IR: ``ops`` (OP_T, ``mat`` indexes ``mats`` [m, 2, 2])."""
        if not 1 <= n <= MAX_QUBITS:
            raise ValueError(f"n_wires must be in 1..{MAX_QUBITS} (got {n})")
        self._n.append(int(n))
        self._z.append(int(z_wire))
        self._ops.append(np.asarray(ops, dtype=OP_T))
        self._mats.append(np.asarray(mats, dtype=np.complex64).reshape(-1, 2, 2))
        return len(self._n) - 1

    def add_gates(self, n: int, gates: Sequence[Dict], z_wire: int = 0) -> int:
        """A circuit as a gate list ``{name, wires, params[, inverse]}`` (params: P reals,
        a scalar or None; wires: a list or one int) -- the format of a device's
        ``op_history`` (upstream functional/gate_wrapper.py:380-391), so a recorded
        circuit can be replayed in a batch.  Consecutive one-qubit gates on a wire are
        fused into one 2x2 matrix; controlled one-qubit gates, CNOT and controlled
        phases use their lower-right 2x2 block; CZ becomes a diagonal op."""
        pending: Dict[int, np.ndarray] = {}
        ops, mats = [], []

        def emit(kind, w0, w1=0, m=None):
            idx = -1
            if m is not None:
                mats.append(m)
                idx = len(mats) - 1
            ops.append((kind, w0, w1, idx))

        def flush(w):
            m = pending.pop(w, None)
            if m is not None:
                emit(DENSE1, w, 0, m)

        for g in gates:
            name = G.canonical_name(g["name"])
            wires = [int(w) for w in np.atleast_1d(g["wires"])]
            gd = G.GATES[name]
            p = g.get("params")
            if p is not None and np.asarray(p).ndim > 1 and np.asarray(p).shape[0] > 1:
                raise ValueError(f"gate {name}: a batch circuit takes one parameter row (got {np.asarray(p).shape})")
            pt = None if p is None else torch.tensor(np.asarray(p, np.float64).reshape(1, -1))
            mat = G.gate_matrix(name, pt, len(wires), dtype=torch.complex128)[0].numpy()
            if g.get("inverse"):
                mat = mat.conj().T
            if len(wires) == 1:
                pending[wires[0]] = mat @ pending.get(wires[0], np.eye(2))
                continue
            if len(wires) != 2 or gd.struct[0] not in ("ctrl", "x", "phase", "diag", "dense"):
                raise ValueError(f"gate {name} on {len(wires)} wires is not supported in a circuit batch")
            for w in wires:
                flush(w)
            off = mat.copy()
            off[2:, 2:] = 0
            if np.abs(off - np.eye(4) * np.array([1, 1, 0, 0])).max() > 1e-12:
                raise ValueError(f"gate {name} is not a controlled one-qubit gate")
            sub = mat[2:, 2:]
            if np.abs(sub - np.diag([1, -1])).max() < 1e-12:
                emit(CZ, wires[0], wires[1])
            else:
                emit(CTRL1, wires[0], wires[1], sub)
        for w in sorted(pending):
            flush(w)
        arr = np.array(ops, dtype=OP_T) if ops else np.zeros(0, dtype=OP_T)
        return self.add_ops(n, arr, np.array(mats) if mats else np.zeros((0, 2, 2)), z_wire)

    def add_layered(self, n: int, ry: np.ndarray, rz: np.ndarray, z_wire: int = 0) -> int:
        """L layers of (RY(ry[l, w]), RZ(rz[l, w]) on every wire w, then CZ(w, w+1) for
        w = 0..n-2): one fused 2x2 per (layer, wire) and one CZ-ladder op per layer."""
        m = layered_matrices(n, ry, rz)
        L = m.shape[0] // n
        per = n + (1 if n >= 2 else 0)
        ops = np.zeros(L * per, dtype=OP_T)
        ops = ops.reshape(L, per)
        ops["kind"][:, :n] = DENSE1
        ops["w0"][:, :n] = np.arange(n)[None, :]
        ops["mat"][:, :n] = np.arange(L * n).reshape(L, n)
        if n >= 2:
            ops["kind"][:, n] = CZ_LADDER
            ops["w0"][:, n] = 0
            ops["w1"][:, n] = n - 1
            ops["mat"][:, n] = -1
        return self.add_ops(n, ops.reshape(-1), m, z_wire)

    # ------------------------------------------------------------------ execution
    def signature(self) -> tuple:
        """Coarse shape of the batch (for the autotuner's cache): circuit count and
        per-width-band counts and work, bucketed by powers of two."""
        def b2(x):
            return int(np.log2(max(1, x)))
        bands = [(1, 10), (11, 12), (13, 14), (15, 17), (18, 20), (21, 24)]
        sig = [b2(len(self._n))]
        for lo, hi in bands:
            idx = [i for i, n in enumerate(self._n) if lo <= n <= hi]
            work = sum(len(self._ops[i]) << self._n[i] for i in idx)
            sig += [b2(len(idx) + 1), b2(work + 1)]
        return tuple(sig)

    def compile(self, return_states: bool = False, tile_bits: int = TILE_BITS):
        """Host tables in execution order (costly circuits first): circuits, planned ops,
        passes, work items, matrices, the execution order and the state buffer size
        (amplitudes), for tiles of 2^tile_bits amplitudes."""
        nc = len(self._n)
        cost = [len(o) * (1 << n) for o, n in zip(self._ops, self._n)]
        order = sorted(range(nc), key=lambda i: -cost[i])
        circ = np.zeros(nc, dtype=CIRC_T)
        ops_l, mats_l = [], []
        nops = nmats = 0
        state_amps = 0
        for slot, i in enumerate(order):
            n = self._n[i]
            o = self._ops[i].copy()
            o["mat"] = np.where(o["mat"] >= 0, o["mat"] + nmats, -1)
            circ[slot] = (n, self._z[i], nops, len(o), -1, 0, 0)
            if return_states or n > tile_bits:
                circ[slot]["state_off"] = state_amps
                state_amps += 1 << n
            ops_l.append(o)
            mats_l.append(self._mats[i])
            nops += len(o)
            nmats += len(self._mats[i])
        ops_in = np.concatenate(ops_l) if ops_l else np.zeros(0, OP_T)
        mats = np.concatenate(mats_l).astype(np.complex64) if mats_l else np.zeros((0, 2, 2), np.complex64)
        ops_out = np.zeros_like(ops_in)
        max_passes = len(ops_in) + nc
        passes = np.zeros(max(1, max_passes), dtype=PASS_T)
        lib = _lib.load()
        npass = lib.tqk_batch_plan(circ.ctypes.data, nc, ops_in.ctypes.data if len(ops_in) else None, len(mats),
                                   ops_out.ctypes.data if len(ops_out) else None, passes.ctypes.data, max_passes,
                                   int(tile_bits))
        if npass < 0:
            raise _lib.TQKError(-npass, lib.tqk_last_error().decode())
        passes = passes[:npass]
        n_items = sum(1 << (int(c["n"]) - bin(int(p["tile_mask"])).count("1"))
                      for c in circ for p in passes[c["first_pass"]:c["first_pass"] + c["num_passes"]])
        items = np.zeros(max(1, n_items), dtype=ITEM_T)
        got = lib.tqk_batch_items(circ.ctypes.data, nc, passes.ctypes.data, items.ctypes.data, n_items)
        if got < 0:
            raise _lib.TQKError(-got, lib.tqk_last_error().decode())
        return circ, ops_out, passes, items[:got], mats, order, state_amps

    def prepare(self, device=None, return_states: bool = False, config=None) -> "PreparedBatch":
        """Compile and upload the batch once; the result launches (or replays a CUDA graph
        of) the persistent kernel any number of times.  ``config``: a ``BatchConfig``,
        ``"auto"`` (the autotuner's choice, measured on this device and cached) or None
        (defaults)."""
        dev = torch.device(device if device is not None else "cuda")
        if dev.type != "cuda":
            raise _lib.TQKError(8, "circuit batches run on a CUDA device only")
        if isinstance(config, str):
            if config != "auto":
                raise ValueError(f"config must be a BatchConfig, 'auto' or None (got {config!r})")
            from . import autotune

            config = autotune.tune_batch(self, dev, return_states)
        return PreparedBatch(self, dev, return_states, config or DEFAULT_CONFIG)

    def run(self, device=None, return_states: bool = False, config=None) -> BatchResult:
        """Compile, upload and launch once (see ``prepare`` for repeated launches)."""
        if len(self._n) == 0:
            return BatchResult(np.zeros(0), np.zeros(0), 0.0, [] if return_states else None)
        pb = self.prepare(device, return_states, config)
        pb.launch()
        return pb.result()


class PreparedBatch:
    """A compiled batch resident on the device: tables, matrices, state and output
    buffers.  ``launch`` zeroes the per-launch counters and starts the persistent kernel
    on the current stream; ``capture`` records that into a CUDA graph which ``replay``
    re-launches with one call; ``set_matrices`` rewrites the gate matrices in place
    (same circuit structure, new angles) between launches."""

    def __init__(self, cb: CircuitBatch, dev: torch.device, return_states: bool, config: BatchConfig):
        self.n = list(cb._n)
        self.ncirc = len(self.n)
        self.device = dev
        self.config = config
        self.return_states = return_states
        circ, ops, passes, items, mats, order, state_amps = cb.compile(return_states, config.tile_bits)
        self.circ, self.order, self.n_items = circ, order, len(items)
        self.mat_counts = [len(cb._mats[i]) for i in order]

        def up(a):
            return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).to(dev)

        self.d_circ, self.d_pass, self.d_items = up(circ), up(passes), up(items)
        self.d_ops = up(ops if len(ops) else np.zeros(1, OP_T))
        self.d_mats = up(mats if len(mats) else np.zeros((1, 2, 2), np.complex64))
        self.d_cfg = config.as_struct()  # host struct, read by the launch call
        self.states = torch.empty(max(1, state_amps), dtype=torch.complex64, device=dev)
        self.z = torch.zeros(self.ncirc, dtype=torch.float64, device=dev)
        self.pass_done = torch.zeros(max(1, len(passes)), dtype=torch.int32, device=dev)
        self.t_done = torch.zeros(self.ncirc + 1, dtype=torch.int64, device=dev)
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
        self.status = _lib.status_word(dev)
        self.graph = None
        self.kernel_ms = 0.0
        self._ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))

    def _enqueue(self, stream) -> None:
        self.z.zero_()
        self.pass_done.zero_()
        self.counter.zero_()
        _lib._check(_lib.load().tqk_batch_run(
            self.d_circ.data_ptr(), self.ncirc, self.d_ops.data_ptr(), self.d_pass.data_ptr(),
            self.d_items.data_ptr(), self.n_items, self.d_mats.data_ptr(), self.states.data_ptr(),
            int(self.return_states), self.z.data_ptr(), self.pass_done.data_ptr(), self.t_done.data_ptr(),
            self.counter.data_ptr(), self.status.data_ptr(), self.d_cfg.ctypes.data, stream.cuda_stream))

    def launch(self) -> None:
        """Zero the counters and launch the persistent kernel (device-timed)."""
        stream = torch.cuda.current_stream(self.device)
        _lib.nvtx_push(f"tqk.batch.launch[{self.ncirc} circuits]")
        self._ev[0].record(stream)
        if self.graph is not None:
            self.graph.replay()
        else:
            self._enqueue(stream)
        self._ev[1].record(stream)
        _lib.nvtx_pop()

    def capture(self) -> "PreparedBatch":
        """Record the counter resets and the kernel launch into a CUDA graph; later
        ``launch`` calls replay it.  A first uncaptured launch is made here so that the
        kernel's one-time device setup happens outside the capture."""
        if self.graph is not None:
            return self
        with torch.cuda.device(self.device):
            self.launch()
            torch.cuda.synchronize(self.device)
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(self.device)
            side.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side):
                    self._enqueue(side)
            torch.cuda.current_stream(self.device).wait_stream(side)
            self.graph = g
        return self

    def set_matrices(self, mats: np.ndarray) -> None:
        """New 2x2 matrices for every circuit, in the order the circuits were added
        (the concatenation of each circuit's matrix list, same counts as before)."""
        mats = np.asarray(mats, dtype=np.complex64).reshape(-1, 2, 2)
        if len(mats) != sum(self.mat_counts):
            raise ValueError(f"expected {sum(self.mat_counts)} matrices, got {len(mats)}")
        starts = np.concatenate([[0], np.cumsum([self.mat_counts[self.order.index(i)] for i in range(self.ncirc)])])
        parts = [mats[starts[i]:starts[i + 1]] for i in self.order]
        flat = np.concatenate(parts) if parts else mats
        src = torch.from_numpy(np.ascontiguousarray(flat).view(np.uint8).reshape(-1))
        self.d_mats[:src.numel()].copy_(src.pin_memory(), non_blocking=True)

    def result(self) -> BatchResult:
        """Wait for the last launch and gather <Z>, latencies and (optionally) states."""
        zh = self.z.cpu().numpy()
        th = self.t_done.cpu().numpy()
        _lib.check_status(self.device)
        self.kernel_ms = self._ev[0].elapsed_time(self._ev[1])
        nc = self.ncirc
        out_z = np.empty(nc)
        lat = np.empty(nc)
        for slot, i in enumerate(self.order):
            out_z[i] = zh[slot]
            lat[i] = (th[slot] - th[nc]) / 1e6
        out_states = None
        if self.return_states:
            out_states = [None] * nc
            for slot, i in enumerate(self.order):
                off = int(self.circ[slot]["state_off"])
                out_states[i] = self.states[off:off + (1 << self.n[i])].clone()
        return BatchResult(out_z, lat, self.kernel_ms, out_states)
