"""ctypes binding of libtqk.so (C ABI declared in include/tqk.h).

The library is loaded from the package directory; if it is missing the import of
any engine function raises -- there is no CPU fallback.  Every wrapper raises
``TQKError`` (a ``RuntimeError``) carrying the library's message when a call
returns a non-zero status.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Optional, Sequence

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libtqk.so")
HEADER = os.path.join(os.path.dirname(_PKG), "include", "tqk.h")

TQK_STATUS = {
    0: "OK", 1: "BAD_WIRES", 2: "BAD_SHAPE", 3: "BAD_POINTER", 4: "TOO_MANY_QUBITS",
    5: "CUDA_ERROR", 6: "TIMEOUT", 7: "SCRATCH_TOO_SMALL", 8: "UNSUPPORTED",
}


class TQKError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{TQK_STATUS.get(code, code)}] {msg}")
        self.code = code


_i32p = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
# tqk_exec_hook: (op index, op kind, after, user)
EXEC_HOOK = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p)

_SIGS = {
    "tqk_last_error": (ctypes.c_char_p, []),
    "tqk_version": (_int, []),
    "tqk_apply_matrix": (_int, [_vp, _i64, _int, _i32p, _int, _vp, _i64, _vp]),
    "tqk_apply_controlled": (_int, [_vp, _i64, _int, _i32p, _int, _i32p, _int, _vp, _i64, _vp]),
    "tqk_apply_mcx": (_int, [_vp, _i64, _int, _i32p, _int, _int, _int, _vp]),
    "tqk_apply_phase": (_int, [_vp, _i64, _int, _i32p, _int, _vp, _i64, _vp]),
    "tqk_apply_diagonal": (_int, [_vp, _i64, _int, _i32p, _int, _vp, _i64, _vp]),
    "tqk_apply_swap": (_int, [_vp, _i64, _int, _i32p, _int, _int, _int, _vp]),
    "tqk_reset_scratch_bytes": (_i64, [_i64, _int]),
    "tqk_reset": (_int, [_vp, _i64, _int, _i32p, _int, _vp, _i64, _vp]),
    "tqk_probs": (_int, [_vp, _i64, _int, _vp, _vp]),
    "tqk_pauli_expval_scratch_bytes": (_i64, [_i64, _int, _int]),
    "tqk_pauli_expval": (_int, [_vp, _i64, _int, _u64p, _u64p, _int, _vp, _vp, _i64, _vp, _vp]),
    "tqk_pauli_apply_sum": (_int, [_vp, _i64, _int, _u64p, _u64p, _int, _vp, _vp, _vp, _vp]),
    "tqk_adjoint_matrix": (_int, [_vp, _vp, _i64, _int, _i32p, _int, _vp, _i64, _vp, _vp, _vp]),
    "tqk_adjoint_controlled": (_int, [_vp, _vp, _i64, _int, _i32p, _int, _i32p, _int, _vp, _i64, _vp, _vp, _vp]),
    "tqk_adjoint_phase": (_int, [_vp, _vp, _i64, _int, _i32p, _int, _vp, _i64, _vp, _vp]),
    "tqk_adjoint_diagonal": (_int, [_vp, _vp, _i64, _int, _i32p, _int, _vp, _i64, _vp, _vp]),
    "tqk_fused_image_bytes": (_i64, [_i64]),
    "tqk_fused_prepare": (_int, [_vp, _i64, _vp, _vp, _vp]),
    "tqk_fused_prepare_adjoint": (_int, [_vp, _i64, _vp, _vp, _vp]),
    "tqk_fused_cross_grad": (_int, [_vp, _vp, _i64, _vp, _vp]),
    "tqk_fused_prepare_many": (_int, [_vp, _int, _i64, _vp]),
    "tqk_fused_cross_add_many": (_int, [_vp, _int, _i64, _vp]),
    "tqk_sample_scratch_bytes": (_i64, [_i64, _int]),
    "tqk_sample": (_int, [_vp, _i64, _int, _vp, _i64, _vp, _vp, _i64, _vp]),
    "tqk_staged_apply": (_int, [_vp, _i64, _int, _vp, _int, _int, _vp, _vp]),
    "tqk_staged_adjoint": (_int, [_vp, _vp, _i64, _int, _vp, _int, _int, _vp, _vp]),
    "tqk_batch_plan": (_int, [_vp, _int, _vp, _int, _vp, _vp, _int, _int]),
    "tqk_batch_items": (_i64, [_vp, _int, _vp, _vp, _i64]),
    "tqk_batch_run": (_int, [_vp, _int, _vp, _vp, _vp, _i64, _vp, _vp, _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "tqk_fused_apply": (_int, [_vp, _i64, _int, _i32p, _vp, _i64, _vp, _vp]),
    "tqk_fused_adjoint": (_int, [_vp, _vp, _i64, _int, _i32p, _vp, _i64, _vp, _vp, _vp]),
    "tqk_fused_apply_to": (_int, [_vp, _vp, _i64, _int, _i32p, _vp, _i64, _vp, _vp]),
    "tqk_fused_adjoint_stored": (_int, [_vp, _vp, _i64, _int, _i32p, _vp, _i64, _vp, _vp, _vp]),
    "tqk_fused_zero_input": (_int, [_vp, _i64, _int, _i32p, _vp, _i64, _vp]),
    "tqk_pauli_expval_noalloc_capacity": (_i64, []),
    "tqk_pauli_expval_noalloc": (_int, [_vp, _i64, _int, _u64p, _u64p, _int, _vp, _vp]),
    "tqk_segment_forward": (_int, [_vp, _i64, _int, _vp, _int, _vp, _vp, _vp, EXEC_HOOK, _vp, _vp]),
    "tqk_segment_backward": (_int, [_vp, _vp, _vp, _i64, _int, _vp, _int, _vp, _vp, _vp, EXEC_HOOK, _vp, _vp]),
    "tqk_gate_operand_size": (_int, [_int]),
    "tqk_gate_operands": (_int, [_vp, _int, _vp]),
    "tqk_param_grads": (_int, [_vp, _int, _vp]),
    "tqk_block_build": (_int, [_vp, _int, _int, _vp, _vp]),
    "tqk_block_unbuild": (_int, [_vp, _int, _int, _vp, _vp]),
}

_lib: Optional[ctypes.CDLL] = None

# Kernels launched by this process through the C ABI (bench.py reports the count of
# its timed region).
LAUNCHES = [0]
# NVTX ranges around segment compilation, forward and backward sweeps, batch launches
# and autotuning probes (for nsys / ncu --nvtx); off unless TQ_GB300_NVTX=1.
NVTX = os.environ.get("TQ_GB300_NVTX") == "1"


def nvtx_push(name: str) -> None:
    if NVTX:
        torch.cuda.nvtx.range_push(name)


def nvtx_pop() -> None:
    if NVTX:
        torch.cuda.nvtx.range_pop()


def _count(k: int = 1) -> None:
    LAUNCHES[0] += k


def header_symbols() -> list:
    """Function names declared in include/tqk.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(tqk_[a-z0-9_]+)\s*\(", text)))


def load() -> ctypes.CDLL:
    """Load libtqk.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python -m torchquantum_gb300.build)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int, launches: int = 1):
    if rc == 0:
        LAUNCHES[0] += launches
    if rc != 0:
        msg = load().tqk_last_error().decode(errors="replace")
        raise TQKError(rc, msg)


def _i32(vals: Sequence[int]):
    arr = (ctypes.c_int32 * max(1, len(vals)))(*vals)
    return arr


def _u64(vals: Sequence[int]):
    return (ctypes.c_uint64 * max(1, len(vals)))(*vals)


def _stream(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


# ------------------------------------------------------------------ gate application
def apply_matrix(state, n, wires, mat, mat_batch):
    _check(load().tqk_apply_matrix(state.data_ptr(), state.shape[0], n, _i32(wires), len(wires), mat.data_ptr(),
                                   mat_batch, _stream(state)))


def apply_controlled(state, n, controls, targets, mat, mat_batch):
    _check(load().tqk_apply_controlled(state.data_ptr(), state.shape[0], n, _i32(controls), len(controls),
                                       _i32(targets), len(targets), mat.data_ptr(), mat_batch, _stream(state)))


def apply_mcx(state, n, controls, ctrl_val, target):
    _check(load().tqk_apply_mcx(state.data_ptr(), state.shape[0], n, _i32(controls), len(controls), ctrl_val, target,
                                _stream(state)))


def apply_phase(state, n, wires, phase, phase_batch):
    _check(load().tqk_apply_phase(state.data_ptr(), state.shape[0], n, _i32(wires), len(wires), phase.data_ptr(),
                                  phase_batch, _stream(state)))


def apply_diagonal(state, n, wires, diag, diag_batch):
    _check(load().tqk_apply_diagonal(state.data_ptr(), state.shape[0], n, _i32(wires), len(wires), diag.data_ptr(),
                                     diag_batch, _stream(state)))


def apply_swap(state, n, controls, w0, w1):
    _check(load().tqk_apply_swap(state.data_ptr(), state.shape[0], n, _i32(controls), len(controls), w0, w1,
                                 _stream(state)))


def reset(state, n, wires):
    lib = load()
    nbytes = lib.tqk_reset_scratch_bytes(state.shape[0], n)
    scratch = torch.empty(max(8, nbytes), dtype=torch.uint8, device=state.device)
    _check(lib.tqk_reset(state.data_ptr(), state.shape[0], n, _i32(wires), len(wires), scratch.data_ptr(), nbytes,
                         _stream(state)), launches=2)


# ------------------------------------------------------------------ measurement
def probs(state, n):
    out = torch.empty(state.shape[0], 1 << n, dtype=torch.float32, device=state.device)
    _check(load().tqk_probs(state.data_ptr(), state.shape[0], n, out.data_ptr(), _stream(state)))
    return out


COSET_TILE_BITS = 13     # a coset pass stages 2^min(n, 13) amplitudes
COSET_MIN_CHUNK_BITS = 4  # in contiguous runs of at least 2^4 amplitudes
MAX_STRINGS_PER_PASS = 8


def gf2_rank(vectors) -> int:
    """Rank over GF(2) of integer bit vectors."""
    basis = []  # (pivot bit, vector), reduced
    for v in vectors:
        for piv, b in basis:
            if (v >> piv) & 1:
                v ^= b
        if v:
            q = v.bit_length() - 1
            basis = [(piv, b ^ v if (b >> q) & 1 else b) for piv, b in basis]
            basis.append((q, v))
    return len(basis)


def coset_groups(xmasks, n: int):
    """The coset passes tqk_pauli_expval (several X-masks) and tqk_pauli_apply_sum make:
    strings in order, a group growing while it holds at most 8 strings and its X-masks'
    parts above the lowest c bits span at most T - c dimensions for c = min(4, T),
    T = min(n, 13).  Returns [(string indices, c, rank)] with the widest such c."""
    T = min(n, COSET_TILE_BITS)
    cmin = min(COSET_MIN_CHUNK_BITS, T)
    groups, cur = [], []
    for j in range(len(xmasks)):
        if cur and (len(cur) == MAX_STRINGS_PER_PASS
                    or gf2_rank([xmasks[i] >> cmin for i in cur + [j]]) > T - cmin):
            groups.append(cur)
            cur = []
        cur.append(j)
    if cur:
        groups.append(cur)
    out = []
    for g in groups:
        c = cmin
        while c < T and gf2_rank([xmasks[i] >> (c + 1) for i in g]) <= T - (c + 1):
            c += 1
        out.append((g, c, gf2_rank([xmasks[i] >> c for i in g])))
    return out


def expval_passes(xmasks, n: int = 64) -> int:
    """Passes tqk_pauli_expval makes: with several X-masks one coset pass per group
    (``coset_groups``); with one X-mask for all strings, one pass per 8 strings."""
    if len(set(xmasks)) > 1:
        return len(coset_groups(list(xmasks), n))
    return (len(xmasks) + 7) // 8


def pauli_expval(state, n, xmasks, zmasks):
    """[bsz, m] float64 expvals of m Pauli strings given by masks."""
    lib = load()
    m = len(xmasks)
    bsz = state.shape[0]
    out = torch.empty(bsz, m, dtype=torch.float64, device=state.device)
    nbytes = lib.tqk_pauli_expval_scratch_bytes(bsz, n, m)
    scratch = torch.empty(max(8, nbytes), dtype=torch.uint8, device=state.device)
    _check(lib.tqk_pauli_expval(state.data_ptr(), bsz, n, _u64(xmasks), _u64(zmasks), m, out.data_ptr(),
                                scratch.data_ptr(), nbytes, status_word(state.device).data_ptr(), _stream(state)),
           launches=2 * expval_passes(xmasks, n))
    return out


def pauli_apply_sum(state, n, xmasks, zmasks, coef):
    """sum_j coef[:, j] * P_j psi; coef float32 [bsz, m] (contiguous, same device)."""
    out = torch.empty_like(state)
    _check(load().tqk_pauli_apply_sum(state.data_ptr(), state.shape[0], n, _u64(xmasks), _u64(zmasks), len(xmasks),
                                      coef.data_ptr(), out.data_ptr(), status_word(state.device).data_ptr(),
                                      _stream(state)), launches=len(coset_groups(list(xmasks), n)))
    return out


# ------------------------------------------------------------------ adjoint
def adjoint_matrix(psi, lam, n, wires, mat, mat_batch, grad, uncompute=None):
    _check(load().tqk_adjoint_matrix(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, _i32(wires), len(wires),
                                     mat.data_ptr(), mat_batch, _ptr(uncompute), _ptr(grad), _stream(psi)))


def adjoint_controlled(psi, lam, n, controls, targets, mat, mat_batch, grad, uncompute=None):
    _check(load().tqk_adjoint_controlled(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, _i32(controls),
                                         len(controls), _i32(targets), len(targets), mat.data_ptr(), mat_batch,
                                         _ptr(uncompute), _ptr(grad), _stream(psi)))


def adjoint_phase(psi, lam, n, wires, phase, phase_batch, grad):
    _check(load().tqk_adjoint_phase(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, _i32(wires), len(wires),
                                    phase.data_ptr(), phase_batch, _ptr(grad), _stream(psi)))


def sample(state, n, uniforms):
    """Inverse-CDF draws: state [bsz, 2^n] complex64, uniforms [bsz, shots] float64 in
    [0, 1) -> outcome indices [bsz, shots] int64 (wire 0 = most significant bit)."""
    lib = load()
    bsz, shots = uniforms.shape
    out = torch.empty(bsz, shots, dtype=torch.int64, device=state.device)
    nbytes = lib.tqk_sample_scratch_bytes(bsz, n)
    scratch = torch.empty(max(1, nbytes // 8), dtype=torch.float64, device=state.device)
    _check(lib.tqk_sample(state.data_ptr(), bsz, n, uniforms.data_ptr(), shots, out.data_ptr(), scratch.data_ptr(),
                          nbytes, _stream(state)), launches=3)
    return out


class ImageJob(ctypes.Structure):
    """tqk_image_job: one operand image (of U, or of U^H when ``adjoint``) to build."""
    _fields_ = [("u", ctypes.c_void_p), ("image", ctypes.c_void_p), ("u_batch", ctypes.c_int64),
                ("wires", ctypes.c_int32 * 6), ("adjoint", ctypes.c_int32), ("pad", ctypes.c_int32)]


class CrossJob(ctypes.Structure):
    """tqk_cross_job: gu += M from the cross term of a stored-input adjoint step."""
    _fields_ = [("mr", ctypes.c_void_p), ("gu", ctypes.c_void_p), ("batch", ctypes.c_int64)]


assert ctypes.sizeof(ImageJob) == 56 and ctypes.sizeof(CrossJob) == 24


def fused_prepare_many(jobs_dev: torch.Tensor, njobs: int, max_u_batch: int) -> None:
    """Build njobs operand images in one launch from a device table of ImageJob records."""
    _check(load().tqk_fused_prepare_many(jobs_dev.data_ptr(), njobs, max_u_batch, _stream(jobs_dev)))


def fused_cross_add_many(jobs_dev: torch.Tensor, njobs: int, max_batch: int) -> None:
    """Add the cross terms of njobs stored-input steps into their cotangents in one launch."""
    _check(load().tqk_fused_cross_add_many(jobs_dev.data_ptr(), njobs, max_batch, _stream(jobs_dev)))


class StagedOp(ctypes.Structure):
    """``tqk_staged_op``: one op of a staged low-qubit run."""
    _fields_ = [("kind", ctypes.c_int32), ("nwires", ctypes.c_int32), ("wires", ctypes.c_int32 * 8),
                ("ctrl_val", ctypes.c_int32), ("pad", ctypes.c_int32), ("operand", ctypes.c_void_p),
                ("batch", ctypes.c_int64), ("grad", ctypes.c_void_p)]


assert ctypes.sizeof(StagedOp) == 72
S_DENSE1, S_X, S_PHASE, S_DIAG = 0, 1, 2, 3
STAGED_MAX_OPS, STAGED_MAX_TILE_BITS, STAGED_MAX_WIRES = 64, 12, 8


# ------------------------------------------------------------------ compiled segments
class ExecOp(ctypes.Structure):
    """``tqk_exec_op``: one op of a compiled segment for tqk_segment_forward / _backward."""
    _fields_ = [("kind", ctypes.c_int32), ("nw", ctypes.c_int32), ("nctrl", ctypes.c_int32),
                ("ctrl_val", ctypes.c_int32), ("wires", ctypes.c_int32 * 16), ("batch", ctypes.c_int64),
                ("operand", ctypes.c_void_p), ("uncompute", ctypes.c_void_p), ("image", ctypes.c_void_p),
                ("image_h", ctypes.c_void_p), ("u", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("stored", ctypes.c_void_p), ("grad", ctypes.c_void_p), ("mr", ctypes.c_void_p),
                ("staged", ctypes.c_void_p), ("nstaged", ctypes.c_int32), ("tile_bits", ctypes.c_int32),
                ("skip_reverse", ctypes.c_int32), ("pad", ctypes.c_int32)]


assert ctypes.sizeof(ExecOp) == 184
X_DENSE, X_CTRL, X_MCX, X_PHASE, X_DIAG, X_SWAP, X_STAGED, X_BLOCK_TC, X_BLOCK_DENSE, X_BLOCK_ZERO = range(10)
# Optional Python callables (exec record, after) the runners call around each op's
# launches, per direction (bench.py installs one to time the dominant kernel's launches
# inside a step).
SEGMENT_HOOKS = {"forward": None, "backward": None}


def _hook(which, table):
    fn = SEGMENT_HOOKS[which]
    if fn is None:
        return EXEC_HOOK()  # a NULL function pointer
    return EXEC_HOOK(lambda i, kind, after, user: fn(table[i], after))


def segment_forward(state, n, table, nops) -> int:
    """Run a host table of ``ExecOp`` forward on ``state``; returns the device address of
    the buffer holding the result."""
    final = ctypes.c_void_p()
    count = ctypes.c_int64(0)
    hook = _hook("forward", table)
    _check(load().tqk_segment_forward(state.data_ptr(), state.shape[0], n, table, nops,
                                      status_word(state.device).data_ptr(), ctypes.byref(final), ctypes.byref(count),
                                      hook, None, _stream(state)), launches=0)
    LAUNCHES[0] += count.value
    return final.value or 0


def segment_backward(psi_end, lam, work, n, table, nops) -> int:
    """Reverse sweep of a host table of ``ExecOp``; returns the device address where the
    sweep's state ended (the segment's start)."""
    start = ctypes.c_void_p()
    count = ctypes.c_int64(0)
    hook = _hook("backward", table)
    _check(load().tqk_segment_backward(psi_end.data_ptr(), lam.data_ptr(), _ptr(work), lam.shape[0], n, table, nops,
                                       status_word(lam.device).data_ptr(), ctypes.byref(start), ctypes.byref(count),
                                       hook, None, _stream(lam)), launches=0)
    LAUNCHES[0] += count.value
    return start.value or 0


def staged_apply(state, n, ops, tile_bits):
    """Apply a run of ``StagedOp`` (sequence) in one shared-memory pass."""
    arr = (StagedOp * max(1, len(ops)))(*ops)
    _check(load().tqk_staged_apply(state.data_ptr(), state.shape[0], n, arr, len(ops), tile_bits,
                                   status_word(state.device).data_ptr(), _stream(state)))


def staged_adjoint(psi, lam, n, ops, tile_bits):
    """Reverse step of a staged run on (psi, lam); ops carry their cotangent slots."""
    arr = (StagedOp * max(1, len(ops)))(*ops)
    _check(load().tqk_staged_adjoint(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, arr, len(ops), tile_bits,
                                     status_word(psi.device).data_ptr(), _stream(psi)))


def adjoint_diagonal(psi, lam, n, wires, diag, diag_batch, grad):
    _check(load().tqk_adjoint_diagonal(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, _i32(wires), len(wires),
                                       diag.data_ptr(), diag_batch, _ptr(grad), _stream(psi)))


# ------------------------------------------------------------------ fused (tensor cores)
_STATUS = {}


def status_word(device) -> torch.Tensor:
    """Per-device int32 that kernels with device-side checks write a status code into
    (TQK_TIMEOUT when a bounded wait gave up, TQK_BAD_SHAPE when a batch work item does
    not fit the launch's tile)."""
    key = str(device)
    t = _STATUS.get(key)
    if t is None:
        t = torch.zeros(1, dtype=torch.int32, device=device)
        _STATUS[key] = t
    return t


def check_status(device) -> None:
    """Raise if a kernel on ``device`` reported a timeout (synchronises); clears the word."""
    t = status_word(device)
    v = int(t.item())
    if v != 0:
        t.zero_()
        why = {6: "a kernel gave up waiting on its pipeline or a dependency (bounded wait timed out)",
               2: "a circuit-batch work item was wider than the launch's tile (plan/config mismatch)"}
        raise TQKError(v, why.get(v, "a kernel reported a device-side error"))


def fused_prepare(u128: torch.Tensor, wires: Sequence[int]) -> torch.Tensor:
    """complex128 [B, 64, 64] -> operand image (uint8 tensor) for fused_apply /
    fused_adjoint on the same 6 wires (the image's layout follows their bit positions)."""
    lib = load()
    b = int(u128.shape[0])
    img = torch.empty(lib.tqk_fused_image_bytes(b), dtype=torch.uint8, device=u128.device)
    _check(lib.tqk_fused_prepare(u128.data_ptr(), b, _i32(wires), img.data_ptr(), _stream(u128)))
    return img


def fused_prepare_adjoint(u128: torch.Tensor, wires: Sequence[int]) -> torch.Tensor:
    """The image of U^H for fused_adjoint, built from U (complex128 [B, 64, 64])."""
    lib = load()
    b = int(u128.shape[0])
    img = torch.empty(lib.tqk_fused_image_bytes(b), dtype=torch.uint8, device=u128.device)
    _check(lib.tqk_fused_prepare_adjoint(u128.data_ptr(), b, _i32(wires), img.data_ptr(), _stream(u128)))
    return img


def fused_cross_grad(mr: torch.Tensor, u128: Optional[torch.Tensor], gu: torch.Tensor) -> None:
    """gu += M U per batch row (M from the adjoint step's cross term ``mr``), or gu += M
    when ``u128`` is None (the cross term of a stored-input step); ``gu`` is a complex128
    [B, 64, 64] tensor or its float64 interleaved view."""
    b = int(mr.shape[0])
    _check(load().tqk_fused_cross_grad(mr.data_ptr(), _ptr(u128), b, gu.data_ptr(), _stream(mr)))


def fused_apply(state, n, wires, image, u_batch):
    _check(load().tqk_fused_apply(state.data_ptr(), state.shape[0], n, _i32(wires), image.data_ptr(), u_batch,
                                  status_word(state.device).data_ptr(), _stream(state)))


def fused_apply_to(src, dst, n, wires, image, u_batch):
    """dst = U src for a fused block (src unchanged)."""
    _check(load().tqk_fused_apply_to(src.data_ptr(), dst.data_ptr(), src.shape[0], n, _i32(wires), image.data_ptr(),
                                     u_batch, status_word(src.device).data_ptr(), _stream(src)))


def fused_zero_input(state, n, wires, u128):
    """A fused block applied to |0...0> (``state`` holds exactly that): U[:, :, 0] written
    at the block's 64 patterns."""
    _check(load().tqk_fused_zero_input(state.data_ptr(), state.shape[0], n, _i32(wires), u128.data_ptr(),
                                       int(u128.shape[0]), _stream(state)))


def fused_adjoint_stored(psi_in, lam, n, wires, image_h, u_batch, mr_out):
    """lam <- U^H lam and the cross term of lam against the block's stored input state."""
    _check(load().tqk_fused_adjoint_stored(psi_in.data_ptr(), lam.data_ptr(), lam.shape[0], n, _i32(wires),
                                           image_h.data_ptr(), u_batch, _ptr(mr_out),
                                           status_word(lam.device).data_ptr(), _stream(lam)))


def fused_adjoint(psi, lam, n, wires, image_h, u_batch, mr_out):
    _check(load().tqk_fused_adjoint(psi.data_ptr(), lam.data_ptr(), psi.shape[0], n, _i32(wires), image_h.data_ptr(),
                                    u_batch, _ptr(mr_out), status_word(psi.device).data_ptr(), _stream(psi)))


def cross_to_complex(mr: torch.Tensor) -> torch.Tensor:
    """[B, 128, 128] real cross term (rows/cols 64p + j, p = 0 real part, 1 imaginary part)
    -> M [B, 64, 64] complex128, M[j][j'] = sum over columns of lam[j] conj(psi[j'])."""
    d = mr.view(-1, 2, 64, 2, 64)
    re = d[:, 0, :, 0, :] + d[:, 1, :, 1, :]
    im = d[:, 1, :, 0, :] - d[:, 0, :, 1, :]
    return torch.complex(re, im)


# ------------------------------------------------------------------ gate programs
def _dstream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def gate_operands(table, ngates, device):
    _check(load().tqk_gate_operands(table.data_ptr(), ngates, _dstream(device)))


def param_grads(table, ngates, device):
    _check(load().tqk_param_grads(table.data_ptr(), ngates, _dstream(device)))


def block_build(blocks, nblocks, max_batch, ops, device):
    _check(load().tqk_block_build(blocks.data_ptr(), nblocks, max_batch, ops.data_ptr(), _dstream(device)))


def block_unbuild(blocks, nblocks, max_batch, ops, device):
    _check(load().tqk_block_unbuild(blocks.data_ptr(), nblocks, max_batch, ops.data_ptr(), _dstream(device)))
