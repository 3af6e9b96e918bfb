"""Reference-side binding: upstream torchquantum's ``apply_unitary_bmm`` on libtqk.so.

Upstream's gate wrapper looks ``apply_unitary_bmm`` up in its own module globals on
every call (``torchquantum/functional/gate_wrapper.py:446``), so assigning
``apply_unitary_bmm`` below to ``torchquantum.functional.gate_wrapper.apply_unitary_bmm``
(``install``) routes every upstream gate -- ``tqf.*``, ``Operator.forward``, encoders,
layers -- through the engine's dense kernel, unchanged upstream code around it.

This module depends only on ctypes, torch and the C ABI (``include/tqk.h``), like the
binding a maintainer would add to upstream.  It keeps upstream's semantics
(``gate_wrapper.py:96-140``): out of place, the input state is never written, and the
result is differentiable with respect to both ``state`` and ``mat`` through a
``torch.autograd.Function`` whose backward is one adjoint step of the engine
(``tqk_adjoint_matrix``): the state cotangent ``U^H g`` and the matrix cotangent
``sum g x^H`` over the batch (per row for a per-row matrix), as torch's own ``bmm``
backward gives them.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Sequence, Union

import torch

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libtqk.so")
_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError(f"{_LIB_PATH} is missing: build the CUDA engine first")
        lib = ctypes.CDLL(_LIB_PATH)
        vp, i64, i32p, c_int = ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), ctypes.c_int
        lib.tqk_last_error.restype = ctypes.c_char_p
        lib.tqk_apply_matrix.restype = c_int
        lib.tqk_apply_matrix.argtypes = [vp, i64, c_int, i32p, c_int, vp, i64, vp]
        lib.tqk_adjoint_matrix.restype = c_int
        lib.tqk_adjoint_matrix.argtypes = [vp, vp, i64, c_int, i32p, c_int, vp, i64, vp, vp, vp]
        _lib = lib
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(_load().tqk_last_error().decode(errors="replace"))


def _wires(wires) -> List[int]:
    return [int(wires)] if isinstance(wires, int) else [int(w) for w in wires]


class _ApplyUnitary(torch.autograd.Function):
    @staticmethod
    def forward(ctx, state: torch.Tensor, mat: torch.Tensor, wires: List[int]):
        lib = _load()
        bsz, n, k = state.shape[0], state.dim() - 1, len(wires)
        if state.device.type != "cuda":
            raise ValueError("apply_unitary_bmm (libtqk): the state must be a CUDA tensor")
        x = state.detach().reshape(bsz, -1).to(torch.complex64).contiguous()
        m = mat.detach().to(x.device, torch.complex64)
        m3 = (m if m.dim() == 3 else m.unsqueeze(0)).resolve_conj().resolve_neg().contiguous()
        out = x.clone()
        w = (ctypes.c_int32 * k)(*wires)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _check(lib.tqk_apply_matrix(out.data_ptr(), bsz, n, w, k, m3.data_ptr(), m3.shape[0], stream))
        ctx.save_for_backward(x, m3)
        ctx.wires, ctx.shape = wires, state.shape
        ctx.mat_shape, ctx.mat_dtype, ctx.mat_device = mat.shape, mat.dtype, mat.device
        return out.view(state.shape)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        lib = _load()
        x, m3 = ctx.saved_tensors
        bsz, n, k = x.shape[0], len(ctx.shape) - 1, len(ctx.wires)
        d = 1 << k
        # one adjoint step: lam <- U^H g, cotangent of U += g x^H; the stored input x is
        # recovered with an identity "uncompute" (exact, also for matrices that are not
        # unitary), on a copy so the saved tensor is never written
        psi = x.clone()
        lam = grad_out.reshape(bsz, -1).to(torch.complex64).resolve_conj().resolve_neg().contiguous().clone()
        eye = torch.eye(d, dtype=torch.complex64, device=x.device).expand(m3.shape[0], d, d).contiguous()
        need_mat = ctx.needs_input_grad[1]
        grad = torch.zeros(m3.shape[0] * d * d * 2, dtype=torch.float64, device=x.device) if need_mat else None
        w = (ctypes.c_int32 * k)(*ctx.wires)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        _check(lib.tqk_adjoint_matrix(psi.data_ptr(), lam.data_ptr(), bsz, n, w, k, m3.data_ptr(), m3.shape[0],
                                      eye.data_ptr(), None if grad is None else grad.data_ptr(), stream))
        g_state = lam.view(ctx.shape) if ctx.needs_input_grad[0] else None
        g_mat = None
        if need_mat:
            # upstream builds constant and some parameterised matrices on the host and lets
            # apply_unitary_bmm move them; the cotangent goes back to where the matrix was
            g_mat = torch.view_as_complex(grad.view(m3.shape[0], d, d, 2)).reshape(ctx.mat_shape)
            g_mat = g_mat.to(device=ctx.mat_device, dtype=ctx.mat_dtype)
        return g_state, g_mat, None


def apply_unitary_bmm(state: torch.Tensor, mat: torch.Tensor, wires: Union[int, Sequence[int]]) -> torch.Tensor:
    """Drop-in for upstream ``apply_unitary_bmm(state, mat, wires)`` (gate_wrapper.py:96):
    ``state`` [bsz, 2, ..., 2] complex on a CUDA device, ``mat`` [2^k, 2^k] or
    [bsz, 2^k, 2^k]; returns the new state (a new tensor), differentiable w.r.t. both."""
    return _ApplyUnitary.apply(state, mat, _wires(wires))


def install(torchquantum_module) -> None:
    """Route every gate of an imported upstream ``torchquantum`` through libtqk.so."""
    import importlib

    gw = importlib.import_module(torchquantum_module.__name__ + ".functional.gate_wrapper")
    gw.apply_unitary_bmm = apply_unitary_bmm
