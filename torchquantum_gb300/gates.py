"""Gate matrices and their kernel structure.

Every builder takes ``params`` as a real ``[B, P]`` tensor (float32 -> complex64,
float64 -> complex128) and returns a batched ``[B, 2^k, 2^k]`` complex matrix, built
from differentiable torch ops so that gradients flow from the engine's matrix
cotangent back to the parameters.  The matrices follow the upstream builders in
``torchquantum/functional/*.py`` entry for entry (cited per gate), including their
quirks: ``cu2`` has no 1/sqrt(2) normalisation (``functional/u2.py:52-80``),
``xxplusyy`` puts ``-i sin(theta/2) e^{+i beta}`` above the diagonal
(``functional/xx_plus_yy.py``), and ``multixcnot`` is an X on the last wire
conditioned on every other wire being 0 (``functional/paulix.py``).

``STRUCT`` tells the engine which kernel applies a gate:

* ``("dense",)``            -- generic dense matrix on all wires;
* ``("ctrl", nc)``          -- first ``nc`` wires are controls (value 1), the
  lower-right ``2x2`` block acts on the last wire;
* ``("ctrl2", nc)``         -- same with a ``4x4`` block on the last two wires;
* ``("x", nc, ctrl_val)``   -- X on the last wire, controls on the first ``nc``
  wires must equal ``ctrl_val`` (1 for cnot/toffoli, 0 for multixcnot);
* ``("phase",)``            -- multiplies amplitudes whose wires are all 1 by the
  matrix's last diagonal entry (z, s, t, u1, cz, ccz, cs, cu1, ...);
* ``("diag",)``             -- general diagonal matrix (rz, rzz, multirz, crz);
* ``("swap", nc)``          -- exchange |..01> and |..10> on the last two wires
  under ``nc`` controls (swap, cswap).
"""
from __future__ import annotations

import math
from typing import Callable, Dict, Tuple

import torch

__all__ = ["GateDef", "GATES", "ALIASES", "canonical_name", "gate_matrix", "const_matrix"]

_SQ2 = 1.0 / math.sqrt(2.0)


def _cdt(params: torch.Tensor) -> torch.dtype:
    return torch.complex128 if params.dtype == torch.float64 else torch.complex64


def _c(x: torch.Tensor) -> torch.Tensor:
    return x.to(_cdt(x))


def _stack2(a, b, c, d):
    """[B] entries -> [B,2,2]."""
    return torch.stack([torch.stack([a, b], -1), torch.stack([c, d], -1)], -2)


def _expi(x: torch.Tensor) -> torch.Tensor:
    return torch.polar(torch.ones_like(x), x)


def _blockdiag_ctrl(sub: torch.Tensor, nc: int) -> torch.Tensor:
    """Embed a [B,d,d] block as the controlled block of a (nc controls) matrix."""
    bsz, d = sub.shape[0], sub.shape[-1]
    dim = d << nc
    eye = torch.eye(dim - d, dtype=sub.dtype, device=sub.device).expand(bsz, -1, -1)
    top = torch.cat([eye, sub.new_zeros(bsz, dim - d, d)], -1)
    bot = torch.cat([sub.new_zeros(bsz, d, dim - d), sub], -1)
    return torch.cat([top, bot], -2)


# ---------------------------------------------------------------- 1-qubit builders
def _rx(p):  # functional/rx.py:19-46
    t = p[:, 0]
    c, s = _c(torch.cos(t / 2)), _c(torch.sin(t / 2))
    js = -1j * s
    return _stack2(c, js, js, c)


def _ry(p):  # functional/ry.py:50-67
    t = p[:, 0]
    c, s = _c(torch.cos(t / 2)), _c(torch.sin(t / 2))
    return _stack2(c, -s, s, c)


def _rz(p):  # functional/rz.py:150-172
    t = p[:, 0]
    e0, e1 = _expi(-t / 2), _expi(t / 2)
    z = torch.zeros_like(e0)
    return _stack2(e0, z, z, e1)


def _phase(p):  # functional/phase_shift.py, functional/u1.py
    e = _expi(p[:, 0])
    o, z = torch.ones_like(e), torch.zeros_like(e)
    return _stack2(o, z, z, e)


def _u2(p):  # functional/u2.py
    phi, lam = p[:, 0], p[:, 1]
    a = _c(torch.full_like(phi, _SQ2))
    return _stack2(a, -_SQ2 * _expi(lam), _SQ2 * _expi(phi), _SQ2 * _expi(phi + lam))


def _u3(p):  # functional/u3.py:52-77
    th, phi, lam = p[:, 0], p[:, 1], p[:, 2]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    return _stack2(c, -s * _expi(lam), s * _expi(phi), c * _expi(phi + lam))


def _rot(p):  # functional/rot.py: RZ(omega) RY(theta) RZ(phi)
    phi, th, om = p[:, 0], p[:, 1], p[:, 2]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    return _stack2(_expi(-(phi + om) / 2) * c, -_expi((phi - om) / 2) * s,
                   _expi(-(phi - om) / 2) * s, _expi((phi + om) / 2) * c)


def _r(p):  # functional/r.py: exp(-i theta/2 (cos phi X + sin phi Y))
    th, phi = p[:, 0], p[:, 1]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    return _stack2(c, -1j * _expi(-phi) * s, -1j * _expi(phi) * s, c)


# ---------------------------------------------------------------- 2-qubit builders
def _zero4(p):
    return torch.zeros(p.shape[0], 4, 4, dtype=_cdt(p), device=p.device)


def _rxx(p):  # functional/rx.py rxx_matrix
    t = p[:, 0]
    c, js = _c(torch.cos(t / 2)), -1j * _c(torch.sin(t / 2))
    z = torch.zeros_like(c)
    rows = [[c, z, z, js], [z, c, js, z], [z, js, c, z], [js, z, z, c]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _ryy(p):  # functional/ry.py ryy_matrix
    t = p[:, 0]
    c, js = _c(torch.cos(t / 2)), 1j * _c(torch.sin(t / 2))
    z = torch.zeros_like(c)
    rows = [[c, z, z, js], [z, c, -js, z], [z, -js, c, z], [js, z, z, c]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _rzz(p):  # functional/rz.py rzz_matrix
    t = p[:, 0]
    a, b = _expi(-t / 2), _expi(t / 2)
    return torch.diag_embed(torch.stack([a, b, b, a], -1))


def _rzx(p):  # functional/rz.py rzx_matrix: exp(-i theta/2 Z(x)X)
    t = p[:, 0]
    c, js = _c(torch.cos(t / 2)), -1j * _c(torch.sin(t / 2))
    z = torch.zeros_like(c)
    rows = [[c, js, z, z], [js, c, z, z], [z, z, c, -js], [z, z, -js, c]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _single_excitation(p):  # functional/single_excitation.py
    t = p[:, 0]
    c, s = _c(torch.cos(t / 2)), _c(torch.sin(t / 2))
    o, z = torch.ones_like(c), torch.zeros_like(c)
    rows = [[o, z, z, z], [z, c, -s, z], [z, s, c, z], [z, z, z, o]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _xxminyy(p):  # functional/xx_min_yy.py
    th, beta = p[:, 0], p[:, 1]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    o, z = torch.ones_like(c), torch.zeros_like(c)
    rows = [[c, z, z, -1j * s * _expi(-beta)], [z, o, z, z], [z, z, o, z],
            [-1j * s * _expi(beta), z, z, c]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _xxplusyy(p):  # functional/xx_plus_yy.py
    th, beta = p[:, 0], p[:, 1]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    o, z = torch.ones_like(c), torch.zeros_like(c)
    rows = [[o, z, z, z], [z, c, -1j * s * _expi(beta), z], [z, -1j * s * _expi(-beta), c, z],
            [z, z, z, o]]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


def _cu2_block(p):  # functional/u2.py cu2_matrix (no 1/sqrt2, as upstream)
    phi, lam = p[:, 0], p[:, 1]
    o = _c(torch.ones_like(phi))
    return _stack2(o, -_expi(lam), _expi(phi), _expi(phi + lam))


def _cu_block(p):  # functional/u3.py:19-49 cu_matrix
    th, phi, lam, gam = p[:, 0], p[:, 1], p[:, 2], p[:, 3]
    c, s = _c(torch.cos(th / 2)), _c(torch.sin(th / 2))
    return _stack2(c * _expi(gam), -s * _expi(lam + gam), s * _expi(phi + gam), c * _expi(phi + lam + gam))


def _multirz(p, n):  # functional/rz.py multirz_matrix: exp(-i theta/2 Z^{(x)n})
    t = p[:, 0]
    idx = torch.arange(1 << n, device=p.device)
    par = torch.zeros_like(idx)
    for b in range(n):
        par = par ^ ((idx >> b) & 1)
    sign = (1 - 2 * par).to(p.dtype)  # +1 even parity, -1 odd
    ph = -t[:, None] / 2 * sign[None, :]
    return torch.diag_embed(_expi(ph))


# ---------------------------------------------------------------- constant matrices
def _const_table() -> Dict[str, list]:
    s2 = _SQ2
    i = 1j
    cp8, sp8 = math.cos(math.pi / 8), math.sin(math.pi / 8)
    h = [[s2, s2], [s2, -s2]]
    x = [[0, 1], [1, 0]]
    y = [[0, -i], [i, 0]]
    sx = [[(1 + i) / 2, (1 - i) / 2], [(1 - i) / 2, (1 + i) / 2]]
    return {
        "hadamard": h,
        "shadamard": [[cp8, -sp8], [sp8, cp8]],
        "paulix": x,
        "pauliy": y,
        "pauliz": [[1, 0], [0, -1]],
        "i": [[1, 0], [0, 1]],
        "s": [[1, 0], [0, i]],
        "sdg": [[1, 0], [0, -i]],
        "t": [[1, 0], [0, complex(math.cos(math.pi / 4), math.sin(math.pi / 4))]],
        "tdg": [[1, 0], [0, complex(math.cos(math.pi / 4), -math.sin(math.pi / 4))]],
        "sx": sx,
        "sxdg": [[(1 - i) / 2, (1 + i) / 2], [(1 + i) / 2, (1 - i) / 2]],
        "swap": [[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]],
        "sswap": [[1, 0, 0, 0], [0, (1 + i) / 2, (1 - i) / 2, 0], [0, (1 - i) / 2, (1 + i) / 2, 0], [0, 0, 0, 1]],
        "iswap": [[1, 0, 0, 0], [0, 0, i, 0], [0, i, 0, 0], [0, 0, 0, 1]],
        "ecr": [[0, 0, s2, i * s2], [0, 0, i * s2, s2], [s2, -i * s2, 0, 0], [-i * s2, s2, 0, 0]],
        "dcx": [[1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1], [0, 1, 0, 0]],
    }


_CONST = _const_table()
_CTRL_CONST_SUB = {  # controlled constant gates: name -> (n controls, target block name)
    "cnot": (1, "paulix"), "cy": (1, "pauliy"), "cz": (1, "pauliz"), "chadamard": (1, "hadamard"),
    "cs": (1, "s"), "csdg": (1, "sdg"), "csx": (1, "sx"), "toffoli": (2, "paulix"), "ccz": (2, "pauliz"),
    "c3x": (3, "paulix"), "c4x": (4, "paulix"), "c3sx": (3, "sx"), "cswap": (1, "swap"),
}
_CONST_CACHE: Dict[Tuple[str, int, torch.dtype, str], torch.Tensor] = {}


def _rccx():
    m = torch.eye(8, dtype=torch.complex128)
    m[5, 5] = -1
    m[6:, 6:] = torch.tensor([[0, -1j], [1j, 0]])
    return m


def _rc3x():
    m = torch.eye(16, dtype=torch.complex128)
    m[12, 12] = 1j
    m[13, 13] = -1j
    m[14:, 14:] = torch.tensor([[0, 1], [-1, 0]], dtype=torch.complex128)
    return m


def _qft(n):  # functional/qft.py: omega^{jk}/sqrt(N), omega = e^{2 pi i / N}
    dim = 1 << n
    j = torch.arange(dim, dtype=torch.float64)
    ph = 2 * math.pi * torch.outer(j, j) / dim
    return torch.polar(torch.full_like(ph, 1 / math.sqrt(dim)), ph)


def _mcx(n, ctrl_val=1):  # functional/paulix.py multicnot / multixcnot
    dim = 1 << n
    m = torch.eye(dim, dtype=torch.complex128)
    a = dim - 2 if ctrl_val == 1 else 0
    m[a:a + 2, a:a + 2] = torch.tensor([[0, 1], [1, 0]], dtype=torch.complex128)
    return m


def const_matrix(name: str, n_wires: int, dtype: torch.dtype, device) -> torch.Tensor:
    """Constant matrix [1, 2^k, 2^k] of a parameter-free gate (cached per device/dtype)."""
    key = (name, n_wires, dtype, str(device))
    m = _CONST_CACHE.get(key)
    if m is not None:
        return m
    if name in _CONST:
        m = torch.tensor(_CONST[name], dtype=torch.complex128)
    elif name in _CTRL_CONST_SUB:
        nc, sub = _CTRL_CONST_SUB[name]
        m = _blockdiag_ctrl(torch.tensor(_CONST[sub], dtype=torch.complex128)[None], nc)[0]
    elif name == "rccx":
        m = _rccx()
    elif name == "rc3x":
        m = _rc3x()
    elif name == "qft":
        m = _qft(n_wires)
    elif name == "multicnot":
        m = _mcx(n_wires, 1)
    elif name == "multixcnot":
        m = _mcx(n_wires, 0)
    else:
        raise KeyError(name)
    m = m.to(dtype=dtype, device=device)[None].contiguous()
    _CONST_CACHE[key] = m
    return m


class GateDef:
    """Static description of one gate type."""

    __slots__ = ("name", "num_params", "num_wires", "builder", "struct")

    def __init__(self, name, num_params, num_wires, builder, struct):
        self.name = name
        self.num_params = num_params
        self.num_wires = num_wires  # -1: any number of wires
        self.builder = builder  # None for constant gates
        self.struct = struct

    def __repr__(self):
        return f"GateDef({self.name}, P={self.num_params}, W={self.num_wires}, {self.struct})"


def _ctrl_builder(block_fn: Callable, nc: int):
    return lambda p: _blockdiag_ctrl(block_fn(p), nc)


GATES: Dict[str, GateDef] = {}


def _def(name, npar, nw, builder, struct):
    GATES[name] = GateDef(name, npar, nw, builder, struct)


# parameterised gates
_def("rx", 1, 1, _rx, ("dense",))
_def("ry", 1, 1, _ry, ("dense",))
_def("rz", 1, 1, _rz, ("diag",))
_def("phaseshift", 1, 1, _phase, ("phase",))
_def("u1", 1, 1, _phase, ("phase",))
_def("u2", 2, 1, _u2, ("dense",))
_def("u3", 3, 1, _u3, ("dense",))
_def("rot", 3, 1, _rot, ("dense",))
_def("r", 2, 1, _r, ("dense",))
_def("rxx", 1, 2, _rxx, ("dense",))
_def("ryy", 1, 2, _ryy, ("dense",))
_def("rzz", 1, 2, _rzz, ("diag",))
_def("rzx", 1, 2, _rzx, ("dense",))
_def("singleexcitation", 1, 2, _single_excitation, ("dense",))
_def("xxminyy", 2, 2, _xxminyy, ("dense",))
_def("xxplusyy", 2, 2, _xxplusyy, ("dense",))
_def("crx", 1, 2, _ctrl_builder(_rx, 1), ("ctrl", 1))
_def("cry", 1, 2, _ctrl_builder(_ry, 1), ("ctrl", 1))
_def("crz", 1, 2, _ctrl_builder(_rz, 1), ("diag",))
_def("crot", 3, 2, _ctrl_builder(_rot, 1), ("ctrl", 1))
_def("cu1", 1, 2, _ctrl_builder(_phase, 1), ("phase",))
_def("cu2", 2, 2, _ctrl_builder(_cu2_block, 1), ("ctrl", 1))
_def("cu3", 3, 2, _ctrl_builder(_u3, 1), ("ctrl", 1))
_def("cu", 4, 2, _ctrl_builder(_cu_block, 1), ("ctrl", 1))
_def("multirz", 1, -1, None, ("diag",))
_def("globalphase", 1, 0, None, ("phase",))
# parameter-free gates
for _n in ("hadamard", "shadamard", "paulix", "pauliy", "sx", "sxdg", "i"):
    _def(_n, 0, 1, None, ("dense",))
for _n in ("pauliz", "s", "sdg", "t", "tdg"):
    _def(_n, 0, 1, None, ("phase",))
_def("paulix", 0, 1, None, ("x", 0, 1))
_def("cnot", 0, 2, None, ("x", 1, 1))
_def("toffoli", 0, 3, None, ("x", 2, 1))
_def("c3x", 0, 4, None, ("x", 3, 1))
_def("c4x", 0, 5, None, ("x", 4, 1))
_def("multicnot", 0, -1, None, ("x", -1, 1))
_def("multixcnot", 0, -1, None, ("x", -1, 0))
_def("cz", 0, 2, None, ("phase",))
_def("ccz", 0, 3, None, ("phase",))
_def("cs", 0, 2, None, ("phase",))
_def("csdg", 0, 2, None, ("phase",))
_def("cy", 0, 2, None, ("ctrl", 1))
_def("chadamard", 0, 2, None, ("ctrl", 1))
_def("csx", 0, 2, None, ("ctrl", 1))
_def("c3sx", 0, 4, None, ("ctrl", 3))
_def("swap", 0, 2, None, ("swap", 0))
_def("cswap", 0, 3, None, ("swap", 1))
for _n in ("sswap", "iswap", "ecr", "dcx"):
    _def(_n, 0, 2, None, ("dense",))
_def("rccx", 0, 3, None, ("dense",))
_def("rc3x", 0, 4, None, ("dense",))
_def("qft", 0, -1, None, ("dense",))
_def("qubitunitary", -1, -1, None, ("dense",))
_def("qubitunitaryfast", -1, -1, None, ("dense",))
_def("qubitunitarystrict", -1, -1, None, ("dense",))

# functional aliases (functional/__init__.py:125-218)
ALIASES = {
    "h": "hadamard", "sh": "shadamard", "x": "paulix", "y": "pauliy", "z": "pauliz",
    "cx": "cnot", "ccnot": "toffoli", "ccx": "toffoli", "xx": "rxx", "yy": "ryy", "zz": "rzz",
    "zx": "rzx", "p": "phaseshift", "cp": "cu1", "cphase": "cu1", "cr": "cu1", "u": "u3",
    "ch": "chadamard", "echoedcrossresonance": "ecr",
}


def canonical_name(name: str) -> str:
    name = name.lower()
    return ALIASES.get(name, name)


def gate_matrix(name: str, params, n_wires: int, dtype=torch.complex64, device="cpu") -> torch.Tensor:
    """Batched matrix ``[B, 2^k, 2^k]`` of gate ``name`` (``B`` = param batch, 1 if none).

    ``params`` is the normalised ``[B, P]`` real tensor for parameterised gates, the
    ``[B, 2^k, 2^k]`` complex matrix for the qubitunitary family, else ``None``.
    """
    name = canonical_name(name)
    g = GATES[name]
    if name in ("qubitunitary", "qubitunitaryfast"):
        return params
    if name == "qubitunitarystrict":  # functional/qubit_unitary.py:72-86 (U @ V, as upstream)
        u, _, v = torch.svd(params)
        return u.matmul(v)
    if name == "multirz":
        return _multirz(params, n_wires)
    if name == "globalphase":
        return _expi(params[:, 0])[:, None, None]
    if g.builder is not None:
        return g.builder(params)
    return const_matrix(name, n_wires, dtype, device)
