"""CPU oracle for the gate-application path -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the upstream torchquantum statevector path, used by
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg as the
checker.  It is never the thing measured on the GPU and never a fallback of the
product: the product package does not import it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against fixtures produced by running the upstream package itself
(``tests/golden/make_golden.py``): 91 gate-matrix variants, 9 random circuits with
autograd gradients, the 4-wire encoder/U3/CNOT model, and the upstream
known-answer tests.

Conventions restated from upstream:

* state ``[bsz, 2^n]``; wire 0 is the most significant bit of the flat index
  (``torchquantum/device/devices.py:64-71,114-117``);
* a k-wire matrix is indexed with ``wires[0]`` most significant and applied as in
  ``apply_unitary_bmm`` (``torchquantum/functional/gate_wrapper.py:96-140``);
* a parameter batch of 1 broadcasts over the state batch, otherwise per sample
  (``gate_wrapper.py:129-136``); ``inverse`` is the conjugate transpose
  (``gate_wrapper.py:427-432``);
* ``expval_joint_analytical`` is ``Re <psi| P_0 (x) ... (x) P_{n-1} |psi>`` with
  ``P[0]`` on wire 0 (``torchquantum/measurement/measurements.py:232-279``).
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence

import numpy as np

C = np.complex128
SQ2 = 1 / math.sqrt(2)

# ----------------------------------------------------------------------- matrices
_X = np.array([[0, 1], [1, 0]], C)
_Y = np.array([[0, -1j], [1j, 0]], C)
_Z = np.array([[1, 0], [0, -1]], C)
_I2 = np.eye(2, dtype=C)
_PAULI = {"I": _I2, "X": _X, "Y": _Y, "Z": _Z}


def _pauli_rot(string: str, theta: np.ndarray) -> np.ndarray:
    """exp(-i theta/2 P) for a Pauli string P, batched over theta [B] -> [B,d,d]."""
    p = np.array([[1]], C)
    for ch in string:
        p = np.kron(p, _PAULI[ch])
    eye = np.eye(p.shape[0], dtype=C)
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    return c[:, None, None] * eye - 1j * s[:, None, None] * p


def _ctrl(block: np.ndarray, nc: int) -> np.ndarray:
    """Controlled embedding: identity unless the first nc wires are all 1."""
    b, d = block.shape[0], block.shape[-1]
    dim = d << nc
    out = np.tile(np.eye(dim, dtype=C), (b, 1, 1))
    out[:, dim - d:, dim - d:] = block
    return out


def _u3(t, p, l):  # functional/u3.py:52-77
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.stack([np.stack([c + 0j, -s * np.exp(1j * l)], -1),
                     np.stack([s * np.exp(1j * p), c * np.exp(1j * (p + l))], -1)], -2)


def _phase(t):
    o = np.ones_like(t)
    return np.stack([np.stack([o + 0j, 0 * o], -1), np.stack([0 * o + 0j, np.exp(1j * t)], -1)], -2)


def _rot(phi, th, om):  # RZ(om) RY(th) RZ(phi)  (functional/rot.py)
    return _pauli_rot("Z", om) @ _pauli_rot("Y", th) @ _pauli_rot("Z", phi)


def _r(th, phi):  # functional/r.py
    c, s = np.cos(th / 2), np.sin(th / 2)
    return np.stack([np.stack([c + 0j, -1j * np.exp(-1j * phi) * s], -1),
                     np.stack([-1j * np.exp(1j * phi) * s, c + 0j], -1)], -2)


def _u2(phi, lam, norm=SQ2):  # functional/u2.py (cu2 keeps norm=1, as upstream)
    o = np.ones_like(phi)
    return norm * np.stack([np.stack([o + 0j, -np.exp(1j * lam)], -1),
                            np.stack([np.exp(1j * phi), np.exp(1j * (phi + lam))], -1)], -2)


def _two_level(theta, beta, lo, hi, sign_upper):
    """XX-YY type: rotation in the {lo,hi} subspace of a 2-qubit space."""
    b = theta.shape[0]
    m = np.tile(np.eye(4, dtype=C), (b, 1, 1))
    c, s = np.cos(theta / 2), np.sin(theta / 2)
    m[:, lo, lo] = c
    m[:, hi, hi] = c
    m[:, lo, hi] = -1j * s * np.exp(sign_upper * 1j * beta)
    m[:, hi, lo] = -1j * s * np.exp(-sign_upper * 1j * beta)
    return m


def _const(name: str, n_wires: int) -> np.ndarray:
    i = 1j
    sx = np.array([[1 + i, 1 - i], [1 - i, 1 + i]], C) / 2
    h = np.array([[1, 1], [1, -1]], C) * SQ2
    table = {
        "hadamard": h, "paulix": _X, "pauliy": _Y, "pauliz": _Z, "i": _I2,
        "shadamard": _pauli_rot("Y", np.array([math.pi / 4]))[0],
        "s": np.diag([1, i]).astype(C), "sdg": np.diag([1, -i]).astype(C),
        "t": np.diag([1, np.exp(i * math.pi / 4)]).astype(C),
        "tdg": np.diag([1, np.exp(-i * math.pi / 4)]).astype(C),
        "sx": sx, "sxdg": sx.conj().T,
        "swap": np.eye(4, dtype=C)[[0, 2, 1, 3]],
        "dcx": np.eye(4, dtype=C)[:, [0, 3, 1, 2]],
        "iswap": np.array([[1, 0, 0, 0], [0, 0, i, 0], [0, i, 0, 0], [0, 0, 0, 1]], C),
        "sswap": np.array([[1, 0, 0, 0], [0, (1 + i) / 2, (1 - i) / 2, 0],
                           [0, (1 - i) / 2, (1 + i) / 2, 0], [0, 0, 0, 1]], C),
        "ecr": SQ2 * np.array([[0, 0, 1, i], [0, 0, i, 1], [1, -i, 0, 0], [-i, 1, 0, 0]], C),
    }
    if name in table:
        return table[name]
    ctrl = {"cnot": (1, _X), "cy": (1, _Y), "cz": (1, _Z), "chadamard": (1, h), "cs": (1, table["s"]),
            "csdg": (1, table["sdg"]), "csx": (1, sx), "toffoli": (2, _X), "ccz": (2, _Z), "c3x": (3, _X),
            "c4x": (4, _X), "c3sx": (3, sx), "cswap": (1, table["swap"])}
    if name in ctrl:
        nc, blk = ctrl[name]
        return _ctrl(blk[None], nc)[0]
    if name == "rccx":
        m = np.eye(8, dtype=C)
        m[5, 5] = -1
        m[6:, 6:] = [[0, -i], [i, 0]]
        return m
    if name == "rc3x":
        m = np.eye(16, dtype=C)
        m[12, 12], m[13, 13] = i, -i
        m[14:, 14:] = [[0, 1], [-1, 0]]
        return m
    if name == "qft":
        d = 1 << n_wires
        j = np.arange(d)
        return np.exp(2j * math.pi * np.outer(j, j) / d) / math.sqrt(d)
    if name in ("multicnot", "multixcnot"):
        d = 1 << n_wires
        m = np.eye(d, dtype=C)
        a = d - 2 if name == "multicnot" else 0
        m[a:a + 2, a:a + 2] = _X
        return m
    raise KeyError(name)


ALIASES = {"h": "hadamard", "sh": "shadamard", "x": "paulix", "y": "pauliy", "z": "pauliz", "cx": "cnot",
           "ccnot": "toffoli", "ccx": "toffoli", "xx": "rxx", "yy": "ryy", "zz": "rzz", "zx": "rzx",
           "p": "phaseshift", "cp": "cu1", "cphase": "cu1", "cr": "cu1", "u": "u3", "ch": "chadamard",
           "echoedcrossresonance": "ecr"}


def gate_matrix(name: str, params: Optional[np.ndarray], n_wires: Optional[int] = None,
                inverse: bool = False) -> np.ndarray:
    """[B, 2^k, 2^k] matrix of a named gate; params is [B, P] (gate_wrapper.py:361-432)."""
    name = ALIASES.get(name, name)
    p = None if params is None else np.asarray(params)
    if p is not None and name not in ("qubitunitary", "qubitunitaryfast", "qubitunitarystrict"):
        p = p.astype(np.float64)
        if p.ndim == 0:
            p = p.reshape(1, 1)
        elif p.ndim == 1:
            p = p[:, None]
    col = (lambda j: p[:, j]) if p is not None else None
    if name in ("qubitunitary", "qubitunitaryfast"):
        m = np.asarray(p, C)
    elif name == "qubitunitarystrict":
        u, _, vh = np.linalg.svd(np.asarray(p, C))
        m = u @ np.conj(np.swapaxes(vh, -1, -2))  # torch.svd's V, as upstream: U @ V
    elif name == "rx":
        m = _pauli_rot("X", col(0))
    elif name == "ry":
        m = _pauli_rot("Y", col(0))
    elif name == "rz":
        m = _pauli_rot("Z", col(0))
    elif name in ("phaseshift", "u1"):
        m = _phase(col(0))
    elif name == "u2":
        m = _u2(col(0), col(1))
    elif name == "u3":
        m = _u3(col(0), col(1), col(2))
    elif name == "rot":
        m = _rot(col(0), col(1), col(2))
    elif name == "r":
        m = _r(col(0), col(1))
    elif name in ("rxx", "ryy", "rzz", "rzx"):
        m = _pauli_rot({"rxx": "XX", "ryy": "YY", "rzz": "ZZ", "rzx": "ZX"}[name], col(0))
    elif name == "multirz":
        m = _pauli_rot("Z" * n_wires, col(0))
    elif name == "singleexcitation":
        m = np.tile(np.eye(4, dtype=C), (p.shape[0], 1, 1))
        m[:, 1:3, 1:3] = _pauli_rot("Y", col(0))
    elif name == "xxminyy":
        m = _two_level(col(0), col(1), 0, 3, -1)
    elif name == "xxplusyy":
        m = _two_level(col(0), col(1), 1, 2, +1)
    elif name in ("crx", "cry", "crz"):
        m = _ctrl(_pauli_rot(name[-1].upper(), col(0)), 1)
    elif name == "crot":
        m = _ctrl(_rot(col(0), col(1), col(2)), 1)
    elif name == "cu1":
        m = _ctrl(_phase(col(0)), 1)
    elif name == "cu2":
        m = _ctrl(_u2(col(0), col(1), norm=1.0), 1)
    elif name == "cu3":
        m = _ctrl(_u3(col(0), col(1), col(2)), 1)
    elif name == "cu":
        m = _ctrl(_u3(col(0), col(1), col(2)) * np.exp(1j * col(3))[:, None, None], 1)
    elif name == "globalphase":
        m = np.exp(1j * col(0))[:, None, None]
    else:
        m = _const(name, n_wires)[None]
    m = np.asarray(m, C)
    if m.ndim == 2:
        m = m[None]
    if inverse:
        m = np.conj(np.swapaxes(m, -1, -2))
    return m


# ----------------------------------------------------------------------- state ops
def init_state(n: int, bsz: int) -> np.ndarray:
    """|0...0> for every batch row (devices.py:64-71)."""
    s = np.zeros((bsz, 1 << n), C)
    s[:, 0] = 1
    return s


def apply(state: np.ndarray, mat: np.ndarray, wires: Sequence[int], n: int) -> np.ndarray:
    """psi' = U psi on ``wires`` (gate_wrapper.py:96-140): move the wire axes to the
    front, contract with the (batched or broadcast) matrix, move back."""
    bsz = state.shape[0]
    k = len(wires)
    mat = np.asarray(mat, C)
    if mat.ndim == 2:
        mat = mat[None]
    t = state.reshape([bsz] + [2] * n)
    axes = [w + 1 for w in wires]
    rest = [a for a in range(1, n + 1) if a not in axes]
    perm = [0] + axes + rest
    tp = np.transpose(t, perm).reshape(bsz, 1 << k, -1)
    out = np.matmul(np.broadcast_to(mat, (bsz,) + mat.shape[1:]), tp)
    out = out.reshape([bsz] + [2] * n)
    return np.transpose(out, np.argsort(perm)).reshape(bsz, -1)


def reset(state: np.ndarray, wires: Sequence[int], n: int) -> np.ndarray:
    """Zero the |1> component of each wire, then renormalise (functional/reset.py)."""
    s = state.copy().reshape([state.shape[0]] + [2] * n)
    for w in wires:
        idx = [slice(None)] * (n + 1)
        idx[w + 1] = 1
        s[tuple(idx)] = 0
    s = s.reshape(state.shape[0], -1)
    norm = np.sqrt((np.abs(s) ** 2).sum(-1, keepdims=True))
    zero = norm[:, 0] == 0
    s[zero, 0] = 1
    norm[zero] = 1
    return s / norm


def run(n: int, bsz: int, gates: List[Dict], state: Optional[np.ndarray] = None) -> np.ndarray:
    """Execute a gate list ({name, wires, params, inverse, n_wires}) from |0..0>."""
    s = init_state(n, bsz) if state is None else np.array(state, C)
    for g in gates:
        wires = [g["wires"]] if isinstance(g["wires"], int) else list(g["wires"])
        if g["name"] == "reset":
            s = reset(s, wires, n)
            continue
        m = gate_matrix(g["name"], g.get("params"), g.get("n_wires") or len(wires), g.get("inverse", False))
        s = apply(s, m, wires, n)
    return s


# ----------------------------------------------------------------------- density matrices
def density_run(n: int, bsz: int, gates: List[Dict], rho: Optional[np.ndarray] = None,
                upstream_bmm: bool = False) -> np.ndarray:
    """rho [bsz, 2^n, 2^n] evolved by a gate list from |0..0><0..0| (or ``rho``).

    Default: rho -> U rho U^H.  ``upstream_bmm``: upstream's density bmm
    (``functional/gate_wrapper.py:265-321``), which multiplies the bra wires by conj(U)
    without transposing -- rho -> U rho conj(U) in the same index convention -- equal to
    U rho U^H only for symmetric U."""
    d = 1 << n
    if rho is None:
        rho = np.zeros((bsz, d, d), C)
        rho[:, 0, 0] = 1
    v = np.array(rho, C).reshape(bsz, d * d)  # vec(rho): ket wires 0..n-1, bra wires n..2n-1
    for g in gates:
        wires = [g["wires"]] if isinstance(g["wires"], int) else list(g["wires"])
        m = np.asarray(gate_matrix(g["name"], g.get("params"), g.get("n_wires") or len(wires),
                                   g.get("inverse", False)), C)
        m3 = m if m.ndim == 3 else m[None]
        v = apply(v, m3, wires, 2 * n)
        # bra side: rho U^H acts on the bra index as conj(U); upstream applies conj(U)^T
        right = np.conj(m3) if not upstream_bmm else np.conj(np.swapaxes(m3, -1, -2))
        v = apply(v, right, [w + n for w in wires], 2 * n)
    return v.reshape(bsz, d, d)


def pauli_masks(pauli: str, n: int):
    """(xmask, zmask, number of Y) with P[0] on wire 0 = bit n-1."""
    x = z = ny = 0
    for w, ch in enumerate(pauli.upper()):
        bit = 1 << (n - 1 - w)
        if ch in "XY":
            x |= bit
        if ch in "ZY":
            z |= bit
        ny += ch == "Y"
    return x, z, ny


def apply_pauli(state: np.ndarray, pauli: str, n: int) -> np.ndarray:
    """P psi via masks: (P psi)_i = i^nY (-1)^popcount((i^x)&z) psi_{i^x}."""
    x, z, ny = pauli_masks(pauli, n)
    idx = np.arange(1 << n)
    src = idx ^ x
    par = np.array([bin(v).count("1") & 1 for v in (src & z)]) if n <= 16 else _parity(src & z)
    ph = (1j ** ny) * (1 - 2 * par)
    return state[:, src] * ph[None, :]


def _parity(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64)
    p = np.zeros_like(v)
    while np.any(v):
        p ^= v & np.uint64(1)
        v >>= np.uint64(1)
    return p.astype(np.int64)


def expval_pauli(state: np.ndarray, pauli: str, n: int) -> np.ndarray:
    """Re <psi|P|psi> per batch row (measurements.py:232-279 restated via masks)."""
    return np.real(np.sum(np.conj(state) * apply_pauli(state, pauli, n), axis=-1))


def expval_kron(state: np.ndarray, pauli: str) -> np.ndarray:
    """Dense-kron form, exactly as measurements.py:269-279 (small n only)."""
    h = np.array([[1]], C)
    for ch in pauli.upper():
        h = np.kron(h, _PAULI[ch])
    return np.real((np.conj(state) * (h @ state.T).T).sum(-1))


def probs(state: np.ndarray) -> np.ndarray:
    return np.abs(state) ** 2


def expval_wire(state: np.ndarray, n: int, wire: int, obs: str = "Z") -> np.ndarray:
    """tq.expval for one wire (measurements.py:282-312): rotate, marginal probs . eigvals."""
    return expval_pauli(state, "".join(obs if w == wire else "I" for w in range(n)), n)


# ----------------------------------------------------------------------- gradients
def loss_expvals(n, bsz, gates, paulis, weights, state=None):
    s = run(n, bsz, gates, state)
    ev = np.stack([expval_pauli(s, p, n) for p in paulis], -1)
    return float((ev * np.asarray(weights)).sum())


def fd_grads(n, bsz, gates, paulis, weights, h=1e-3, state=None):
    """Central finite differences of sum(w * expvals) w.r.t. every real gate parameter."""
    out = []
    for gi, g in enumerate(gates):
        if g.get("params") is None or g["name"].startswith("qubitunitary"):
            out.append(None)
            continue
        p0 = np.array(g["params"], np.float64)
        gr = np.zeros_like(p0)
        for idx in np.ndindex(p0.shape):
            for sgn in (1, -1):
                pp = p0.copy()
                pp[idx] += sgn * h
                gg = list(gates)
                gg[gi] = dict(g, params=pp)
                gr[idx] += sgn * loss_expvals(n, bsz, gg, paulis, weights, state) / (2 * h)
        out.append(gr)
    return out


# ----------------------------------------------------------------------- CPU baseline
def forward_saving(n: int, bsz: int, gates: List[Dict], dtype=np.complex64):
    """Forward pass that keeps every gate's input state, as torch autograd does for
    upstream's apply_unitary_bmm (gate_wrapper.py:127-136); returns (final, saved, mats)."""
    s = init_state(n, bsz).astype(dtype)
    saved, mats = [], []
    for g in gates:
        wires = list(g["wires"])
        m = gate_matrix(g["name"], g.get("params"), len(wires), g.get("inverse", False)).astype(dtype)
        saved.append(s)
        mats.append(m)
        s = apply(s, m, wires, n).astype(dtype)
    return s, saved, mats


def backward_sweep(n: int, gates: List[Dict], saved, mats, lam: np.ndarray):
    """Reverse sweep of the saved-state forward: per gate, the matrix cotangent
    sum_cols lam psi_in^H (what torch.bmm's backward computes) and lam <- U^H lam."""
    grads = [None] * len(gates)
    bsz = lam.shape[0]
    for i in range(len(gates) - 1, -1, -1):
        wires = list(gates[i]["wires"])
        k = len(wires)
        m = mats[i]
        axes = [w + 1 for w in wires]
        rest = [a for a in range(1, n + 1) if a not in axes]
        perm = [0] + axes + rest
        lp = np.transpose(lam.reshape([bsz] + [2] * n), perm).reshape(bsz, 1 << k, -1)
        pp = np.transpose(saved[i].reshape([bsz] + [2] * n), perm).reshape(bsz, 1 << k, -1)
        g = np.matmul(lp, np.conj(np.swapaxes(pp, -1, -2)))
        grads[i] = g.sum(0, keepdims=True) if m.shape[0] == 1 else g
        lam = apply(lam, np.conj(np.swapaxes(m, -1, -2)), wires, n).astype(lam.dtype)
    return grads, lam
