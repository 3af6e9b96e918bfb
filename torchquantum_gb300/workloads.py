"""Seeded synthetic workloads with the shapes of the benchmark configurations.

All inputs are synthetic (no datasets): angles are drawn from seeded generators with
the stated distributions.  A circuit is a list of gate dicts ``{name, wires,
params_slice}`` over one packed parameter tensor ``theta [bsz, P]`` so that a step
moves all its inputs with a single host->device copy.

* ``random_circuit`` -- plain method at scale: depth-D circuit where each gate is a
  U3 on a uniform wire with probability 0.6, else a uniform choice of CNOT / CZ /
  CRX on a uniform ordered pair of distinct wires; angles ~ U[-pi, pi) per sample.
* ``hea_circuit`` -- hardware-efficient ansatz: L layers of RY, RZ on every wire
  (shared parameters) followed by a CZ ladder (i, i+1).
* ``random_paulis`` -- Pauli strings with per-site uniform {I, X, Y, Z}.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np
import torch

_NP = {"u3": 3, "crx": 1, "cnot": 0, "cz": 0, "ry": 1, "rz": 1, "rx": 1}


def random_circuit(n: int, depth: int, seed: int = 0, p1q: float = 0.6) -> Tuple[List[Dict], int]:
    """Gate list + number of parameter columns (config: n=24, depth=400)."""
    rng = np.random.default_rng(seed)
    gates, off = [], 0
    for _ in range(depth):
        if rng.random() < p1q:
            name, wires = "u3", [int(rng.integers(n))]
        else:
            name = ("cnot", "cz", "crx")[int(rng.integers(3))]
            a, b = rng.choice(n, size=2, replace=False)
            wires = [int(a), int(b)]
        npar = _NP[name]
        gates.append({"name": name, "wires": wires, "off": off, "np": npar})
        off += npar
    return gates, off


def hea_circuit(n: int, layers: int) -> Tuple[List[Dict], int]:
    """RY, RZ on every wire + CZ ladder, per layer (shared parameters)."""
    gates, off = [], 0
    for _ in range(layers):
        for name in ("ry", "rz"):
            for w in range(n):
                gates.append({"name": name, "wires": [w], "off": off, "np": 1})
                off += 1
        for w in range(n - 1):
            gates.append({"name": "cz", "wires": [w, w + 1], "off": off, "np": 0})
    return gates, off


def random_params(bsz: int, ncols: int, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(-np.pi, np.pi, size=(bsz, ncols)).astype(np.float32)


def random_paulis(n: int, m: int, seed: int = 2) -> List[str]:
    rng = np.random.default_rng(seed)
    return ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(m)]


def apply_circuit(qdev, gates: List[Dict], theta: torch.Tensor) -> None:
    """Apply ``gates`` through the public functional API, slicing ``theta`` per gate."""
    from . import functional as tqf

    fns = tqf.func_name_dict
    for g in gates:
        p = theta[:, g["off"]:g["off"] + g["np"]] if g["np"] else None
        fns[g["name"]](qdev, wires=g["wires"], params=p)


def oracle_gates(gates: List[Dict], theta: np.ndarray) -> List[Dict]:
    """The same circuit in the oracle's gate-dict format (float64 params)."""
    out = []
    for g in gates:
        p = theta[:, g["off"]:g["off"] + g["np"]].astype(np.float64) if g["np"] else None
        out.append({"name": g["name"], "wires": g["wires"], "params": p})
    return out
