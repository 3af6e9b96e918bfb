"""Loaders for the committed golden fixtures (produced by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(d["__meta__"])) if "__meta__" in d.files else None
    return d, meta


def circuit_cases():
    """Yield (case meta, gates with numeric params, arrays dict) for circuits.npz."""
    d, meta = load("circuits")
    for case in meta:
        key = case["key"]
        gates = []
        for g in case["gates"]:
            g = dict(g)
            if g["params"] == "unitary":
                g["params"] = d[key + "__unitary"]
            elif g["params"] is not None:
                g["params"] = np.asarray(g["params"], np.float64)
            gates.append(g)
        arrays = {k[len(key) + 2:]: d[k] for k in d.files if k.startswith(key + "__")}
        yield case, gates, arrays
