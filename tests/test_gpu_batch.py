"""Persistent circuit batches on the GPU (tqk_batch_run) against the oracle: <Z> and
final states of mixed batches -- one-tile circuits that live in shared memory and
multi-pass circuits (n > 14) that stream their state -- and the uneven-batch workload
(layered RY/RZ + CZ-ladder circuits of random width and depth) at a reduced size."""
import numpy as np
import pytest

from oracle import statevec as O
from tests.test_batch_plan import _random_gates

pytestmark = pytest.mark.gpu


def _z(state, n, wire):
    return float(O.expval_pauli(state[None], "".join("Z" if w == wire else "I" for w in range(n)), n)[0])


def test_mixed_batch_vs_oracle():
    from torchquantum_gb300 import batch as B

    rng = np.random.default_rng(11)
    cb = B.CircuitBatch()
    refs = []
    for n in [1, 2, 5, 9, 13, 14, 15, 16, 17, 6]:
        zw = int(rng.integers(n))
        if n % 3 == 0 and n > 1:
            L = int(rng.integers(1, 5))
            ry, rz = rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n))
            cb.add_layered(n, ry, rz, z_wire=zw)
            gates = []
            for l in range(L):
                gates += [{"name": "ry", "wires": [w], "params": np.array([[ry[l, w]]])} for w in range(n)]
                gates += [{"name": "rz", "wires": [w], "params": np.array([[rz[l, w]]])} for w in range(n)]
                gates += [{"name": "cz", "wires": [w, w + 1], "params": None} for w in range(n - 1)]
        else:
            gl = _random_gates(rng, n, 50) if n > 1 else [{"name": "u3", "wires": [0], "params": [0.3, 0.2, 0.1]}]
            cb.add_gates(n, gl, z_wire=zw)
            gates = [dict(g, params=None if g["params"] is None else np.asarray(g["params"])[None]) for g in gl]
        refs.append((n, zw, O.run(n, 1, gates)[0]))
    res = cb.run(return_states=True)
    for (n, zw, ref), z, st in zip(refs, res.z, res.states):
        np.testing.assert_allclose(st.cpu().numpy(), ref, atol=2e-5)
        assert abs(z - _z(ref, n, zw)) < 2e-5
    assert (res.latency_ms > 0).all() and res.latency_ms.max() <= res.kernel_ms + 1.0


def test_uneven_batch_vs_oracle():
    from torchquantum_gb300 import batch as B

    rng = np.random.default_rng(4)
    cb = B.CircuitBatch()
    refs = []
    for _ in range(24):
        n, L = int(rng.integers(8, 19)), int(rng.integers(2, 9))
        ry, rz = rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n))
        cb.add_layered(n, ry, rz)
        refs.append((n, L, ry, rz))
    res = cb.run()
    for (n, L, ry, rz), z in zip(refs, res.z):
        gates = []
        for l in range(L):
            gates += [{"name": "ry", "wires": [w], "params": np.array([[ry[l, w]]])} for w in range(n)]
            gates += [{"name": "rz", "wires": [w], "params": np.array([[rz[l, w]]])} for w in range(n)]
            gates += [{"name": "cz", "wires": [w, w + 1], "params": None} for w in range(n - 1)]
        assert abs(z - _z(O.run(n, 1, gates)[0], n, 0)) < 2e-5
    assert res.kernel_ms > 0 and np.isfinite(res.latency_ms).all()
