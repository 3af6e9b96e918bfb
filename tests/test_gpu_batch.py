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


def _layered_ref(n, ry, rz):
    gates = []
    for l in range(ry.shape[0]):
        gates += [{"name": "ry", "wires": [w], "params": np.array([[ry[l, w]]])} for w in range(n)]
        gates += [{"name": "rz", "wires": [w], "params": np.array([[rz[l, w]]])} for w in range(n)]
        gates += [{"name": "cz", "wires": [w, w + 1], "params": None} for w in range(n - 1)]
    return O.run(n, 1, gates)[0]


def _layered_batch(rng, sizes, L):
    from torchquantum_gb300 import batch as B

    cb = B.CircuitBatch()
    spec = []
    for n in sizes:
        ry, rz = rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n))
        cb.add_layered(n, ry, rz)
        spec.append((n, ry, rz))
    return cb, spec


@pytest.mark.parametrize("cfg_idx", range(6))
def test_every_launch_shape_vs_oracle(cfg_idx):
    """Each candidate the autotuner may pick (tile 2^11..2^14, 128..512 threads, 1..8 CTAs
    per SM) gives the oracle's states: tiles narrower than a circuit split it into more
    passes."""
    from torchquantum_gb300 import autotune as A

    cands = A.batch_candidates(17)
    if cfg_idx >= len(cands):
        pytest.skip("fewer candidates")
    cfg = cands[cfg_idx]
    rng = np.random.default_rng(20 + cfg_idx)
    cb, spec = _layered_batch(rng, [5, 9, 11, 12, 13, 15, 17], 3)
    res = cb.run(return_states=True, config=cfg)
    for (n, ry, rz), z, st in zip(spec, res.z, res.states):
        ref = _layered_ref(n, ry, rz)
        np.testing.assert_allclose(st.cpu().numpy(), ref, atol=2e-5)
        assert abs(z - _z(ref, n, 0)) < 2e-5


def test_graph_replay_autotuned_and_new_angles(tmp_path, monkeypatch):
    """config="auto" picks a launch shape by timing the candidates; the batch is captured
    in a CUDA graph; replays give the same <Z>; set_matrices + replay gives the oracle's
    values for new angles."""
    from torchquantum_gb300 import autotune as A
    from torchquantum_gb300 import batch as B

    monkeypatch.setenv("TQ_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    A.clear()
    rng = np.random.default_rng(7)
    sizes = [int(rng.integers(8, 17)) for _ in range(24)]
    cb, spec = _layered_batch(rng, sizes, 4)
    pb = cb.prepare(config="auto").capture()
    assert A.lookup(next(k for k in A._MEM if k.startswith("batch|")))["config"]["tile_bits"] == pb.config.tile_bits
    pb.launch()
    z1 = pb.result().z
    pb.launch()
    r2 = pb.result()
    np.testing.assert_allclose(z1, r2.z, atol=1e-12)  # multi-tile circuits add partials atomically
    for (n, ry, rz), z in zip(spec, z1):
        assert abs(z - _z(_layered_ref(n, ry, rz), n, 0)) < 2e-5
    new = [(n, rng.uniform(-np.pi, np.pi, (4, n)), rng.uniform(-np.pi, np.pi, (4, n))) for n in sizes]
    pb.set_matrices(np.concatenate([B.layered_matrices(n, ry, rz) for n, ry, rz in new]))
    pb.launch()
    r3 = pb.result()
    for (n, ry, rz), z in zip(new, r3.z):
        assert abs(z - _z(_layered_ref(n, ry, rz), n, 0)) < 2e-5
    assert r3.kernel_ms > 0 and (r3.latency_ms > 0).all()
    A.clear()


def test_bounded_wait_reports_timeout():
    """Failure detection without a GPU fault: a work list missing every tile of a
    circuit's first pass leaves the second pass's tiles waiting on a counter that nothing
    raises; their bounded waits (~2 s) give up, the kernel finishes, and the host reads
    TQK_TIMEOUT from the status word."""
    import torch

    from torchquantum_gb300 import _lib
    from torchquantum_gb300 import batch as B

    n = 16
    rng = np.random.default_rng(3)
    cb = B.CircuitBatch()
    cb.add_layered(n, rng.uniform(-np.pi, np.pi, (2, n)), rng.uniform(-np.pi, np.pi, (2, n)))
    circ, ops, passes, items, mats, order, state_amps = cb.compile(tile_bits=14)
    assert circ[0]["num_passes"] >= 2
    first = int(circ[0]["first_pass"])
    kept = items[items["pass"] != first]  # pass 1 waits for tiles that are never run
    dev = torch.device("cuda")

    def up(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).to(dev)

    d_circ, d_ops, d_pass, d_items, d_mats = up(circ), up(ops), up(passes), up(kept), up(mats)
    states = torch.zeros(max(1, state_amps), dtype=torch.complex64, device=dev)
    z = torch.zeros(1, dtype=torch.float64, device=dev)
    pass_done = torch.zeros(len(passes), dtype=torch.int32, device=dev)
    counter = torch.zeros(1, dtype=torch.int32, device=dev)
    status = _lib.status_word(dev)
    status.zero_()
    cfg = B.DEFAULT_CONFIG.as_struct()
    rc = _lib.load().tqk_batch_run(d_circ.data_ptr(), 1, d_ops.data_ptr(), d_pass.data_ptr(), d_items.data_ptr(),
                                   len(kept), d_mats.data_ptr(), states.data_ptr(), 0, z.data_ptr(),
                                   pass_done.data_ptr(), None, counter.data_ptr(), status.data_ptr(),
                                   cfg.ctypes.data, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    with pytest.raises(_lib.TQKError, match="TIMEOUT|bounded wait"):
        _lib.check_status(dev)
    assert int(status.item()) == 0  # check_status clears the word; the context stays usable
    res = cb.run(config=B.DEFAULT_CONFIG)
    assert np.isfinite(res.z).all()
