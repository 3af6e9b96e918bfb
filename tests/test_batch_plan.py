"""Circuit batches on the CPU: the IR compiler (torchquantum_gb300.batch) and the host
planner (tqk_batch_plan, host code in libtqk.so) checked with the oracle.

* the IR a gate list compiles to (fused one-qubit matrices, controlled blocks, CZ)
  simulates to the oracle's state;
* the planner only regroups ops of one circuit, keeps every pass's targets inside its
  tile of 2^tile_bits amplitudes (tile_bits 10, 12, 14; with address bits 0-4, for
  coalescing), flags the first and last passes, and its regrouped order simulates to
  the same state as the original;
* invalid circuits are rejected with the library's status codes.
"""
import numpy as np
import pytest

from oracle import statevec as O
from torchquantum_gb300 import batch as B


def _simulate_ir(n, ops, mats):
    """The IR's semantics, op by op, with the oracle's dense application."""
    s = O.init_state(n, 1).astype(np.complex128)
    for op in ops:
        k, w0, w1 = int(op["kind"]), int(op["w0"]), int(op["w1"])
        if k == B.DENSE1:
            s = O.apply(s, mats[op["mat"]][None], [w0], n)
        elif k == B.CTRL1:
            m = np.eye(4, dtype=np.complex128)
            m[2:, 2:] = mats[op["mat"]]
            s = O.apply(s, m[None], [w0, w1], n)
        elif k == B.CZ:
            s = O.apply(s, np.diag([1, 1, 1, -1]).astype(np.complex128)[None], [w0, w1], n)
        else:
            for w in range(w0, w1):
                s = O.apply(s, np.diag([1, 1, 1, -1]).astype(np.complex128)[None], [w, w + 1], n)
    return s[0]


def _random_gates(rng, n, depth):
    names1 = ["u3", "rx", "ry", "rz", "hadamard", "s", "t", "sx"]
    names2 = ["cnot", "cz", "crx", "cry", "crz", "cu3", "cu1"]
    from torchquantum_gb300 import gates as G

    out = []
    for _ in range(depth):
        if rng.random() < 0.6:
            name = names1[rng.integers(len(names1))]
            wires = [int(rng.integers(n))]
        else:
            name = names2[rng.integers(len(names2))]
            wires = [int(w) for w in rng.choice(n, 2, replace=False)]
        npar = G.GATES[G.canonical_name(name)].num_params
        p = rng.uniform(-np.pi, np.pi, size=npar) if npar else None
        out.append({"name": name, "wires": wires, "params": p})
    return out


@pytest.mark.parametrize("n", [3, 6, 9])
def test_compiled_ir_matches_oracle(n):
    rng = np.random.default_rng(n)
    gates = _random_gates(rng, n, 60)
    cb = B.CircuitBatch()
    cb.add_gates(n, gates)
    got = _simulate_ir(n, cb._ops[0], cb._mats[0].astype(np.complex128))
    ref = O.run(n, 1, [dict(g, params=None if g["params"] is None else np.asarray(g["params"])[None]) for g in gates])
    np.testing.assert_allclose(got, ref[0], atol=1e-5)
    assert len(cb._ops[0]) < len(gates)  # consecutive one-qubit gates were fused


def test_layered_ir_matches_gate_list():
    n, L = 5, 3
    rng = np.random.default_rng(1)
    ry, rz = rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n))
    cb = B.CircuitBatch()
    cb.add_layered(n, ry, rz)
    gates = []
    for l in range(L):
        gates += [{"name": "ry", "wires": [w], "params": np.array([[ry[l, w]]])} for w in range(n)]
        gates += [{"name": "rz", "wires": [w], "params": np.array([[rz[l, w]]])} for w in range(n)]
        gates += [{"name": "cz", "wires": [w, w + 1], "params": None} for w in range(n - 1)]
    got = _simulate_ir(n, cb._ops[0], cb._mats[0].astype(np.complex128))
    np.testing.assert_allclose(got, O.run(n, 1, gates)[0], atol=1e-6)


@pytest.mark.parametrize("tile_bits", [10, 12, 14])
def test_plan_regroups_legally(tile_bits):
    T = tile_bits
    rng = np.random.default_rng(3)
    cb = B.CircuitBatch()
    sizes = [15, 4, 16, 12, 17, 11]
    for n in sizes:
        if n % 2:
            L = int(rng.integers(2, 5))
            cb.add_layered(n, rng.uniform(-np.pi, np.pi, (L, n)), rng.uniform(-np.pi, np.pi, (L, n)), z_wire=n - 1)
        else:
            cb.add_gates(n, _random_gates(rng, n, 40))
    circ, ops, passes, items, mats, order, state_amps = cb.compile(tile_bits=T)
    # work items: one per (circuit, pass, tile); a pass's items come after all items of
    # the circuit's previous pass
    seen = {}
    for k, it in enumerate(items):
        seen.setdefault(int(it["pass"]), []).append(k)
    for slot in range(len(circ)):
        c = circ[slot]
        for w in range(int(c["num_passes"])):
            pi = int(c["first_pass"]) + w
            ks = seen[pi]
            assert len(ks) == 1 << (int(c["n"]) - bin(int(passes[pi]["tile_mask"])).count("1"))
            assert all(int(items[k]["circuit"]) == slot for k in ks)
            if w:
                assert min(ks) > max(seen[pi - 1])
    assert sorted(order) == list(range(len(sizes)))
    assert state_amps == sum(1 << n for n in sizes if n > T)
    for slot, i in enumerate(order):
        c = circ[slot]
        n = int(c["n"])
        assert n == sizes[i]
        mine = ops[c["first_op"]:c["first_op"] + c["num_ops"]]
        orig = cb._ops[i]
        key = lambda a: sorted(map(tuple, np.stack([a["kind"], a["w0"], a["w1"]], 1).tolist()))
        assert key(mine) == key(orig)  # a permutation of the circuit's own ops
        ps = passes[c["first_pass"]:c["first_pass"] + c["num_passes"]]
        assert ps[0]["flags"] & 1 and ps[-1]["flags"] & 2
        covered = 0
        for p in ps:
            tm = int(p["tile_mask"])
            assert bin(tm).count("1") == min(n, T) and tm < (1 << n)
            if n > T:
                assert tm & 0x1F == 0x1F
            for op in ops[p["first_op"]:p["first_op"] + p["num_ops"]]:
                k = int(op["kind"])
                tgt = int(op["w0"]) if k == B.DENSE1 else int(op["w1"]) if k == B.CTRL1 else None
                if tgt is not None:
                    assert (tm >> (n - 1 - tgt)) & 1
            covered += int(p["num_ops"])
        assert covered == len(orig)
        m64 = cb._mats[i].astype(np.complex128)
        mine_local = mine.copy()
        mine_local["mat"] = np.where(mine["mat"] >= 0, mine["mat"] - _mat_base(cb, order, slot), -1)
        np.testing.assert_allclose(_simulate_ir(n, mine_local, m64), _simulate_ir(n, orig, m64), atol=1e-9)


def _mat_base(cb, order, slot):
    return sum(len(cb._mats[j]) for j in order[:slot])


def test_plan_rejects_invalid():
    from torchquantum_gb300 import _lib

    cb = B.CircuitBatch()
    cb.add_ops(3, np.array([(B.CTRL1, 1, 1, 0)], dtype=B.OP_T), np.eye(2)[None])
    with pytest.raises(_lib.TQKError, match="BAD_WIRES"):
        cb.compile()
    cb = B.CircuitBatch()
    cb.add_ops(3, np.array([(B.DENSE1, 5, 0, 0)], dtype=B.OP_T), np.eye(2)[None])
    with pytest.raises(_lib.TQKError, match="BAD_WIRES"):
        cb.compile()
    cb = B.CircuitBatch()
    cb.add_ops(4, np.array([(B.CZ_LADDER, 2, 1, -1)], dtype=B.OP_T), np.zeros((0, 2, 2)))
    with pytest.raises(_lib.TQKError, match="BAD_WIRES"):
        cb.compile()
    cb = B.CircuitBatch()
    cb.add_ops(3, np.array([(B.DENSE1, 0, 0, 1)], dtype=B.OP_T), np.eye(2)[None])  # only matrix 0 exists
    with pytest.raises(_lib.TQKError, match="BAD_SHAPE"):
        cb.compile()
    with pytest.raises(ValueError):
        B.CircuitBatch().add_ops(25, np.zeros(0, B.OP_T), np.zeros((0, 2, 2)))
    cb = B.CircuitBatch()
    cb.add_ops(3, np.array([(B.DENSE1, 0, 0, 0)], dtype=B.OP_T), np.eye(2)[None])
    for bad in (9, 15):
        with pytest.raises(_lib.TQKError, match="BAD_SHAPE"):
            cb.compile(tile_bits=bad)
    with pytest.raises(ValueError, match="not supported"):
        B.CircuitBatch().add_gates(3, [{"name": "swap", "wires": [0, 1], "params": None}])


def test_op_history_ingestion():
    """A device's op_history (scalar wires for one-qubit gates, scalar or list params,
    inverse flags) compiles to a batch circuit with the oracle's state."""
    n = 4
    hist = [{"name": "u3", "wires": 2, "params": [0.3, -0.7, 1.1], "inverse": False, "trainable": True},
            {"name": "rx", "wires": 0, "params": 0.4, "inverse": True, "trainable": False},
            {"name": "crx", "wires": [0, 3], "params": 1.3, "inverse": True, "trainable": True},
            {"name": "cnot", "wires": [3, 1], "params": None, "inverse": False, "trainable": False},
            {"name": "sx", "wires": 1, "params": None, "inverse": True, "trainable": False},
            {"name": "cz", "wires": [1, 2], "params": None, "inverse": False, "trainable": False}]
    cb = B.CircuitBatch()
    cb.add_gates(n, hist)
    got = _simulate_ir(n, cb._ops[0], cb._mats[0].astype(np.complex128))
    og = [{"name": h["name"], "wires": list(np.atleast_1d(h["wires"])), "inverse": h["inverse"],
           "params": None if h["params"] is None else np.atleast_1d(np.asarray(h["params"], np.float64))[None]}
          for h in hist]
    np.testing.assert_allclose(got, O.run(n, 1, og)[0], atol=1e-6)
    with pytest.raises(ValueError, match="one parameter row"):
        B.CircuitBatch().add_gates(2, [{"name": "rx", "wires": 0, "params": [[0.1], [0.2]]}])


def _local_pos(tmask, b):
    return bin(tmask & ((1 << b) - 1)).count("1")


def _cz_terms(tmask, base, b0, b1, st):
    """Host model of batch.cu's cz_terms: split a CZ's sign into tile-local terms."""
    in0, in1 = (tmask >> b0) & 1, (tmask >> b1) & 1
    if in0 and in1:
        p0, p1 = _local_pos(tmask, b0), _local_pos(tmask, b1)
        lo, hi = min(p0, p1), max(p0, p1)
        if hi == lo + 1:
            st["quad"] |= 1 << lo
        else:
            st["pairs"] |= (1 << lo) | (1 << hi)
    elif in0:
        if (base >> b1) & 1:
            st["lin"] ^= 1 << _local_pos(tmask, b0)
    elif in1:
        if (base >> b0) & 1:
            st["lin"] ^= 1 << _local_pos(tmask, b1)
    else:
        st["c0"] ^= (base >> b0) & (base >> b1) & 1


def test_cz_sign_split_matches_global_index():
    """The batch kernel's CZ / CZ-ladder signs, computed from the tile-local index with
    per-tile constants, equal the signs computed from each amplitude's global index."""
    rng = np.random.default_rng(0)
    for _ in range(60):
        n = int(rng.integers(3, 16))
        tb = int(rng.integers(1, n + 1))
        bits = sorted(rng.choice(n, size=tb, replace=False))
        tmask = sum(1 << int(b) for b in bits)
        other = [b for b in range(n) if not (tmask >> b) & 1]
        base = sum(1 << b for b in other if rng.random() < 0.5)
        locs = np.arange(1 << tb)
        glob = np.full(1 << tb, base)
        for j, b in enumerate(bits):
            glob |= ((locs >> j) & 1) << int(b)
        # a ladder over wires w0..w1 and a single CZ
        w0 = int(rng.integers(0, n - 1))
        w1 = int(rng.integers(w0 + 1, n))
        st = {"c0": 0, "lin": 0, "quad": 0, "pairs": 0}
        for w in range(w0, w1):
            _cz_terms(tmask, base, n - 1 - w, n - 2 - w, st)
        assert st["pairs"] == 0
        got = (st["c0"] + np.array([bin(l & st["lin"]).count("1") + bin(l & (l >> 1) & st["quad"]).count("1")
                                    for l in locs])) & 1
        want = np.zeros(1 << tb, dtype=int)
        for w in range(w0, w1):
            want ^= ((glob >> (n - 1 - w)) & (glob >> (n - 2 - w)) & 1)
        assert (got == want).all()
        a, c = [int(x) for x in rng.choice(n, 2, replace=False)]
        st = {"c0": 0, "lin": 0, "quad": 0, "pairs": 0}
        _cz_terms(tmask, base, n - 1 - a, n - 1 - c, st)
        if st["pairs"]:
            got = np.array([(l & st["pairs"]) == st["pairs"] for l in locs]).astype(int)
        else:
            got = (st["c0"] + np.array([bin(l & st["lin"]).count("1") + bin(l & (l >> 1) & st["quad"]).count("1")
                                        for l in locs])) & 1
        want = (glob >> (n - 1 - a)) & (glob >> (n - 1 - c)) & 1
        assert (got == want).all()

