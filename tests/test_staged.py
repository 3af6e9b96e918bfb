"""Staged low-qubit runs of the plain method (tqk_staged_apply / tqk_staged_adjoint).

* CPU: which ops the plain method groups into one shared-memory pass (targets in the
  lowest 12 index bits, diagonal ops anywhere, at most 64 ops, runs of two or more) and
  that grouping keeps the gate order.
* GPU: states, expvals and gradients of random circuits weighted towards the low wires
  (dense, controlled, controlled-X, phase and diagonal gates, shared and per-sample
  parameters) are the same with staging on and off, and match the oracle; the C ABI
  rejects a run whose target lies outside the tile.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from torchquantum_gb300 import engine
from torchquantum_gb300 import program as P


def _op(kind, wires, nc=0, rows=1, k=1):
    if kind == engine.KIND_X:
        return engine.TapeOp(kind, wires, controls=wires[:nc], targets=wires[nc:])
    if kind == engine.KIND_PHASE:
        return engine.TapeOp(kind, wires, operand=torch.ones(rows, dtype=torch.complex64))
    if kind == engine.KIND_DIAG:
        return engine.TapeOp(kind, wires, operand=torch.ones(rows, 1 << len(wires), dtype=torch.complex64))
    if kind == engine.KIND_SWAP:
        return engine.TapeOp(kind, wires, controls=wires[:nc], targets=wires[nc:])
    m = torch.eye(2, dtype=torch.complex64).repeat(rows, 1, 1)
    if kind == engine.KIND_CTRL:
        return engine.TapeOp(kind, wires, controls=wires[:nc], targets=wires[nc:], operand=m)
    return engine.TapeOp(kind, wires, operand=m if len(wires) == 1 else torch.eye(4, dtype=torch.complex64)[None])


def test_stage_runs_grouping():
    n = 20  # tile = wires 8..19
    D, C, X, PH, DG, SW = (engine.KIND_DENSE, engine.KIND_CTRL, engine.KIND_X, engine.KIND_PHASE, engine.KIND_DIAG,
                           engine.KIND_SWAP)
    ops = [_op(D, [19]), _op(C, [0, 12], nc=1), _op(X, [3, 9], nc=1), _op(PH, [0, 1]), _op(DG, [2, 5]),
           _op(D, [2]),                                  # target outside the tile: breaks the run
           _op(D, [10]),                                 # a lone stageable op stays on its own kernel
           _op(SW, [18, 19]),                            # swaps are not staged
           _op(X, [1, 2, 15], nc=2), _op(D, [8]), _op(DG, [0, 1, 2]),  # 3-wire diagonal breaks the run
           _op(D, [9]), _op(D, [11, 12])]                # 2-wire dense is not staged
    out = P.stage_runs(ops, n)
    kinds = [("run", len(o.ops)) if isinstance(o, P.StagedRun) else o.kind for o in out]
    assert kinds == [("run", 5), D, D, SW, ("run", 2), DG, D, D]
    flat = [m for o in out for m in (o.ops if isinstance(o, P.StagedRun) else [o])]
    assert flat == ops
    assert all(o.tile_bits == 12 for o in out if isinstance(o, P.StagedRun))
    long = [_op(D, [19]) for _ in range(150)]
    runs = P.stage_runs(long, n)
    assert [len(r.ops) for r in runs] == [64, 64, 22]
    small = P.stage_runs([_op(D, [0]), _op(D, [1]), _op(C, [1, 0], nc=1)], 4)
    assert len(small) == 1 and small[0].tile_bits == 4
    nonunitary = _op(D, [19])
    nonunitary.uncompute = nonunitary.operand
    assert not P.stageable(nonunitary, n, 12)


def _random_low_circuit(rng, n, depth, bsz):
    """Gate dicts for the public API and the oracle; targets mostly on the low wires."""
    low = list(range(max(0, n - 12), n))
    gates = []
    for _ in range(depth):
        r = rng.random()
        def pick(k, pool_low=True):
            pool = low if (pool_low and rng.random() < 0.85) else list(range(n))
            return [int(w) for w in rng.choice(pool, size=k, replace=False)] if len(pool) >= k else \
                [int(w) for w in rng.choice(n, size=k, replace=False)]
        if r < 0.35:
            name, npar = ["u3", "rx", "ry", "rz", "hadamard", "sx"][int(rng.integers(6))], None
        elif r < 0.55:
            name = ["crx", "cry", "crz", "cu3"][int(rng.integers(4))]
        elif r < 0.7:
            name = ["cnot", "toffoli"][int(rng.integers(2))]
        elif r < 0.85:
            name = ["cz", "cu1", "rzz"][int(rng.integers(3))]
        else:
            name = ["swap", "rxx"][int(rng.integers(2))]
        from torchquantum_gb300 import gates as G

        gd = G.GATES[G.canonical_name(name)]
        wires = pick(gd.num_wires)
        p = None
        if gd.num_params:
            rows = bsz if rng.random() < 0.5 else 1
            p = rng.uniform(-np.pi, np.pi, size=(rows, gd.num_params))
        gates.append({"name": name, "wires": wires, "params": p})
    return gates


@pytest.mark.gpu
@pytest.mark.parametrize("n,bsz,seed", [(5, 3, 0), (12, 2, 1), (14, 3, 2), (17, 2, 3)])
def test_staged_matches_gate_by_gate_and_oracle(n, bsz, seed):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(seed)
    gates = _random_low_circuit(rng, n, 80, bsz)
    paulis = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(3)]
    dev = torch.device("cuda")
    res = {}
    for stage in (True, False):
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
        q.stage_low = stage
        leaves = []
        for g in gates:
            p = None
            if g["params"] is not None:
                p = torch.tensor(g["params"], dtype=torch.float32, device=dev, requires_grad=True)
                leaves.append(p)
            tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=p)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        ev.sum().backward()
        nruns = sum(isinstance(o, P.StagedRun) for sg in q._tape for o in sg.exec_ops)
        res[stage] = (q.get_states_1d().detach().cpu().numpy(), ev.detach().cpu().numpy(),
                      [l.grad.cpu().numpy() for l in leaves], nruns)
    assert res[True][3] > 0 and res[False][3] == 0
    ref = O.run(n, bsz, [dict(g, params=None if g["params"] is None else np.asarray(g["params"])) for g in gates])
    for stage in (True, False):
        assert np.abs(res[stage][0] - ref).max() < 1e-5
    assert np.abs(res[True][1] - res[False][1]).max() < 1e-5
    for a, b in zip(res[True][2], res[False][2]):
        assert np.abs(a - b).max() < 1e-5


@pytest.mark.gpu
def test_staged_abi_rejects_target_outside_tile():
    from torchquantum_gb300 import _lib

    n = 14
    psi = torch.zeros(1, 1 << n, dtype=torch.complex64, device="cuda")
    m = torch.eye(2, dtype=torch.complex64, device="cuda")[None]
    d = _lib.StagedOp()
    d.kind, d.nwires, d.batch, d.operand = _lib.S_DENSE1, 1, 1, m.data_ptr()
    d.wires[0] = 0  # bit 13, outside a 12-bit tile
    with pytest.raises(_lib.TQKError, match="outside the tile"):
        _lib.staged_apply(psi, n, [d], 12)
    d.wires[0] = 13
    _lib.staged_apply(psi, n, [d], 12)
    with pytest.raises(_lib.TQKError, match="tile_bits"):
        _lib.staged_apply(psi, n, [d], 13)


def _pair_base(q, lb):
    """Host model of staged.cu's pair_base (index of the first pair of pair-pair q)."""
    if lb == 0:
        return q << 1
    lowm = (1 << (lb - 1)) - 1
    return ((q >> (lb - 1)) << (lb + 1)) | ((q & lowm) << 1)


@pytest.mark.parametrize("m", [1, 2, 3, 5, 8, 12])
def test_staged_pair_indexing_covers_every_pair_once(m):
    """The staged kernels visit, for a target bit lb of a 2^m tile, every amplitude pair
    (i, i | 2^lb) with bit lb of i clear exactly once, through 16-byte-aligned float4
    accesses inside the tile (checked on the CPU before any launch)."""
    tsz = 1 << m
    for lb in range(m):
        nq = tsz >> 1 if lb == 0 else tsz >> 2
        seen = []
        for q in range(nq):
            i0 = _pair_base(q, lb)
            assert i0 % 2 == 0 and (i0 >> lb) & 1 == 0
            if lb == 0:
                seen.append((i0, i0 + 1))
            else:
                i1 = i0 | (1 << lb)
                assert i1 < tsz and i1 % 2 == 0
                seen += [(i0, i1), (i0 + 1, i1 + 1)]
        want = [(i, i | (1 << lb)) for i in range(tsz) if not (i >> lb) & 1]
        assert sorted(seen) == want
