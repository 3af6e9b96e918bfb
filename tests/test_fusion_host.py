"""Fusion planner and block-unitary build (host logic, CPU)."""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from torchquantum_gb300 import engine, fusion
from torchquantum_gb300 import functional as F
from torchquantum_gb300 import gates as G
from torchquantum_gb300 import workloads as W


@pytest.mark.parametrize("k", [2, 3, 4, 5, 6])
def test_plan_respects_dependencies_and_width(k):
    gates, _ = W.random_circuit(12, 300, seed=k)
    wl = [g["wires"] for g in gates]
    blocks = fusion.plan_blocks(wl, k)
    order = [i for _, idxs in blocks for i in idxs]
    assert sorted(order) == list(range(len(wl)))
    pos = {g: p for p, g in enumerate(order)}
    for _, idxs in blocks:
        assert len(set(w for i in idxs for w in wl[i])) <= k
    for a in range(len(wl)):
        for b in range(a + 1, len(wl)):
            if set(wl[a]) & set(wl[b]):
                assert pos[a] < pos[b], (a, b)


def test_plan_fuses_runs():
    gates, _ = W.random_circuit(24, 400, seed=0)
    blocks = fusion.plan_blocks([g["wires"] for g in gates], 6)
    assert len(blocks) < 60  # ~9 gates per 6-wire block on this circuit


def _op(name, wires, params, inverse=False):
    gd = G.GATES[name]
    n_w = gd.num_wires if gd.num_wires > 0 else len(wires)
    p = None if params is None else torch.tensor(params, dtype=torch.float64)
    m = G.gate_matrix(name, p, n_w, dtype=torch.complex128)
    if inverse:
        m = m.conj().transpose(-1, -2)
    return F._op_from_matrix(name, m, list(wires), torch.device("cpu"))


def test_block_unitary_matches_oracle_product():
    rng = np.random.default_rng(0)
    names = ["u3", "cnot", "cz", "crx", "rzz", "swap", "toffoli", "s", "cswap", "ry", "multicnot"]
    for trial in range(20):
        k = int(rng.integers(2, 6))
        bw = sorted(int(w) for w in rng.permutation(8)[:k])
        ops, ogates = [], []
        for _ in range(8):
            nm = names[rng.integers(len(names))]
            gd = G.GATES[nm]
            nw = gd.num_wires if gd.num_wires > 0 else 3
            if nw > k:
                continue
            wires = [int(w) for w in rng.permutation(bw)[:nw]]
            p = rng.uniform(-np.pi, np.pi, size=(2, gd.num_params)) if gd.num_params else None
            inv = bool(rng.random() < 0.3)
            ops.append(_op(nm, wires, p, inv))
            ogates.append({"name": nm, "wires": wires, "params": p, "inverse": inv, "n_wires": nw})
        if not ops:
            continue
        u = fusion.build_block_unitary(ops, bw, torch.device("cpu")).numpy()
        # oracle: apply the gates to the 2^k basis states of the block wires (relabelled 0..k-1)
        relabel = {w: i for i, w in enumerate(bw)}
        eye = np.eye(1 << k, dtype=np.complex128)
        for b in range(u.shape[0]):
            og = [dict(g, wires=[relabel[w] for w in g["wires"]],
                       params=None if g["params"] is None else g["params"][b:b + 1]) for g in ogates]
            cols = O.run(k, 1 << k, og, state=eye)  # row j = U e_j
            np.testing.assert_allclose(u[b], cols.T, atol=1e-12)


def test_ops_blocks_cannot_hold_stay_alone_on_small_states():
    """An op the block kernels cannot hold (a 3-wire dense matrix, an op with an explicit
    uncompute) is a planner barrier: on a 4-wire state, where all wires fit one 6-wire
    block, every planner still leaves it alone and moves no gate across it."""
    from torchquantum_gb300 import program as P

    n = 4

    def dense(wires):
        d = 1 << len(wires)
        return engine.TapeOp(engine.KIND_DENSE, wires, operand=torch.eye(d, dtype=torch.complex64)[None])

    wide = dense([0, 1, 2])
    nonunitary = dense([3])
    nonunitary.uncompute = torch.eye(2, dtype=torch.complex64)[None]
    ops = [dense([0]), dense([1]), wide, dense([2]), dense([3]), nonunitary, dense([0]), dense([1, 2])]
    assert not P.fusable(wide) and not P.fusable(nonunitary) and P.fusable(ops[0])
    wl = P.planner_wires(ops, n)
    assert len(wl[2]) > 6 and len(wl[5]) > 6
    for plan in (fusion.plan_blocks(wl, 6), fusion.plan_blocks(wl, 6, 8), fusion.plan_beam(wl, 6, 4, 8)):
        where = {i: b for b, (_, idxs) in enumerate(plan) for i in idxs}
        for barrier in (2, 5):
            assert plan[where[barrier]][1] == [barrier]
            # no gate after the barrier sits in a block before it, and none before it after
            assert all(where[i] < where[barrier] for i in range(barrier))
            assert all(where[i] > where[barrier] for i in range(barrier + 1, len(ops)))
