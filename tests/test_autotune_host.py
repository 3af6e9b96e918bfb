"""Autotuner host logic on the CPU: the tuning cache (JSON file keyed by GPU and
workload, reloaded by a fresh process), the plan cost model that picks the fusion width,
planner variant and per-block kernel from measured pass costs, the lookahead planner's
legality, and the batch candidates and signature."""
import json

import numpy as np

from torchquantum_gb300 import autotune as A
from torchquantum_gb300 import batch as B
from torchquantum_gb300 import fusion as F
from torchquantum_gb300 import workloads as W


def test_cache_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("TQ_GB300_TUNE_CACHE", str(path))
    A.clear()
    A._store("k1", {"config": {"tile_bits": 13}})
    assert json.loads(path.read_text())["k1"]["config"]["tile_bits"] == 13
    A.clear(memory_only=True)
    monkeypatch.setattr(A, "_LOADED", False)
    assert A.lookup("k1") == {"config": {"tile_bits": 13}}
    monkeypatch.setenv("TQ_GB300_TUNE_CACHE", "off")
    A.clear()
    A._store("k2", {"x": 1})
    assert A.lookup("k2") == {"x": 1}
    A.clear()


def _fake_costs(tc_fwd, tc_adj, dense_slope):
    return {"dense": {str(k): (dense_slope * k, 2 * dense_slope * k) for k in range(1, 7)},
            "tc": (tc_fwd, tc_adj), "rows": 1}


def test_plan_cost_picks_cheaper_kernel():
    plan = [([0, 1, 2, 3, 4, 5], [0, 1, 2]), ([1, 2], [3]), ([0, 1, 2, 3], [4, 5])]
    c, flags = A.plan_cost(plan, _fake_costs(1.0, 2.0, 1.0), True, False)
    assert flags == [True, False, True] and c == 1.0 + 2.0 + 1.0
    c, flags = A.plan_cost(plan, _fake_costs(100.0, 200.0, 0.1), True, True)
    assert flags == [False, False, False]
    assert abs(c - (0.6 + 1.2 + 0.2 + 0.4 + 0.4 + 0.8)) < 1e-12
    c, flags = A.plan_cost(plan, _fake_costs(1.0, 2.0, 1.0), False, False)
    assert flags == [False, False, False]


def test_lone_dense_gate_may_run_as_tensor_core_block():
    """A gate alone in its block keeps its own kernel unless it is a dense / controlled gate
    and a tensor-core block costs less than its dense pass with a cotangent; structured
    lone gates are costed with the measured light pass."""
    plan = [([0, 1, 2, 3, 4, 5], [0, 1, 2]), ([1, 2], [3]), ([7], [4]), ([0] * 30, [5])]
    costs = {"dense": {str(k): (1.0, 4.0) for k in range(1, 7)}, "tc": (0.7, 1.4, 1.1), "rows": 1}
    c, flags = A.plan_cost(plan, costs, True, True, stored=True)
    assert flags == [True, False, False, False] and abs(c - (1.8 + 3 * 5.0)) < 1e-12
    D, L, O = A.LONE_DENSE, A.LONE_LIGHT, A.LONE_OTHER
    lone = [D, D, D, D, L, O]
    c, flags = A.plan_cost(plan, costs, True, True, stored=True, lone_kind=lone)
    # gate 3 (dense, 2 wires) runs as a block; gate 4 (light) keeps its kernel, costed as a
    # dense pass while no light cost was measured; the 30-wire barrier op never is a block
    assert flags == [True, True, False, False] and abs(c - (1.8 + 1.8 + 5.0 + 5.0)) < 1e-12
    costs["light"] = (0.4, 0.8)
    c, flags = A.plan_cost(plan, costs, True, True, stored=True, lone_kind=lone)
    assert flags == [True, True, False, False] and abs(c - (1.8 + 1.8 + 1.2 + 5.0)) < 1e-12
    # without tensor cores the dense lone gate keeps its own kernel
    c, flags = A.plan_cost(plan, costs, False, True, stored=True, lone_kind=lone)
    assert flags == [False] * 4 and abs(c - (5.0 + 5.0 + 1.2 + 5.0)) < 1e-12


def test_choose_fusion_picks_cheapest_candidate(monkeypatch):
    gates, _ = W.random_circuit(24, 200, seed=0)
    wl = [g["wires"] for g in gates]
    monkeypatch.setattr(A, "pass_costs", lambda n, bsz, dev, tc_ok: _fake_costs(1.0, 2.0, 5.0))
    plan, flags, k, _ = A.choose_fusion(wl, 24, 16, None, True, True)
    assert k == 6 and all(flags[i] for i, (_, idx) in enumerate(plan) if len(idx) > 1)
    costs = _fake_costs(1.0, 2.0, 5.0)
    cands = [F.plan_cached(wl, kk, la, bm) for kk in (4, 5, 6) for la, bm in ((0, 0), (8, 0), (8, 4))]
    # 16 x 2^24 amplitudes: the wide beams are candidates for 6-wire blocks as well
    wide = [F.plan_cached(wl, 6, la, bm) for la, bm in A.WIDE_BEAMS]
    for w in wide:
        _check_legal(wl, w, 6)
        assert len(w) <= len(F.plan_cached(wl, 6, 8, 4))
    best = min(A.plan_cost(c, costs, True, True)[0] for c in cands + wide)
    assert A.plan_cost(plan, costs, True, True)[0] == best
    assert best <= A.plan_cost(F.plan_blocks(wl, 6), costs, True, True)[0]
    # a small state (16 x 2^20 amplitudes) keeps the three cheaper candidates only
    plan_s, _, _, _ = A.choose_fusion(wl, 20, 16, None, True, True)
    assert any(plan_s is F.plan_cached(wl, kk, la, bm) for kk in (4, 5, 6) for la, bm in ((0, 0), (8, 0), (8, 4)))


def test_lookahead_plan_is_legal_and_not_worse():
    for seed in range(3):
        gates, _ = W.random_circuit(20, 150, seed=seed)
        wl = [g["wires"] for g in gates]
        for k in (4, 6):
            base, look = F.plan_blocks(wl, k), F.plan_blocks(wl, k, 8)
            beam = F.plan_beam(wl, k, 4)
            assert len(look) <= len(base) + 1 and len(beam) <= len(look)
            for plan in (look, beam):
                _check_legal(wl, plan, k)
    assert F.plan_cached(wl, 6, 8) is F.plan_cached([list(w) for w in wl], 6, 8)


def _check_legal(wl, plan, k):
    """Every gate exactly once; a gate never moves ahead of an earlier gate sharing a wire."""
    if True:
        if True:
            pos = {}
            for bi, (bw, idxs) in enumerate(plan):
                assert len(bw) <= k
                for gi in idxs:
                    assert set(wl[gi]) <= set(bw)
                    pos[gi] = bi
            assert sorted(pos) == list(range(len(wl)))
            for a in range(len(wl)):
                for b in range(a + 1, len(wl)):
                    if set(wl[a]) & set(wl[b]):
                        assert pos[a] <= pos[b]


def test_batch_candidates_and_signature():
    cands = A.batch_candidates(20)
    assert {c.tile_bits for c in cands} >= {12, 13, 14}
    assert all(c.tile_bits <= 11 for c in A.batch_candidates(9))
    for c in cands:
        assert (8 << c.tile_bits) * min(c.ctas_per_sm, 1) <= 227 * 1024
        assert c.as_struct().dtype == B.CONFIG_T
    rng = np.random.default_rng(0)
    cb = B.CircuitBatch()
    for _ in range(10):
        n = int(rng.integers(8, 21))
        cb.add_layered(n, rng.uniform(size=(3, n)), rng.uniform(size=(3, n)))
    s1 = cb.signature()
    cb.add_layered(9, rng.uniform(size=(3, 9)), rng.uniform(size=(3, 9)))
    assert len(s1) == 13 and cb.signature() != s1


def test_choose_fusion_without_room_for_probes(monkeypatch):
    """If the cost probes cannot allocate their scratch states, the plan is still chosen
    (fewest passes, tensor cores for multi-gate blocks when allowed)."""
    import torch

    def oom(*a, **k):
        raise torch.cuda.OutOfMemoryError("no room")

    monkeypatch.setattr(A, "pass_costs", oom)
    gates, _ = W.random_circuit(20, 120, seed=1)
    wl = [g["wires"] for g in gates]
    plan, flags, k, costs = A.choose_fusion(wl, 20, 4, None, True, True)
    assert costs["rows"] == 0 and k in (4, 5, 6)
    assert all(flags[i] for i, (_, idx) in enumerate(plan) if len(idx) > 1)
    plan, flags, k, costs = A.choose_fusion(wl, 20, 4, None, False, False)
    assert not any(flags)


def test_plan_cost_uses_stored_input_adjoint_when_inputs_are_kept():
    """With stored block inputs the tensor-core reverse step is the stored-input one (the
    third cost entry); without it, or when the cost table predates it, the in-place one."""
    plan = [([0, 1, 2, 3, 4, 5], [0, 1, 2]), ([0, 1, 2, 3, 4, 5], [3, 4])]
    costs = {"dense": {str(k): (10.0, 20.0) for k in range(1, 7)}, "tc": (1.0, 2.0, 1.5), "rows": 1}
    assert A.plan_cost(plan, costs, True, True, stored=False)[0] == 2 * (1.0 + 2.0)
    assert A.plan_cost(plan, costs, True, True, stored=True)[0] == 2 * (1.0 + 1.5)
    assert A.plan_cost(plan, costs, True, False, stored=True)[0] == 2 * 1.0
    old = dict(costs, tc=(1.0, 2.0))
    assert A.plan_cost(plan, old, True, True, stored=True)[0] == 2 * (1.0 + 2.0)
