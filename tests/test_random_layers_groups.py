"""Upstream RandomLayer / RandomLayerAllTypes (layer/layers/random_layers.py:80-298) and
find_observable_groups (measurement/measurements.py:77-111) against fixtures made by
running upstream (tests/golden/random_layers.npz); sampled expectation values
(measurements.py:114-229) against the analytic ones.

* CPU: a seeded layer draws upstream's op sequence, wires and parameters; the grouping
  of observable lists equals upstream's, dict order included.
* GPU: the seeded layers' states match upstream's complex128 states; sampled expvals
  (single and grouped) agree with the analytic values within 5 standard errors.
"""
import json

import numpy as np
import pytest
import torch

from tests.golden_data import load


def _meta():
    d, _ = load("random_layers")
    return d, json.loads(str(d["__meta__"]))


def _build(case):
    import torchquantum_gb300 as tq

    torch.manual_seed(case["seed"])
    return getattr(tq, case["cls"])(n_ops=case["n_ops"], wires=list(range(case["n"])), seed=case["seed"])


def test_random_layer_draws_match_upstream():
    _, meta = _meta()
    for case in meta["layers"]:
        layer = _build(case)
        got = [(o.name, [int(w) for w in np.atleast_1d(o.wires)]) for o in layer.op_list]
        assert got == [(o["name"], o["wires"]) for o in case["ops"]]
        for o, ref in zip(layer.op_list, case["ops"]):
            if ref["params"] is not None:
                np.testing.assert_allclose(o.params.detach().double().numpy(), np.array(ref["params"]), atol=1e-6)


def test_find_observable_groups_matches_upstream():
    import torchquantum_gb300 as tq

    _, meta = _meta()
    for g in meta["groups"]:
        got = tq.find_observable_groups(g["observables"])
        assert list(got.items()) == list(g["groups"].items())


@pytest.mark.gpu
def test_random_layer_states_match_upstream():
    import torchquantum_gb300 as tq

    d, meta = _meta()
    for case in meta["layers"]:
        if not case["state"]:
            continue
        layer = _build(case).to("cuda")
        q = tq.QuantumDevice(n_wires=case["n"], bsz=1, device="cuda")
        layer(q)
        got = q.get_states_1d().detach().cpu().numpy()
        assert np.abs(got - d[case["key"] + "__state"]).max() < 1e-5


@pytest.mark.gpu
def test_sampled_expvals_vs_analytic():
    import torchquantum_gb300 as tq

    torch.manual_seed(1)
    n = 4
    layer = tq.RandomLayer(n_ops=60, wires=list(range(n)), seed=5).to("cuda")
    q = tq.QuantumDevice(n_wires=n, bsz=2, device="cuda")
    layer(q)
    rng = np.random.default_rng(0)
    obs = sorted({"".join(rng.choice(list("XYZI"), size=n)) for _ in range(12)} - {"IIII"})
    shots = 200000
    gen = torch.Generator(device="cuda").manual_seed(3)
    grouped = tq.expval_joint_sampling_grouping(q, obs, n_shots_per_group=shots, generator=gen)
    assert set(grouped) == set(obs)
    tol = 5 / np.sqrt(shots)
    for o in obs:
        ana = tq.expval_joint_analytical(q, o).detach().cpu().numpy()
        assert np.abs(grouped[o].cpu().numpy() - ana).max() < tol, o
        single = tq.expval_joint_sampling(q, o, n_shots=shots, generator=gen).cpu().numpy()
        assert np.abs(single - ana).max() < tol, o
    # the device state is unchanged by the basis rotations (they act on a copy)
    before = q.get_states_1d().detach().clone()
    tq.expval_joint_sampling(q, "XYZX", n_shots=10)
    assert torch.equal(before, q.get_states_1d().detach())
