"""Static mode (``module.static_on(wires_per_block=k)``: upstream ``module/modules.py:230-313``
and ``graph/graphs.py``) routed to the engine's fused method, and op-history replay.

* Against the oracle: a seeded ``RandomLayer`` model in static mode gives the oracle's
  states and Pauli expvals (complex128 restatement of the model's own op list) and its
  parameter gradients equal float64 central differences of the oracle loss.
* Against upstream: the fixture's seeded layers in static mode reproduce the states
  upstream computed (``tests/golden/random_layers.npz``), and, when upstream is installed
  (``baseline/_ref``), upstream's own static mode (``QuantumGraph`` block fusion, run live
  on the host with the same ``wires_per_block``) on the same seeded layer.
* Upstream's self-consistency checks (``test/static_mode_test.py:258-401``): static and
  dynamic runs agree; ``get_unitary`` is the circuit's unitary; a device's
  ``op_history`` replayed through ``QuantumModule.from_op_history`` gives the same state.
"""
import json

import numpy as np
import pytest
import torch

from oracle import statevec as O
from oracle import upstream as U
from tests.golden_data import load

pytestmark = pytest.mark.gpu

OPS = ("RX", "RY", "RZ", "U3", "CNOT", "CZ", "CRX", "RZZ")


def _model(tq, n, n_ops, seed, op_types=None, device="cuda"):
    class M(tq.QuantumModule):
        def __init__(self):
            super().__init__()
            self.n_wires = n
            kw = {} if op_types is None else {"op_types": tuple(getattr(tq, o) for o in op_types)}
            self.layer = tq.RandomLayer(n_ops=n_ops, wires=list(range(n)), seed=seed, **kw)

        @tq.static_support
        def forward(self, q_device):
            self.q_device = q_device  # upstream's static_support reads it
            self.layer(q_device)

    torch.manual_seed(seed)
    return M().to(device)


def _oracle_gates(layer):
    gates = []
    for o in layer.op_list:
        p = o.params.detach().double().cpu().numpy() if getattr(o, "params", None) is not None else None
        gates.append({"name": o.name.lower(), "wires": [int(w) for w in np.atleast_1d(o.wires)], "params": p})
    return gates


@pytest.mark.parametrize("k", [2, 3, 4, 6])
def test_static_matches_oracle(k):
    import torchquantum_gb300 as tq

    n, bsz = 7, 3
    m = _model(tq, n, 120, seed=k, op_types=OPS)
    gates = _oracle_gates(m.layer)
    obs = ["ZIXIYZI", "IIIIIIZ", "XXYYZZI"]
    w = np.array([0.7, -1.3, 0.4])
    m.static_on(wires_per_block=k)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    m(q)
    assert any(getattr(op, "members", None) for sg in q._tape for op in sg.exec_ops)
    ev = tq.expval_joint_analytical_batch(q, obs)
    (ev * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
    ref = O.run(n, bsz, gates)
    assert np.abs(q.get_states_1d().detach().cpu().numpy() - ref).max() < 1e-5
    ref_ev = np.stack([O.expval_pauli(ref, p, n) for p in obs], -1)
    assert np.abs(ev.detach().cpu().numpy() - ref_ev).max() < 1e-5
    fd = O.fd_grads(n, bsz, gates, obs, w, h=1e-4)
    got = [o.params.grad.cpu().numpy() for o in m.layer.op_list if getattr(o, "params", None) is not None]
    want = [f for f in fd if f is not None]
    assert len(got) == len(want) and len(got) > 0
    err = max(np.abs(g - f.reshape(g.shape)).max() for g, f in zip(got, want))
    assert err < 1e-5, err
    m.static_off()


@pytest.mark.parametrize("k", [2, 3, 4])
def test_static_matches_upstream(k):
    import torchquantum_gb300 as tq

    d, _ = load("random_layers")
    meta = json.loads(str(d["__meta__"]))
    cases = [c for c in meta["layers"] if c["state"] and c["cls"] == "RandomLayer"]
    up = U.import_upstream() if U.available() else None
    for case in cases:
        n = case["n"]
        m = _model(tq, n, case["n_ops"], case["seed"])
        m.static_on(wires_per_block=k)
        q = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda")
        m(q)
        got = q.get_states_1d().detach().cpu().numpy()
        m.static_off()
        assert np.abs(got - d[case["key"] + "__state"]).max() < 1e-5, case["key"]
        if up is not None:
            # upstream's own static mode on the same seeded layer (host, complex64)
            U.set_precision(False)
            mu = _model(up, n, case["n_ops"], case["seed"], device="cpu")
            mu.static_on(wires_per_block=k)
            qu = up.QuantumDevice(n_wires=n, bsz=1)
            mu(qu)
            want = qu.get_states_1d().detach().numpy()
            assert np.abs(got - want).max() < 1e-5, (case["key"], "upstream static mode")


@pytest.mark.parametrize("k", [2, 3, 4, 6])
def test_static_matches_dynamic(k):
    import torchquantum_gb300 as tq

    n, bsz = 7, 3
    m = _model(tq, n, 120, seed=k, op_types=OPS)
    obs = ["ZIXIYZI", "IIIIIIZ"]
    res = {}
    for static in (False, True):
        if static:
            m.static_on(wires_per_block=k)
        else:
            m.static_off()
        m.zero_grad()
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
        m(q)
        ev = tq.expval_joint_analytical_batch(q, obs)
        ev.sum().backward()
        grads = torch.cat([p.grad.reshape(-1) for p in m.parameters()])
        res[static] = (q.get_states_1d().detach().cpu().numpy(), grads.cpu().numpy())
    m.static_off()
    assert np.abs(res[True][0] - res[False][0]).max() < 1e-5
    assert np.abs(res[True][1] - res[False][1]).max() < 1e-5


def test_get_unitary_and_op_history_replay():
    import torchquantum_gb300 as tq

    n = 5
    m = _model(tq, n, 60, seed=9, op_types=OPS)
    u = m.get_unitary().detach()
    ud = u.to(torch.complex128).cpu().numpy()
    assert np.abs(ud @ ud.conj().T - np.eye(1 << n)).max() < 1e-5
    q = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda", record_op=True)
    m(q)
    psi = q.get_states_1d().detach().cpu().numpy()[0]
    assert np.abs(ud[:, 0] - psi).max() < 1e-5
    replay = tq.QuantumModule.from_op_history(q.op_history).to("cuda")
    q2 = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda")
    replay(q2)
    assert np.abs(q2.get_states_1d().detach().cpu().numpy()[0] - psi).max() < 1e-5
