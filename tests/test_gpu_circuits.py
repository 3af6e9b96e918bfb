"""Circuits through the public API against upstream fixtures and the oracle (GPU).

* ``circuits.npz``: random circuits over every gate type, run by upstream in
  complex128: final states and expvals within 1e-5, adjoint gradients within 1e-5.
* ``config1.npz``: the 4-wire encoder + U3 + CNOT-ring model, forward and backward.
* finite differences: adjoint gradients against complex128 central differences
  (h = 1e-3) of the oracle.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from tests.golden_data import circuit_cases, load

pytestmark = pytest.mark.gpu


def _run_api(n, bsz, gates, requires_grad=True):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    leaves = []
    for g in gates:
        p = g["params"]
        pt = None
        if p is not None:
            if g["name"] == "qubitunitaryfast":
                pt = torch.tensor(np.asarray(p), dtype=torch.complex64, device="cuda")
            else:
                pt = torch.tensor(np.asarray(p), dtype=torch.float32, device="cuda", requires_grad=requires_grad)
                leaves.append(pt)
        kw = {"n_wires": g["n_wires"]} if g.get("n_wires") else {}
        tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=pt, inverse=g["inverse"], **kw)
    return q, leaves


@pytest.mark.parametrize("case_idx", range(9))
def test_upstream_random_circuit(case_idx):
    import torchquantum_gb300 as tq

    case, gates, arr = list(circuit_cases())[case_idx]
    n, bsz = case["n"], case["bsz"]
    q, leaves = _run_api(n, bsz, gates)
    st = q.get_states_1d()
    assert np.abs(st.detach().cpu().numpy() - arr["state"]).max() < 1e-5
    ev = tq.expval_joint_analytical_batch(q, case["paulis"])
    assert np.abs(ev.detach().cpu().numpy() - arr["expval"]).max() < 1e-5
    loss = (ev * torch.tensor(arr["weights"], dtype=torch.float32, device="cuda")).sum()
    loss.backward()
    # compare in order of the parameterised (real) leaves
    refs = [arr[f"grad{i}"] for i in range(case["n_grads"])]
    refs = [r for r, g in zip(refs, [g for g in gates if g["params"] is not None]) if g["name"] != "qubitunitaryfast"]
    assert len(refs) == len(leaves)
    for lf, ref in zip(leaves, refs):
        assert np.abs(lf.grad.cpu().numpy() - ref.reshape(lf.shape)).max() < 1e-5


def test_config1_model_matches_upstream():
    import torchquantum_gb300 as tq

    d, _ = load("config1")
    n, bsz = 4, 32
    funcs = ["rx", "ry", "rz", "rx"]
    enc = tq.GeneralEncoder([{"input_idx": [4 * g + w], "func": funcs[g], "wires": [w]} for g in range(4)
                             for w in range(4)])
    layers = []
    for layer in range(2):
        l1 = tq.Op1QAllLayer(op=tq.U3, n_wires=n, has_params=True, trainable=True)
        for wi in range(n):
            l1.ops_all[wi].params.data = torch.tensor(d["u3_params"][layer, wi][None], dtype=torch.float32)
        layers += [l1, tq.Op2QAllLayer(op=tq.CNOT, n_wires=n, circular=True)]
    model = torch.nn.ModuleList([enc] + layers).cuda()
    x = torch.tensor(d["x"], dtype=torch.float32, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    enc(q, x)
    for lay in layers:
        lay(q)
    obs = ["".join("Z" if i == j else "I" for i in range(n)) for j in range(n)]
    ev = torch.stack([tq.expval_joint_analytical(q, o) for o in obs], dim=-1)
    assert np.abs(ev.detach().cpu().numpy() - d["c128__expval"]).max() < 1e-5
    assert np.abs(ev.detach().cpu().numpy() - d["c64__expval"]).max() < 1e-5
    (ev * torch.tensor(d["loss_weights"], dtype=torch.float32, device="cuda")).sum().backward()
    assert np.abs(x.grad.cpu().numpy() - d["c128__grad_x"]).max() < 1e-5
    gu3 = np.stack([np.stack([layers[2 * l].ops_all[w].params.grad.cpu().numpy()[0] for w in range(n)])
                    for l in range(2)])
    assert np.abs(gu3 - d["c128__grad_u3"]).max() < 1e-5


def _random_circuit(rng, n, bsz, depth, names=("u3", "rx", "ry", "rz", "crx", "cnot", "cz", "cry", "rzz", "cu3")):
    from torchquantum_gb300 import gates as G

    gates = []
    for _ in range(depth):
        name = names[rng.integers(len(names))]
        gd = G.GATES[name]
        wires = [int(w) for w in rng.permutation(n)[:gd.num_wires]]
        p = None
        if gd.num_params:
            p = rng.uniform(-np.pi, np.pi, size=(bsz if rng.random() < 0.5 else 1, gd.num_params))
        gates.append({"name": name, "wires": wires, "params": p, "inverse": bool(rng.random() < 0.2)})
    return gates


def test_adjoint_vs_central_differences():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(11)
    n, bsz = 7, 2
    gates = _random_circuit(rng, n, bsz, 30)
    paulis = ["ZIIXIIY", "IIZZIII", "XXXXXXX"]
    w = rng.normal(size=len(paulis))
    q, leaves = _run_api(n, bsz, gates)
    ev = tq.expval_joint_analytical_batch(q, paulis)
    (ev * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
    fd = O.fd_grads(n, bsz, gates, paulis, w, h=1e-3)
    fd = [f for f in fd if f is not None]
    assert len(fd) == len(leaves)
    err = max(np.abs(lf.grad.cpu().numpy() - f).max() for lf, f in zip(leaves, fd))
    assert err < 1e-5, err


def test_large_state_vs_oracle_and_norm():
    """n = 16, bsz = 3, 120 gates: state within 1e-5 of the oracle, norm within 1e-5."""
    rng = np.random.default_rng(5)
    n, bsz = 16, 3
    gates = _random_circuit(rng, n, bsz, 120)
    q, _ = _run_api(n, bsz, gates, requires_grad=False)
    got = q.get_states_1d().detach().cpu().numpy()
    ref = O.run(n, bsz, gates)
    assert np.abs(got - ref).max() < 1e-5
    assert np.abs(np.linalg.norm(got, axis=1) - 1).max() < 1e-5


def test_forward_then_inverse_round_trip_n22():
    """Size-independent property at n = 22: U^-1 U |psi> = |psi> (complex64, 200 gates)."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(9)
    n, bsz = 22, 2
    gates = _random_circuit(rng, n, bsz, 200)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    tqf.hadamard(q, wires=0)
    s0 = q.get_states_1d().detach().clone()
    for g in gates:
        p = None if g["params"] is None else torch.tensor(g["params"], dtype=torch.float32, device="cuda")
        tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=p, inverse=g["inverse"])
    for g in reversed(gates):
        p = None if g["params"] is None else torch.tensor(g["params"], dtype=torch.float32, device="cuda")
        tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=p, inverse=not g["inverse"])
    assert (q.get_states_1d().detach() - s0).abs().max().item() < 1e-5


def test_states_reads_are_snapshots():
    """Reading states then applying more gates leaves the earlier tensor unchanged."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.QuantumDevice(n_wires=3, bsz=1)
    tqf.hadamard(q, wires=0)
    s1 = q.states
    snap = s1.detach().clone()
    tqf.paulix(q, wires=2)
    assert torch.equal(s1.detach(), snap)
    assert not torch.equal(q.states.detach(), snap)


def test_phase_encoders_vs_oracle():
    """PhaseEncoder (upstream encodings.py:133-160) and MultiPhaseEncoder (:163-205)."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    n, bsz = 4, 3
    x = torch.rand(bsz, 12, device="cuda")
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    tq.PhaseEncoder(tqf.ry)(q, x)
    tq.MultiPhaseEncoder(["u3", "rz", "u2", "rx"], wires=[0, 1, 2, 3])(q, x[:, 4:])
    xh = x.cpu().double().numpy()
    gates = [{"name": "ry", "wires": [k], "params": xh[:, k:k + 1]} for k in range(n)]
    gates += [{"name": "u3", "wires": [0], "params": xh[:, 4:7]}, {"name": "rz", "wires": [1], "params": xh[:, 7:8]},
              {"name": "u2", "wires": [2], "params": xh[:, 8:10]}, {"name": "rx", "wires": [3], "params": xh[:, 10:11]}]
    assert np.abs(q.get_states_1d().cpu().numpy() - O.run(n, bsz, gates)).max() < 1e-5
