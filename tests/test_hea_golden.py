"""Differentiation workload pinned against upstream's own autograd gradients.

``tests/golden/hea.npz`` holds, for three reduced-size instances of the layered
RY/RZ + CZ-ladder ansatz with one shared parameter row (optionally behind a per-sample
RY(x) input layer), upstream's forward expvals and its autograd gradients of
``sum_b sum_j w_j <P_j>`` with respect to the shared angles and the inputs, computed by
``tqf.ry/rz/cz`` -> ``gate_wrapper`` -> ``apply_unitary_bmm``
(``functional/gate_wrapper.py:96-140,324-446``) and ``expval_joint_analytical``
(``measurement/measurements.py:232-279``).

* CPU: the oracle's central differences reproduce upstream's complex128 gradients.
* GPU: the engine's adjoint backward (plain and fused methods) reproduces them within
  1e-5 absolute, and its forward expvals within 1e-5.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from tests.golden_data import load


def _cases():
    d, meta = load("hea")
    for case in meta:
        k = case["key"]
        arr = {f[len(k) + 2:]: d[f] for f in d.files if f.startswith(k + "__")}
        yield case, arr


def _gates(n, layers, theta, x, bsz):
    """The instance as an oracle gate list (shared params broadcast over the batch)."""
    gates = []
    if x is not None:
        gates += [{"name": "ry", "wires": [w], "params": x[:, w:w + 1]} for w in range(n)]
    off = 0
    for _ in range(layers):
        for name in ("ry", "rz"):
            for w in range(n):
                gates.append({"name": name, "wires": [w], "params": np.repeat(theta[:, off:off + 1], bsz, 0),
                              "shared": off})
                off += 1
        gates += [{"name": "cz", "wires": [w, w + 1], "params": None} for w in range(n - 1)]
    return gates


CASES = list(_cases())


@pytest.mark.parametrize("ci", range(len(CASES)))
def test_oracle_fd_matches_upstream_autograd(ci):
    case, arr = CASES[ci]
    n, bsz, layers = case["n"], case["bsz"], case["layers"]
    x = arr["x"] if case["per_sample"] else None
    gates = _gates(n, layers, arr["theta"], x, bsz)
    s = O.run(n, bsz, gates)
    ev = np.stack([O.expval_pauli(s, p, n) for p in case["paulis"]], -1)
    np.testing.assert_allclose(ev, arr["c128__expval"], atol=1e-10)
    # upstream's complex64 default agrees with its complex128 mode to complex64 rounding
    np.testing.assert_allclose(arr["c64__expval"], arr["c128__expval"], atol=1e-5)
    fd = O.fd_grads(n, bsz, gates, case["paulis"], arr["weights"], h=1e-4)
    g_theta = np.zeros(arr["theta"].shape[1])
    g_x = np.zeros_like(arr["x"])
    for g, gr in zip(gates, fd):
        if gr is None:
            continue
        if "shared" in g:
            g_theta[g["shared"]] += gr.sum()
        else:
            g_x[:, g["wires"][0]] += gr[:, 0]
    np.testing.assert_allclose(g_theta, arr["c128__grad_theta"][0], atol=1e-6)
    if x is not None:
        np.testing.assert_allclose(g_x, arr["c128__grad_x"], atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["plain", "fused"])
@pytest.mark.parametrize("ci", range(len(CASES)))
def test_engine_adjoint_matches_upstream_autograd(ci, method):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    case, arr = CASES[ci]
    n, bsz, layers = case["n"], case["bsz"], case["layers"]
    dev = torch.device("cuda")
    th = torch.tensor(arr["theta"], dtype=torch.float32, device=dev, requires_grad=True)
    xt = torch.tensor(arr["x"], dtype=torch.float32, device=dev, requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
    q.method = method
    q.fuse_wires = 6
    if case["per_sample"]:
        for w in range(n):
            tqf.ry(q, wires=w, params=xt[:, w:w + 1])
    off = 0
    for _ in range(layers):
        for fn in (tqf.ry, tqf.rz):
            for w in range(n):
                fn(q, wires=w, params=th[:, off:off + 1])
                off += 1
        for w in range(n - 1):
            tqf.cz(q, wires=[w, w + 1])
    ev = tq.expval_joint_analytical_batch(q, case["paulis"])
    (ev * torch.tensor(arr["weights"], dtype=torch.float32, device=dev)).sum().backward()
    tol = 1e-5
    e_ev = np.abs(ev.detach().cpu().numpy() - arr["c128__expval"]).max()
    e_th = np.abs(th.grad.cpu().numpy() - arr["c128__grad_theta"]).max()
    e_x = np.abs(xt.grad.cpu().numpy() - arr["c128__grad_x"]).max() if case["per_sample"] else 0.0
    print(f"hea case {ci} ({method}, n={n}, bsz={bsz}): max |expval err| {e_ev:.2e}, max |grad err| "
          f"shared angles {e_th:.2e}, inputs {e_x:.2e} vs upstream complex128 autograd")
    assert e_ev < tol and e_th < tol and e_x < tol
