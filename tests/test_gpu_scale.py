"""Configurations at scale on the GPU.

* Fusion accuracy (n = 26, bsz = 8 with fused block widths k = 4, 5, 6; n = 28, bsz = 1
  with k = 6): final amplitudes and 8 Pauli expectation values of a depth-400 random
  circuit against a complex128 torch reference, within 1e-5.
* Differentiation workload (layered RY/RZ + CZ-ladder ansatz with shared parameters,
  observable = weighted sum of Pauli strings): fused adjoint gradients against the plain
  method and against complex128 central differences at a reduced size, for the literal
  configuration and for the variant with a per-sample RY input layer; at full size
  (n = 20, bsz = 64, 10 layers, 50 strings) the step's peak device memory stays a small
  multiple of one state with the in-place reverse sweep, and one more state per
  tensor-core block with stored block inputs, where per-gate autograd storage would need
  ~590 states.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from tests import torch_ref as TR

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,bsz,k", [(26, 8, 4), (26, 8, 5), (26, 8, 6), (28, 1, 6)])
def test_fusion_accuracy_at_scale(n, bsz, k):
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    dev = torch.device("cuda")
    gates, ncols = W.random_circuit(n, 400, seed=0)
    theta = W.random_params(bsz, ncols, seed=1)
    paulis = W.random_paulis(n, 8, seed=2)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
    q.method = "fused"
    q.fuse_wires = k
    W.apply_circuit(q, gates, torch.tensor(theta, device=dev))
    got = q.get_states_1d().detach()
    ev = tq.expval_joint_analytical_batch(q, paulis).detach().double()
    ntc = sum(1 for sg in q._tape for op in sg.exec_ops if getattr(op, "tc", False))
    del q
    ref = TR.run(n, bsz, W.oracle_gates(gates, theta), dev)
    err = (got.to(torch.complex128) - ref).abs().max().item()
    del got
    ev_ref = torch.stack([TR.expval_pauli(ref, p, n) for p in paulis], 1)
    eerr = (ev - ev_ref).abs().max().item()
    print(f"fusion n={n} bsz={bsz} k={k}: tensor-core blocks {ntc}, max |amplitude error| {err:.2e} "
          f"(max |amplitude| {ref.abs().max().item():.2e}), max |expval error| {eerr:.2e}")
    assert ntc > 0
    assert err < 1e-5 and eerr < 1e-5


def _vqe(n, bsz, layers, m, seed, per_sample):
    """(gates in the workload format, shared theta [1, P], input angles [bsz, n] or None,
    Pauli strings, weights)."""
    from torchquantum_gb300 import workloads as W

    gates, ncols = W.hea_circuit(n, layers)
    rng = np.random.default_rng(seed)
    theta = rng.uniform(-np.pi, np.pi, size=(1, ncols)).astype(np.float32)
    x = rng.uniform(0, np.pi, size=(bsz, n)).astype(np.float32) if per_sample else None
    paulis = W.random_paulis(n, m, seed=seed + 1)
    w = rng.normal(size=m).astype(np.float32)
    return gates, theta, x, paulis, w


def _engine_loss_grad(n, bsz, gates, theta, x, paulis, w, method, checkpoint="auto", blocks=None):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300 import workloads as W

    dev = torch.device("cuda")
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
    q.method = method
    q.fuse_wires = 6
    q.checkpoint = checkpoint
    if x is not None:
        xt = torch.tensor(x, device=dev)
        for wi in range(n):
            tqf.ry(q, wires=wi, params=xt[:, wi:wi + 1])
    th = torch.tensor(theta, device=dev, requires_grad=True)
    W.apply_circuit(q, gates, th)
    ev = tq.expval_joint_analytical_batch(q, paulis)
    loss = (ev * torch.tensor(w, device=dev)).sum()
    loss.backward()
    if blocks is not None:
        blocks.append(sum(1 for sg in q._tape for op in sg.blocks
                          if getattr(op, "kept_input", False)))
    return loss.item(), th.grad.detach().cpu().numpy()[0]


def _oracle_loss(n, bsz, gates, theta, x, paulis, w):
    from torchquantum_gb300 import workloads as W

    og = W.oracle_gates(gates, np.repeat(theta.astype(np.float64), bsz, axis=0))
    if x is not None:
        og = [{"name": "ry", "wires": [wi], "params": x[:, wi:wi + 1].astype(np.float64)} for wi in range(n)] + og
    s = O.run(n, bsz, og)
    return float(sum(wj * O.expval_pauli(s, p, n).sum() for wj, p in zip(w, paulis)))


@pytest.mark.parametrize("per_sample", [False, True])
def test_vqe_gradients_vs_plain_and_fd(per_sample):
    n, bsz, layers = 14, 4, 3
    gates, theta, x, paulis, w = _vqe(n, bsz, layers, 10, seed=5 + per_sample, per_sample=per_sample)
    lf, gf = _engine_loss_grad(n, bsz, gates, theta, x, paulis, w, "fused")
    lp, gp = _engine_loss_grad(n, bsz, gates, theta, x, paulis, w, "plain")
    assert abs(lf - lp) < 1e-5 * max(1.0, abs(lp))
    assert np.abs(gf - gp).max() < 1e-5
    rng = np.random.default_rng(0)
    h = 1e-3
    for j in rng.choice(theta.shape[1], size=6, replace=False):
        tp, tm = theta.astype(np.float64).copy(), theta.astype(np.float64).copy()
        tp[0, j] += h
        tm[0, j] -= h
        fd = (_oracle_loss(n, bsz, gates, tp, x, paulis, w) - _oracle_loss(n, bsz, gates, tm, x, paulis, w)) / (2 * h)
        assert abs(gf[j] - fd) < 1e-5 * max(1.0, abs(fd)), (j, gf[j], fd)


def test_vqe_full_size_memory():
    """Peak memory of the differentiation workload: the in-place reverse sweep holds a few
    states whatever the depth; with stored block inputs it holds one more state per
    tensor-core block, still far below per-gate autograd storage; both give the same loss
    and gradients."""
    n, bsz, layers = 20, 64, 10
    gates, theta, x, paulis, w = _vqe(n, bsz, layers, 50, seed=9, per_sample=True)
    state_bytes = bsz * (1 << n) * 8
    res = {}
    for mode in (False, True):
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        blocks = []
        loss, g = _engine_loss_grad(n, bsz, gates, theta, x, paulis, w, "fused", checkpoint=mode, blocks=blocks)
        torch.cuda.synchronize()
        peak = torch.cuda.max_memory_allocated() - base
        print(f"differentiation workload n={n} bsz={bsz} stored inputs={mode}: peak {peak / 2**30:.2f} GiB = "
              f"{peak / state_bytes:.1f} states ({blocks[0]} stored); per-gate autograd storage ~{len(gates)} "
              f"states = {len(gates) * state_bytes / 2**30:.0f} GiB")
        assert np.isfinite(loss) and np.isfinite(g).all() and g.shape == (theta.shape[1],)
        res[mode] = (loss, g, peak, blocks[0])
    assert res[False][3] == 0 and res[False][2] < 8 * state_bytes
    assert res[True][3] > 0 and res[True][2] < (res[True][3] + 8) * state_bytes
    assert abs(res[True][0] - res[False][0]) < 1e-5 * max(1.0, abs(res[False][0]))
    assert np.abs(res[True][1] - res[False][1]).max() < 1e-5 * max(1.0, np.abs(res[False][1]).max())
