"""Stored block inputs on the GPU: the out-of-place tensor-core forward, the adjoint step
that reads a block's stored input, and circuits run with and without stored inputs
(same states, same gradients, repeated backward)."""
import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu


def _unitaries(rng, b):
    us = []
    for _ in range(b):
        z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
        q_, r_ = np.linalg.qr(z)
        us.append(q_ * (np.diag(r_) / np.abs(np.diag(r_))))
    return torch.tensor(np.stack(us), dtype=torch.complex128, device="cuda")


def _state(rng, bsz, n):
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    return torch.tensor(s / np.linalg.norm(s, axis=1, keepdims=True), dtype=torch.complex64, device="cuda")


@pytest.mark.parametrize("n,bsz,per_row", [(13, 1, False), (14, 3, True), (20, 3, True), (20, 2, False)])
def test_apply_to_matches_in_place(n, bsz, per_row):
    """tqk_fused_apply_to writes exactly what tqk_fused_apply computes in place and
    leaves its input untouched."""
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(7 * n + bsz)
    b = bsz if per_row else 1
    for trial in range(2):
        wires = [int(w) for w in rng.permutation(n)[:6]] if trial == 0 else list(range(n - 6, n))
        img = _lib.fused_prepare(_unitaries(rng, b), wires)
        src = _state(rng, bsz, n)
        keep = src.clone()
        dst = torch.full_like(src, complex(7.0, -7.0))
        _lib.fused_apply_to(src, dst, n, wires, img, b)
        ref = src.clone()
        _lib.fused_apply(ref, n, wires, img, b)
        torch.cuda.synchronize()
        _lib.check_status(src.device)
        assert torch.equal(src, keep)
        assert torch.equal(dst, ref)


def test_apply_to_rejects_partial_overlap():
    from torchquantum_gb300 import _lib

    n, bsz = 13, 2
    rng = np.random.default_rng(0)
    img = _lib.fused_prepare(_unitaries(rng, 1), list(range(6)))
    big = torch.zeros(bsz * 2 + 1, 1 << n, dtype=torch.complex64, device="cuda")
    with pytest.raises(_lib.TQKError):
        _lib.fused_apply_to(big[0:bsz], big[1:bsz + 1], n, list(range(6)), img, 1)


@pytest.mark.parametrize("n,bsz,per_row", [(13, 1, False), (14, 3, True), (15, 2, False), (20, 3, True)])
def test_adjoint_stored_vs_cuda_cores(n, bsz, per_row):
    """lam <- U^H lam and the cotangent sum lam conj(psi_in)^T from the stored input,
    against the CUDA-core dense adjoint run on psi_out = U psi_in."""
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(300 + n)
    b = bsz if per_row else 1
    for trial in range(3):
        wires = [int(w) for w in rng.permutation(n)[:6]] if trial != 1 else list(range(n - 6, n))
        u = _unitaries(rng, b)
        psi_in, lam = _state(rng, bsz, n), _state(rng, bsz, n)
        keep = psi_in.clone()
        psi_r, lam_r = psi_in.clone(), lam.clone()
        u64 = u.to(torch.complex64).contiguous()
        _lib.apply_matrix(psi_r, n, wires, u64, b)  # psi_out
        g_ref = torch.zeros(b * 64 * 64 * 2, dtype=torch.float64, device="cuda")
        _lib.adjoint_matrix(psi_r, lam_r, n, wires, u64, b, g_ref)
        mr = torch.zeros(b, 128, 128, dtype=torch.float64, device="cuda")
        _lib.fused_adjoint_stored(psi_in, lam, n, wires, _lib.fused_prepare_adjoint(u, wires), b, mr)
        g = torch.zeros(b, 64, 64, dtype=torch.complex128, device="cuda")
        _lib.fused_cross_grad(mr, None, torch.view_as_real(g))
        torch.cuda.synchronize()
        _lib.check_status(lam.device)
        assert torch.equal(psi_in, keep)
        assert (lam - lam_r).abs().max().item() < 2e-5 * lam_r.abs().max().item()
        gr = torch.view_as_complex(g_ref.view(-1, 2)).view(b, 64, 64)
        assert (g - gr).abs().max().item() < 1e-5 * max(1.0, gr.abs().max().item()), trial
        # u = NULL adds the cross term itself
        assert (g - _lib.cross_to_complex(mr)).abs().max().item() == 0.0


def _circuit_run(n, bsz, gates, theta, paulis, checkpoint, retain=False):
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    th = torch.tensor(theta, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.method = "fused"
    q.fuse_wires = 6
    q.checkpoint = checkpoint
    W.apply_circuit(q, gates, th)
    ev = tq.expval_joint_analytical_batch(q, paulis)
    ev.sum().backward(retain_graph=retain)
    g1 = th.grad.detach().clone()
    if retain:
        th.grad = None
        ev.sum().backward()
        assert torch.equal(th.grad, g1)
    return q, q.get_states_1d().detach().cpu().numpy(), g1.cpu().numpy()


def test_circuit_with_stored_inputs_matches_recompute():
    """The same circuit with stored block inputs and with the in-place reverse sweep:
    identical forward state (and the oracle's), gradients within float32 accuracy, and a
    second backward over the retained graph gives the same gradients."""
    from torchquantum_gb300 import workloads as W

    n, bsz = 14, 3
    gates, ncols = W.random_circuit(n, 160, seed=11)
    theta = W.random_params(bsz, ncols, seed=12)
    paulis = W.random_paulis(n, 4, seed=13)
    q1, s1, g1 = _circuit_run(n, bsz, gates, theta, paulis, True, retain=True)
    q0, s0, g0 = _circuit_run(n, bsz, gates, theta, paulis, False)
    tc1 = [op for sg in q1._tape for op in sg.blocks if op.tc]
    tc0 = [op for sg in q0._tape for op in sg.blocks if op.tc]
    # from |0...0> the circuit's first block keeps nothing (its reverse step is a gather)
    first = q1._tape[0].exec_ops[0]
    assert getattr(first, "zero_input", False) == bool(getattr(first, "tc", False))
    assert tc1 and all(getattr(op, "kept_input", False) or getattr(op, "zero_input", False) for op in tc1)
    assert all(not getattr(op, "kept_input", False) for op in tc0)
    assert np.array_equal(s1, s0)
    assert np.abs(s1 - O.run(n, bsz, W.oracle_gates(gates, theta))).max() < 1e-5
    assert np.abs(g1 - g0).max() < 1e-5 * max(1.0, np.abs(g0).max())
    # a backward that does not retain the graph releases the stored inputs, like torch's
    # own saved tensors (the segments keep only weak references)
    q2, _, g2 = _circuit_run(n, bsz, gates, theta, paulis, True)
    blocks = [op for sg in q2._tape for op in sg.blocks if op.tc and not getattr(op, "zero_input", False)]
    assert blocks and all(op.kept_input and op.stored_ref() is None for op in blocks)
    assert np.array_equal(g2, g1)


def test_mixed_segment_with_stored_inputs():
    """CUDA-core ops (an 8-wire multi-controlled X, an 8-wire multirz with a gradient)
    between tensor-core blocks: the reverse sweep copies a stored input before
    uncomputing through them; state and gradients match the plain method."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(5)
    n, bsz, layers = 14, 2, 5
    th_np = rng.uniform(-np.pi, np.pi, size=(bsz, layers * n))
    rz_np = rng.uniform(-np.pi, np.pi, size=(1, layers))
    mcx_wires = [[int(w) for w in rng.permutation(n)[:8]] for _ in range(layers)]
    res = {}
    for method in ("fused", "plain"):
        q = tq.QuantumDevice(n_wires=n, bsz=bsz)
        q.method = method
        q.fuse_wires = 6
        q.checkpoint = True
        th = torch.tensor(th_np, dtype=torch.float32, device="cuda", requires_grad=True)
        rz = torch.tensor(rz_np, dtype=torch.float32, device="cuda", requires_grad=True)
        for layer in range(layers):
            for w in range(n):
                tqf.ry(q, wires=w, params=th[:, layer * n + w:layer * n + w + 1])
            for w in range(0, n - 1):
                tqf.cnot(q, wires=[w, w + 1])
            tqf.multicnot(q, wires=mcx_wires[layer])
            tqf.multirz(q, wires=list(range(layer, layer + 8)), params=rz[:, layer:layer + 1])
        ev = tq.expval_joint_analytical(q, "Z" * n)
        ev.sum().backward()
        res[method] = (q.get_states_1d().detach().cpu().numpy(), th.grad.cpu().numpy(), rz.grad.cpu().numpy())
        if method == "fused":
            ops = [op for sg in q._tape for op in sg.exec_ops]
            assert any(getattr(op, "kept_input", False) for op in ops)
            assert any(getattr(op, "members", None) is None for op in ops)
    for a, b in zip(res["fused"], res["plain"]):
        assert np.abs(a - b).max() < 1e-5 * max(1.0, np.abs(b).max())


def test_auto_mode_stores_only_when_needed(monkeypatch):
    """checkpoint="auto" keeps nothing without autograd and nothing when the states would
    not fit the memory share."""
    from torchquantum_gb300 import device as D
    from torchquantum_gb300 import workloads as W
    import torchquantum_gb300 as tq

    n, bsz = 14, 2
    gates, ncols = W.random_circuit(n, 80, seed=1)
    theta = W.random_params(bsz, ncols, seed=2)

    def stored_blocks(grad):
        th = torch.tensor(theta, device="cuda", requires_grad=grad)
        q = tq.QuantumDevice(n_wires=n, bsz=bsz)
        q.method = "fused"
        q.fuse_wires = 6
        W.apply_circuit(q, gates, th)
        q.get_states_1d()
        return [getattr(op, "kept_input", False) for sg in q._tape for op in sg.blocks
                if op.tc and not getattr(op, "zero_input", False)]

    assert all(stored_blocks(True))
    assert not any(stored_blocks(False))
    with torch.no_grad():
        assert not any(stored_blocks(True))
    monkeypatch.setattr(D, "CHECKPOINT_MEMORY_SHARE", 0.0)
    assert not any(stored_blocks(True))


def test_out_of_memory_midway_falls_back_in_place(monkeypatch):
    """When a stored input cannot be allocated the segment runs its remaining blocks in
    place; the reverse sweep then mixes stored-input steps and in-place steps and still
    gives the in-place sweep's state and gradients."""
    from torchquantum_gb300 import program as P
    from torchquantum_gb300 import workloads as W

    n, bsz = 14, 2
    gates, ncols = W.random_circuit(n, 160, seed=21)
    theta = W.random_params(bsz, ncols, seed=22)
    paulis = W.random_paulis(n, 4, seed=23)
    _, s0, g0 = _circuit_run(n, bsz, gates, theta, paulis, False)
    real = P._new_state
    calls = {"n": 0}

    def limited(like):
        calls["n"] += 1
        return real(like) if calls["n"] <= 3 else None

    monkeypatch.setattr(P, "_new_state", limited)
    q, s1, g1 = _circuit_run(n, bsz, gates, theta, paulis, True, retain=True)
    flags = [getattr(op, "kept_input", False) for sg in q._tape for op in sg.blocks if op.tc]
    assert sum(flags) == 3 and len(flags) > 3
    assert np.array_equal(s1, s0)
    assert np.abs(g1 - g0).max() < 1e-5 * max(1.0, np.abs(g0).max())


def _two_reads(n, bsz, gates, theta, paulis, init, checkpoint):
    """Gradients (angles, initial state) of <P> read twice: after the first half of the
    circuit and after all of it (two autograd nodes over shared segments)."""
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    th = torch.tensor(theta, device="cuda", requires_grad=True)
    s0 = torch.tensor(init, dtype=torch.complex64, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.method = "fused"
    q.fuse_wires = 6
    q.checkpoint = checkpoint
    q.set_states(s0)
    half = len(gates) // 2
    W.apply_circuit(q, gates[:half], th)
    e1 = tq.expval_joint_analytical_batch(q, paulis)
    W.apply_circuit(q, gates[half:], th)
    e2 = tq.expval_joint_analytical_batch(q, paulis)
    (e1.sum() + 2.0 * e2.sum()).backward()
    kept = sum(1 for sg in q._tape for op in sg.blocks if getattr(op, "kept_input", False))
    return th.grad.cpu().numpy(), s0.grad.cpu().numpy(), kept


def test_two_reads_and_initial_state_gradient():
    """Two reads of one device (the second node's segments include the first's) and a
    differentiable initial state: stored block inputs give the in-place sweep's gradients
    for the angles and for the initial state."""
    from torchquantum_gb300 import workloads as W

    n, bsz = 14, 2
    gates, ncols = W.random_circuit(n, 200, seed=31)
    theta = W.random_params(bsz, ncols, seed=32)
    paulis = W.random_paulis(n, 3, seed=33)
    rng = np.random.default_rng(34)
    init = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    init /= np.linalg.norm(init, axis=1, keepdims=True)
    g1, s1, k1 = _two_reads(n, bsz, gates, theta, paulis, init, True)
    g0, s0, k0 = _two_reads(n, bsz, gates, theta, paulis, init, False)
    assert k1 > 0 and k0 == 0
    assert np.abs(g1 - g0).max() < 1e-5 * max(1.0, np.abs(g0).max())
    assert np.abs(s1 - s0).max() < 1e-5 * max(1.0, np.abs(s0).max())


@pytest.mark.parametrize("per_row", [False, True])
def test_first_block_from_zero_state(per_row):
    """The circuit's first tensor-core block acting on |0...0> takes the gather reverse
    step (cotangent lam conj(e_0)^T, no lam update): gradients equal the plain method's,
    for one U shared by every row and for per-row U."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300 import workloads as W

    n, bsz = 14, 3
    gates, ncols = W.random_circuit(n, 120, seed=41 + per_row)
    theta = W.random_params(1 if not per_row else bsz, ncols, seed=42)
    paulis = W.random_paulis(n, 3, seed=43)
    res = {}
    for method in ("fused", "plain"):
        th = torch.tensor(theta, device="cuda", requires_grad=True)
        q = tq.QuantumDevice(n_wires=n, bsz=bsz)
        q.method = method
        q.fuse_wires = 6
        for w in range(6):  # a first block of several gates on wires 0-5
            tqf.ry(q, wires=w, params=th[:, w:w + 1])
        W.apply_circuit(q, gates, th)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        (ev * torch.tensor([1.0, -0.5, 2.0], device="cuda")).sum().backward()
        res[method] = (ev.detach().cpu().numpy(), th.grad.cpu().numpy())
        if method == "fused":
            first = q._tape[0].exec_ops[0]
            assert getattr(first, "tc", False) and first.zero_input and first.block_batch == (bsz if per_row else 1)
    assert np.abs(res["fused"][0] - res["plain"][0]).max() < 1e-5
    assert np.abs(res["fused"][1] - res["plain"][1]).max() < 1e-5 * max(1.0, np.abs(res["plain"][1]).max())
