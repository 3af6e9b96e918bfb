"""Fused method on the GPU: forward against the oracle, gradients against the plain
method and against complex128 central differences; dense k-wire adjoint."""
import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu


def _circuit(rng, n, bsz, depth):
    from torchquantum_gb300 import gates as G

    names = ("u3", "rx", "ry", "rz", "crx", "cnot", "cz", "cry", "rzz", "cu3", "swap", "toffoli", "hadamard", "s",
             "cu2", "rxx")
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


def _tc_blocks(q):
    return sum(1 for sg in q._tape for op in sg.exec_ops if getattr(op, "tc", False))


def _run(n, bsz, gates, method, k=5, grad=True):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.method = method
    q.fuse_wires = k
    leaves = []
    for g in gates:
        p = None
        if g["params"] is not None:
            p = torch.tensor(g["params"], dtype=torch.float32, device="cuda", requires_grad=grad)
            leaves.append(p)
        tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=p, inverse=g["inverse"])
    return q, leaves


@pytest.mark.parametrize("k", [3, 4, 5, 6])
def test_fused_forward_vs_oracle(k):
    rng = np.random.default_rng(k)
    n, bsz = 10, 3
    gates = _circuit(rng, n, bsz, 120)
    q, _ = _run(n, bsz, gates, "fused", k, grad=False)
    got = q.get_states_1d().detach().cpu().numpy()
    assert np.abs(got - O.run(n, bsz, gates)).max() < 1e-5
    assert sum(len(sg.exec_ops) for sg in q._tape) < 120


@pytest.mark.parametrize("k", [3, 5, 6])
def test_fused_gradients_match_plain_and_fd(k):
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(10 + k)
    n, bsz = 8, 2
    gates = _circuit(rng, n, bsz, 40)
    paulis = ["ZIIXIIYI", "XXXXXXXX", "IZIZIZIZ"]
    w = rng.normal(size=3)
    grads = {}
    for method in ("plain", "fused"):
        q, leaves = _run(n, bsz, gates, method, k)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        (ev * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
        grads[method] = [lf.grad.cpu().numpy() for lf in leaves]
    fd = [f for f in O.fd_grads(n, bsz, gates, paulis, w, h=1e-3) if f is not None]
    for gp, gf, gd in zip(grads["plain"], grads["fused"], fd):
        assert np.abs(gf - gp).max() < 1e-5
        assert np.abs(gf - gd).max() < 1e-5


@pytest.mark.parametrize("kw", [3, 4, 6])
def test_dense_k_wire_adjoint_vs_fd(kw):
    """Trainable dense unitary on kw wires: gradient w.r.t. the matrix entries."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(kw)
    n, bsz = 8, 2
    z = rng.normal(size=(1 << kw, 1 << kw)) + 1j * rng.normal(size=(1 << kw, 1 << kw))
    u0, _ = np.linalg.qr(z)
    wires = [int(w) for w in rng.permutation(n)[:kw]]
    ut = torch.tensor(u0[None], dtype=torch.complex64, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    for w_ in range(n):
        tqf.hadamard(q, wires=w_)
    tqf.ry(q, wires=0, params=torch.tensor([[0.3], [1.1]], device="cuda"))
    tqf.qubitunitaryfast(q, wires=wires, params=ut)
    ev = tq.expval_joint_analytical(q, "ZXIYIIZI")
    ev.sum().backward()
    # analytic: dL/dU = sum_b 2 * (P psi_after)_cols psi_before^H  (torch convention: grad = dL/dRe + i dL/dIm)
    base = [{"name": "hadamard", "wires": [w]} for w in range(n)]
    base.append({"name": "ry", "wires": [0], "params": np.array([[0.3], [1.1]])})
    s_before = O.run(n, bsz, base)
    eps = 1e-6
    gnum = np.zeros_like(u0)
    for i in range(1 << kw):
        for j in range(1 << kw):
            for part, unit in ((0, 1.0), (1, 1j)):
                vals = []
                for sgn in (1, -1):
                    up = u0.copy()
                    up[i, j] += sgn * eps * unit
                    s = O.apply(s_before, up[None], wires, n)
                    vals.append(O.expval_pauli(s, "ZXIYIIZI", n).sum())
                d = (vals[0] - vals[1]) / (2 * eps)
                gnum[i, j] += d * unit
    assert np.abs(ut.grad.cpu().numpy()[0] - gnum).max() < 1e-5


@pytest.mark.parametrize(
    "n,bsz,per_row", [(13, 1, False), (14, 3, True), (16, 2, False), (14, 2, True), (20, 3, True), (20, 3, False)]
)
def test_tensor_core_block_vs_cuda_cores(n, bsz, per_row):
    """The tcgen05 split-BF16 kernel against the CUDA-core dense kernel on random 6-wire unitaries.

    n = 20, bsz = 3 gives every CTA several tiles (accumulator and A-buffer reuse) and a
    batch-row change inside a CTA (per-row U reload).
    """
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(n * 10 + bsz)
    for trial in range(4):
        wires = [int(w) for w in rng.permutation(n)[:6]]
        if trial == 1:
            wires = list(range(n - 6, n))  # the lowest bits
        b = bsz if per_row else 1
        us = []
        for _ in range(b):
            z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
            q_, r_ = np.linalg.qr(z)
            us.append(q_ * (np.diag(r_) / np.abs(np.diag(r_))))
        u128 = torch.tensor(np.stack(us), dtype=torch.complex128, device="cuda")
        s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
        s /= np.linalg.norm(s, axis=1, keepdims=True)
        st = torch.tensor(s, dtype=torch.complex64, device="cuda")
        ref = st.clone()
        _lib.apply_matrix(ref, n, wires, u128.to(torch.complex64).contiguous(), b)
        img = _lib.fused_prepare(u128, wires)
        _lib.fused_apply(st, n, wires, img, b)
        torch.cuda.synchronize()
        _lib.check_status(st.device)
        err = (st - ref).abs().max().item()
        scale = ref.abs().max().item()
        assert err < 2e-5 * scale, (trial, wires, err, scale)


def test_fused_tensor_core_circuit_vs_oracle():
    rng = np.random.default_rng(21)
    n, bsz = 14, 2
    gates = _circuit(rng, n, bsz, 150)
    q, _ = _run(n, bsz, gates, "fused", 6, grad=False)
    got = q.get_states_1d().detach().cpu().numpy()
    assert _tc_blocks(q) > 0
    assert np.abs(got - O.run(n, bsz, gates)).max() < 1e-5


@pytest.mark.parametrize(
    "n,bsz,per_row", [(13, 1, False), (14, 3, True), (15, 2, False), (20, 3, True), (20, 3, False)]
)
def test_tensor_core_adjoint_vs_cuda_cores(n, bsz, per_row):
    """tcgen05 adjoint step (psi, lam <- U^H, cotangent M U) against the CUDA-core dense adjoint."""
    from torchquantum_gb300 import _lib

    rng = np.random.default_rng(100 + n)
    b = bsz if per_row else 1
    for trial in range(3):
        wires = [int(w) for w in rng.permutation(n)[:6]] if trial != 1 else list(range(n - 6, n))
        us = []
        for _ in range(b):
            z = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
            q_, r_ = np.linalg.qr(z)
            us.append(q_ * (np.diag(r_) / np.abs(np.diag(r_))))
        u = torch.tensor(np.stack(us), dtype=torch.complex128, device="cuda")

        def rand_state():
            s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
            return torch.tensor(s / np.linalg.norm(s, axis=1, keepdims=True), dtype=torch.complex64, device="cuda")

        psi, lam = rand_state(), rand_state()
        psi_r, lam_r = psi.clone(), lam.clone()
        g_ref = torch.zeros(b * 64 * 64 * 2, dtype=torch.float64, device="cuda")
        _lib.adjoint_matrix(psi_r, lam_r, n, wires, u.to(torch.complex64).contiguous(), b, g_ref)
        uh = u.conj().transpose(-1, -2).contiguous()
        mr = torch.zeros(b, 128, 128, dtype=torch.float64, device="cuda")
        _lib.fused_adjoint(psi, lam, n, wires, _lib.fused_prepare(uh, wires), b, mr)
        torch.cuda.synchronize()
        _lib.check_status(psi.device)
        assert (psi - psi_r).abs().max().item() < 2e-5 * psi_r.abs().max().item()
        assert (lam - lam_r).abs().max().item() < 2e-5 * lam_r.abs().max().item()
        g = torch.matmul(_lib.cross_to_complex(mr), u)
        gr = torch.view_as_complex(g_ref.view(-1, 2)).view(b, 64, 64)
        assert (g - gr).abs().max().item() < 1e-5 * max(1.0, gr.abs().max().item()), trial


def test_fused_tensor_core_gradients_vs_plain():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(33)
    n, bsz = 14, 2
    gates = _circuit(rng, n, bsz, 80)
    paulis = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(3)]
    w = rng.normal(size=3)
    grads, evs = {}, {}
    for method in ("plain", "fused"):
        q, leaves = _run(n, bsz, gates, method, 6)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        (ev * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
        grads[method] = [lf.grad.cpu().numpy() for lf in leaves]
        evs[method] = ev.detach().cpu().numpy()
        if method == "fused":
            assert _tc_blocks(q) > 0
    assert np.abs(evs["fused"] - evs["plain"]).max() < 1e-5
    for gp, gf in zip(grads["plain"], grads["fused"]):
        assert np.abs(gf - gp).max() < 1e-5


def test_autotuned_fusion_vs_oracle(tmp_path, monkeypatch):
    """fuse_wires="auto": the width / planner / kernel choice made from measured pass
    costs gives the oracle's state and the plain method's gradients."""
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import autotune as A
    from torchquantum_gb300 import workloads as W

    monkeypatch.setenv("TQ_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    A.clear()
    dev = torch.device("cuda")
    n, bsz = 14, 3
    gates, ncols = W.random_circuit(n, 120, seed=3)
    theta = W.random_params(bsz, ncols, seed=4)
    paulis = W.random_paulis(n, 4, seed=5)
    res = {}
    for method in ("fused", "plain"):
        th = torch.tensor(theta, device=dev, requires_grad=True)
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
        q.method = method
        W.apply_circuit(q, gates, th)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        ev.sum().backward()
        res[method] = (q.get_states_1d().detach().cpu().numpy(), th.grad.cpu().numpy())
        if method == "fused":
            seg = q._tape[0]
            assert seg.fuse_width in (4, 5, 6) and any(getattr(op, "members", None) for op in seg.exec_ops)
    ref = O.run(n, bsz, W.oracle_gates(gates, theta))
    assert np.abs(res["fused"][0] - ref).max() < 1e-5
    assert np.abs(res["fused"][1] - res["plain"][1]).max() < 1e-5
    assert any(k.startswith("fusion3|") for k in A._MEM)
    A.clear()


@pytest.mark.parametrize("checkpoint", ["auto", False])
def test_lone_gates_as_tensor_core_blocks(monkeypatch, checkpoint):
    """A plan that leaves every gate alone, with the tensor-core flag set on each (what the
    autotuner does for a lone dense gate when a padded 6-wire block costs less than the
    gate's own pass): every fusable gate runs as its own tensor-core block (the others on
    their own kernels), the first one on |0...0> written directly.  States, expvals and
    gradients match the oracle and the plain method."""
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import autotune as A

    def every_gate_alone(wl, n, bsz, dev, tc_ok, with_adj, widths=(4, 5, 6), stored=False, lone_kind=None):
        assert lone_kind is not None and len(lone_kind) == len(wl)
        plan = [(list(w), [i]) for i, w in enumerate(wl)]
        return plan, [True] * len(plan), 6, None

    rng = np.random.default_rng(41)
    n, bsz = 14, 2
    gates = [g for g in _circuit(rng, n, bsz, 30) if len(g["wires"]) <= 2]
    paulis = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(3)]
    res = {}
    for method in ("plain", "fused"):
        if method == "fused":
            monkeypatch.setattr(A, "choose_fusion", every_gate_alone)
        q, leaves = _run(n, bsz, gates, method, "auto")
        q.checkpoint = checkpoint
        ev = tq.expval_joint_analytical_batch(q, paulis)
        ev.sum().backward()
        res[method] = (q.get_states_1d().detach().cpu().numpy(), ev.detach().cpu().numpy(),
                       [lf.grad.cpu().numpy() for lf in leaves])
        if method == "fused":
            from torchquantum_gb300 import program as P

            seg = q._tape[0]
            blocks = [op for op in seg.exec_ops if getattr(op, "members", None) is not None]
            assert all(op.tc and len(op.members) == 1 and len(op.wires) == 6 for op in blocks)
            assert sum(1 for op in seg.records if P.fusable(op)) == len(blocks) > 0
            if getattr(seg.exec_ops[0], "members", None) is not None:
                assert getattr(seg.exec_ops[0], "zero_input", False)
    assert np.abs(res["fused"][0] - O.run(n, bsz, gates)).max() < 1e-5
    assert np.abs(res["fused"][1] - res["plain"][1]).max() < 1e-5
    for gp, gf in zip(res["plain"][2], res["fused"][2]):
        assert np.abs(gf - gp).max() < 1e-5


def test_adjoint_image_and_cross_grad_kernels():
    """tqk_fused_prepare_adjoint(U) is byte-identical to tqk_fused_prepare(U^H), and
    tqk_fused_cross_grad adds M U (M from the real cross term) into a float64 cotangent
    within float32 accuracy."""
    from torchquantum_gb300 import _lib

    dev = torch.device("cuda")
    rng = np.random.default_rng(5)
    b = 3
    z = rng.normal(size=(b, 64, 64)) + 1j * rng.normal(size=(b, 64, 64))
    u = torch.tensor(np.linalg.qr(z)[0], dtype=torch.complex128, device=dev)
    wires = [3, 9, 0, 14, 7, 11]
    img_h = _lib.fused_prepare_adjoint(u, wires)
    ref_h = _lib.fused_prepare(u.conj().transpose(-1, -2).contiguous(), wires)
    assert torch.equal(img_h, ref_h)
    mr = torch.tensor(rng.normal(size=(b, 128, 128)), dtype=torch.float64, device=dev)
    gu = torch.tensor(rng.normal(size=(b, 64, 64)) + 1j * rng.normal(size=(b, 64, 64)), dtype=torch.complex128,
                      device=dev)
    want = gu + torch.matmul(_lib.cross_to_complex(mr), u)
    _lib.fused_cross_grad(mr, u, torch.view_as_real(gu))
    assert (gu - want).abs().max().item() < 1e-4 * want.abs().max().item()


def test_batched_image_and_cross_add_kernels():
    """tqk_fused_prepare_many builds the same bytes as one tqk_fused_prepare /
    tqk_fused_prepare_adjoint call per block (blocks of different batch and wires in one
    launch), and tqk_fused_cross_add_many adds each cross term into its own cotangent as
    tqk_fused_cross_grad(mr, NULL) does."""
    from torchquantum_gb300 import _lib
    from torchquantum_gb300.program import _to_device_table

    dev = torch.device("cuda")
    rng = np.random.default_rng(9)
    specs = [(3, [3, 9, 0, 14, 7, 11]), (1, [0, 1, 2, 3, 4, 5]), (2, [13, 2, 8, 5, 10, 1])]
    jobs, want, got = [], [], []
    for b, wires in specs:
        z = rng.normal(size=(b, 64, 64)) + 1j * rng.normal(size=(b, 64, 64))
        u = torch.tensor(np.linalg.qr(z)[0], dtype=torch.complex128, device=dev)
        for adj in (0, 1):
            img = torch.zeros(_lib.load().tqk_fused_image_bytes(b), dtype=torch.uint8, device=dev)
            j = _lib.ImageJob()
            j.u, j.image, j.u_batch, j.adjoint = u.data_ptr(), img.data_ptr(), b, adj
            for i, w in enumerate(wires):
                j.wires[i] = w
            jobs.append(j)
            got.append((img, u))
            want.append(_lib.fused_prepare_adjoint(u, wires) if adj else _lib.fused_prepare(u, wires))
    table, host = _to_device_table(jobs, dev)
    _lib.fused_prepare_many(table, len(jobs), 3)
    torch.cuda.synchronize()
    for (img, _), ref in zip(got, want):
        assert torch.equal(img, ref)
    cjobs, outs = [], []
    for b, _ in specs:
        mr = torch.tensor(rng.normal(size=(b, 128, 128)), dtype=torch.float64, device=dev)
        gu = torch.tensor(rng.normal(size=(b, 64, 64)) + 1j * rng.normal(size=(b, 64, 64)), dtype=torch.complex128,
                          device=dev)
        ref = gu.clone()
        _lib.fused_cross_grad(mr, None, torch.view_as_real(ref))
        j = _lib.CrossJob()
        j.mr, j.gu, j.batch = mr.data_ptr(), gu.data_ptr(), b
        cjobs.append(j)
        outs.append((gu, ref, mr))
    ctable, chost = _to_device_table(cjobs, dev)
    _lib.fused_cross_add_many(ctable, len(cjobs), 3)
    torch.cuda.synchronize()
    for gu, ref, _ in outs:
        assert torch.equal(gu, ref)
