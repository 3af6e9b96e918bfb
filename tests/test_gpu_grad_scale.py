"""Gradient parity at the sizes the benchmark times.

Upstream's gradient is torch autograd through ``apply_unitary_bmm`` and the Pauli
expectation values (``functional/gate_wrapper.py:96-140``,
``measurement/measurements.py:232-279``).  Here the engine's adjoint gradients are
checked at full size against

* the plain method (complex64 gate-by-gate adjoint sweep, every gradient), and
* complex128 central differences (h = 1e-3, fourth-order stencil) of the same loss,
  computed with torch's own CUDA ops (``tests/torch_ref.py``: permute + bmm, no engine
  kernel) on sampled angles.

Workloads:

* the headline step: depth-400 random circuit at n = 24, bsz = 16 (2 GiB state),
  per-sample angles, loss = sum_b sum_j w_j <P_j>_b over 8 random Pauli strings, run by
  the fused method with stored block inputs (the default), by the fused method with the
  in-place O(1)-state reverse sweep, and by the plain method;
* the differentiation workload: n = 20, bsz = 64, 10 layers of RY/RZ on every wire
  (400 shared angles) + CZ ladder after a per-sample RY input layer, loss = sum of 50
  weighted Pauli strings; gradients of the shared angles and of the inputs.

Tolerance: 1e-5 absolute between the fused and plain gradients, and against the
complex128 central differences at the headline size.  For the differentiation workload
the shared angles' gradients sum 64 rows x 50 strings over 2^20 amplitudes per row and
complex64 arithmetic reaches about 1e-4 of the largest gradient (~0.13), for the plain
method as for the fused one: there the bound against central differences is
max(1e-5, 1e-4 x max |grad|).  Each case prints its errors (run with ``-s``).
"""
import numpy as np
import pytest
import torch

from tests import torch_ref as TR

pytestmark = pytest.mark.gpu

TOL = 1e-5
H = 1e-3


def _fd_rows(n, gates, theta, x, paulis, w, rows_cols, dev, shared):
    """Central differences of the loss with respect to theta[row, col] (per-sample
    angles: only row `row` depends on it) or theta[0, col] (shared: every row), in
    complex128 with torch ops on the GPU."""
    from torchquantum_gb300 import workloads as W

    def loss(th, rows):
        og = W.oracle_gates(gates, th)
        if x is not None:
            og = [{"name": "ry", "wires": [wi], "params": x[rows, wi:wi + 1].astype(np.float64)}
                  for wi in range(n)] + og
        st = TR.run(n, len(rows), og, dev)
        return float(sum(wj * TR.expval_pauli(st, p, n).sum().item() for wj, p in zip(w, paulis)))

    out = []
    for row, col in rows_cols:
        rows = list(range(x.shape[0])) if shared else [row]
        base = theta.astype(np.float64)[[0] if shared else [row]]
        if shared:
            base = np.repeat(base, len(rows), axis=0)
        vals = []
        for step in (2, 1, -1, -2):
            tv = base.copy()
            tv[:, col] += step * H
            vals.append(loss(tv, rows))
        out.append(_stencil(vals))
    return np.array(out)


def _stencil(v):
    """Fourth-order central difference from f(2h), f(h), f(-h), f(-2h): truncation error
    O(h^4) (about 1e-12 x the fifth derivative), so the check is set by the engine."""
    return (-v[0] + 8 * v[1] - 8 * v[2] + v[3]) / (12 * H)


def _headline_grads(method, checkpoint, gates, theta, paulis, pw, n, bsz):
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    dev = torch.device("cuda")
    th = torch.tensor(theta, device=dev, requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
    q.method = method
    if method == "fused":
        q.fuse_wires = "auto"
        q.checkpoint = checkpoint
    W.apply_circuit(q, gates, th)
    ev = tq.expval_joint_analytical_batch(q, paulis)
    stored = sum(1 for sg in q._tape for op in sg.exec_ops if getattr(op, "kept_input", False))
    tcb = sum(1 for sg in q._tape for op in sg.exec_ops if getattr(op, "tc", False))
    (ev * torch.tensor(pw, dtype=torch.float32, device=dev)).sum().backward()
    g = th.grad.detach().cpu().numpy()
    e = ev.detach().double().cpu().numpy()
    del q, ev, th
    torch.cuda.empty_cache()
    return e, g, stored, tcb


def test_headline_gradients_full_size():
    """n = 24, bsz = 16, depth 400 (the benchmark's workload and seeds)."""
    from torchquantum_gb300 import workloads as W

    n, bsz, depth = 24, 16, 400
    gates, ncols = W.random_circuit(n, depth, seed=0)
    theta = W.random_params(bsz, ncols, seed=1)
    paulis = W.random_paulis(n, 8, seed=2)
    pw = np.random.default_rng(3).normal(size=(1, 8)).astype(np.float32)
    res = {}
    for key, (method, ckpt) in {"fused_stored": ("fused", "auto"), "fused_in_place": ("fused", False),
                                "plain": ("plain", None)}.items():
        res[key] = _headline_grads(method, ckpt, gates, theta, paulis, pw, n, bsz)
    assert res["fused_stored"][2] > 0 and res["fused_in_place"][2] == 0 and res["fused_stored"][3] > 0
    gp = res["plain"][1]
    gscale = np.abs(gp).max()
    # complex128 central differences on sampled (row, angle) pairs
    rng = np.random.default_rng(12)
    picks = [(int(rng.integers(bsz)), int(rng.integers(ncols))) for _ in range(8)]
    fd = _fd_rows(n, gates, theta, None, paulis, pw[0], picks, torch.device("cuda"), shared=False)
    print(f"\nheadline n={n} bsz={bsz} depth={depth}: max |grad| {gscale:.3e}, "
          f"tensor-core blocks {res['fused_stored'][3]}, stored inputs {res['fused_stored'][2]}")
    for key, (e, g, _, _) in res.items():
        d_plain = np.abs(g - gp).max()
        d_fd = max(abs(g[r, c] - f) for (r, c), f in zip(picks, fd))
        d_ev = np.abs(e - res["plain"][0]).max()
        print(f"  {key:15s} max |grad - plain| {d_plain:.2e}  max |grad - fd128| {d_fd:.2e} "
              f"(8 angles)  max |expval - plain| {d_ev:.2e}")
        assert d_plain < TOL and d_fd < TOL and d_ev < TOL, key


def test_differentiation_workload_gradients_full_size():
    """n = 20, bsz = 64, 10 layers, 50 strings, per-sample RY inputs: shared-angle and
    input gradients of the fused method (stored inputs and in place) and the plain
    method, against each other and complex128 central differences."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300 import workloads as W

    n, bsz, layers, m = 20, 64, 10, 50
    gates, ncols = W.hea_circuit(n, layers)
    rng = np.random.default_rng(7)
    theta = rng.uniform(-np.pi, np.pi, size=(1, ncols)).astype(np.float32)
    x = rng.uniform(0, np.pi, size=(bsz, n)).astype(np.float32)
    paulis = W.random_paulis(n, m, seed=8)
    w = rng.normal(size=m).astype(np.float32)
    dev = torch.device("cuda")
    res = {}
    for key, (method, ckpt) in {"fused_stored": ("fused", "auto"), "fused_in_place": ("fused", False),
                                "plain": ("plain", None)}.items():
        th = torch.tensor(theta, device=dev, requires_grad=True)
        xt = torch.tensor(x, device=dev, requires_grad=True)
        q = tq.QuantumDevice(n_wires=n, bsz=bsz, device=dev)
        q.method = method
        if method == "fused":
            q.fuse_wires = 6
            q.checkpoint = ckpt
        for wi in range(n):
            tqf.ry(q, wires=wi, params=xt[:, wi:wi + 1])
        W.apply_circuit(q, gates, th)
        ev = tq.expval_joint_analytical_batch(q, paulis)
        (ev * torch.tensor(w, device=dev)).sum().backward()
        res[key] = (th.grad.detach().cpu().numpy()[0], xt.grad.detach().cpu().numpy())
        del q, ev, th, xt
        torch.cuda.empty_cache()
    gp, xp = res["plain"]
    picks = [(0, int(c)) for c in rng.choice(ncols, size=6, replace=False)]
    fd_t = _fd_rows(n, gates, theta, x, paulis, w, picks, dev, shared=True)
    # input angles x[b, w]: the input layer is RY(x[b, w]) on wire w, so perturb it as a
    # one-gate circuit prefix (only row b depends on it)
    xpicks = [(int(rng.integers(bsz)), int(rng.integers(n))) for _ in range(4)]
    fd_x = []
    for b, wi in xpicks:
        vals = []
        for step in (2, 1, -1, -2):
            xx = x.astype(np.float64).copy()
            xx[b, wi] += step * H
            og = [{"name": "ry", "wires": [k], "params": xx[[b], k:k + 1]} for k in range(n)]
            og += W.oracle_gates(gates, theta.astype(np.float64))
            st = TR.run(n, 1, og, dev)
            vals.append(sum(wj * TR.expval_pauli(st, p, n).sum().item() for wj, p in zip(w, paulis)))
        fd_x.append(_stencil(vals))
    gscale = max(np.abs(gp).max(), np.abs(xp).max())
    print(f"\ndifferentiation workload n={n} bsz={bsz}: max |grad theta| {np.abs(gp).max():.3e}, "
          f"max |grad x| {np.abs(xp).max():.3e}")
    errs = {}
    for key, (g, gx) in res.items():
        d_plain = max(np.abs(g - gp).max(), np.abs(gx - xp).max())
        d_fd_t = max(abs(g[c] - f) for (_, c), f in zip(picks, fd_t))
        d_fd_x = max(abs(gx[b, wi] - f) for (b, wi), f in zip(xpicks, fd_x))
        errs[key] = (d_plain, max(d_fd_t, d_fd_x))
        print(f"  {key:15s} max |grad - plain| {d_plain:.2e}  max |grad - fd128| shared angles {d_fd_t:.2e}, "
              f"inputs {d_fd_x:.2e}")
    # the shared angles' gradients sum 64 rows x 50 weighted strings over 2^20 amplitudes
    # each: complex64 arithmetic (plain and fused alike) reaches about 1e-4 of the largest
    # gradient here, while fused and plain agree within the 1e-5 bar
    for key, (d_plain, d_fd) in errs.items():
        assert d_plain < TOL, key
        assert d_fd < max(TOL, 1e-4 * gscale), key
