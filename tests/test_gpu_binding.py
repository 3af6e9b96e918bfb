"""The drop-in ``apply_unitary_bmm`` functions, on the GPU.

* ``torchquantum_gb300.functional.apply_unitary_bmm`` (the package's drop-in) and
  ``torchquantum_gb300.binding.apply_unitary_bmm`` (the ctypes binding a maintainer adds
  to upstream) against upstream's own algorithm (``gate_wrapper.py:96-140``: permute,
  ``bmm``, permute back) in complex128 torch with torch autograd: outputs and the
  gradients with respect to the state and the matrix, for a shared and a per-row matrix,
  plus central differences of the loss in float64 on the CPU oracle.
* Upstream itself (imported from the offline install in ``baseline/_ref``) with the
  binding assigned to ``torchquantum.functional.gate_wrapper.apply_unitary_bmm`` (the
  lookup at ``gate_wrapper.py:446``): the 4-wire encoder / U3 / CNOT model and the nine
  random circuits, forward and backward, against the fixtures upstream produced on its
  own (complex128), within 1e-5.  Skipped when upstream is not installed.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from oracle import upstream as U
from tests.golden_data import circuit_cases, load

pytestmark = pytest.mark.gpu


def _upstream_bmm(state, mat, wires):
    """Upstream's algorithm with torch ops (permute the wires to the front, bmm, back)."""
    n = state.dim() - 1
    dims = [w + 1 for w in wires]
    perm = list(range(state.dim()))
    for d in sorted(dims, reverse=True):
        del perm[d]
    perm = perm[:1] + dims + perm[1:]
    back = list(np.argsort(perm))
    shape = state.shape
    x = state.permute(perm).reshape(shape[0], mat.shape[-1], -1)
    m = mat if mat.dim() == 3 else mat.expand(shape[0], *mat.shape)
    return m.bmm(x).view(shape).permute(back)


def _case(rng, n, bsz, k, per_row):
    d = 1 << k
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    m = rng.normal(size=(bsz if per_row else 1, d, d)) + 1j * rng.normal(size=(bsz if per_row else 1, d, d))
    if not per_row:
        m = m[0]
    wts = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    wires = [int(w) for w in rng.permutation(n)[:k]]
    return s, m, wts, wires


def _loss_grads(fn, s, m, wts, wires, n, dtype, device):
    st = torch.tensor(s, dtype=dtype, device=device).view([s.shape[0]] + [2] * n).requires_grad_(True)
    mt = torch.tensor(m, dtype=dtype, device=device, requires_grad=True)
    out = fn(st, mt, wires)
    w = torch.tensor(wts, dtype=dtype, device=device).view(out.shape)
    loss = (out * w).real.sum() + (out.abs() ** 2).sum() * 0.25
    loss.backward()
    return (out.detach().reshape(s.shape[0], -1).cpu().numpy(), st.grad.reshape(s.shape[0], -1).cpu().numpy(),
            mt.grad.cpu().numpy(), float(loss.item()))


@pytest.mark.parametrize("which", ["package", "binding"])
@pytest.mark.parametrize("n,bsz,k,per_row", [(5, 3, 1, False), (6, 2, 2, True), (7, 4, 3, False), (9, 2, 2, True)])
def test_apply_unitary_bmm_grads(which, n, bsz, k, per_row):
    if which == "package":
        from torchquantum_gb300.functional import apply_unitary_bmm as fn
    else:
        from torchquantum_gb300.binding import apply_unitary_bmm as fn
    rng = np.random.default_rng(100 * n + k)
    s, m, wts, wires = _case(rng, n, bsz, k, per_row)
    out, gs, gm, _ = _loss_grads(fn, s, m, wts, wires, n, torch.complex64, "cuda")
    out_r, gs_r, gm_r, _ = _loss_grads(_upstream_bmm, s, m, wts, wires, n, torch.complex128, "cpu")
    scale = max(1.0, np.abs(out_r).max())
    assert np.abs(out - out_r).max() < 1e-5 * scale
    assert np.abs(gs - gs_r).max() < 1e-5 * max(1.0, np.abs(gs_r).max())
    assert np.abs(gm - gm_r).max() < 1e-5 * max(1.0, np.abs(gm_r).max())
    # central differences of the loss (float64 oracle) along a few matrix and state entries
    def f(sv, mv):
        st = sv.reshape([bsz] + [2] * n)
        o = _upstream_bmm(torch.tensor(st), torch.tensor(mv), wires).reshape(bsz, -1).numpy()
        return float((o * wts).real.sum() + (np.abs(o) ** 2).sum() * 0.25)

    h = 1e-6
    for _ in range(3):
        idx = tuple(int(rng.integers(x)) for x in np.shape(m))
        for unit in (1.0, 1j):
            mp, mm = np.array(m, dtype=np.complex128), np.array(m, dtype=np.complex128)
            mp[idx] += h * unit
            mm[idx] -= h * unit
            fd = (f(s, mp) - f(s, mm)) / (2 * h)
            # torch's complex gradient g = dL/dRe + i dL/dIm
            got = gm[idx].real if unit == 1.0 else gm[idx].imag
            assert abs(got - fd) < 1e-4 * max(1.0, abs(fd)), (idx, unit, got, fd)
    for _ in range(3):
        idx = (int(rng.integers(bsz)), int(rng.integers(1 << n)))
        sp, sm = s.copy(), s.copy()
        sp[idx] += h
        sm[idx] -= h
        fd = (f(sp, m) - f(sm, m)) / (2 * h)
        assert abs(gs[idx].real - fd) < 1e-4 * max(1.0, abs(fd)), (idx, gs[idx], fd)


def test_binding_does_not_write_its_input():
    from torchquantum_gb300.binding import apply_unitary_bmm

    rng = np.random.default_rng(1)
    s = torch.tensor(rng.normal(size=(2, 64)) + 1j * rng.normal(size=(2, 64)), dtype=torch.complex64,
                     device="cuda").view(2, 2, 2, 2, 2, 2, 2)
    keep = s.clone()
    u = torch.tensor(np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0], dtype=torch.complex64,
                     device="cuda")
    out = apply_unitary_bmm(s, u, [1, 4])
    torch.cuda.synchronize()
    assert torch.equal(s, keep) and out.data_ptr() != s.data_ptr()


def _upstream():
    if not U.available():
        pytest.skip("upstream torchquantum is not installed (baseline/_ref)")
    return U.import_upstream()


@pytest.fixture
def upstream_with_binding():
    """Upstream with every gate routed through the binding (restored afterwards)."""
    import importlib

    from torchquantum_gb300 import binding

    tq = _upstream()
    U.set_precision(False)
    gw = importlib.import_module("torchquantum.functional.gate_wrapper")
    saved = gw.apply_unitary_bmm
    binding.install(tq)
    try:
        yield tq
    finally:
        gw.apply_unitary_bmm = saved


def test_upstream_config1_through_binding(upstream_with_binding):
    tq = upstream_with_binding
    from torchquantum.measurement import expval_joint_analytical

    d, _ = load("config1")
    n, bsz = 4, 32
    funcs = ["rx", "ry", "rz", "rx"]
    enc = tq.GeneralEncoder([{"input_idx": [4 * g + w], "func": funcs[g], "wires": [w]} for g in range(4)
                             for w in range(4)])
    layers = []
    for layer in range(2):
        l1 = tq.layer.Op1QAllLayer(op=tq.U3, n_wires=n, has_params=True, trainable=True)
        for wi in range(n):
            l1.ops_all[wi].params.data = torch.tensor(d["u3_params"][layer, wi][None, :], dtype=torch.float32)
        layers += [l1, tq.layer.Op2QAllLayer(op=tq.CNOT, n_wires=n, circular=True)]
    model = torch.nn.ModuleList([enc] + layers).cuda()
    x = torch.tensor(d["x"], dtype=torch.float32, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    enc(q, x)
    for lay in layers:
        lay(q)
    assert np.abs(q.get_states_1d().detach().cpu().numpy() - d["c128__state"]).max() < 1e-5
    obs = ["".join("Z" if i == j else "I" for i in range(n)) for j in range(n)]
    ev = torch.stack([expval_joint_analytical(q, o) for o in obs], dim=-1)
    assert np.abs(ev.detach().cpu().numpy() - d["c128__expval"]).max() < 1e-5
    (ev * torch.tensor(d["loss_weights"], dtype=torch.float32, device="cuda")).sum().backward()
    assert np.abs(x.grad.cpu().numpy() - d["c128__grad_x"]).max() < 1e-5
    gu3 = np.stack([np.stack([layers[2 * l].ops_all[w].params.grad.cpu().numpy()[0] for w in range(n)])
                    for l in range(2)])
    assert np.abs(gu3 - d["c128__grad_u3"]).max() < 1e-5
    del model


@pytest.mark.parametrize("case_idx", range(9))
def test_upstream_random_circuits_through_binding(upstream_with_binding, case_idx):
    """Every gate type upstream's gate wrapper dispatches (parameterised, fixed, inverse,
    variable width, a dense unitary) through the binding, forward and backward."""
    import importlib

    tq = upstream_with_binding
    import torchquantum.functional as tqf
    from torchquantum.measurement import expval_joint_analytical

    gw = importlib.import_module("torchquantum.functional.gate_wrapper")
    case, gates, arr = list(circuit_cases())[case_idx]
    n, bsz = case["n"], case["bsz"]
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    leaves = []
    for g in gates:
        name, params = g["name"], None
        if g["params"] is not None:
            # parameters stay on the host: several upstream builders (xx_min_yy.py:37, ...)
            # mix in host tensors and fail for CUDA parameters; upstream's apply_unitary_bmm
            # (gate_wrapper.py:113) and the binding move the built matrix to the state
            unitary = name == "qubitunitaryfast"
            params = torch.tensor(np.asarray(g["params"]), dtype=torch.complex64 if unitary else torch.float32,
                                  requires_grad=not unitary)
            leaves.append(params)
        gw.gate_wrapper(name=name, mat=tqf.mat_dict[name], method="bmm", q_device=q, wires=g["wires"],
                        params=params, n_wires=g.get("n_wires"), inverse=g["inverse"])
    assert np.abs(q.get_states_1d().detach().cpu().numpy() - arr["state"]).max() < 1e-5
    ev = torch.stack([expval_joint_analytical(q, p) for p in case["paulis"]], dim=-1)
    assert np.abs(ev.detach().cpu().numpy() - arr["expval"]).max() < 1e-5
    (ev * torch.tensor(arr["weights"], dtype=torch.float32, device="cuda")).sum().backward()
    checked = 0
    for i, lf in enumerate(leaves):
        ref = arr[f"grad{i}"]
        if np.isnan(ref).any() or not lf.requires_grad:
            continue  # upstream's builder left the graph (recorded as NaN), or a fixed unitary
        got = lf.grad
        assert got is not None, (i, gates[i]["name"] if i < len(gates) else None)
        assert np.abs(got.cpu().numpy() - ref.reshape(lf.shape)).max() < 1e-5, i
        checked += 1
    assert checked > 0
