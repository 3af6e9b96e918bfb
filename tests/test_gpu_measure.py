"""Measurement kernels against the oracle (GPU): multi-string Pauli expvals, their
backward, probabilities, per-wire expval/MeasureAll, reset; determinism."""
import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu


def _dev(n, bsz, rng):
    import torchquantum_gb300 as tq

    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.set_states(torch.tensor(s, dtype=torch.complex64))
    return q, s


@pytest.mark.parametrize("n", [1, 2, 3, 6, 12])
def test_pauli_expvals_vs_oracle(n):
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(n)
    q, s = _dev(n, 3, rng)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(20)]
    strings += ["Z" * n, "X" * n, "Y" * n, "I" * n]
    ev = tq.expval_joint_analytical_batch(q, strings).cpu().numpy()
    ref = np.stack([O.expval_pauli(s, p, n) for p in strings], -1)
    assert np.abs(ev - ref).max() < 1e-5


def test_expval_backward_is_two_g_p_psi():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(1)
    n, bsz = 8, 2
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    st = torch.tensor(s, dtype=torch.complex64, device="cuda", requires_grad=True)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.set_states(st)
    strings = ["XYZIXYZI", "ZZZZIIII", "IIIIIIIY"]
    w = rng.normal(size=(bsz, 3))
    ev = tq.expval_joint_analytical_batch(q, strings)
    (ev * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
    ref = sum(2 * w[:, j:j + 1] * O.apply_pauli(s, p, n) for j, p in enumerate(strings))
    assert np.abs(st.grad.cpu().numpy() - ref).max() < 1e-5


def test_expval_deterministic():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(2)
    q, _ = _dev(18, 2, rng)
    strings = ["".join(rng.choice(list("IXYZ"), size=18)) for _ in range(10)]
    a = tq.measurement.expval_joint_analytical_batch(q, strings)
    b = tq.measurement.expval_joint_analytical_batch(q, strings)
    assert torch.equal(a, b)


def test_probs_vs_oracle():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(3)
    q, s = _dev(10, 3, rng)
    p = tq.probs(q).cpu().numpy()
    assert np.abs(p - O.probs(s)).max() < 1e-6


def test_measure_all_and_expval_vs_oracle():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(4)
    n = 5
    for obs_cls, ch in ((tq.PauliZ, "Z"), (tq.PauliX, "X"), (tq.PauliY, "Y"), (tq.Hadamard, None)):
        q, s = _dev(n, 2, rng)
        got = tq.MeasureAll(obs_cls)(q).cpu().numpy()
        if ch is not None:
            ref = np.stack([O.expval_pauli(s, "".join(ch if w == j else "I" for w in range(n)), n)
                            for j in range(n)], -1)
        else:  # H = (X + Z) / sqrt(2)
            ref = np.stack([(O.expval_pauli(s, "".join("X" if w == j else "I" for w in range(n)), n)
                             + O.expval_pauli(s, "".join("Z" if w == j else "I" for w in range(n)), n))
                            / np.sqrt(2) for j in range(n)], -1)
        # MeasureAll rotates each wire in place; wires are measured on the rotated state
        # of all wires together, which is exact for single-wire observables.
        assert np.abs(got - ref).max() < 1e-5, obs_cls


def test_reset_vs_oracle():
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(5)
    n = 6
    q, s = _dev(n, 3, rng)
    tqf.reset(q, wires=[1, 4])
    ref = O.reset(s, [1, 4], n)
    assert np.abs(q.get_states_1d().cpu().numpy() - ref).max() < 1e-5


@pytest.mark.parametrize("n,bsz,m", [(6, 5, 3), (10, 3, 20), (14, 2, 17), (22, 2, 9), (24, 1, 9)])
def test_coset_expvals_vs_per_mask_passes(n, bsz, m):
    """Strings with several X-masks take the coset passes (partners staged in shared
    memory): against the oracle where it is cheap, and against the per-X-mask passes of
    the no-allocation entry point at every size, including diagonal strings, X-mask 1 and
    groups of 8 with a remainder."""
    import ctypes

    from torchquantum_gb300 import _lib
    from torchquantum_gb300.measurement import pauli_masks

    rng = np.random.default_rng(40 + n)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(m - 2)]
    strings += ["Z" * n, "I" * (n - 1) + "Y"]
    xs, zs = zip(*[pauli_masks(p, n) for p in strings])
    assert len(set(xs)) > 1 and _lib.expval_passes(list(xs), n) == len(_lib.coset_groups(list(xs), n))
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    st = torch.tensor(s, dtype=torch.complex64, device="cuda")
    got = _lib.pauli_expval(st, n, list(xs), list(zs))
    lib = _lib.load()
    per_mask = torch.full((bsz, m), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.tqk_pauli_expval_noalloc(st.data_ptr(), bsz, n, _lib._u64(list(xs)), _lib._u64(list(zs)), m,
                                      per_mask.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.tqk_last_error().decode()
    torch.cuda.synchronize()
    assert (got - per_mask).abs().max().item() < 2e-6
    if n <= 14:
        s64 = st.cpu().numpy().astype(np.complex128)
        want = np.stack([O.expval_pauli(s64, p, n) for p in strings], -1)
        assert np.abs(got.cpu().numpy() - want).max() < 1e-6
        assert np.abs(per_mask.cpu().numpy() - want).max() < 1e-6


@pytest.mark.parametrize("n,bsz,m", [(3, 2, 6), (13, 2, 12), (14, 3, 20), (16, 2, 30), (17, 1, 9)])
def test_coset_passes_vs_oracle(n, bsz, m):
    """Coset passes (strings with different X-masks: partners staged in shared memory,
    groups of <= 8 strings spanning <= 13 - c dimensions above c contiguous bits): the
    expvals and the backward seed sum_j c_j P_j psi against the oracle, including a
    diagonal string, X-mask 1, strings whose masks share the top bits, and several groups."""
    from torchquantum_gb300 import _lib
    from torchquantum_gb300.measurement import pauli_masks

    rng = np.random.default_rng(70 + n)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(m - 3)]
    strings += ["Z" * n, "I" * (n - 1) + "X", "X" + "I" * (n - 1)]
    xs, zs = zip(*[pauli_masks(p, n) for p in strings])
    groups = _lib.coset_groups(list(xs), n)
    assert sum(len(g) for g, _, _ in groups) == m
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    st = torch.tensor(s, dtype=torch.complex64, device="cuda")
    got = _lib.pauli_expval(st, n, list(xs), list(zs)).cpu().numpy()
    s64 = st.cpu().numpy().astype(np.complex128)
    want = np.stack([O.expval_pauli(s64, p, n) for p in strings], -1)
    assert np.abs(got - want).max() < 1e-6
    coef = rng.normal(size=(bsz, m)).astype(np.float32)
    seed = _lib.pauli_apply_sum(st, n, list(xs), list(zs), torch.tensor(coef, device="cuda")).cpu().numpy()
    want_seed = sum(coef[:, j:j + 1].astype(np.float64) * O.apply_pauli(s64, p, n) for j, p in enumerate(strings))
    assert np.abs(seed - want_seed).max() < 1e-5
    _lib.check_status(st.device)


def test_coset_pass_at_bench_size_matches_per_mask_passes():
    """n = 24, bsz = 4: 8 random strings in one coset pass against the per-X-mask passes
    of the no-allocation entry point (each string's partner stream read from HBM)."""
    from torchquantum_gb300 import _lib
    from torchquantum_gb300.measurement import pauli_masks

    n, bsz = 24, 4
    rng = np.random.default_rng(24)
    strings = ["".join(rng.choice(list("IXYZ"), size=n)) for _ in range(8)]
    xs, zs = zip(*[pauli_masks(p, n) for p in strings])
    assert _lib.expval_passes(list(xs), n) == 1
    g = torch.Generator(device="cuda").manual_seed(5)
    st = torch.randn(bsz, 1 << n, dtype=torch.complex64, device="cuda", generator=g)
    st /= st.abs().pow(2).sum(1, keepdim=True).sqrt()
    got = _lib.pauli_expval(st, n, list(xs), list(zs))
    lib = _lib.load()
    ref = torch.full((bsz, 8), float("nan"), dtype=torch.float64, device="cuda")
    rc = lib.tqk_pauli_expval_noalloc(st.data_ptr(), bsz, n, _lib._u64(list(xs)), _lib._u64(list(zs)), 8,
                                      ref.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.tqk_last_error().decode()
    torch.cuda.synchronize()
    assert (got - ref).abs().max().item() < 2e-6
    _lib.check_status(st.device)
