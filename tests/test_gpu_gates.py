"""Every gate kernel against the CPU oracle, on random states (GPU).

Tolerance: 1e-5 absolute per amplitude (complex64 arithmetic against the complex128
oracle), the bar the upstream test-suite uses for state comparisons.
"""
import zlib

import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu

ATOL = 1e-5


def _rand_state(rng, bsz, n):
    s = rng.normal(size=(bsz, 1 << n)) + 1j * rng.normal(size=(bsz, 1 << n))
    return s / np.linalg.norm(s, axis=1, keepdims=True)


def _gate_cases():
    from torchquantum_gb300 import gates as G

    cases = []
    for name, gd in sorted(G.GATES.items()):
        if name.startswith("qubitunitary"):
            continue
        if gd.num_wires == -1:
            for k in (1, 2, 3, 4):
                if name in ("multicnot", "multixcnot") and k < 2:
                    continue
                cases.append((name, k))
        else:
            cases.append((name, gd.num_wires))
    return cases


def _run_one(name, k, n, bsz, per_sample, inverse, rng, low_wires=False):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300 import gates as G

    gd = G.GATES[name]
    s0 = _rand_state(rng, bsz, n)
    wires = [int(w) for w in (rng.permutation(n)[:k] if not low_wires else list(range(n - k, n))[::-1])]
    params = None
    if gd.num_params > 0:
        b = bsz if per_sample else 1
        params = rng.uniform(-np.pi, np.pi, size=(b, gd.num_params))
    q = tq.QuantumDevice(n_wires=n, bsz=bsz)
    q.set_states(torch.tensor(s0, dtype=torch.complex64))
    kw = {}
    if gd.num_wires == -1:
        kw["n_wires"] = k
    p_t = None if params is None else torch.tensor(params, dtype=torch.float32, device="cuda")
    tqf.func_name_dict[name](q, wires=wires if k != 0 else [], params=p_t, inverse=inverse, **kw)
    got = q.get_states_1d().detach().cpu().numpy()
    m = O.gate_matrix(name, params, k, inverse)
    ref = O.apply(s0, m, wires, n) if k > 0 else s0 * m.reshape(-1, 1)
    return np.abs(got - ref).max()


@pytest.mark.parametrize("name,k", _gate_cases())
def test_gate_vs_oracle(name, k):
    rng = np.random.default_rng(zlib.crc32(name.encode()) + k)
    for n in sorted({max(k, 1), k + 1, 5, 9}):
        if n < k or (k == 0 and n < 1):
            continue
        for per_sample in (False, True):
            for inverse in (False, True):
                err = _run_one(name, k, n, 3, per_sample, inverse, rng)
                assert err < ATOL, f"{name} n={n} per_sample={per_sample} inverse={inverse}: {err}"


@pytest.mark.parametrize("name", ["u3", "cnot", "cz", "crx", "rzz", "swap", "cswap", "toffoli", "s", "qft"])
def test_gate_on_lowest_bits(name):
    """Targets on the least significant bits exercise the paired-float4 (MODE_LOW) paths."""
    from torchquantum_gb300 import gates as G

    rng = np.random.default_rng(7)
    k = G.GATES[name].num_wires if G.GATES[name].num_wires > 0 else 3
    for n in (k, k + 1, 7):
        err = _run_one(name, k, n, 2, True, False, rng, low_wires=True)
        assert err < ATOL, f"{name} n={n}: {err}"


def test_dense_wide_gates():
    """Generic dense kernel: qubitunitaryfast on 3..9 wires, per-sample and broadcast."""
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    rng = np.random.default_rng(3)
    n, bsz = 10, 2
    for k in (3, 5, 7, 9):
        for b in (1, bsz):
            us = np.stack([O.gate_matrix("qubitunitaryfast", _unitary(rng, 1 << k)[None])[0] for _ in range(b)])
            s0 = _rand_state(rng, bsz, n)
            wires = [int(w) for w in rng.permutation(n)[:k]]
            q = tq.QuantumDevice(n_wires=n, bsz=bsz)
            q.set_states(torch.tensor(s0, dtype=torch.complex64))
            tqf.qubitunitaryfast(q, wires=wires, params=torch.tensor(us, dtype=torch.complex64))
            got = q.get_states_1d().detach().cpu().numpy()
            ref = O.apply(s0, us, wires, n)
            assert np.abs(got - ref).max() < ATOL, (k, b)


def _unitary(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def test_bad_wires_raise():
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf
    from torchquantum_gb300._lib import TQKError

    q = tq.QuantumDevice(n_wires=3, bsz=1)
    with pytest.raises(TQKError, match="out of range"):
        tqf.hadamard(q, wires=5)
    with pytest.raises(TQKError, match="used twice"):
        tqf.cnot(q, wires=[1, 1])
    with pytest.raises(ValueError, match="does not match"):
        tqf.rx(q, wires=0, params=torch.zeros(2, 1, device="cuda"))
    # the device is still usable after the rejected calls
    tqf.hadamard(q, wires=0)
    assert abs(float(q.get_states_1d()[0, 0].real) - 2 ** -0.5) < 1e-6
