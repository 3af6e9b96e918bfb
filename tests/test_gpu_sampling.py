"""Measurement family on the GPU against the oracle.

* ``measure`` (upstream measurement/measurements.py:37-74): the device inverse-CDF
  sampler returns, for the same uniforms, the same outcomes as the oracle's float64
  CDF search; the dicts have upstream's format (every bitstring, qubit 0 first, sorted);
  counts follow |psi|^2 (chi-square) at n = 10 and wide states (n = 22) keep only observed
  outcomes.
* ``MeasureMultipleTimes`` / ``MeasureMultiPauliSum`` / ``MeasureMultiQubitPauliSum``
  (measurements.py:346-456): per-wire single-site expectation values per layer, as the
  oracle computes them, including a non-Pauli observable (Hadamard) on a copied state.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu


def _random_state_device(n, bsz, seed):
    import torchquantum_gb300 as tq
    from torchquantum_gb300 import workloads as W

    gates, ncols = W.random_circuit(n, 40, seed=seed)
    theta = W.random_params(bsz, ncols, seed=seed + 1)
    q = tq.QuantumDevice(n_wires=n, bsz=bsz, device="cuda")
    W.apply_circuit(q, gates, torch.tensor(theta, device="cuda"))
    return q, O.run(n, bsz, W.oracle_gates(gates, theta))


@pytest.mark.parametrize("n,bsz", [(3, 2), (10, 3), (13, 1)])
def test_sampler_matches_oracle_cdf(n, bsz):
    from torchquantum_gb300 import _lib

    q, ref = _random_state_device(n, bsz, seed=n)
    st = q.get_states_1d().detach().contiguous()
    g = torch.Generator(device="cuda").manual_seed(5)
    u = torch.rand(bsz, 4000, dtype=torch.float64, device="cuda", generator=g)
    idx = _lib.sample(st, n, u).cpu().numpy()
    p = np.abs(st.cpu().numpy().astype(np.complex128)) ** 2
    cdf = np.cumsum(p, axis=1)
    want = np.stack([np.searchsorted(cdf[b], u[b].cpu().numpy() * cdf[b, -1], side="right") for b in range(bsz)])
    assert (idx == np.minimum(want, (1 << n) - 1)).mean() > 0.999
    assert (idx >= 0).all() and (idx < (1 << n)).all()
    assert (p[np.arange(bsz)[:, None], idx] > 0).all()


def test_measure_format_and_statistics():
    import torchquantum_gb300 as tq

    n, bsz, shots = 10, 2, 200000
    q, ref = _random_state_device(n, bsz, seed=3)
    out = tq.measure(q, n_shots=shots, generator=torch.Generator(device="cuda").manual_seed(0))
    assert len(out) == bsz
    keys = tq.gen_bitstrings(n)
    for b in range(bsz):
        assert list(out[b].keys()) == keys and sum(out[b].values()) == shots
        cnt = np.array(list(out[b].values()), dtype=np.float64)
        p = np.abs(ref[b]) ** 2
        m = p * shots > 20
        chi2 = ((cnt[m] - shots * p[m]) ** 2 / (shots * p[m])).sum()
        dof = m.sum() - 1
        assert chi2 < dof + 6 * np.sqrt(2 * dof), (chi2, dof)


def test_measure_wide_state_keeps_observed_outcomes():
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    n = 22
    q = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda")
    tqf.hadamard(q, wires=0)
    tqf.cnot(q, wires=[0, n - 1])
    out = tq.measure(q, n_shots=5000)[0]
    assert set(out) <= {"0" * n, "1" + "0" * (n - 2) + "1"} and sum(out.values()) == 5000
    assert min(out.values()) > 2000


def test_measure_multiple_times_and_pauli_sums():
    import torchquantum_gb300 as tq

    n, bsz = 5, 3
    q, ref = _random_state_device(n, bsz, seed=11)
    layers = [{"wires": [0, 2, 3, 1], "observables": ["x", "y", "z", "i"], "coefficient": [1, 0.5, 0.4, 0.3]},
              {"wires": [4, 1], "observables": ["z", "x"], "coefficient": [1, 1]}]
    got = tq.MeasureMultipleTimes(layers)(q).detach().cpu().numpy()
    want = []
    for layer in layers:
        names = ["I"] * n
        for w, ob in zip(layer["wires"], layer["observables"]):
            names[w] = ob.upper()
        want.append(np.stack([O.expval_pauli(ref, "".join(names[w] if j == w else "I" for j in range(n)), n)
                              for w in range(n)], -1))
    want = np.concatenate(want)
    assert got.shape == (2 * bsz, n) and np.abs(got - want).max() < 1e-5
    s = tq.MeasureMultiPauliSum(layers)(q).detach().cpu().numpy()
    assert np.abs(s - want.sum(-1)).max() < 1e-5
    coef_layers = [{"coefficient": [0.5, 0.2, 0.1, 0.3, 0.7]}] + layers
    s2 = tq.MeasureMultiQubitPauliSum(coef_layers)(q).detach().cpu().numpy()
    assert np.abs(s2 - (want * np.array([0.5, 0.2, 0.1, 0.3, 0.7])).sum(-1)).max() < 1e-5
    # a non-Pauli observable is measured on a copy: the device state is unchanged
    before = q.get_states_1d().detach().clone()
    h = tq.MeasureMultipleTimes([{"wires": [2], "observables": ["hadamard"]}])(q).detach().cpu().numpy()
    assert torch.equal(before, q.get_states_1d().detach())
    hmat = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    hv = O.apply(ref, hmat[None].astype(np.complex128), [2], n)
    assert np.abs(h[:, 2] - np.real(np.sum(np.conj(ref) * hv, axis=1))).max() < 1e-5
