"""Density-matrix device (upstream device/noisedevices.py:36-105 and the density bmm of
functional/gate_wrapper.py:265-321, 434-440).

* CPU: the oracle's rho -> U rho U^H reproduces upstream's fixtures (tests/golden/
  density.npz) on circuits of symmetric gates; on a circuit with RY upstream's result
  is rho -> U rho conj(U) (its bra side skips the transpose), which the oracle
  reproduces with ``upstream_bmm=True`` and which is not a density matrix (negative
  diagonal entries).
* GPU: ``NoiseDevice`` matches upstream on the symmetric circuits, U rho U^H everywhere
  (including per-sample parameters, which upstream's density bmm cannot take), mixed
  initial states, probabilities and sampling, and its adjoint gradients match central
  differences.
"""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from tests.golden_data import load


def _cases():
    d, meta = load("density")
    for c in meta:
        gates = [dict(g, params=None if g["params"] is None else np.asarray(g["params"], np.float64))
                 for g in c["gates"]]
        yield c, gates, d[c["key"] + "__rho"]


CASES = list(_cases())


def test_oracle_density_matches_upstream():
    for c, gates, rho in CASES:
        mine = O.density_run(c["n"], c["bsz"], gates)
        up = O.density_run(c["n"], c["bsz"], gates, upstream_bmm=True)
        # upstream keeps its constant gate matrices (H, SX) in complex64 even in complex128
        # mode, so 1e-7 is the pin (as for the statevector fixtures)
        np.testing.assert_allclose(up, rho, atol=1e-7)
        if c["symmetric"]:
            np.testing.assert_allclose(mine, rho, atol=1e-7)
        else:
            assert np.abs(mine - rho).max() > 1e-3
            assert np.diagonal(rho, axis1=1, axis2=2).real.min() < -1e-3  # not positive semidefinite
            assert np.diagonal(mine, axis1=1, axis2=2).real.min() > -1e-12


def _run_device(n, bsz, gates, rho0=None, requires_grad=False):
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.NoiseDevice(n_wires=n, bsz=bsz, device="cuda")
    if rho0 is not None:
        q.set_densities(torch.tensor(rho0, dtype=torch.complex64, device="cuda"))
    leaves = []
    for g in gates:
        p = None
        if g["params"] is not None:
            p = torch.tensor(g["params"], dtype=torch.float32, device="cuda", requires_grad=requires_grad)
            leaves.append(p)
        tqf.func_name_dict[g["name"]](q, wires=g["wires"], params=p)
    return q, leaves


@pytest.mark.gpu
def test_noise_device_vs_upstream_and_oracle():
    for c, gates, rho in CASES:
        q, _ = _run_device(c["n"], c["bsz"], gates)
        got = q.get_densities_2d().detach().cpu().numpy()
        assert np.abs(got - O.density_run(c["n"], c["bsz"], gates)).max() < 1e-5
        if c["symmetric"]:
            assert np.abs(got - rho).max() < 1e-5
        assert q.densities.shape == (c["bsz"],) + (2,) * (2 * c["n"])


@pytest.mark.gpu
def test_noise_device_per_sample_mixed_probs_and_grad():
    import torchquantum_gb300 as tq

    rng = np.random.default_rng(3)
    n, bsz = 4, 3
    gates = []
    for _ in range(30):
        name = ["u3", "ry", "crx", "cnot", "cz", "rzz", "sx"][int(rng.integers(7))]
        k = {"crx": 2, "cnot": 2, "cz": 2, "rzz": 2}.get(name, 1)
        npar = {"u3": 3, "ry": 1, "crx": 1, "rzz": 1}.get(name, 0)
        p = rng.uniform(-np.pi, np.pi, size=(bsz, npar)) if npar else None
        gates.append({"name": name, "wires": [int(w) for w in rng.permutation(n)[:k]], "params": p})
    # a mixed initial state: random density matrices of rank 2
    v = rng.normal(size=(bsz, 16, 2)) + 1j * rng.normal(size=(bsz, 16, 2))
    rho0 = np.einsum("bik,bjk->bij", v, v.conj())
    rho0 /= np.trace(rho0, axis1=1, axis2=2)[:, None, None]
    q, leaves = _run_device(n, bsz, gates, rho0, requires_grad=True)
    ref = O.density_run(n, bsz, gates, rho0)
    got = q.get_densities_2d()
    assert np.abs(got.detach().cpu().numpy() - ref).max() < 1e-5
    probs = q.get_probs_1d()
    assert np.abs(probs.detach().cpu().numpy() - np.diagonal(ref, axis1=1, axis2=2)).max() < 1e-5
    # <Z_0> = Tr(rho Z_0) through the adjoint backward vs central differences
    z = torch.tensor([1.0 if (i >> (n - 1)) == 0 else -1.0 for i in range(16)], device="cuda")
    loss = (probs.real * z).sum()
    loss.backward()
    gi = next(i for i, g in enumerate(gates) if g["params"] is not None)
    g0 = leaves[0].grad.cpu().numpy()
    h = 1e-4
    for j in range(gates[gi]["params"].shape[1]):
        vals = []
        for sgn in (1, -1):
            gg = [dict(g) for g in gates]
            pp = gates[gi]["params"].copy()
            pp[0, j] += sgn * h
            gg[gi]["params"] = pp
            r = O.density_run(n, bsz, gg, rho0)
            vals.append((np.diagonal(r, axis1=1, axis2=2).real * z.cpu().numpy()).sum())
        assert abs(g0[0, j] - (vals[0] - vals[1]) / (2 * h)) < 1e-3
    # sampling draws from the diagonal
    out = tq.measure(q, n_shots=20000, generator=torch.Generator(device="cuda").manual_seed(1))
    emp = np.array(list(out[0].values())) / 20000
    assert np.abs(emp - np.diagonal(ref[0]).real).max() < 0.02
