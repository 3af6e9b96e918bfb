"""The product's gate-matrix library against the upstream builders (fixture: gate_matrices.npz)."""
import numpy as np
import torch

from tests.golden_data import load
from torchquantum_gb300 import gates as G


def test_product_gate_matrices_match_upstream():
    d, meta = load("gate_matrices")
    for key, m in meta.items():
        p = torch.tensor(d[key + "__params"]) if key + "__params" in d.files else None
        mine = G.gate_matrix(m["name"], p, m["n_wires"], dtype=torch.complex128).detach().numpy()
        ref = d[key + "__mat"]
        ref = ref[None] if ref.ndim == 2 else ref
        np.testing.assert_allclose(mine, ref, atol=1e-12, err_msg=key)


def test_float32_params_give_complex64():
    m = G.gate_matrix("u3", torch.zeros(2, 3), 1)
    assert m.dtype == torch.complex64 and m.shape == (2, 2, 2)
