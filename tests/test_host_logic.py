"""Host-side logic that needs no GPU: Pauli masks, gate structure table, op construction."""
import numpy as np
import pytest
import torch

from oracle import statevec as O
from torchquantum_gb300 import gates as G
from torchquantum_gb300.measurement import pauli_masks


@pytest.mark.parametrize("obs", ["ZIII", "IXYZ", "YYYY", "XIZY", "IIII"])
def test_pauli_masks_match_oracle(obs):
    x, z, _ = O.pauli_masks(obs, 4)
    assert pauli_masks(obs, 4) == (x, z)


def test_every_upstream_gate_name_present():
    from tests.golden_data import load

    _, meta = load("gate_matrices")
    names = {m["name"] for m in meta.values()}
    for nm in names:
        assert G.canonical_name(nm) in G.GATES, nm


def test_structured_ops_are_consistent_with_matrix():
    """The block the engine reads for ctrl/phase/diag gates reproduces the full matrix."""
    for name, gd in G.GATES.items():
        if gd.num_wires <= 0 or name.startswith("qubitunitary"):
            continue
        p = torch.rand(2, gd.num_params, dtype=torch.float64) if gd.num_params > 0 else None
        m = G.gate_matrix(name, p, gd.num_wires, dtype=torch.complex128)
        d = m.shape[-1]
        kind = gd.struct[0]
        if kind == "ctrl":
            full = torch.eye(d, dtype=m.dtype).expand_as(m).clone()
            full[:, -2:, -2:] = m[:, -2:, -2:]
            assert torch.allclose(full, m), name
        elif kind == "phase":
            full = torch.eye(d, dtype=m.dtype).expand_as(m).clone()
            full[:, -1, -1] = m[:, -1, -1]
            assert torch.allclose(full, m), name
        elif kind == "diag":
            assert torch.allclose(torch.diag_embed(torch.diagonal(m, dim1=-2, dim2=-1)), m), name
        elif kind == "x":
            nc = gd.struct[1] if gd.struct[1] >= 0 else gd.num_wires - 1
            ref = O.gate_matrix(name, None, gd.num_wires)[0]
            assert np.allclose(m[0].numpy(), ref), name


def test_upstream_top_level_names():
    """Names user code reaches through ``import torchquantum as tq`` on this path."""
    import torchquantum_gb300 as tq

    for name in ["C_DTYPE", "F_DTYPE", "ABC", "ABC_ARRAY", "INV_SQRT2", "QuantumDevice", "NoiseDevice",
                 "QuantumModule", "QuantumModuleList", "static_support", "op_name_dict", "func_name_dict",
                 "mat_dict", "gate_wrapper", "apply_unitary_bmm", "rx", "cnot", "u3", "rx_matrix", "u3_matrix",
                 "GeneralEncoder", "PhaseEncoder", "MultiPhaseEncoder", "StateEncoder", "AmplitudeEncoder",
                 "Op1QAllLayer", "Op2QAllLayer", "TwoLocal", "EfficientSU2", "RandomLayer", "RandomLayerAllTypes",
                 "expval_joint_analytical", "expval_joint_sampling", "expval_joint_sampling_grouping",
                 "find_observable_groups", "expval", "measure", "gen_bitstrings", "MeasureAll",
                 "MeasureMultipleTimes", "MeasureMultiPauliSum", "MeasureMultiQubitPauliSum"]:
        assert hasattr(tq, name), name
    assert tq.RX is not tq.rx and tq.C_DTYPE == __import__("torch").complex64


def test_engine_defaults_roundtrip():
    import pytest

    import torchquantum_gb300 as tq
    from torchquantum_gb300 import device as D

    prev = tq.set_engine_defaults(method="fused", fuse_wires=5, fused_backend="tc", stage_low=False, checkpoint=False)
    try:
        assert D.ENGINE_DEFAULTS == {"method": "fused", "fuse_wires": 5, "fused_backend": "tc", "stage_low": False,
                                     "checkpoint": False}
        for bad in ({"method": "x"}, {"fuse_wires": 7}, {"fused_backend": "gpu"}, {"checkpoint": "yes"}):
            with pytest.raises(ValueError):
                tq.set_engine_defaults(**bad)
    finally:
        tq.set_engine_defaults(**prev)
    assert D.ENGINE_DEFAULTS == prev
