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


def test_state_cursor_allocates_its_work_buffer_once():
    """engine.StateCursor: the saved final state and stored block inputs are only read; the
    reverse sweep's in-place steps use one work buffer per backward, made on first need."""
    from torchquantum_gb300 import engine

    final = torch.arange(8, dtype=torch.float32)
    cur = engine.StateCursor(final)
    assert cur.state is final and not cur.owned and cur.work is None
    w = cur.work_buffer()
    assert w is not final and w.shape == final.shape and cur.work_buffer() is w


def test_exec_records_follow_the_abi():
    """program._plain_record / _exec: the tqk_exec_op records the segment runner reads --
    controls first for the controlled kinds, operand / cotangent addresses, the kind codes
    of include/tqk.h, and the 16-wire limit of one op."""
    import re

    from torchquantum_gb300 import _lib, engine, program

    with open(_lib.HEADER) as f:
        hdr = f.read()
    for name in ("DENSE", "CTRL", "MCX", "PHASE", "DIAG", "SWAP", "STAGED", "BLOCK_TC", "BLOCK_DENSE"):
        code = int(re.search(rf"TQK_X_{name} = (\d+)", hdr).group(1))
        assert code == getattr(_lib, f"X_{name}")
    assert "} tqk_exec_op;             /* 184 bytes */" in hdr
    mat = torch.zeros(3, 2, 2, dtype=torch.complex64)
    op = engine.TapeOp(engine.KIND_CTRL, [4, 1, 6], controls=[4, 1], targets=[6], operand=mat)
    g = torch.zeros(24, dtype=torch.float64)
    r = program._plain_record(op, g)
    assert (r.kind, r.nw, r.nctrl, list(r.wires[:3]), r.batch) == (_lib.X_CTRL, 3, 2, [4, 1, 6], 3)
    assert r.operand == mat.data_ptr() and r.grad == g.data_ptr() and not r.uncompute
    x = program._plain_record(engine.TapeOp(engine.KIND_X, [0, 5], controls=[0], targets=[5], ctrl_val=0))
    assert (x.kind, x.nctrl, x.ctrl_val, list(x.wires[:2]), x.operand) == (_lib.X_MCX, 1, 0, [0, 5], None)
    sw = program._plain_record(engine.TapeOp(engine.KIND_SWAP, [2, 3, 7], controls=[2], targets=[3, 7]))
    assert (sw.kind, sw.nw, sw.nctrl, list(sw.wires[:3])) == (_lib.X_SWAP, 3, 1, [2, 3, 7])
    with pytest.raises(_lib.TQKError):
        program._exec(_lib.X_MCX, list(range(17)), nctrl=16)


def test_stored_inputs_move_to_the_autograd_node():
    """Segment.take_stored_inputs hands each kept input to the caller once and keeps a weak
    reference: a second node finds the input while the first holds it, and the input is
    gone once every holder has dropped it."""
    import gc
    import types

    from torchquantum_gb300 import program

    a, b = types.SimpleNamespace(stored_input=torch.zeros(4)), types.SimpleNamespace(stored_input=None)
    seg = types.SimpleNamespace(blocks=[a, b])
    first = program.Segment.take_stored_inputs(seg)
    assert [op for op, _ in first] == [a] and a.stored_input is None
    held = first[0][1]
    second = program.Segment.take_stored_inputs(seg)
    assert len(second) == 1 and second[0][1] is held
    del first, second, held
    gc.collect()
    assert a.stored_ref() is None and program.Segment.take_stored_inputs(seg) == []


def test_expval_pass_count_follows_the_coset_grouping():
    """_lib.expval_passes mirrors tqk_pauli_expval: one X-mask for every string -> one pass
    per 8 strings; several X-masks -> one coset pass per group, a group taking strings in
    order while it holds <= 8 and its X-masks above the lowest 4 bits span <= 9 dimensions
    (13 - 4; rows of n < 13 bits: everything fits one stage)."""
    from torchquantum_gb300 import _lib

    xs = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10]  # all below bit 4: rank 0 above the chunk
    assert _lib.expval_passes(xs, 20) == 2 and _lib.expval_passes(xs, 25) == 2
    assert _lib.expval_passes([0] * 9, 20) == 2  # one X-mask: grouped passes
    assert _lib.expval_passes([0, 0, 3], 26) == 1
    hi = [1 << (4 + k) for k in range(12)]  # independent above the chunk: 8 per group (<= 9 dims)
    assert [len(g) for g, _, _ in _lib.coset_groups(hi, 20)] == [8, 4]
    assert _lib.expval_passes(hi, 12) == 2  # n < 13: a whole row is one stage, 8 strings per pass
    for g, c, r in _lib.coset_groups(hi, 24):
        assert c + r == 13


def test_stored_input_policy(monkeypatch):
    """QuantumDevice._store_block_inputs: keep block inputs only with tensor-core blocks, grad
    mode on, something differentiable reaching the segment, and (for "auto") room in half
    of the memory still available; True / False force the choice."""
    import types

    from torchquantum_gb300 import device as D

    free = {"b": 100 << 30}
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda dev=None: (free["b"], 280 << 30))
    monkeypatch.setattr(torch.cuda, "memory_reserved", lambda dev=None: 10 << 30)
    monkeypatch.setattr(torch.cuda, "memory_allocated", lambda dev=None: 4 << 30)
    tc = types.SimpleNamespace(tc=True)
    seg = types.SimpleNamespace(blocks=[tc, tc], diff_inputs=["theta"], stored_bytes=lambda buf: 40 << 30)
    dev = types.SimpleNamespace(checkpoint="auto", _init=None, _tape=[], _buf=None, device="cuda:0")
    decide = lambda s=seg: D.QuantumDevice._store_block_inputs(dev, s)
    assert decide()                                  # 40 GiB <= (100 + 6) / 2
    free["b"] = 60 << 30
    assert not decide()                              # 40 GiB > (60 + 6) / 2
    dev.checkpoint = True
    assert decide()
    dev.checkpoint = False
    free["b"] = 200 << 30
    assert not decide()
    dev.checkpoint = "auto"
    with torch.no_grad():
        assert not decide()
    assert not decide(types.SimpleNamespace(blocks=[types.SimpleNamespace(tc=False)], diff_inputs=["t"],
                                            stored_bytes=lambda buf: 0))
    quiet = types.SimpleNamespace(blocks=[tc], diff_inputs=[], stored_bytes=lambda buf: 1)
    assert not decide(quiet)                         # nothing differentiable reaches it
    dev._tape = [types.SimpleNamespace(diff_inputs=["earlier"])]
    assert decide(quiet)                             # an earlier segment's inputs need its lam
