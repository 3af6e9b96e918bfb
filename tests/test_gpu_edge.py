"""Edge cases on the GPU: an empty circuit, one wire, the widest state a test can hold
(n = 30, 8 GiB), batch-size and width limits rejected by the host checks before any
launch, and a circuit whose parameters do not require gradients."""
import numpy as np
import pytest
import torch

from oracle import statevec as O

pytestmark = pytest.mark.gpu


def test_empty_circuit_and_single_wire():
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.QuantumDevice(n_wires=3, bsz=2, device="cuda")
    ev = tq.expval_joint_analytical(q, "ZZZ")
    assert torch.allclose(ev, torch.ones(2, device="cuda"))
    q1 = tq.QuantumDevice(n_wires=1, bsz=5, device="cuda")
    th = torch.rand(5, 3, device="cuda", requires_grad=True)
    for name in ("hadamard", "sx", "s", "t", "paulix", "pauliy"):
        tqf.func_name_dict[name](q1, wires=0)
    tqf.u3(q1, wires=0, params=th)
    tqf.rz(q1, wires=0, params=th[:, :1])
    e = tq.expval_joint_analytical(q1, "X")
    e.sum().backward()
    gates = [{"name": nm, "wires": [0], "params": None} for nm in ("hadamard", "sx", "s", "t", "paulix", "pauliy")]
    thn = th.detach().cpu().double().numpy()
    gates += [{"name": "u3", "wires": [0], "params": thn}, {"name": "rz", "wires": [0], "params": thn[:, :1]}]
    ref = O.run(1, 5, gates)
    assert np.abs(q1.get_states_1d().detach().cpu().numpy() - ref).max() < 1e-6
    assert np.abs(e.detach().cpu().numpy() - O.expval_pauli(ref, "X", 1)).max() < 1e-6
    assert th.grad is not None and torch.isfinite(th.grad).all()


def test_widest_state_n30():
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    n = 30
    q = tq.QuantumDevice(n_wires=n, bsz=1, device="cuda")
    tqf.hadamard(q, wires=0)
    tqf.cnot(q, wires=[0, n - 1])
    tqf.rx(q, wires=n // 2, params=torch.tensor([[0.5]], device="cuda"))
    zz = tq.expval_joint_analytical(q, "Z" + "I" * (n - 2) + "Z")
    z_mid = tq.expval_joint_analytical(q, "I" * (n // 2) + "Z" + "I" * (n - n // 2 - 1))
    assert abs(zz.item() - 1.0) < 1e-5 and abs(z_mid.item() - np.cos(0.5)) < 1e-5
    p = tq.probs(q)
    assert abs(p.sum().item() - 1.0) < 1e-4
    del q, p
    torch.cuda.empty_cache()


def test_host_checks_reject_before_launch():
    from torchquantum_gb300 import _lib

    buf = torch.zeros(1, 4, dtype=torch.complex64, device="cuda")
    mat = torch.eye(2, dtype=torch.complex64, device="cuda")[None]
    lib = _lib.load()
    w = _lib._i32([0])
    s = torch.cuda.current_stream().cuda_stream
    assert lib.tqk_apply_matrix(buf.data_ptr(), 1, 35, w, 1, mat.data_ptr(), 1, s) == 4  # TOO_MANY_QUBITS
    assert lib.tqk_apply_matrix(buf.data_ptr(), 70000, 2, w, 1, mat.data_ptr(), 1, s) == 2  # BAD_SHAPE
    assert lib.tqk_apply_matrix(buf.data_ptr() + 8, 1, 2, w, 1, mat.data_ptr(), 1, s) == 3  # misaligned
    assert lib.tqk_apply_matrix(buf.data_ptr(), 1, 2, _lib._i32([2]), 1, mat.data_ptr(), 1, s) == 1  # wire
    assert lib.tqk_apply_matrix(buf.data_ptr(), 1, 2, w, 1, mat.data_ptr(), 3, s) == 2  # operand batch
    torch.cuda.synchronize()
    assert torch.equal(buf, torch.zeros_like(buf))


def test_no_grad_parameters_and_no_grad_mode():
    import torchquantum_gb300 as tq
    import torchquantum_gb300.functional as tqf

    q = tq.QuantumDevice(n_wires=4, bsz=2, device="cuda")
    tqf.ry(q, wires=1, params=torch.tensor([[0.3], [0.4]], device="cuda"))
    tqf.cnot(q, wires=[1, 2])
    with torch.no_grad():
        ev = tq.expval_joint_analytical(q, "IZZI")
    assert not ev.requires_grad
    ref = O.run(4, 2, [{"name": "ry", "wires": [1], "params": np.array([[0.3], [0.4]])},
                       {"name": "cnot", "wires": [1, 2], "params": None}])
    assert np.abs(ev.cpu().numpy() - O.expval_pauli(ref, "IZZI", 4)).max() < 1e-6
